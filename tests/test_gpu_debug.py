"""The debug build (mhd-gpu_gb300/build.py --debug -> lib/libmhdgpu_debug.so):
every shared-memory, global and halo index of the kernels is checked where it
is formed (csrc/mhd_debug.cuh); an index outside its array is skipped and
recorded instead of accessed.

The cases of tests/debug_cases.py (the subroutines on odd and non-cubic
shapes and the register-blocked lengths, whole steps on both paths with
both row stagings, full and partial row tiles, a batched ensemble of uneven
boxes) run through the debug build in a child process with poisoned
(NaN-filled) scratch: no index may fall outside its array, and every output
must equal the release build's bit for bit.  The record itself is checked
with mhdgpu_debug_selftest, whose kernel checks an index without accessing
anything through it."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from util import bits_equal

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def debug_lib():
    sys.path.insert(0, os.path.join(REPO, "mhd-gpu_gb300"))
    import build
    return build.build(debug=True)   # a minute or two the first time, then only when sources change


def _child(debug_lib, code_or_args, timeout=900):
    env = dict(os.environ, MHDGPU_LIB=debug_lib)
    return subprocess.run([sys.executable, *code_or_args], env=env, capture_output=True, text=True,
                          timeout=timeout, cwd=REPO)


def test_debug_record_reports_a_failed_check(gpu, debug_lib):
    code = ("import sys, json; sys.path.insert(0, 'mhd-gpu_gb300'); import mhdgpu;"
            "ok_in = mhdgpu.debug_selftest(2, 3); ok_out = mhdgpu.debug_selftest(7, 3);"
            "print(json.dumps([mhdgpu.debug_build(), ok_in, ok_out, mhdgpu.debug_faults(), mhdgpu.debug_faults()]))")
    r = _child(debug_lib, ["-c", code])
    assert r.returncode == 0, r.stderr[-3000:]
    is_debug, ok_in, ok_out, first, again = json.loads(r.stdout.strip().splitlines()[-1])
    assert is_debug and ok_in and not ok_out
    assert first["count"] == 1 and first["kind"] == "index" and first["file"] == "debug.cu"
    assert first["index"] == 7 and first["extent"] == 3
    assert again == {"count": 0}   # the read clears the count
    # the release build has no checks
    assert not gpu.debug_build()
    assert gpu.debug_selftest(7, 3) and gpu.debug_faults() == {"count": 0}


def test_debug_build_every_kernel_in_bounds_and_bitwise(gpu, debug_lib, tmp_path):
    out = tmp_path / "debug_cases.npz"
    r = _child(debug_lib, [os.path.join(HERE, "debug_cases.py"), str(out), "--poison"])
    assert r.returncode == 0, r.stderr[-3000:]
    z = np.load(out)
    assert bool(z["debug"])
    faults = json.loads(str(z["faults"]))
    assert faults["count"] == 0, faults
    import debug_cases
    rel = debug_cases.run_cases()
    assert set(rel) <= set(z.files)
    bad = [k for k, v in rel.items() if not bits_equal(v, z[k])]
    assert not bad, bad
