"""The near-boundary windows of the faithful policy cover the float-float
error on GB300 (tests/window_probe.cu).

Each exactly rounded helper (total pressure, van Leer quotient, fast speed,
CFL speed; mhd-gpu_gb300/csrc/mhd_math.cuh) forms its value as r + d in
float-float and takes the C path's double expression only where r + d lies
within 2^-K of d of a float rounding boundary.  That is exact only if the
float-float value never lies further than the window from the double value:
the probe measures the largest distance on the GPU's own approximate
reciprocal and root over seeded random operands, and every window must be
at least twice that distance."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
SAMPLES = 1 << 26


def _nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    return None


def test_windows_cover_the_float_float_error(tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("no nvcc")
    exe = tmp_path / "window_probe"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-o", str(exe),
                    os.path.join(HERE, "window_probe.cu")], check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe), str(SAMPLES), "20261204"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    seen = {}
    for line in r.stdout.strip().splitlines():
        name, count, log2_dist, k = line.split()
        seen[name] = (int(count), float(log2_dist), int(k))
    assert set(seen) == {"pressure", "slope", "speed", "cfl"}, r.stdout
    print("largest float-float distance, log2 of half-ulps (window K):",
          {n: (d, k) for n, (_, d, k) in seen.items()})
    for name, (count, log2_dist, k) in seen.items():
        assert count > SAMPLES // 4, (name, count)
        # the window 2^-K (of d, about half an ulp near a boundary) at least
        # twice the largest distance in half-ulps
        assert log2_dist <= -(k + 1), (name, log2_dist, k)
