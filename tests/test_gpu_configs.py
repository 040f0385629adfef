"""Parity of the benchmarked configurations at their own sizes, through the C ABI.

  - config 2: the 128^3 diagonal Alfven wave, 200 steps at CFL 0.7, on the
    plain per-subroutine step and the transpose-free step, against the FP32
    oracle (the C path's own time loop, Heterogeneous_MHD/C/mhd.c:60-125):
    the faithful kernels reproduce the C path bit for bit, so the bar is
    bit equality (and, as the contract's floor, 1e-5 per field);
  - the same run against the FP64 oracle replaying the GPU run's dt sequence:
    the accuracy of the FP32 step on the wave fields, per field;
  - the benchmark's own ensemble (64 boxes, sizes along each axis from
    {32,48,64,96,128} by seed 0, 27.2 M cells): all boxes batched for five
    steps against the oracle run box by box.

The oracle runs on every host core; at these sizes each case takes tens of
seconds of CPU time.
"""
import os

import numpy as np
import pytest

from util import B_FIELDS, U_FIELDS, bits_equal, field_errors

pytestmark = pytest.mark.gpu
TOL = 1e-5
CFL = 0.7
# the benchmark's ensemble workload (bench.py ENSEMBLE)
ENSEMBLE = {"nbox": 64, "seed": 0, "sizes": (32, 48, 64, 96, 128), "amp_range": (1e-4, 1e-1)}


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _advance(gpu, u, b, dims, nsteps, path):
    import torch
    du, db = dev(u), dev(b)
    work = torch.empty(gpu.step_workspace_bytes(*dims, path), dtype=torch.uint8, device="cuda")
    clock = gpu.new_clock()
    log = torch.zeros(nsteps, dtype=torch.float32, device="cuda")
    gpu.advance(du, db, *dims, nsteps, CFL, gpu.MHD_CFL_C, 0.0, clock, log, work, path)
    return host(du), host(db), host(log), gpu.read_clock(clock)


@pytest.fixture(scope="module")
def config2(oracle_lib):
    """The FP32 oracle's run of config 2: (u0, b0, u, b, dts)."""
    import ics
    n = 128
    u0, b0 = ics.alfven_oblique(n)
    ru, rb = u0.copy(), b0.copy()
    oracle_lib.set_threads(os.cpu_count() or 1)
    try:
        steps, _t, dts = oracle_lib.oracle("f32").run(ru, rb, n, n, n, cfl_number=CFL, max_steps=200)
    finally:
        oracle_lib.set_threads(1)
    assert steps == 200
    return u0, b0, ru, rb, dts


@pytest.mark.parametrize("path", [0, 1])   # MHD_PATH_PLAIN, MHD_PATH_FUSED
def test_config2_128_200_steps_matches_oracle(gpu, config2, path):
    """128^3 diagonal wave, 200 steps: the GPU run's dt sequence and final state
    equal the FP32 oracle's bit for bit."""
    import ics
    n = 128
    u0, b0, ru, rb, rdts = config2
    gu, gb, dts, clk = _advance(gpu, u0, b0, (n, n, n), 200, path)
    assert clk.iter == 200 and clk.health == 0
    eu, eb = field_errors(gu, ru, 5), field_errors(gb, rb, 3)
    print("CONFIG2", path, dict(zip(U_FIELDS + B_FIELDS, eu + eb)))
    assert max(eu) < TOL and max(eb) < TOL, (eu, eb)
    assert bits_equal(dts, rdts)
    assert bits_equal(gu, ru) and bits_equal(gb, rb)
    assert ics.div_b(gb, n, n, n) < 2.0 * ics.div_b(rb, n, n, n) + 1e-6


def test_config2_128_200_steps_against_fp64(gpu, oracle_lib, config2):
    """The FP32 step's error per field against the FP64 oracle on the same dt
    sequence (128^3 diagonal wave, A = 1e-3, 200 steps).  The wave lives in the
    momentum and field components perpendicular to B0; errors are per-field
    max-norms relative to the field (vector fields: their largest component)."""
    n = 128
    u0, b0, ru, rb, rdts = config2
    gu, gb, dts, clk = _advance(gpu, u0, b0, (n, n, n), 200, gpu.MHD_PATH_FUSED)
    O64 = oracle_lib.oracle("f64")
    oracle_lib.set_threads(os.cpu_count() or 1)
    try:
        uu, bb = u0.astype(np.float64), b0.astype(np.float64)
        wu, wb = np.empty_like(uu), np.empty_like(bb)
        for dt in dts:
            O64.step(uu, bb, n, n, n, np.float64(dt), wu, wb)
    finally:
        oracle_lib.set_threads(1)
    err = dict(zip(U_FIELDS + B_FIELDS, field_errors(gu, uu, 5) + field_errors(gb, bb, 3)))
    print("CONFIG2_FP64", err)
    for f, e in err.items():
        assert e < FP64_BOUND[f], (f, err)


# Per-field bound of the FP32 step against the FP64 oracle at 128^3 after 200
# steps (set from the oracle's own FP32-vs-FP64 distance on this run, which the
# bit-exact GPU run shares).
FP64_BOUND = {f: TOL for f in U_FIELDS + B_FIELDS}


@pytest.fixture(scope="module")
def ensemble64():
    import ics
    return ics.ensemble(**ENSEMBLE)


def test_ensemble64_batched_matches_oracle(gpu, oracle_lib, ensemble64):
    """The benchmark's 64-box ensemble, batched, five steps: every box equals the
    oracle run on that box alone (its own CFL and dt sequence), bit for bit."""
    ens = ensemble64
    assert sum(int(np.prod(e["dims"])) for e in ens) == 27246592
    boxes = [(dev(e["u"]), dev(e["b"]), e["dims"]) for e in ens]
    bt = gpu.Batch(boxes, cfl_number=CFL, cfl_mode=gpu.MHD_CFL_C)
    bt.advance(5)
    clocks = bt.clocks()
    got = [(host(u), host(b)) for u, b, _ in boxes]
    bt.close()
    del boxes
    O = oracle_lib.oracle("f32")
    oracle_lib.set_threads(os.cpu_count() or 1)
    worst = 0.0
    mismatched = []
    try:
        for i, e in enumerate(ens):
            ru, rb = e["u"].copy(), e["b"].copy()
            steps, t, _dts = O.run(ru, rb, *e["dims"], cfl_number=CFL, max_steps=5)
            gu, gb = got[i]
            c = clocks[i]
            assert c.iter == 5 and np.float32(c.t) == t, (i, e["dims"])
            assert c.health & (gpu.MHD_HEALTH_NONFINITE | gpu.MHD_HEALTH_DENSITY | gpu.MHD_HEALTH_STALL) == 0
            errs = field_errors(gu, ru, 5) + field_errors(gb, rb, 3)
            worst = max(worst, max(errs))
            if not (bits_equal(gu, ru) and bits_equal(gb, rb)):
                mismatched.append((i, e["dims"], max(errs)))
    finally:
        oracle_lib.set_threads(1)
    print("ENSEMBLE64", {"worst_field_error": worst, "boxes_not_bit_equal": mismatched})
    assert worst < TOL
    assert not mismatched, mismatched


def test_copy_matrix_and_compat_copies_bit_exact(gpu, oracle_lib):
    """mhdgpu_copy_matrix (device) and the reference-named host entries
    copy_matrix and transpose12 (include/mhdgpu_compat.h) against the oracle
    (Heterogeneous_MHD/C/copy_matrix.c:9-38, transpose12.c:7-47), non-cubic."""
    import ctypes as C
    import torch
    import ics
    L = gpu.lib()
    O = oracle_lib.oracle("f32")
    nx, ny, nz = 12, 20, 28
    u, b = ics.random_state(nx, ny, nz, seed=31)
    du, db = dev(u), dev(b)
    ou = torch.full_like(du, float("nan"))
    ob = torch.full_like(db, float("nan"))
    P = C.c_void_p
    st = L.mhdgpu_copy_matrix(P(ou.data_ptr()), P(ob.data_ptr()), P(du.data_ptr()), P(db.data_ptr()),
                              nx, ny, nz, None)
    assert st == gpu.MHD_OK, L.mhdgpu_last_error()
    assert bits_equal(host(ou), u) and bits_equal(host(ob), b)

    def ip(x):
        return C.byref(C.c_int(x))

    def fp(a):
        return a.ctypes.data_as(C.c_void_p)

    # copy_matrix(u, b, nx, ny, nz, update_u, update_b): update <- u
    cu, cb = np.full_like(u, np.nan), np.full_like(b, np.nan)
    L.copy_matrix(fp(u), fp(b), ip(nx), ip(ny), ip(nz), fp(cu), fp(cb))
    assert L.mhdgpu_compat_status() == 0
    su, sb = np.full_like(u, np.nan), np.full_like(b, np.nan)
    O.copy_matrix(u.copy(), b.copy(), nx, ny, nz, su, sb)
    assert bits_equal(cu, su) and bits_equal(cb, sb) and bits_equal(cu, u)
    # transpose12(u, b, update_u, update_b, ...): u/b <- update, permuted
    tu, tb = np.full_like(u, np.nan), np.full_like(b, np.nan)
    L.transpose12(fp(tu), fp(tb), fp(u.copy()), fp(b.copy()), ip(nx), ip(ny), ip(nz), 0)
    assert L.mhdgpu_compat_status() == 0
    ru, rb = np.full_like(u, np.nan), np.full_like(b, np.nan)
    O.transpose12(ru, rb, u.copy(), b.copy(), nx, ny, nz)
    assert bits_equal(tu, ru) and bits_equal(tb, rb)
