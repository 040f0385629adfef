"""Precision studies on the GPU against the FP64 oracle, through the C ABI.

  - mhdgpu_diagnostics (FP64 totals, max |div B|, min p) against numpy in
    float64 on the same state;
  - the FP64 pressure-recovery policy (MHD_MATH_FP64P): bit-identical to the
    faithful policy where beta >= 0.1, and on the low-beta blast compared with
    the faithful FP32 run and the FP64 oracle on positivity, energy
    conservation and max |div B|;
  - the turbulent start: per-field error of the FP32 step against the FP64
    oracle fed the same dt sequence.

The FP64 oracle runs replay the GPU run's dt sequence (dt_log) so that the
comparison isolates the arithmetic precision from the CFL's rounding.
Studies marked `slow` run the full-size configurations and are skipped unless
MHDGPU_SLOW=1.
"""
import os

import numpy as np
import pytest

from util import U_FIELDS, B_FIELDS, bits_equal, field_errors

pytestmark = pytest.mark.gpu
SLOW = os.environ.get("MHDGPU_SLOW") == "1"


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def gas_pressure(u, b, nx, ny, nz):
    """p = (gamma-1)(E - m^2/2rho - Bc^2/2) in float64, Bc face -> centre."""
    g = float(np.float32(5.0 / 3.0))
    uu = np.asarray(u, dtype=np.float64).reshape(nz, ny, nx, 5)
    bb = np.asarray(b, dtype=np.float64).reshape(nz, ny, nx, 3)
    cx = 0.5 * (bb[..., 0] + np.roll(bb[..., 0], -1, axis=2))
    cy = 0.5 * (bb[..., 1] + np.roll(bb[..., 1], -1, axis=1))
    cz = 0.5 * (bb[..., 2] + np.roll(bb[..., 2], -1, axis=0))
    q = (uu[..., 1] ** 2 + uu[..., 2] ** 2 + uu[..., 3] ** 2) / uu[..., 0]
    return (g - 1.0) * (uu[..., 4] - 0.5 * q - 0.5 * (cx ** 2 + cy ** 2 + cz ** 2))


def gpu_run(gpu, u, b, dims, nsteps, cfl, math, path=1):
    """nsteps on the device under a math policy; returns (u, b, dt_log, clock,
    diagnostics before, diagnostics after)."""
    import torch
    prev = gpu.set_math(math)
    try:
        du, db = dev(u), dev(b)
        d0 = gpu.diagnostics(du, db, *dims)
        work = torch.empty(gpu.step_workspace_bytes(*dims, path), dtype=torch.uint8, device="cuda")
        clock = gpu.new_clock()
        log = torch.zeros(nsteps, dtype=torch.float32, device="cuda")
        gpu.advance(du, db, *dims, nsteps, cfl, 0, 0.0, clock, log, work, path)
        d1 = gpu.diagnostics(du, db, *dims)
        return host(du), host(db), host(log), gpu.read_clock(clock), d0, d1
    finally:
        gpu.set_math(prev)


def oracle64_replay(oracle_lib, u, b, dims, dts, threads=None):
    """The FP64 oracle from the same initial state with a given dt sequence."""
    O = oracle_lib.oracle("f64")
    if threads:
        oracle_lib.set_threads(threads)
    uu = np.asarray(u, dtype=np.float64).copy()
    bb = np.asarray(b, dtype=np.float64).copy()
    wu, wb = np.empty_like(uu), np.empty_like(bb)
    for dt in dts:
        O.step(uu, bb, *dims, np.float64(dt), wu, wb)
    return uu, bb


def test_diagnostics_match_numpy(gpu):
    import ics
    dims = (24, 16, 20)
    u, b = ics.random_state(*dims, seed=12, amp=0.3)
    d = gpu.diagnostics(dev(u), dev(b), *dims)
    uu = np.asarray(u, dtype=np.float64).reshape(-1, 5)
    for i, k in enumerate(("mass", "m_x", "m_y", "m_z", "energy")):
        ref = uu[:, i].sum()
        assert abs(d[k] - ref) <= 1e-12 * max(1.0, np.abs(uu[:, i]).sum()), k
    assert d["max_div_b"] == pytest.approx(ics.div_b(b, *dims), rel=1e-12)
    p = gas_pressure(u, b, *dims)
    assert d["min_p"] == pytest.approx(p.min(), rel=1e-12)
    assert d["cells_p_nonpositive"] == float((p <= 0).sum())
    d2 = gpu.diagnostics(dev(u), dev(b), *dims)
    assert d2 == d          # fixed reduction order: repeatable bit for bit


def test_fp64_pressure_equals_faithful_at_high_beta(gpu):
    """Where beta >= 0.1 the FP64 recovery is not taken: same bits."""
    import ics
    dims = (32, 16, 24)
    u, b = ics.turbulence(*dims, seed=4, mach=0.3, b_mean=0.3, db_rms=0.3)
    bb = np.asarray(b, dtype=np.float64).reshape(dims[2], dims[1], dims[0], 3)
    bc2 = sum((0.5 * (bb[..., a] + np.roll(bb[..., a], -1, axis=2 - a))) ** 2 for a in range(3))
    assert (2 * gas_pressure(u, b, *dims) / bc2).min() > 0.5   # beta far above 0.1
    a = gpu_run(gpu, u, b, dims, 3, 0.7, gpu.MHD_MATH_FAITHFUL)
    c = gpu_run(gpu, u, b, dims, 3, 0.7, gpu.MHD_MATH_FP64P)
    assert bits_equal(a[0], c[0]) and bits_equal(a[1], c[1])


def _blast_study(gpu, oracle_lib, n, nsteps, threads=None):
    import ics
    dims = (n, n, n)
    u, b = ics.blast(n)
    res = {}
    for name, math in (("fp32", gpu.MHD_MATH_FAITHFUL), ("fp64_pressure", gpu.MHD_MATH_FP64P)):
        gu, gb, dts, clk, d0, d1 = gpu_run(gpu, u, b, dims, nsteps, 0.7, math)
        ru, rb = oracle64_replay(oracle_lib, u, b, dims, dts, threads)
        p, p64 = gas_pressure(gu, gb, *dims), gas_pressure(ru, rb, *dims)
        res[name] = {
            "health": clk.health, "min_p": d1["min_p"], "cells_p_nonpositive": d1["cells_p_nonpositive"],
            "energy_drift": abs(d1["energy"] - d0["energy"]) / abs(d0["energy"]),
            "max_div_b": d1["max_div_b"], "oracle64_min_p": float(p64.min()),
            "p_err_vs_fp64_over_p_out": float(np.abs(p - p64).max() / 0.1),
            "field_err_vs_fp64": dict(zip(U_FIELDS + B_FIELDS,
                                          field_errors(gu, ru, 5) + field_errors(gb, rb, 3))),
        }
    return res


def test_lowbeta_blast_fp64_pressure_small(gpu, oracle_lib):
    """32^3 blast (beta = 0.002 outside), 20 steps: both policies stay finite
    with rho > 0 and conserve energy to round-off; the FP64 recovery's gas
    pressure is at least as close to the FP64 oracle's as the FP32 one."""
    res = _blast_study(gpu, oracle_lib, 32, 20)
    print(res)
    for name, r in res.items():
        assert r["health"] & (gpu.MHD_HEALTH_NONFINITE | gpu.MHD_HEALTH_DENSITY) == 0, name
        assert r["energy_drift"] < 1e-6, name
        assert r["max_div_b"] < 1e-4, name
    assert res["fp64_pressure"]["p_err_vs_fp64_over_p_out"] <= res["fp32"]["p_err_vs_fp64_over_p_out"] * 1.05


@pytest.mark.slow
@pytest.mark.skipif(not SLOW, reason="full-size study: set MHDGPU_SLOW=1")
def test_lowbeta_blast_study_128(gpu, oracle_lib):
    res = _blast_study(gpu, oracle_lib, 128, 300, threads=os.cpu_count())
    print("LOWBETA_STUDY", res)
    for r in res.values():
        assert r["health"] & (gpu.MHD_HEALTH_NONFINITE | gpu.MHD_HEALTH_DENSITY) == 0


@pytest.mark.slow
@pytest.mark.skipif(not SLOW, reason="full-size study: set MHDGPU_SLOW=1")
def test_lowbeta_blast_study_256(gpu, oracle_lib):
    """Config 5 at its full size (256^3, 300 steps); the FP64 oracle replays
    each run's dt sequence on the host cores (about 5e9 FP64 cell-updates)."""
    res = _blast_study(gpu, oracle_lib, 256, 300, threads=os.cpu_count())
    print("LOWBETA_STUDY_256", res)
    for r in res.values():
        assert r["health"] & (gpu.MHD_HEALTH_NONFINITE | gpu.MHD_HEALTH_DENSITY) == 0


def _turbulence_study(gpu, oracle_lib, n, nsteps, threads=None):
    import ics
    dims = (n, n, n)
    u, b = ics.turbulence(n, seed=7, mach=0.5, b_mean=0.3)
    out = {}
    for name, math in (("faithful", gpu.MHD_MATH_FAITHFUL), ("fast", gpu.MHD_MATH_FAST)):
        gu, gb, dts, clk, d0, d1 = gpu_run(gpu, u, b, dims, nsteps, 0.7, math)
        ru, rb = oracle64_replay(oracle_lib, u, b, dims, dts, threads)
        out[name] = dict(zip(U_FIELDS + B_FIELDS, field_errors(gu, ru, 5) + field_errors(gb, rb, 3)))
        out[name]["energy_drift"] = abs(d1["energy"] - d0["energy"]) / abs(d0["energy"])
        out[name]["max_div_b"] = d1["max_div_b"]
    return out


def test_turbulence_fp32_vs_fp64_small(gpu, oracle_lib):
    """48^3 turbulent start (k^-2 velocity at rms Mach 0.5, k^-3 potential,
    mean field 0.3), 10 steps: the FP32 step is within 1e-5 per field of the
    FP64 oracle on the same dt sequence."""
    out = _turbulence_study(gpu, oracle_lib, 48, 10)
    print(out)
    for f in U_FIELDS + B_FIELDS:
        assert out["faithful"][f] < 1e-5, (f, out["faithful"][f])


@pytest.mark.slow
@pytest.mark.skipif(not SLOW, reason="full-size study: set MHDGPU_SLOW=1")
def test_turbulence_precision_study_256(gpu, oracle_lib):
    out = _turbulence_study(gpu, oracle_lib, 256, 50, threads=os.cpu_count())
    print("TURBULENCE_STUDY", out)


def _alfven_vs_fp64(gpu, oracle_lib, n, nsteps, oblique, threads=None):
    import ics
    dims = (n, n, n)
    u, b = ics.alfven_oblique(n) if oblique else ics.alfven_x(n)
    gu, gb, dts, clk, d0, d1 = gpu_run(gpu, u, b, dims, nsteps, 0.7, gpu.MHD_MATH_FAITHFUL)
    ru, rb = oracle64_replay(oracle_lib, u, b, dims, dts, threads)
    # the wave's fields: m and b perpendicular to B0 carry the wave; the
    # vector floors measure them against the wave amplitude (util.field_errors)
    return dict(zip(U_FIELDS + B_FIELDS, field_errors(gu, ru, 5) + field_errors(gb, rb, 3)))


def test_alfven_x_32_fp32_vs_fp64(gpu, oracle_lib):
    """Config 1 (32^3 x-Alfven wave, A = 1e-3, CFL 0.7, 100 steps): the wave's
    fields (rho, m_y, E, b_y) stay within 1e-5 of the FP64 oracle on the same
    dt sequence.  m_x is second order in A (~1e-7 of the state) and sits at the
    FP32 noise floor: it is held to 1e-6 absolute (err x the wave's 1e-3)."""
    err = _alfven_vs_fp64(gpu, oracle_lib, 32, 100, oblique=False)
    print(err)
    for f in ("rho", "m_y", "m_z", "E", "b_x", "b_y", "b_z"):
        assert err[f] < 1e-5, (f, err)
    assert err["m_x"] * 1e-3 < 1e-6, err


@pytest.mark.slow
@pytest.mark.skipif(not SLOW, reason="full-size study: set MHDGPU_SLOW=1")
def test_alfven_diag_128_fp32_vs_fp64_study(gpu, oracle_lib):
    err = _alfven_vs_fp64(gpu, oracle_lib, 128, 200, oblique=True, threads=os.cpu_count())
    print("ALFVEN128_STUDY", err)
    assert all(np.isfinite(v) for v in err.values())


def restrict2(u, b, n):
    """2x2x2 restriction of an n^3 state to (n/2)^3 in float64: cell averages of
    u, and face averages of b (each coarse left face is the mean of the four
    fine faces it covers), which keeps the discrete div B of the fine field."""
    h = n // 2
    uu = np.asarray(u, dtype=np.float64).reshape(h, 2, h, 2, h, 2, 5).mean(axis=(1, 3, 5))
    bb = np.asarray(b, dtype=np.float64).reshape(h, 2, h, 2, h, 2, 3)
    bx = bb[:, :, :, :, :, 0, 0].mean(axis=(1, 3))     # fine x-face 2I, averaged over j, k pairs
    by = bb[:, :, :, 0, :, :, 1].mean(axis=(1, 4))     # fine y-face 2J, averaged over k, i pairs
    bz = bb[:, 0, :, :, :, :, 2].mean(axis=(2, 4))     # fine z-face 2K, averaged over j, i pairs
    return uu.reshape(-1), np.stack([bx, by, bz], axis=-1).reshape(-1)


@pytest.mark.slow
@pytest.mark.skipif(not SLOW, reason="full-size study: set MHDGPU_SLOW=1")
def test_turbulence_512_against_fp64_256_by_restriction(gpu, oracle_lib):
    """Config 3 as stated: the 512^3 turbulent start (k^-2 velocity at rms Mach
    0.5, k^-3 potential, mean field 0.3, rho = p = 1), 50 FP32 steps on the GPU,
    against an FP64 run of the same solver at 256^3 from the 2x2x2 restriction
    of the same initial state, run to the same physical time (the 256^3 grid's
    solver time is half the 512^3 one's: the solver counts time in cells).
    Per-field error of the restricted 512^3 FP32 state; beside it, the FP32 run
    at 256^3 against the same FP64 run (the same-resolution precision error),
    so the part of the first that is resolution rather than precision shows."""
    import json
    import ics
    n, h = 512, 256
    u, b = ics.turbulence(n, seed=7, mach=0.5, b_mean=0.3)
    gu, gb, dts, clk, d0, d1 = gpu_run(gpu, u, b, (n, n, n), 50, 0.7, gpu.MHD_MATH_FAITHFUL,
                                       path=gpu.MHD_PATH_AUTO)
    t512 = float(clk.t)
    ru, rb = restrict2(gu, gb, n)
    cu, cb = restrict2(u, b, n)
    del u, b, gu, gb
    # FP64 oracle at 256^3 to t512 / 2 (its own CFL steps)
    O64 = oracle_lib.oracle("f64")
    oracle_lib.set_threads(os.cpu_count())
    uu, bb = cu.copy(), cb.copy()
    steps64, t64, _ = O64.run(uu, bb, h, h, h, cfl_number=0.7, tf=t512 / 2, max_steps=int(clk.iter))
    # FP32 GPU at 256^3 from the same restricted start, to the same time
    import torch
    du, db = dev(cu.astype(np.float32)), dev(cb.astype(np.float32))
    work = torch.empty(gpu.step_workspace_bytes(h, h, h, gpu.MHD_PATH_AUTO), dtype=torch.uint8, device="cuda")
    clock = gpu.new_clock()
    gpu.advance(du, db, h, h, h, int(clk.iter), 0.7, 0, float(np.float32(t512 / 2)), clock, None, work,
                gpu.MHD_PATH_AUTO)   # ~half the steps reach tf; the rest take dt = 0
    c256 = gpu.read_clock(clock)
    fu, fb = host(du), host(db)
    rec = {"t512": t512, "steps512": int(clk.iter), "t256_fp64": float(t64), "steps256_fp64": int(steps64),
           "t256_fp32": float(c256.t), "steps256_fp32": int(c256.iter),
           "fp32_512_restricted_vs_fp64_256": dict(zip(U_FIELDS + B_FIELDS,
                                                       field_errors(ru, uu, 5) + field_errors(rb, bb, 3))),
           "fp32_256_vs_fp64_256": dict(zip(U_FIELDS + B_FIELDS,
                                            field_errors(fu, uu, 5) + field_errors(fb, bb, 3))),
           "energy_drift_512": abs(d1["energy"] - d0["energy"]) / abs(d0["energy"]),
           "max_div_b_512": d1["max_div_b"], "health_512": int(clk.health)}
    print("CONFIG3_STUDY", json.dumps(rec))
    assert clk.health & (gpu.MHD_HEALTH_NONFINITE | gpu.MHD_HEALTH_DENSITY) == 0
    assert abs(c256.t / t64 - 1) < 1e-5


BLAST_RECORD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "blast256_f64.json")


@pytest.mark.skipif(not os.path.exists(BLAST_RECORD), reason="FP64 blast record not generated")
def test_lowbeta_blast_256_against_fp64_record(gpu):
    """Config 5 at its own size (256^3 low-beta blast, 300 steps at CFL 0.7)
    in FP32 and FP32 + FP64 pressure recovery on the GPU, against the
    diagnostics of the FP64 oracle's run of the same configuration
    (tests/golden/blast256_f64.json, made by gen_blast256_f64.py): both
    policies stay finite with rho > 0, conserve mass and energy to FP32
    round-off, keep div B at round-off of |B| = 10, and lose positivity in the
    same cells as FP64 does (the scheme's own loss: the count of cells with
    p <= 0 within 3% of the FP64 run's, the minimum within a factor of 1.5)."""
    import json
    import ics
    rec = json.load(open(BLAST_RECORD))
    n = rec["config"]["n"]
    u, b = ics.blast(n)
    out = {}
    for name, math in (("fp32", gpu.MHD_MATH_FAITHFUL), ("fp64_pressure", gpu.MHD_MATH_FP64P)):
        gu, gb, dts, clk, d0, d1 = gpu_run(gpu, u, b, (n, n, n), rec["config"]["steps"], rec["config"]["cfl"],
                                           math, path=gpu.MHD_PATH_AUTO)
        out[name] = {"health": int(clk.health), "t": float(clk.t), "min_p": d1["min_p"],
                     "cells_p_nonpositive": d1["cells_p_nonpositive"],
                     "energy_drift": abs(d1["energy"] - d0["energy"]) / abs(d0["energy"]),
                     "mass_drift": abs(d1["mass"] - d0["mass"]) / abs(d0["mass"]),
                     "max_div_b": d1["max_div_b"]}
    print("BLAST256", json.dumps({"gpu": out, "fp64_record": rec["final"], "fp64_t": rec["t_end"]}))
    ref = rec["final"]
    for name, r in out.items():
        assert r["health"] & (gpu.MHD_HEALTH_NONFINITE | gpu.MHD_HEALTH_DENSITY) == 0, name
        assert r["energy_drift"] < 1e-6 and r["mass_drift"] < 1e-6, (name, r)
        assert r["max_div_b"] < 2e-4, (name, r)
        assert abs(r["cells_p_nonpositive"] / ref["cells_p_nonpositive"] - 1) < 0.03, (name, r, ref)
        assert ref["min_p"] * 1.5 < r["min_p"] < ref["min_p"] / 1.5, (name, r, ref)
