"""CPU tests of the oracle: pinned to the reference's own C path through the
golden vectors (which the reference produced, tests/golden/gen_golden.py)
and, where the reference has been compiled here (oracle/_ref), directly."""
import os

import numpy as np
import pytest

from util import bits_equal, field_errors

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_oracle_matches_reference_goldens_per_subroutine(oracle_lib):
    O = oracle_lib.oracle("f32")
    g = np.load(os.path.join(GOLD, "subroutines_f32.npz"))
    tags = sorted({k.split("_")[0] for k in g.files})
    assert tags
    for tag in tags:
        nx, ny, nz = (int(x) for x in g[f"{tag}_dims"])
        dt = np.float32(g[f"{tag}_dt"][0])
        u, b = g[f"{tag}_u"], g[f"{tag}_b"]
        uu = np.zeros_like(u)
        O.fluidx(uu, b.copy(), nx, ny, nz, dt, u.copy(), b.copy())
        assert bits_equal(uu, g[f"{tag}_fluidx_u"]), tag
        bb = b.copy()
        O.advectbyzx(u.copy(), bb, nx, ny, nz, dt, u.copy(), b.copy())
        assert bits_equal(bb, g[f"{tag}_advect_b"]), tag
        tu, tb = np.zeros_like(u), np.zeros_like(b)
        O.transpose12(tu, tb, u.copy(), b.copy(), nx, ny, nz)
        assert bits_equal(tu, g[f"{tag}_t12_u"]) and bits_equal(tb, g[f"{tag}_t12_b"]), tag
        if f"{tag}_t13_u" in g.files:
            tu, tb = np.zeros_like(u), np.zeros_like(b)
            O.transpose13(tu, tb, u.copy(), b.copy(), nx, ny, nz)
            assert bits_equal(tu, g[f"{tag}_t13_u"]) and bits_equal(tb, g[f"{tag}_t13_b"]), tag
        assert bits_equal(np.array([O.calcfl(u, b, nx, ny, nz)]), g[f"{tag}_calcfl"]), tag


def test_oracle_matches_reference_run_on_shipped_alfven_state(oracle_lib):
    """54 steps to tf=64 from data/source_init_alfvenlinear_16cube.dat, CFL 0.9:
    the reference's own run (Heterogeneous_MHD/C/mhd.c:59-125), bit for bit."""
    O = oracle_lib.oracle("f32")
    g = np.load(os.path.join(GOLD, "alfven16_dat.npz"))
    u, b = g["u0"].copy(), g["b0"].copy()
    s, t, dts = O.run(u, b, 16, 16, 16, cfl_number=0.9, tf=64.0, max_steps=100000)
    assert s == int(g["steps"][0]) == 54
    assert bits_equal(dts, g["dtsf"])
    assert np.float32(t) == g["t"][0]
    assert bits_equal(u, g["uf"]) and bits_equal(b, g["bf"])


def test_oracle_matches_reference_cfl07_alfven_x(oracle_lib):
    O = oracle_lib.oracle("f32")
    g = np.load(os.path.join(GOLD, "alfvenx16_cfl07.npz"))
    u, b = g["u0"].copy(), g["b0"].copy()
    s, t, dts = O.run(u, b, 16, 16, 16, cfl_number=0.7, tf=0.0, max_steps=20)
    assert s == 20 and bits_equal(dts, g["dts"])
    assert bits_equal(u, g["u"]) and bits_equal(b, g["b"])


def test_oracle64_matches_reference_fp64_build(oracle_lib):
    O = oracle_lib.oracle("f64")
    g = np.load(os.path.join(GOLD, "run8_f64.npz"))
    u, b = g["u0"].copy(), g["b0"].copy()
    s, t, dts = O.run(u, b, 8, 8, 8, cfl_number=0.9, tf=0.0, max_steps=3)
    assert bits_equal(dts, g["dts"])
    assert bits_equal(u, g["u"]) and bits_equal(b, g["b"])


def test_oracle_thread_count_invariant(oracle_lib):
    import ics
    O = oracle_lib.oracle("f32")
    u0, b0 = ics.random_state(12, 10, 8, seed=3)
    res = []
    for th in (1, 4):
        oracle_lib.set_threads(th)
        u, b = u0.copy(), b0.copy()
        O.run(u, b, 12, 10, 8, cfl_number=0.8, max_steps=2)
        res.append((u, b))
    oracle_lib.set_threads(1)
    assert bits_equal(res[0][0], res[1][0]) and bits_equal(res[0][1], res[1][1])


def test_oracle_fp32_close_to_fp64_on_alfven(oracle_lib):
    import ics
    O32, O64 = oracle_lib.oracle("f32"), oracle_lib.oracle("f64")
    u, b = ics.alfven_x(16)
    u64, b64 = u.astype(np.float64), b.astype(np.float64)
    O32.run(u, b, 16, 16, 16, cfl_number=0.7, max_steps=10)
    O64.run(u64, b64, 16, 16, 16, cfl_number=0.7, max_steps=10)
    eu, eb = field_errors(u, u64, 5), field_errors(b, b64, 3)
    # the wave (rho, m_y, E, b_x, b_y) to 1e-5 of each field
    for e in (eu[0], eu[2], eu[4], eb[0], eb[1]):
        assert e < 1e-5, (eu, eb)
    # m_x is second order (~3e-7) and FP32 pressure round-off (~1e-7
    # absolute) dominates it; bound it against the total pressure scale
    ux, u64x = u.reshape(-1, 5), u64.reshape(-1, 5)
    assert np.abs(ux[:, 1] - u64x[:, 1]).max() < 1e-6


def test_oracle_transpose13_noncubic_is_the_fortran_formula(oracle_lib):
    """nx != nz: dst(ii,k,j,i) = src(perm(ii),i,j,k), perm_u=(1,4,3,2,5),
    perm_b=(3,2,1) (OpenMP/mhd.f90:433-474); applying it twice is the identity."""
    import ics
    O = oracle_lib.oracle("f32")
    nx, ny, nz = 6, 5, 9
    u, b = ics.random_state(nx, ny, nz, seed=5)
    tu, tb = np.zeros_like(u), np.zeros_like(b)
    O.transpose13(tu, tb, u.copy(), b.copy(), nx, ny, nz)
    U = u.reshape(nz, ny, nx, 5)
    T = tu.reshape(nx, ny, nz, 5)   # dims (nz, ny, nx) -> index [i][j][k]
    assert np.array_equal(T, U[..., [0, 3, 2, 1, 4]].transpose(2, 1, 0, 3))
    bu, bb = np.zeros_like(u), np.zeros_like(b)
    O.transpose13(bu, bb, tu, tb, nz, ny, nx)
    assert bits_equal(bu, u) and bits_equal(bb, b)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(os.path.dirname(
    os.path.abspath(__file__))), "oracle", "_ref", "libref_f32.so")),
    reason="reference C path not compiled here (make -C oracle ref)")
def test_oracle_bit_exact_against_reference_build(oracle_lib):
    import ics
    R, O = oracle_lib.reference("f32"), oracle_lib.oracle("f32")
    for dims, seed in [((8, 8, 8), 1), ((12, 6, 10), 2), ((5, 7, 9), 3), ((16, 4, 16), 4)]:
        nx, ny, nz = dims
        u0, b0 = ics.random_state(*dims, seed=seed)
        out = []
        for P in (R, O):
            u, b = u0.copy(), b0.copy()
            if nx == ny == nz:
                P.run(u, b, nx, ny, nz, cfl_number=0.9, max_steps=2)
            else:
                uu = np.zeros_like(u)
                P.fluidx(uu, b.copy(), nx, ny, nz, np.float32(0.05), u.copy(), b.copy())
                bb = b.copy()
                P.advectbyzx(u.copy(), bb, nx, ny, nz, np.float32(0.05), u.copy(), b.copy())
                u, b = uu, bb
            out.append((u, b))
        assert bits_equal(out[0][0], out[1][0]) and bits_equal(out[0][1], out[1][1]), dims


def test_flop_count_per_cell_update(oracle_lib):
    """The operation count of one step (oracle/flopcount.cpp: every +, -, *, /
    and sqrt of the restatement as the reference writes them) is the figure the
    roofline's flop rate uses (bench.py FLOPS_PER_CELL_UPDATE)."""
    import subprocess
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, repo)
    import bench
    odir = os.path.join(repo, "oracle")
    subprocess.run(["make", "-s", "-C", odir, "flopcount"], check=True)
    out = subprocess.run([os.path.join(odir, "lib", "flopcount"), "64", "64", "64"], check=True,
                         capture_output=True, text=True).stdout
    total = float(out.split("flops per cell-update:")[1].split()[0])
    assert abs(total - bench.FLOPS_PER_CELL_UPDATE) < 5, (total, out)


def test_oracle_matches_reference_run_on_shipped_32cube_state(oracle_lib):
    """108 steps to tf = 128 from data/source_init_alfvenlinear_32cube.dat at
    CFL 0.9: the reference's own run, bit for bit (digests of the final state)."""
    import hashlib
    O = oracle_lib.oracle("f32")
    g = np.load(os.path.join(GOLD, "alfven32_dat.npz"))
    u, b = g["u0"].copy(), g["b0"].copy()
    s, t, dts = O.run(u, b, 32, 32, 32, cfl_number=0.9, tf=128.0, max_steps=100000)
    assert s == int(g["steps"][0]) == 108
    assert bits_equal(dts, g["dtsf"])
    assert hashlib.sha256(u.tobytes()).hexdigest() == str(g["uf_sha"][0])
    assert hashlib.sha256(b.tobytes()).hexdigest() == str(g["bf_sha"][0])


def test_oracle64_keeps_div_b_and_conserves_on_a_noncubic_state(oracle_lib):
    """Size-independent properties of the scheme, pinned on the FP64 oracle
    with a turbulent non-cubic start: constrained transport keeps max |div B|
    at round-off of the initial field, and mass and total energy (fluxes in
    conservation form on a periodic box) are conserved to round-off."""
    import ics
    O = oracle_lib.oracle("f64")
    nx, ny, nz = 24, 16, 20
    u32, b32 = ics.random_state(nx, ny, nz, seed=12, amp=0.3)
    u, b = u32.astype(np.float64), b32.astype(np.float64)
    d0 = ics.div_b(b, nx, ny, nz)
    t0 = ics.totals(u, nx, ny, nz)
    s, _t, _dts = O.run(u, b, nx, ny, nz, cfl_number=0.7, tf=0.0, max_steps=6)
    assert s == 6
    assert ics.div_b(b, nx, ny, nz) < d0 + 1e-12
    t1 = ics.totals(u, nx, ny, nz)
    assert abs(t1[0] - t0[0]) < 1e-12 * abs(t0[0])
    assert abs(t1[4] - t0[4]) < 1e-12 * abs(t0[4])


def test_tie_pencil_fixture_is_a_double_tie(oracle_lib):
    """The fixture of tests/golden/gen_tie_pencil.py: the oracle reproduces
    its stored fluidx output, and cell 70's half-step total pressure is the
    double-rounding case the fixture is kept for -- the exact value lies half
    a double ulp above a float midpoint, the C path's RN_d(RN_d(A G) + M)
    one ulp above it (rounds up), a fused A G + M on the midpoint (rounds to
    even, down)."""
    from fractions import Fraction as Fr
    O = oracle_lib.oracle("f32")
    z = np.load(os.path.join(GOLD, "tie_pencil.npz"))
    nx, ny, nz = (int(x) for x in z["dims"])
    dt = np.float32(z["dt"][0])
    out = np.zeros_like(z["u"])
    O.fluidx(out, z["b"].copy(), nx, ny, nz, dt, z["u"].copy(), z["b"].copy())
    assert bits_equal(out, z["out"])
    # cell 70 of pencil (0, 0) before the half step: u and the cell-centred b
    f32 = np.float32
    u = z["u"].reshape(nz, ny, nx, 5)[0, 0, 70]
    bb = z["b"].reshape(nz, ny, nx, 3)
    bx = f32(f32(0.5) * bb[0, 0, 70, 0]) + f32(f32(0.5) * bb[0, 0, 71, 0])
    by = f32(f32(0.5) * bb[0, 0, 70, 1]) + f32(bb[0, 1, 70, 1] / f32(2))
    bz = f32(f32(0.5) * bb[0, 0, 70, 2]) + f32(bb[1, 0, 70, 2] / f32(2))
    r, m1, m2, m3, e = u
    q = f32(f32(f32(f32(m1 * m1) + f32(m2 * m2)) + f32(m3 * m3)) / r)
    b2 = f32(f32(f32(bx * bx) + f32(by * by)) + f32(bz * bz))
    g = float(f32(5.0 / 3.0))
    a = float(e) - float(q) / 2.0
    m = (2.0 - g) * float(b2) / 2.0
    c_path = a * (g - 1.0) + m                       # two double roundings
    exact = Fr(a) * (Fr(g) - 1) + Fr(m)
    assert Fr(a) == Fr(float(e)) - Fr(float(q)) / 2 and Fr(m) == (2 - Fr(g)) * Fr(float(b2)) / 2
    lo = float(f32(c_path))
    lo = float(np.nextafter(f32(lo), f32(0)))
    mid = (Fr(lo) + Fr(float(f32(c_path)))) / 2
    ulp_d = Fr(2.0 ** -52)                           # the double ulp at ps ~ 1.03
    assert 1.0 <= c_path < 2.0
    assert exact - mid == ulp_d / 2                  # a tie in double
    assert Fr(c_path) - mid == ulp_d                 # the C path's double, above
    assert float(f32(c_path)) > float(mid)           # rounds up in float
