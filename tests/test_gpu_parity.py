"""GPU parity of the sm_103a kernels against the oracle, through the C ABI.

Tolerances (written here, per the task's contract):
  - transposes: bit-exact;
  - fluidx / advectbyzx / whole step: per-field max-norm relative error
    <= 1e-5 (util.field_errors; momentum and b components are measured
    against the largest component of their vector field);
  - cfl: 1/c within 2 ulp (the reference forms the root and the final sum
    in double; the kernel reproduces that in float-float).
"""
import os

import numpy as np
import pytest

from util import bits_equal, field_errors

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = 1e-5


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def scalar(x):
    import torch
    return torch.tensor([x], dtype=torch.float32, device="cuda")


SHAPES = [(16, 16, 16), (8, 6, 10), (5, 7, 9), (32, 4, 3), (48, 3, 5), (64, 5, 4), (100, 3, 2),
          (128, 4, 3), (200, 2, 3), (256, 2, 2), (512, 2, 1), (1024, 1, 2), (12, 20, 28), (1, 4, 5)]


@pytest.mark.parametrize("dims", SHAPES)
def test_fluidx_matches_oracle(gpu, oracle_lib, dims):
    import ics
    O = oracle_lib.oracle("f32")
    nx, ny, nz = dims
    u, b = ics.random_state(nx, ny, nz, seed=nx + ny + nz)
    dt = np.float32(0.03)
    ref = np.zeros_like(u)
    O.fluidx(ref, b.copy(), nx, ny, nz, dt, u.copy(), b.copy())
    du, db = dev(u), dev(b)
    gpu.fluidx(du, du, db, nx, ny, nz, scalar(dt))         # in place
    got = host(du)
    assert max(field_errors(got, ref, 5)) < TOL, field_errors(got, ref, 5)
    out = dev(np.zeros_like(u))
    du2 = dev(u)
    gpu.fluidx(out, du2, db, nx, ny, nz, scalar(dt))       # out of place
    assert bits_equal(host(out), got)
    assert bits_equal(host(du2), u)                        # input untouched


def test_fluidx_pressure_on_a_double_tie(gpu):
    """tests/golden/tie_pencil.npz: a cell whose total pressure the C path
    rounds twice in double away from a tie (mhdflux.c:28).  The rare-operand
    fallback must round the product and the sum separately, as the C path
    does; a contracted FMA lands on the float midpoint and rounds the other
    way.  Bit-exact, all math policies that claim the C path's rounding."""
    z = np.load(os.path.join(GOLD, "tie_pencil.npz"))
    nx, ny, nz = (int(x) for x in z["dims"])
    du, db = dev(z["u"]), dev(z["b"])
    out = dev(np.zeros_like(z["u"]))
    gpu.fluidx(out, du, db, nx, ny, nz, scalar(np.float32(z["dt"][0])))
    assert bits_equal(host(out), z["out"])


@pytest.mark.parametrize("dims", SHAPES)
def test_advectbyzx_matches_oracle(gpu, oracle_lib, dims):
    import ics
    O = oracle_lib.oracle("f32")
    nx, ny, nz = dims
    u, b = ics.random_state(nx, ny, nz, seed=7 * nx + ny)
    dt = np.float32(0.04)
    ref = b.copy()
    O.advectbyzx(u.copy(), ref, nx, ny, nz, dt, u.copy(), b.copy())
    du, db = dev(u), dev(b)
    import torch
    scr = torch.empty(gpu.advectbyzx_scratch_bytes(nx, ny, nz) // 4, dtype=torch.float32, device="cuda")
    gpu.advectbyzx(db, du, nx, ny, nz, scalar(dt), scr)
    got = host(db)
    assert max(field_errors(got, ref, 3)) < TOL, field_errors(got, ref, 3)


@pytest.mark.parametrize("dims", [(16, 16, 16), (8, 6, 10), (5, 7, 9), (33, 31, 2), (64, 1, 40),
                                  (1, 1, 1), (7, 70, 3),
                                  # full 32x32 tiles on 16-byte rows (vector copies), with
                                  # ragged edge tiles beside them, and unaligned strides
                                  (64, 96, 32), (96, 40, 68), (64, 36, 44), (32, 64, 30), (36, 64, 64)])
def test_transposes_bit_exact(gpu, oracle_lib, dims):
    import ics
    O = oracle_lib.oracle("f32")
    nx, ny, nz = dims
    u, b = ics.random_state(nx, ny, nz, seed=3)
    for which in (12, 13):
        ru, rb = np.zeros_like(u), np.zeros_like(b)
        (O.transpose12 if which == 12 else O.transpose13)(ru, rb, u.copy(), b.copy(), nx, ny, nz)
        du, db = dev(u), dev(b)
        ou, ob = dev(np.full_like(u, np.nan)), dev(np.full_like(b, np.nan))
        (gpu.transpose12 if which == 12 else gpu.transpose13)(ou, ob, du, db, nx, ny, nz)
        assert bits_equal(host(ou), ru) and bits_equal(host(ob), rb), (which, dims)


def test_transposes_match_reference_goldens(gpu):
    g = np.load(os.path.join(GOLD, "subroutines_f32.npz"))
    for tag in sorted({k.split("_")[0] for k in g.files}):
        nx, ny, nz = (int(x) for x in g[f"{tag}_dims"])
        u, b = g[f"{tag}_u"], g[f"{tag}_b"]
        ou, ob = dev(np.zeros_like(u)), dev(np.zeros_like(b))
        gpu.transpose12(ou, ob, dev(u), dev(b), nx, ny, nz)
        assert bits_equal(host(ou), g[f"{tag}_t12_u"]) and bits_equal(host(ob), g[f"{tag}_t12_b"])
        if f"{tag}_t13_u" in g.files:
            gpu.transpose13(ou, ob, dev(u), dev(b), nx, ny, nz)
            assert bits_equal(host(ou), g[f"{tag}_t13_u"]) and bits_equal(host(ob), g[f"{tag}_t13_b"])


def _ulps(a, b):
    a = np.float32(a).view(np.int32).astype(np.int64)
    b = np.float32(b).view(np.int32).astype(np.int64)
    return abs(int(a) - int(b))


@pytest.mark.parametrize("dims", [(16, 16, 16), (8, 6, 10), (5, 7, 9), (64, 32, 16), (1, 1, 1)])
@pytest.mark.parametrize("mode", [0, 1])
def test_cfl_matches_oracle(gpu, oracle_lib, dims, mode):
    import ics
    import torch
    O = oracle_lib.oracle("f32")
    nx, ny, nz = dims
    u, b = ics.random_state(nx, ny, nz, seed=nx * 3 + mode)
    ref = (O.calcfl_averaged if mode else O.calcfl)(u, b, nx, ny, nz)
    inv = torch.zeros(1, dtype=torch.float32, device="cuda")
    word = torch.zeros(1, dtype=torch.int32, device="cuda")
    gpu.cfl(dev(u), dev(b), nx, ny, nz, mode, inv, word)
    got = host(inv)[0]
    assert _ulps(got, ref) <= 2, (got, ref)


def test_cfl_matches_reference_goldens(gpu):
    import torch
    g = np.load(os.path.join(GOLD, "subroutines_f32.npz"))
    for tag in sorted({k.split("_")[0] for k in g.files}):
        nx, ny, nz = (int(x) for x in g[f"{tag}_dims"])
        inv = torch.zeros(1, dtype=torch.float32, device="cuda")
        word = torch.zeros(1, dtype=torch.int32, device="cuda")
        gpu.cfl(dev(g[f"{tag}_u"]), dev(g[f"{tag}_b"]), nx, ny, nz, 0, inv, word)
        assert _ulps(host(inv)[0], g[f"{tag}_calcfl"][0]) <= 2


def test_dt_update_follows_the_driver_rule(gpu, oracle_lib):
    O = oracle_lib.oracle("f32")
    for inv, cfl, t, tf in [(0.3, 0.9, 0.0, 64.0), (0.37, 0.7, 63.5, 64.0), (0.25, 0.8, 10.0, 0.0)]:
        d_t, d_dt = scalar(t), scalar(0.0)
        gpu.dt_update(scalar(inv), cfl, tf, d_t, d_dt)
        ref_dt = O.dt_from_cfl(np.float32(inv), cfl, np.float32(t), np.float32(tf))
        assert host(d_dt)[0] == ref_dt
        assert host(d_t)[0] == np.float32(np.float32(t) + np.float32(2) * ref_dt)


def _step_parity(gpu, O, u, b, nx, ny, nz, dt):
    import torch
    ru, rb = u.copy(), b.copy()
    O.step(ru, rb, nx, ny, nz, dt)
    du, db = dev(u), dev(b)
    work = torch.empty(gpu.step_workspace_bytes(nx, ny, nz), dtype=torch.uint8, device="cuda")
    health = torch.zeros(1, dtype=torch.int32, device="cuda")
    gpu.step(du, db, nx, ny, nz, scalar(dt), work, health)
    return host(du), host(db), ru, rb, int(host(health)[0])


@pytest.mark.parametrize("dims", [(16, 16, 16), (12, 10, 8), (32, 16, 24), (5, 7, 9)])
def test_step_matches_oracle(gpu, oracle_lib, dims):
    import ics
    O = oracle_lib.oracle("f32")
    nx, ny, nz = dims
    u, b = ics.random_state(nx, ny, nz, seed=17, amp=0.2)
    gu, gb, ru, rb, health = _step_parity(gpu, O, u, b, nx, ny, nz, np.float32(0.05))
    assert health == 0
    assert max(field_errors(gu, ru, 5)) < TOL, field_errors(gu, ru, 5)
    assert max(field_errors(gb, rb, 3)) < TOL, field_errors(gb, rb, 3)


def _advance(gpu, u, b, nx, ny, nz, nsteps, cfl_number, mode=0, tf=0.0, path=0):
    import torch
    du, db = dev(u), dev(b)
    work = torch.empty(gpu.step_workspace_bytes(nx, ny, nz, path), dtype=torch.uint8, device="cuda")
    clock = gpu.new_clock()
    log = torch.zeros(max(nsteps, 1), dtype=torch.float32, device="cuda")
    gpu.advance(du, db, nx, ny, nz, nsteps, cfl_number, mode, tf, clock, log, work, path)
    clk = gpu.read_clock(clock)
    return host(du), host(db), host(log)[:clk.iter], clk


PATHS = [0, 1]   # MHD_PATH_PLAIN, MHD_PATH_FUSED


@pytest.mark.parametrize("dims", [(16, 16, 16), (12, 10, 8), (32, 16, 24), (5, 7, 9), (64, 40, 24)])
def test_fused_step_equals_plain_step_bitwise(gpu, dims):
    """The transpose-free step does the same arithmetic per pencil as the
    transposing one: equal bit for bit, on cubic and non-cubic boxes."""
    import ics
    import torch
    nx, ny, nz = dims
    u, b = ics.random_state(nx, ny, nz, seed=23, amp=0.2)
    out = []
    for path in PATHS:
        du, db = dev(u), dev(b)
        work = torch.empty(gpu.step_workspace_bytes(nx, ny, nz, path), dtype=torch.uint8, device="cuda")
        (gpu.step if path == 0 else gpu.step_fused)(du, db, nx, ny, nz, scalar(0.05), work)
        out.append((host(du), host(db)))
    assert bits_equal(out[0][0], out[1][0]) and bits_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("path", PATHS)
def test_shipped_alfven_state_full_run_matches_reference(gpu, path):
    """The reference's own run from data/source_init_alfvenlinear_16cube.dat:
    54 steps to tf = 64 at CFL 0.9 (Heterogeneous_MHD/C/mhd.c:59-125)."""
    g = np.load(os.path.join(GOLD, "alfven16_dat.npz"))
    gu, gb, dts, clk = _advance(gpu, g["u0"], g["b0"], 16, 16, 16, 60, 0.9, tf=64.0, path=path)
    # this state has plasma beta ~1e-3: the FP32 pressure recovery touches 0
    # at round-off (the warning bit), nothing worse
    assert clk.iter == 54
    assert clk.health & (gpu.MHD_HEALTH_NONFINITE | gpu.MHD_HEALTH_DENSITY) == 0
    assert np.float32(clk.t) == g["t"][0]
    assert np.abs(dts / g["dtsf"] - 1).max() < 1e-6
    eu, eb = field_errors(gu, g["uf"], 5), field_errors(gb, g["bf"], 3)
    assert max(eu) < TOL and max(eb) < TOL, (eu, eb)


@pytest.mark.parametrize("path", PATHS)
def test_shipped_32cube_state_full_run_matches_reference(gpu, path):
    """The reference's own run from data/source_init_alfvenlinear_32cube.dat:
    108 steps to tf = 128 at CFL 0.9.  The fixture carries digests of the final
    state and every 97th value; the faithful kernels reproduce the digests."""
    import hashlib
    g = np.load(os.path.join(GOLD, "alfven32_dat.npz"))
    gu, gb, dts, clk = _advance(gpu, g["u0"], g["b0"], 32, 32, 32, 120, 0.9, tf=128.0, path=path)
    assert clk.iter == 108
    assert clk.health & (gpu.MHD_HEALTH_NONFINITE | gpu.MHD_HEALTH_DENSITY) == 0
    assert np.array_equal(dts, g["dtsf"])
    eu = field_errors(gu[::97], g["uf_sample"], 1, vector_floor=False)
    eb = field_errors(gb[::97], g["bf_sample"], 1, vector_floor=False)
    assert max(eu) < TOL and max(eb) < TOL, (eu, eb)
    assert hashlib.sha256(gu.tobytes()).hexdigest() == str(g["uf_sha"][0])
    assert hashlib.sha256(gb.tobytes()).hexdigest() == str(g["bf_sha"][0])


@pytest.mark.parametrize("path", PATHS)
def test_config1_alfven_x_32_100_steps(gpu, oracle_lib, path):
    """32^3 Alfven wave along x, A=1e-3, CFL 0.7, 100 steps."""
    import ics
    O = oracle_lib.oracle("f32")
    oracle_lib.set_threads(os.cpu_count() or 1)
    u, b = ics.alfven_x(32)
    ru, rb = u.copy(), b.copy()
    s, t, rdts = O.run(ru, rb, 32, 32, 32, cfl_number=0.7, max_steps=100)
    gu, gb, dts, clk = _advance(gpu, u, b, 32, 32, 32, 100, 0.7, path=path)
    oracle_lib.set_threads(1)
    assert clk.iter == 100 and clk.health == 0
    assert np.abs(dts / rdts - 1).max() < 1e-6
    eu, eb = field_errors(gu, ru, 5), field_errors(gb, rb, 3)
    assert max(eu) < TOL and max(eb) < TOL, (eu, eb)
    assert ics.div_b(gb, 32, 32, 32) < 1e-6


@pytest.mark.parametrize("path", PATHS)
def test_oblique_alfven_64_matches_oracle(gpu, oracle_lib, path):
    """The diagonal wave of the 128^3 configuration, at 64^3 for 30 steps."""
    import ics
    O = oracle_lib.oracle("f32")
    oracle_lib.set_threads(os.cpu_count() or 1)
    n = 64
    u, b = ics.alfven_oblique(n)
    ru, rb = u.copy(), b.copy()
    O.run(ru, rb, n, n, n, cfl_number=0.7, max_steps=30)
    gu, gb, dts, clk = _advance(gpu, u, b, n, n, n, 30, 0.7, path=path)
    oracle_lib.set_threads(1)
    eu, eb = field_errors(gu, ru, 5), field_errors(gb, rb, 3)
    assert max(eu) < TOL and max(eb) < TOL, (eu, eb)
    # div B is FP32 round-off of the face updates (|B| ~ 1): the same size
    # as the oracle's own
    assert ics.div_b(gb, n, n, n) < 2.0 * ics.div_b(rb, n, n, n) + 1e-6


@pytest.mark.parametrize("path", PATHS)
def test_config2_full_size_invariants(gpu, path):
    """128^3 diagonal Alfven wave, 200 steps: div B stays at round-off, mass and
    energy are conserved to FP32 round-off, the wave amplitude decays only by
    the scheme's diffusion."""
    import ics
    n = 128
    u, b = ics.alfven_oblique(n)
    tot0 = ics.totals(u, n, n, n)
    gu, gb, dts, clk = _advance(gpu, u, b, n, n, n, 200, 0.7, path=path)
    assert clk.iter == 200 and clk.health == 0
    assert ics.div_b(gb, n, n, n) < 1e-5
    tot = ics.totals(gu, n, n, n)
    assert abs(tot[0] / tot0[0] - 1) < 1e-6
    assert abs(tot[4] / tot0[4] - 1) < 1e-6
    amp0 = np.abs(u.reshape(-1, 5)[:, 1:4]).max()
    amp = np.abs(gu.reshape(-1, 5)[:, 1:4]).max()
    assert 0.5 * amp0 < amp <= 1.01 * amp0


@pytest.mark.parametrize("path", PATHS)
def test_run_host_matches_device_path(gpu, path):
    import ics
    u, b = ics.alfven_x(16)
    gu, gb, dts, clk = _advance(gpu, u, b, 16, 16, 16, 5, 0.7, path=path)
    hu, hb = u.copy(), b.copy()
    log = np.zeros(5, np.float32)
    st, t, done = gpu.run_host(hu, hb, 16, 16, 16, 0.7, 0, 0.0, 0.0, 5, log, path=path)
    assert st == gpu.MHD_OK and done == 5
    assert bits_equal(hu, gu) and bits_equal(hb, gb) and bits_equal(log, dts)


def test_run_host_cache_grows_and_releases(gpu):
    """The host entry keeps its device buffers per thread: a small box, a
    larger one (the buffer grows), the small one again inside the larger
    buffer, and a call after mhdgpu_release_host_cache all equal the device
    path bit for bit."""
    import ics
    cases = [((16, 16, 16), ics.alfven_x(16)), ((24, 16, 32), ics.random_state(24, 16, 32, seed=9, amp=0.1))]
    refs = {}
    for dims, (u, b) in cases:
        gu, gb, _dts, _clk = _advance(gpu, u, b, *dims, 3, 0.7, path=gpu.MHD_PATH_FUSED)
        refs[dims] = (gu, gb)
    for k, release in ((0, False), (1, False), (0, False), (1, True), (0, True)):
        dims, (u, b) = cases[k]
        if release:
            gpu.release_host_cache()
        hu, hb = u.copy(), b.copy()
        st, _t, done = gpu.run_host(hu, hb, *dims, 0.7, 0, 0.0, 0.0, 3, path=gpu.MHD_PATH_FUSED)
        assert st == gpu.MHD_OK and done == 3
        assert bits_equal(hu, refs[dims][0]) and bits_equal(hb, refs[dims][1])


def test_health_word_flags_unphysical_state(gpu):
    """Fault injection on the host: a negative density uploaded into the
    state.  The kernels keep running; the health word reports it."""
    import ics
    import torch
    u, b = ics.alfven_x(16)
    u = u.copy()
    u[5 * 100] = -1.0                                     # rho < 0 in one cell
    du, db = dev(u), dev(b)
    health = torch.zeros(1, dtype=torch.int32, device="cuda")
    gpu.fluidx(du, du, db, 16, 16, 16, scalar(0.1), health)
    h = int(host(health)[0])
    assert h & (gpu.MHD_HEALTH_DENSITY | gpu.MHD_HEALTH_PRESSURE | gpu.MHD_HEALTH_NONFINITE)
    hu, hb = u.copy(), b.copy()
    st, t, done = gpu.run_host(hu, hb, 16, 16, 16, 0.7, 0, 0.0, 0.0, 1)
    assert st == gpu.MHD_ERR_UNPHYSICAL


def test_compat_shims_match_oracle(gpu, oracle_lib):
    """The reference-named host entry points (include/mhdgpu_compat.h) driven
    like the reference driver drives its own subroutines."""
    import ctypes as C
    import ics
    L = gpu.lib()
    O = oracle_lib.oracle("f32")
    nx, ny, nz = 8, 6, 8
    u, b = ics.random_state(nx, ny, nz, seed=9)

    def ip(x):
        return C.byref(C.c_int(x))

    def fp(a):
        return a.ctypes.data_as(C.c_void_p)

    dt = C.c_float(0.05)
    gu = np.zeros_like(u)
    L.fluidx(fp(gu), fp(b.copy()), ip(nx), ip(ny), ip(nz), C.byref(dt), fp(u.copy()), fp(b.copy()), 0)
    ru = np.zeros_like(u)
    O.fluidx(ru, b.copy(), nx, ny, nz, np.float32(0.05), u.copy(), b.copy())
    assert L.mhdgpu_compat_status() == 0
    assert max(field_errors(gu, ru, 5)) < TOL
    gb = b.copy()
    L.advectbyzx(fp(u.copy()), fp(gb), ip(nx), ip(ny), ip(nz), C.byref(dt), fp(u.copy()), fp(b.copy()))
    rb = b.copy()
    O.advectbyzx(u.copy(), rb, nx, ny, nz, np.float32(0.05), u.copy(), b.copy())
    assert max(field_errors(gb, rb, 3)) < TOL
    tu, tb = np.zeros_like(u), np.zeros_like(b)
    L.transpose13(fp(tu), fp(tb), fp(u.copy()), fp(b.copy()), ip(nx), ip(ny), ip(nz))
    su, sb = np.zeros_like(u), np.zeros_like(b)
    O.transpose13(su, sb, u.copy(), b.copy(), nx, ny, nz)
    assert bits_equal(tu, su) and bits_equal(tb, sb)
    inv = L.calcfl(fp(u), fp(b), ip(nx), ip(ny), ip(nz))
    assert _ulps(inv, O.calcfl(u, b, nx, ny, nz)) <= 2


SHAPES_COMPILED = [(1, 1), (2, 1), (4, 1), (1, 2), (2, 2), (4, 2), (1, 4), (2, 4), (4, 4), (2, 8), (4, 8)]


@pytest.mark.parametrize("n", [16, 48, 100, 128, 256, 512])
def test_every_team_shape_matches_oracle(gpu, oracle_lib, n):
    """fluidx and advectbyzx under every compiled team shape that covers the
    pencil (the shapes the autotuner chooses from)."""
    import ics
    import torch
    O = oracle_lib.oracle("f32")
    ny, nz = 3, 2
    u, b = ics.random_state(n, ny, nz, seed=n)
    dt = np.float32(0.03)
    ref_u = np.zeros_like(u)
    O.fluidx(ref_u, b.copy(), n, ny, nz, dt, u.copy(), b.copy())
    ref_b = b.copy()
    O.advectbyzx(u.copy(), ref_b, n, ny, nz, dt, u.copy(), b.copy())
    saved = {k: gpu.get_tile(k, n) for k in ("fluidx", "advectbyzx")}
    scr = torch.empty(gpu.advectbyzx_scratch_bytes(n, ny, nz) // 4, dtype=torch.float32, device="cuda")
    tested = 0
    try:
        for cpl, wpp in SHAPES_COMPILED:
            if n > 32 * wpp * cpl:
                continue
            for ppc in (1, 2, 4, 8):
                if 32 * wpp * ppc > 256:
                    continue
                gpu.set_tile("fluidx", n, cpl, wpp, ppc)
                gpu.set_tile("advectbyzx", n, cpl, wpp, ppc)
                du, db = dev(u), dev(b)
                out = dev(np.zeros_like(u))
                gpu.fluidx(out, du, db, n, ny, nz, scalar(dt))
                gpu.advectbyzx(db, du, n, ny, nz, scalar(dt), scr)
                eu = field_errors(host(out), ref_u, 5)
                eb = field_errors(host(db), ref_b, 3)
                assert max(eu) < TOL and max(eb) < TOL, ((cpl, wpp, ppc), eu, eb)
                tested += 1
    finally:
        for k, (c, w, p) in saved.items():
            gpu.set_tile(k, n, c, w, p)
    assert tested > 0


@pytest.mark.parametrize("n", [16, 48, 100])
def test_every_team_shape_fused_step_bitwise(gpu, n):
    """The transpose-free step stages pencils that run across memory through
    shared memory in rows; every compiled team shape must give the plain
    step's bits."""
    import ics
    import torch
    u, b = ics.random_state(n, n, n, seed=n + 1, amp=0.2)
    du, db = dev(u), dev(b)
    work = torch.empty(gpu.step_workspace_bytes(n, n, n), dtype=torch.uint8, device="cuda")
    gpu.step(du, db, n, n, n, scalar(0.04), work)
    ref_u, ref_b = host(du), host(db)
    saved = {(k, r): gpu.get_tile(k, n, rows=r) for k in ("fluidx", "advectbyzx") for r in (False, True)}
    wf = torch.empty(gpu.step_workspace_bytes(n, n, n, 1), dtype=torch.uint8, device="cuda")
    try:
        for cpl, wpp in SHAPES_COMPILED:
            if n > 32 * wpp * cpl:
                continue
            for ppc in (1, 2, 4, 8):
                if 32 * wpp * ppc > 256:
                    continue
                for k in ("fluidx", "advectbyzx"):
                    for r in (False, True):
                        gpu.set_tile(k, n, cpl, wpp, ppc, rows=r)
                du, db = dev(u), dev(b)
                gpu.step_fused(du, db, n, n, n, scalar(0.04), wf)
                assert bits_equal(host(du), ref_u) and bits_equal(host(db), ref_b), (cpl, wpp, ppc)
    finally:
        for (k, r), (c, w, p) in saved.items():
            gpu.set_tile(k, n, c, w, p, rows=r)


def test_fast_math_policy_matches_oracle(gpu, oracle_lib):
    """The fast policy (FMA contraction, hardware reciprocal and root): one
    fluidx and one advectbyzx within the same 1e-5 tolerance."""
    import ics
    import torch
    O = oracle_lib.oracle("f32")
    nx, ny, nz = 64, 8, 6
    u, b = ics.random_state(nx, ny, nz, seed=77)
    dt = np.float32(0.03)
    ref_u = np.zeros_like(u)
    O.fluidx(ref_u, b.copy(), nx, ny, nz, dt, u.copy(), b.copy())
    ref_b = b.copy()
    O.advectbyzx(u.copy(), ref_b, nx, ny, nz, dt, u.copy(), b.copy())
    prev = gpu.set_math(gpu.MHD_MATH_FAST)
    try:
        du, db = dev(u), dev(b)
        scr = torch.empty(gpu.advectbyzx_scratch_bytes(nx, ny, nz) // 4, dtype=torch.float32, device="cuda")
        gpu.fluidx(du, du, db, nx, ny, nz, scalar(dt))
        gpu.advectbyzx(db, dev(u), nx, ny, nz, scalar(dt), scr)
        assert max(field_errors(host(du), ref_u, 5)) < TOL
        assert max(field_errors(host(db), ref_b, 3)) < TOL
    finally:
        gpu.set_math(prev)


def test_autotune_keeps_parity(gpu, oracle_lib):
    import ics
    O = oracle_lib.oracle("f32")
    nx, ny, nz = 48, 32, 20
    saved = {(k, n, r): gpu.get_tile(k, n, rows=r) for k in ("fluidx", "advectbyzx")
             for n in (nx, ny, nz) for r in (False, True)}
    try:
        picks = gpu.autotune(nx, ny, nz)
        for (k, n, r), (c, w, p) in picks.items():
            assert n <= 32 * w * c and 32 * w * p <= 256
        u, b = ics.random_state(nx, ny, nz, seed=5, amp=0.2)
        gu, gb, ru, rb, health = _step_parity(gpu, O, u, b, nx, ny, nz, np.float32(0.05))
        assert max(field_errors(gu, ru, 5)) < TOL and max(field_errors(gb, rb, 3)) < TOL
        import torch
        du, db = dev(u), dev(b)
        wf = torch.empty(gpu.step_workspace_bytes(nx, ny, nz, 1), dtype=torch.uint8, device="cuda")
        gpu.step_fused(du, db, nx, ny, nz, scalar(0.05), wf)
        assert bits_equal(host(du), gu) and bits_equal(host(db), gb)
    finally:
        for (k, n, r), (c, w, p) in saved.items():
            gpu.set_tile(k, n, c, w, p, rows=r)
