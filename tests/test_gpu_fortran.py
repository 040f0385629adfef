"""The Fortran original's analytic initial states (ics.fortran_ic, restating
OpenMP/mhd.f90:130-247) advanced on the GPU two ways and checked against the
oracle (the C path) on the same dt sequence:

  - the Fortran main loop (mhd.f90:41-72) driven through the Fortran-ABI shim
    (include/mhdgpu_fortran.h: fluidx_, advectbyzx_, transpose12_/13_ in
    place, cfl_), host arrays, dt = 0.9*cfl in float as the Fortran forms it;
  - the device time loop mhdgpu_advance on the transpose-free path.

Tolerance: 1e-5 per field (util.field_errors), as for the other whole-step
parity tests; the original runs a 2-D slab (ny = 1, nz = nx), covered here
beside a 3-D box."""
import ctypes as C

import numpy as np
import pytest

from util import field_errors

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def fortran_loop(L, u, b, nx, ny, nz, nsteps, tf):
    """mhd.f90:41-72 through the shim; returns the dt sequence (float32)."""
    ip = lambda v: C.byref(C.c_int(v))   # noqa: E731
    t = np.float32(0.0)
    dts = []
    fu, fb = _fp(u), _fp(b)
    for _ in range(nsteps):
        if t >= np.float32(tf):
            break
        dt = np.float32(0.9) * np.float32(L.cfl_(fu, fb, ip(nx), ip(ny), ip(nz)))
        dt = min(dt, (np.float32(tf) - t) / np.float32(2))
        t = np.float32(t + np.float32(2) * dt)
        d = C.byref(C.c_float(dt))
        L.fluidx_(fu, fb, ip(nx), ip(ny), ip(nz), d)
        L.advectbyzx_(fu, fb, ip(nx), ip(ny), ip(nz), d)
        L.transpose12_(fu, fb, fu, fb, ip(nx), ip(ny), ip(nz))
        L.fluidx_(fu, fb, ip(ny), ip(nx), ip(nz), d)
        L.advectbyzx_(fu, fb, ip(ny), ip(nx), ip(nz), d)
        L.transpose13_(fu, fb, fu, fb, ip(ny), ip(nx), ip(nz))
        L.fluidx_(fu, fb, ip(nz), ip(nx), ip(ny), d)
        L.advectbyzx_(fu, fb, ip(nz), ip(nx), ip(ny), d)
        L.advectbyzx_(fu, fb, ip(nz), ip(nx), ip(ny), d)
        L.fluidx_(fu, fb, ip(nz), ip(nx), ip(ny), d)
        L.transpose13_(fu, fb, fu, fb, ip(nz), ip(nx), ip(ny))
        L.advectbyzx_(fu, fb, ip(ny), ip(nx), ip(nz), d)
        L.fluidx_(fu, fb, ip(ny), ip(nx), ip(nz), d)
        L.transpose12_(fu, fb, fu, fb, ip(ny), ip(nx), ip(nz))
        L.advectbyzx_(fu, fb, ip(nx), ip(ny), ip(nz), d)
        L.fluidx_(fu, fb, ip(nx), ip(ny), ip(nz), d)
        dts.append(dt)
    return np.array(dts, dtype=np.float32)


@pytest.mark.parametrize("dims", [(24, 1, 24), (16, 4, 16)])
@pytest.mark.parametrize("kind", ["sound", "cp_alfven", "alfven", "magnetic", "magnetosonic", "oblique"])
def test_fortran_driver_through_shim_matches_oracle(gpu, oracle_lib, kind, dims):
    import ics
    nx, ny, nz = dims
    u0, b0 = ics.fortran_ic(kind, nx, ny, nz)
    L = gpu.lib()
    L.mhdgpu_compat_status()
    u, b = u0.copy(), b0.copy()
    dts = fortran_loop(L, u, b, nx, ny, nz, 6, tf=10.0 * nx)
    assert L.mhdgpu_compat_status() == 0
    assert len(dts) == 6 and np.all(dts > 0)
    O = oracle_lib.oracle("f32")
    ru, rb = u0.copy(), b0.copy()
    for i, dt in enumerate(dts):
        inv = O.calcfl_averaged(ru, rb, nx, ny, nz)
        assert np.float32(0.9) * np.float32(inv) == dt, i     # the shim's CFL is the oracle's
        O.step(ru, rb, nx, ny, nz, dt)
    assert max(field_errors(u, ru, 5)) < TOL, field_errors(u, ru, 5)
    assert max(field_errors(b, rb, 3)) < TOL, field_errors(b, rb, 3)


@pytest.mark.parametrize("kind", ["cp_alfven", "magnetosonic", "oblique"])
def test_fortran_states_on_device_loop(gpu, oracle_lib, kind):
    """mhdgpu_advance (transpose-free step, averaged CFL) vs the oracle run."""
    import ics
    import torch
    nx, ny, nz = 32, 2, 32
    u0, b0 = ics.fortran_ic(kind, nx, ny, nz)
    du, db = torch.from_numpy(u0.copy()).cuda(), torch.from_numpy(b0.copy()).cuda()
    work = torch.empty(gpu.step_workspace_bytes(nx, ny, nz, gpu.MHD_PATH_FUSED), dtype=torch.uint8, device="cuda")
    clock = gpu.new_clock()
    log = torch.zeros(10, dtype=torch.float32, device="cuda")
    gpu.advance(du, db, nx, ny, nz, 10, 0.9, gpu.MHD_CFL_AVERAGED, 0.0, clock, log, work, gpu.MHD_PATH_FUSED)
    torch.cuda.synchronize()
    O = oracle_lib.oracle("f32")
    ru, rb = u0.copy(), b0.copy()
    steps, _t, dts = O.run(ru, rb, nx, ny, nz, cfl_number=0.9, cfl_mode=1, max_steps=10)
    assert steps == 10 and np.array_equal(dts, log.cpu().numpy())
    assert max(field_errors(du.cpu().numpy(), ru, 5)) < TOL
    assert max(field_errors(db.cpu().numpy(), rb, 3)) < TOL
