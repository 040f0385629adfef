"""The transpose-free step with its y/z fluid tiles moved by TMA tensor copies
(MHD_STAGING_TMA, tma_rows.cuh) against the same step with the default
staging (MHD_STAGING_CPASYNC: 16-byte quads of four pencils for full tiles,
4-byte row copies otherwise) and against the plain step: bit for bit.

The boxes cover pencils of 32, 64 and 128 cells along y and z (the lengths
that take the TMA tile), full and partial last tiles (a j extent that is not
a multiple of 8), the periodic j+1 column of the last tile, one- and
two-tile planes, and a box whose row stride is not a multiple of 4 cells
(nx = 10: both modes fall back to the row copies)."""
import numpy as np
import pytest

from util import bits_equal, field_errors

pytestmark = pytest.mark.gpu

BOXES = [(20, 32, 64), (12, 64, 32), (8, 128, 16), (36, 32, 128), (16, 64, 64), (10, 32, 32),
         (4, 32, 128), (128, 128, 8)]


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _fused(gpu, u, b, dims, staging, nsteps=2):
    import torch
    prev = gpu.set_row_staging(staging)
    try:
        du, db = dev(u), dev(b)
        work = torch.empty(gpu.step_workspace_bytes(*dims, gpu.MHD_PATH_FUSED), dtype=torch.uint8, device="cuda")
        d_dt = torch.tensor([0.04], dtype=torch.float32, device="cuda")
        health = torch.zeros(1, dtype=torch.int32, device="cuda")
        for _ in range(nsteps):
            gpu.step_fused(du, db, *dims, d_dt, work, health)
        return host(du), host(db), int(host(health)[0])
    finally:
        gpu.set_row_staging(prev)


@pytest.mark.parametrize("dims", BOXES)
def test_tma_staging_equals_row_copies_and_plain(gpu, dims):
    import torch
    import ics
    u, b = ics.random_state(*dims, seed=sum(dims), amp=0.2)
    tu, tb, th = _fused(gpu, u, b, dims, gpu.MHD_STAGING_TMA)
    cu, cb, ch = _fused(gpu, u, b, dims, gpu.MHD_STAGING_CPASYNC)
    assert th & gpu.MHD_HEALTH_STALL == 0
    assert bits_equal(tu, cu) and bits_equal(tb, cb), (field_errors(tu, cu, 5), field_errors(tb, cb, 3))
    du, db = dev(u), dev(b)
    work = torch.empty(gpu.step_workspace_bytes(*dims), dtype=torch.uint8, device="cuda")
    d_dt = torch.tensor([0.04], dtype=torch.float32, device="cuda")
    for _ in range(2):
        gpu.step(du, db, *dims, d_dt, work)
    assert bits_equal(host(du), tu) and bits_equal(host(db), tb)
