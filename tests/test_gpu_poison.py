"""Poison mode (mhdgpu_set_poison): every entry that takes scratch fills it
with NaN before use, so a kernel that read scratch before writing it would
carry NaN into the state.  Each path is run with and without poison on odd
and uneven boxes; the results must be equal bit for bit and finite."""
import numpy as np
import pytest

from util import bits_equal

pytestmark = pytest.mark.gpu

SHAPES = [(12, 20, 28), (5, 7, 9), (32, 48, 20), (64, 40, 12), (1, 4, 3), (96, 8, 16)]


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _run(gpu, poison, fn):
    prev = gpu.set_poison(poison)
    try:
        return fn()
    finally:
        gpu.set_poison(prev)


@pytest.mark.parametrize("dims", SHAPES)
@pytest.mark.parametrize("path", [0, 1])
def test_steps_read_no_scratch_before_writing_it(gpu, dims, path):
    import torch
    import ics
    u, b = ics.random_state(*dims, seed=3 + sum(dims), amp=0.2)

    def go():
        du, db = dev(u), dev(b)
        work = torch.empty(gpu.step_workspace_bytes(*dims, path), dtype=torch.uint8, device="cuda")
        clock = gpu.new_clock()
        gpu.advance(du, db, *dims, 2, 0.7, gpu.MHD_CFL_C, 0.0, clock, None, work, path)
        return host(du), host(db)

    pu, pb = _run(gpu, True, go)
    cu, cb = _run(gpu, False, go)
    assert np.isfinite(pu).all() and np.isfinite(pb).all()
    assert bits_equal(pu, cu) and bits_equal(pb, cb)


def test_advectbyzx_and_batch_with_poison(gpu):
    import torch
    import ics
    dims = (12, 20, 28)
    u, b = ics.random_state(*dims, seed=5, amp=0.2)

    def adv():
        db = dev(b)
        scr = torch.empty(gpu.advectbyzx_scratch_bytes(*dims) // 4, dtype=torch.float32, device="cuda")
        gpu.advectbyzx(db, dev(u), *dims, torch.tensor([0.04], device="cuda"), scr)
        return host(db)

    assert bits_equal(_run(gpu, True, adv), _run(gpu, False, adv))
    boxes_dims = [(8, 16, 24), (32, 48, 20), (5, 7, 9), (16, 96, 8), (48, 32, 64)]
    states = [ics.random_state(*d, seed=11 + i, amp=0.2) for i, d in enumerate(boxes_dims)]

    def batch():
        boxes = [(dev(x), dev(y), d) for (x, y), d in zip(states, boxes_dims)]
        bt = gpu.Batch(boxes, cfl_number=0.7)
        bt.advance(2)
        bt.clocks()
        out = [(host(x), host(y)) for x, y, _ in boxes]
        bt.close()
        return out

    p, c = _run(gpu, True, batch), _run(gpu, False, batch)
    for (pu, pb), (cu, cb) in zip(p, c):
        assert np.isfinite(pu).all() and bits_equal(pu, cu) and bits_equal(pb, cb)
