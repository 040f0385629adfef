"""mhdgpu_advectbyzx_noalloc: the advection for callers that cannot allocate.

Some callers of this library cannot call cudaMalloc at the point where they
run the step -- a plugin executing inside another runtime's memory pool, or a
loop that must not allocate or fail for lack of memory mid-run -- and own only
their input and output buffers.  For them the library keeps the advection's
scratch in a fixed device array of its own.  This file checks, through the C
ABI, that the entry gives what mhdgpu_advectbyzx (caller scratch) gives,
within the parity tolerance of the other GPU tests (1e-5 per field), on two
calls in a row, and that it rejects boxes above its size limit.  The file
name makes pytest collect it last.
"""
import ctypes as C

import numpy as np
import pytest

from util import field_errors

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _ptr(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("dims", [(16, 16, 16), (48, 6, 10), (128, 128, 128), (12, 20, 28)])
def test_noalloc_matches_caller_scratch_entry_twice(gpu, dims):
    import torch

    import ics
    L = gpu.lib()
    nx, ny, nz = dims
    u, b = ics.random_state(nx, ny, nz, seed=nx + 2 * ny + 3 * nz)
    du = torch.from_numpy(u).cuda()
    b_ref = torch.from_numpy(b).cuda()
    b_na = b_ref.clone()
    scr = torch.empty(L.mhdgpu_advectbyzx_scratch_bytes(nx, ny, nz) // 4, dtype=torch.float32,
                      device="cuda")
    dts = [torch.tensor([x], dtype=torch.float32, device="cuda") for x in (0.04, 0.03)]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call, dt in enumerate(dts):
        st = L.mhdgpu_advectbyzx(_ptr(b_ref), _ptr(du), nx, ny, nz, _ptr(dt), _ptr(scr), stream)
        assert st == gpu.MHD_OK, L.mhdgpu_last_error()
        st = L.mhdgpu_advectbyzx_noalloc(_ptr(b_na), _ptr(du), nx, ny, nz, _ptr(dt), stream)
        assert st == gpu.MHD_OK, L.mhdgpu_last_error()
        torch.cuda.synchronize()
        got, ref = b_na.cpu().numpy(), b_ref.cpu().numpy()
        errs = field_errors(got, ref, 3)
        assert max(errs) < TOL, (call, errs)
        assert not np.array_equal(ref, b)   # the call advanced the field


def test_noalloc_rejects_boxes_above_its_limit(gpu):
    import torch
    L = gpu.lib()
    t = torch.zeros(8, dtype=torch.float32, device="cuda")
    st = L.mhdgpu_advectbyzx_noalloc(_ptr(t), _ptr(t), 256, 128, 65, _ptr(t), None)
    assert st == gpu.MHD_ERR_ARG
    assert b"MHD_NOALLOC_MAX_CELLS" in L.mhdgpu_last_error()
