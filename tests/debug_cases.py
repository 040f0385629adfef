"""Cases of the debug-build test (tests/test_gpu_debug.py): every kernel family
on odd shapes, run through whichever library mhdgpu loads.

    MHDGPU_LIB=mhd-gpu_gb300/lib/libmhdgpu_debug.so python tests/debug_cases.py out.npz [--poison]

writes every case's output state into out.npz, with the debug build's fault
record ('faults', JSON) and whether the library is the debug build.  The test
runs the same cases through the release library in its own process and
compares the arrays bit for bit.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
for _p in (os.path.join(REPO, "mhd-gpu_gb300"), HERE):
    if _p not in sys.path:
        sys.path.insert(0, _p)

# subroutine shapes: non-cubic, odd, tiny, long x pencils, register-blocked
# lengths (32/48/64/96/128) and team-tile lengths
SUB_SHAPES = [(12, 20, 28), (5, 7, 9), (33, 17, 9), (100, 3, 2), (48, 40, 24), (128, 4, 3), (1, 4, 5),
              (64, 6, 10), (96, 5, 3)]
# whole steps, both paths: full and partial row tiles, row strides that are
# and are not multiples of 4 cells (vector staging and its fallback)
STEP_SHAPES = [(12, 20, 28), (48, 40, 24), (36, 32, 64), (10, 32, 32), (32, 48, 96), (20, 30, 40)]
# batched boxes: the 32/48/64/96/128 classes and others along each axis
BATCH_DIMS = [(32, 48, 64), (96, 32, 48), (48, 64, 32), (20, 30, 40), (128, 32, 16), (64, 96, 20)]


def run_cases() -> dict:
    import torch

    import ics
    import mhdgpu

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()

    def host(t):
        torch.cuda.synchronize()
        return t.cpu().numpy()

    out = {}
    dt = torch.tensor([0.03], dtype=torch.float32, device="cuda")
    for dims in SUB_SHAPES:
        tag = "x".join(map(str, dims))
        u, b = ics.random_state(*dims, seed=sum(dims))
        du, db = dev(u), dev(b)
        fo = torch.zeros_like(du)
        mhdgpu.fluidx(fo, du, db, *dims, dt)
        out[f"fluidx_{tag}"] = host(fo)
        bb = dev(b)
        scr = torch.empty(mhdgpu.advectbyzx_scratch_bytes(*dims) // 4, device="cuda")
        mhdgpu.advectbyzx(bb, du, *dims, dt, scr)
        out[f"advect_{tag}"] = host(bb)
        for name, fn in (("t12", mhdgpu.transpose12), ("t13", mhdgpu.transpose13)):
            tu, tb = torch.zeros_like(du), torch.zeros_like(db)
            fn(tu, tb, du, db, *dims)
            out[f"{name}_u_{tag}"], out[f"{name}_b_{tag}"] = host(tu), host(tb)
        for mode in (mhdgpu.MHD_CFL_C, mhdgpu.MHD_CFL_AVERAGED):
            inv = torch.zeros(1, dtype=torch.float32, device="cuda")
            word = torch.zeros(1, dtype=torch.int32, device="cuda")
            mhdgpu.cfl(du, db, *dims, mode, inv, word)
            out[f"cfl{mode}_{tag}"] = host(inv)
    for dims in STEP_SHAPES:
        tag = "x".join(map(str, dims))
        u, b = ics.random_state(*dims, seed=3 * sum(dims), amp=0.2)
        for path in (mhdgpu.MHD_PATH_PLAIN, mhdgpu.MHD_PATH_FUSED):
            for staging in ((mhdgpu.MHD_STAGING_CPASYNC, mhdgpu.MHD_STAGING_TMA)
                            if path == mhdgpu.MHD_PATH_FUSED else (mhdgpu.MHD_STAGING_CPASYNC,)):
                prev = mhdgpu.set_row_staging(staging)
                du, db = dev(u), dev(b)
                work = torch.empty(mhdgpu.step_workspace_bytes(*dims, path), dtype=torch.uint8, device="cuda")
                clock = mhdgpu.new_clock()
                mhdgpu.advance(du, db, *dims, 2, 0.7, mhdgpu.MHD_CFL_C, 0.0, clock, None, work, path)
                mhdgpu.set_row_staging(prev)
                out[f"step{path}_{staging}_u_{tag}"], out[f"step{path}_{staging}_b_{tag}"] = host(du), host(db)
    boxes = []
    for i, dims in enumerate(BATCH_DIMS):
        u, b = ics.turbulence(*dims, seed=i, v_rms=0.05, db_rms=0.05)
        boxes.append((dev(u), dev(b), dims))
    bt = mhdgpu.Batch(boxes, cfl_number=0.7, cfl_mode=mhdgpu.MHD_CFL_C)
    bt.advance(2)
    for i, (du, db, dims) in enumerate(boxes):
        out[f"batch_u_{i}"], out[f"batch_b_{i}"] = host(du), host(db)
    bt.close()
    return out


def main() -> None:
    import torch

    import mhdgpu
    torch.cuda.set_device(0)
    poison = "--poison" in sys.argv
    if poison:
        mhdgpu.set_poison(True)
    out = run_cases()
    faults = mhdgpu.debug_faults()
    np.savez(sys.argv[1], faults=np.array(json.dumps(faults)), debug=np.array(mhdgpu.debug_build()), **out)


if __name__ == "__main__":
    main()
