"""Python front end of libmhdgpu.so (ctypes over the C ABI in include/mhdgpu.h).

Device buffers are torch CUDA tensors (flat float32, reference layout); the
calls are issued on torch's current CUDA stream.  The library is required:
importing works without it, but every call raises if libmhdgpu.so is missing
or fails to load.  There is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# MHDGPU_LIB selects another build of the library, e.g. the debug build
# lib/libmhdgpu_debug.so (build.py --debug)
LIB_PATH = os.environ.get("MHDGPU_LIB") or os.path.join(HERE, "lib", "libmhdgpu.so")

MHD_OK = 0
MHD_ERR_ARG = 1
MHD_ERR_CUDA = 2
MHD_ERR_TIMEOUT = 3
MHD_ERR_UNPHYSICAL = 4
MHD_ERR_NOMEM = 5
MHD_CFL_C = 0
MHD_CFL_AVERAGED = 1
MHD_ADVANCE_RESUME = 0x100   # or'ed into cfl_mode of advance(): reuse the folded CFL word
MHD_HEALTH_NONFINITE = 1
MHD_HEALTH_DENSITY = 2
MHD_HEALTH_PRESSURE = 4
MHD_HEALTH_STALL = 8
MHD_BATCH_MAX_PENCIL = 256
KCLASS = {"fluidx": 0, "advectbyzx": 1, "transpose": 2, "cfl": 3, "batch": 4}

# every symbol the C headers declare
EXPORTS = [
    "mhdgpu_status_string", "mhdgpu_last_error", "mhdgpu_version",
    "mhdgpu_fluidx", "mhdgpu_advectbyzx_scratch_bytes", "mhdgpu_advectbyzx",
    "mhdgpu_advectbyzx_noalloc",
    "mhdgpu_transpose12", "mhdgpu_transpose13", "mhdgpu_cfl", "mhdgpu_dt_update",
    "mhdgpu_copy_matrix", "mhdgpu_step_workspace_bytes", "mhdgpu_step", "mhdgpu_advance",
    "mhdgpu_step_fused_workspace_bytes", "mhdgpu_step_fused",
    "mhdgpu_run_host", "mhdgpu_release_host_cache", "mhdgpu_resolve_path", "mhdgpu_path_workspace_bytes",
    "mhdgpu_set_math", "mhdgpu_set_row_staging", "mhdgpu_set_poison", "mhdgpu_set_tile", "mhdgpu_get_tile",
    "mhdgpu_debug_build", "mhdgpu_debug_faults", "mhdgpu_debug_selftest",
    "mhdgpu_autotune", "mhdgpu_tile_cache_save", "mhdgpu_tile_cache_load", "mhdgpu_profiler_create", "mhdgpu_profiler_destroy",
    "mhdgpu_profiler_attach", "mhdgpu_profiler_reset", "mhdgpu_profiler_summary",
    "mhdgpu_diagnostics_scratch_bytes", "mhdgpu_diagnostics",
    "mhdgpu_read_state", "mhdgpu_write_state", "mhdgpu_write_result", "mhdgpu_write_check",
    "mhdgpu_batch_workspace_bytes", "mhdgpu_batch_create", "mhdgpu_batch_destroy",
    "mhdgpu_batch_advance", "mhdgpu_batch_resume", "mhdgpu_batch_run_host", "mhdgpu_batch_read_clocks",
    "mhdgpu_batch_set_schedule",
    "mhdgpu_batch_get_schedule", "mhdgpu_batch_tune", "mhdgpu_batch_inject_stall",
    "mhdgpu_batch_schedule_save", "mhdgpu_batch_schedule_load",
    # include/mhdgpu_compat.h
    "fluidx", "advectbyzx", "transpose12", "transpose13", "calcfl", "copy_matrix",
    "mhdgpu_compat_status",
    # include/mhdgpu_fortran.h
    "fluidx_", "advectbyzx_", "transpose12_", "transpose13_", "cfl_",
]


class MhdError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"status {status}: {msg}")
        self.status = status


class Clock(C.Structure):
    """mhdgpu_clock"""
    _fields_ = [("t", C.c_float), ("dt", C.c_float), ("inv_c", C.c_float),
                ("cmax", C.c_uint), ("health", C.c_uint), ("iter", C.c_int)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build() "
                               "or python mhd-gpu_gb300/build.py")
        L = C.CDLL(LIB_PATH, mode=os.RTLD_LOCAL)
        P, I, F, D, S = C.c_void_p, C.c_int, C.c_float, C.c_double, C.c_size_t
        sig = {
            "mhdgpu_status_string": (C.c_char_p, [I]),
            "mhdgpu_last_error": (C.c_char_p, []),
            "mhdgpu_version": (C.c_char_p, []),
            "mhdgpu_fluidx": (I, [P, P, P, I, I, I, P, P, P]),
            "mhdgpu_advectbyzx_scratch_bytes": (S, [I, I, I]),
            "mhdgpu_advectbyzx": (I, [P, P, I, I, I, P, P, P]),
            "mhdgpu_advectbyzx_noalloc": (I, [P, P, I, I, I, P, P]),
            "mhdgpu_transpose12": (I, [P, P, P, P, I, I, I, P]),
            "mhdgpu_transpose13": (I, [P, P, P, P, I, I, I, P]),
            "mhdgpu_cfl": (I, [P, P, I, I, I, I, P, P, P]),
            "mhdgpu_dt_update": (I, [P, D, F, P, P, P]),
            "mhdgpu_copy_matrix": (I, [P, P, P, P, I, I, I, P]),
            "mhdgpu_step_workspace_bytes": (S, [I, I, I]),
            "mhdgpu_step": (I, [P, P, I, I, I, P, P, P, P]),
            "mhdgpu_step_fused_workspace_bytes": (S, [I, I, I]),
            "mhdgpu_resolve_path": (I, [I, I, I]),
            "mhdgpu_path_workspace_bytes": (S, [I, I, I, I]),
            "mhdgpu_step_fused": (I, [P, P, I, I, I, P, P, P, P]),
            "mhdgpu_advance": (I, [P, P, I, I, I, I, D, I, F, P, P, P, I, P]),
            "mhdgpu_run_host": (I, [P, P, I, I, I, D, I, P, F, I, P, P, I]),
            "mhdgpu_release_host_cache": (I, []),
            "mhdgpu_set_math": (I, [I]),
            "mhdgpu_set_row_staging": (I, [I]),
            "mhdgpu_set_poison": (I, [I]),
            "mhdgpu_debug_build": (I, []),
            "mhdgpu_debug_faults": (I, [P, P, P, P, P, P]),
            "mhdgpu_debug_selftest": (I, [C.c_longlong, C.c_longlong, P]),
            "mhdgpu_set_tile": (I, [I, I, I, I, I]),
            "mhdgpu_get_tile": (I, [I, I, P, P, P]),
            "mhdgpu_autotune": (I, [I, I, I, I]),
            "mhdgpu_tile_cache_save": (I, [C.c_char_p]),
            "mhdgpu_tile_cache_load": (I, [C.c_char_p, P]),
            "mhdgpu_profiler_create": (I, [P, I]),
            "mhdgpu_profiler_destroy": (I, [P]),
            "mhdgpu_profiler_attach": (I, [P]),
            "mhdgpu_profiler_reset": (I, [P]),
            "mhdgpu_profiler_summary": (I, [P, I, P, P, P]),
            "mhdgpu_diagnostics_scratch_bytes": (S, [I, I, I]),
            "mhdgpu_diagnostics": (I, [P, P, I, I, I, P, P, P]),
            "mhdgpu_read_state": (I, [C.c_char_p, P, P, I, I, I]),
            "mhdgpu_write_state": (I, [C.c_char_p, P, P, I, I, I]),
            "mhdgpu_write_result": (I, [C.c_char_p, C.c_char_p, P, P, I, I, I]),
            "mhdgpu_write_check": (I, [C.c_char_p, P, P, I, I, I]),
            "mhdgpu_batch_workspace_bytes": (S, [I, P]),
            "mhdgpu_batch_create": (I, [P, I, P, P, P, D, I, P]),
            "mhdgpu_batch_destroy": (I, [P]),
            "mhdgpu_batch_advance": (I, [P, I, P]),
            "mhdgpu_batch_resume": (I, [P, I, P]),
            "mhdgpu_batch_run_host": (I, [P, P, P, I, P]),
            "mhdgpu_batch_read_clocks": (I, [P, P, P]),
            "mhdgpu_batch_set_schedule": (I, [P, I, I, I]),
            "mhdgpu_batch_get_schedule": (I, [P, I, P, P]),
            "mhdgpu_batch_tune": (I, [P, P]),
            "mhdgpu_batch_schedule_save": (I, [P, C.c_char_p]),
            "mhdgpu_batch_schedule_load": (I, [P, C.c_char_p, P]),
            "mhdgpu_batch_inject_stall": (I, [P]),
            "calcfl": (F, [P, P, P, P, P]),
            "cfl_": (F, [P, P, P, P, P]),
            "mhdgpu_compat_status": (I, []),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(status: int):
    if status != MHD_OK:
        raise MhdError(status, lib().mhdgpu_last_error().decode())


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _host_ptr(x):
    """Address of a host float32 buffer: a CPU tensor (pinned or not) or a
    C-contiguous numpy array."""
    if hasattr(x, "data_ptr"):
        assert not x.is_cuda and x.is_contiguous()
        return x.data_ptr()
    assert x.flags["C_CONTIGUOUS"]
    return x.ctypes.data


def _stream(stream=None):
    import torch
    s = torch.cuda.current_stream() if stream is None else stream
    return C.c_void_p(s.cuda_stream)


def fluidx(u_out, u_in, b, nx, ny, nz, d_dt, health=None, stream=None):
    _check(lib().mhdgpu_fluidx(_p(u_out), _p(u_in), _p(b), nx, ny, nz, _p(d_dt), _p(health),
                               _stream(stream)))


def advectbyzx_scratch_bytes(nx, ny, nz) -> int:
    return int(lib().mhdgpu_advectbyzx_scratch_bytes(nx, ny, nz))


def advectbyzx(b, u, nx, ny, nz, d_dt, scratch, stream=None):
    _check(lib().mhdgpu_advectbyzx(_p(b), _p(u), nx, ny, nz, _p(d_dt), _p(scratch), _stream(stream)))


def transpose12(dst_u, dst_b, src_u, src_b, nx, ny, nz, stream=None):
    _check(lib().mhdgpu_transpose12(_p(dst_u), _p(dst_b), _p(src_u), _p(src_b), nx, ny, nz,
                                    _stream(stream)))


def transpose13(dst_u, dst_b, src_u, src_b, nx, ny, nz, stream=None):
    _check(lib().mhdgpu_transpose13(_p(dst_u), _p(dst_b), _p(src_u), _p(src_b), nx, ny, nz,
                                    _stream(stream)))


def cfl(u, b, nx, ny, nz, mode, d_inv_c, d_word, stream=None):
    _check(lib().mhdgpu_cfl(_p(u), _p(b), nx, ny, nz, mode, _p(d_inv_c), _p(d_word), _stream(stream)))


def dt_update(d_inv_c, cfl_number, tf, d_t, d_dt, stream=None):
    _check(lib().mhdgpu_dt_update(_p(d_inv_c), float(cfl_number), float(tf), _p(d_t), _p(d_dt),
                                  _stream(stream)))


MHD_PATH_PLAIN = 0
MHD_PATH_FUSED = 1
MHD_PATH_AUTO = 2


def step_workspace_bytes(nx, ny, nz, path=MHD_PATH_PLAIN) -> int:
    return int(lib().mhdgpu_path_workspace_bytes(nx, ny, nz, int(path)))


def resolve_path(nx, ny, nz) -> int:
    """The path MHD_PATH_AUTO takes for the box (mhdgpu_resolve_path)."""
    return int(lib().mhdgpu_resolve_path(nx, ny, nz))


def step(u, b, nx, ny, nz, d_dt, work, health=None, stream=None):
    _check(lib().mhdgpu_step(_p(u), _p(b), nx, ny, nz, _p(d_dt), _p(work), _p(health),
                             _stream(stream)))


def step_fused(u, b, nx, ny, nz, d_dt, work, health=None, stream=None):
    _check(lib().mhdgpu_step_fused(_p(u), _p(b), nx, ny, nz, _p(d_dt), _p(work), _p(health),
                                   _stream(stream)))


def advance(u, b, nx, ny, nz, nsteps, cfl_number, cfl_mode, tf, clock, dt_log, work,
            path=MHD_PATH_PLAIN, stream=None, resume=False):
    """clock: a torch uint8 CUDA tensor of sizeof(Clock) bytes (see new_clock).
    resume: the first step takes the CFL speed folded into the clock by the
    previous advance of this unchanged state (MHD_ADVANCE_RESUME)."""
    mode = int(cfl_mode) | (MHD_ADVANCE_RESUME if resume else 0)
    _check(lib().mhdgpu_advance(_p(u), _p(b), nx, ny, nz, int(nsteps), float(cfl_number),
                                mode, float(tf), _p(clock), _p(dt_log), _p(work),
                                int(path), _stream(stream)))


def new_clock(device="cuda", t=0.0):
    import torch
    host = Clock()
    host.t = t
    raw = bytes(host)
    return torch.tensor(list(raw), dtype=torch.uint8, device=device)


def read_clock(clock) -> Clock:
    data = bytes(clock.cpu().numpy().tobytes())
    return Clock.from_buffer_copy(data)


def run_host(u, b, nx, ny, nz, cfl_number=0.9, cfl_mode=MHD_CFL_C, t=0.0, tf=0.0,
             max_steps=1, dt_log=None, path=MHD_PATH_PLAIN):
    """End-to-end call on host numpy arrays (float32, modified in place).

    Returns (status, t, steps_done); status MHD_ERR_UNPHYSICAL is returned, not
    raised, so that the caller can inspect the state."""
    import numpy as np
    assert u.dtype == np.float32 and b.dtype == np.float32
    tt = C.c_float(t)
    done = C.c_int(0)
    log_ptr = None if dt_log is None else dt_log.ctypes.data_as(C.c_void_p)
    st = lib().mhdgpu_run_host(u.ctypes.data_as(C.c_void_p), b.ctypes.data_as(C.c_void_p), nx, ny,
                               nz, float(cfl_number), int(cfl_mode), C.byref(tt), float(tf),
                               int(max_steps), log_ptr, C.byref(done), int(path))
    if st not in (MHD_OK, MHD_ERR_UNPHYSICAL):
        _check(st)
    return st, tt.value, done.value


def release_host_cache():
    """Frees this thread's device buffers and stream kept by run_host."""
    _check(lib().mhdgpu_release_host_cache())


MHD_MATH_FAITHFUL = 0
MHD_MATH_FAST = 1
MHD_MATH_FP64P = 2


def set_math(mode: int) -> int:
    """Select the arithmetic policy of the pencil kernels; returns the previous one."""
    prev = lib().mhdgpu_set_math(int(mode))
    if prev < 0:
        raise MhdError(MHD_ERR_ARG, lib().mhdgpu_last_error().decode())
    return prev


MHD_STAGING_TMA = 0
MHD_STAGING_CPASYNC = 1


def set_row_staging(mode: int) -> int:
    """How the transpose-free step moves its y/z pencils (MHD_STAGING_TMA or
    MHD_STAGING_CPASYNC; the calling thread's setting); returns the previous one."""
    prev = lib().mhdgpu_set_row_staging(int(mode))
    if prev < 0:
        raise MhdError(MHD_ERR_ARG, lib().mhdgpu_last_error().decode())
    return prev


# source files of the debug build's index checks, by their number in a record
DEBUG_FILES = {1: "fluidx_reg.cuh", 2: "fluidx_kernel.cuh", 3: "advect_reg.cuh", 4: "advect_kernel.cuh",
               5: "batch_kernel.cuh", 6: "transpose.cu", 7: "cfl_kernel.cuh", 8: "tma_rows.cuh",
               9: "mhd_common.cuh", 10: "debug.cu"}
DEBUG_KINDS = {1: "index", 2: "shared", 3: "global"}


def debug_build() -> bool:
    """True when the loaded library is the debug build (every kernel index checked)."""
    return bool(lib().mhdgpu_debug_build())


def debug_faults() -> dict:
    """Synchronises the device and returns the index faults recorded by the
    debug build since the last call: {'count', 'kind', 'file', 'line',
    'index', 'extent'} of the first one (count 0 in the release build)."""
    c, k, f, ln = C.c_uint(), C.c_uint(), C.c_uint(), C.c_uint()
    i, n = C.c_longlong(), C.c_longlong()
    _check(lib().mhdgpu_debug_faults(C.byref(c), C.byref(k), C.byref(f), C.byref(ln), C.byref(i), C.byref(n)))
    if c.value == 0:
        return {"count": 0}
    return {"count": c.value, "kind": DEBUG_KINDS.get(k.value, k.value), "file": DEBUG_FILES.get(f.value, f.value),
            "line": ln.value, "index": i.value, "extent": n.value}


def debug_selftest(index: int, extent: int) -> bool:
    """Checks index against extent in a one-thread kernel (mhdgpu_debug_selftest):
    whether the check passed (always True in the release build)."""
    r = C.c_int()
    _check(lib().mhdgpu_debug_selftest(int(index), int(extent), C.byref(r)))
    return bool(r.value)


def set_poison(on: bool) -> bool:
    """Fill every entry's scratch with NaN before use (a debugging aid; the
    calling thread's setting); returns the previous setting."""
    return bool(lib().mhdgpu_set_poison(1 if on else 0))


MHD_TILE_ROWS = 16


def set_tile(kclass: str, n: int, cpl: int, wpp: int, ppc: int, rows: bool = False):
    """rows: the shape for pencils that run across memory (transpose-free y/z sweeps)."""
    _check(lib().mhdgpu_set_tile(KCLASS[kclass] | (MHD_TILE_ROWS if rows else 0), n, cpl, wpp, ppc))


def get_tile(kclass: str, n: int, rows: bool = False):
    c, w, p = C.c_int(), C.c_int(), C.c_int()
    _check(lib().mhdgpu_get_tile(KCLASS[kclass] | (MHD_TILE_ROWS if rows else 0), n,
                                 C.byref(c), C.byref(w), C.byref(p)))
    return c.value, w.value, p.value


def autotune(nx: int, ny: int, nz: int, math: int = MHD_MATH_FAITHFUL):
    """Time every compiled team shape for the pencil lengths of this box and
    keep the fastest (mhdgpu_autotune); returns {(kclass, n, rows): shape}."""
    _check(lib().mhdgpu_autotune(nx, ny, nz, int(math)))
    out = {}
    for k in ("fluidx", "advectbyzx"):
        for n in sorted({nx, ny, nz}):
            out[(k, n, False)] = get_tile(k, n)
        for n in sorted({ny, nz}):
            out[(k, n, True)] = get_tile(k, n, rows=True)
    return out


def tile_cache_save(path: str) -> None:
    """Write the tile shapes set in this process (mhdgpu_tile_cache_save)."""
    _check(lib().mhdgpu_tile_cache_save(os.fsencode(path)))


def tile_cache_load(path: str) -> int:
    """Set the tile shapes a cache file holds for this device; returns how many."""
    n = C.c_int()
    _check(lib().mhdgpu_tile_cache_load(os.fsencode(path), C.byref(n)))
    return n.value


class Profiler:
    """Per-kernel-class device time from CUDA events (mhdgpu_profiler_*).

    Use as a context manager around the C-ABI calls to time; ``summary()``
    returns {class: (records, launches, total_ms)}."""

    def __init__(self, max_records=100000):
        self.h = C.c_void_p()
        _check(lib().mhdgpu_profiler_create(C.byref(self.h), int(max_records)))

    def __enter__(self):
        _check(lib().mhdgpu_profiler_attach(self.h))
        return self

    def __exit__(self, *exc):
        lib().mhdgpu_profiler_attach(None)
        return False

    def reset(self):
        _check(lib().mhdgpu_profiler_reset(self.h))

    def summary(self):
        out = {}
        for name, k in KCLASS.items():
            r, n, ms = C.c_int(), C.c_int(), C.c_double()
            _check(lib().mhdgpu_profiler_summary(self.h, k, C.byref(r), C.byref(n), C.byref(ms)))
            out[name] = (r.value, n.value, ms.value)
        return out

    def close(self):
        if self.h:
            lib().mhdgpu_profiler_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _host_f32(a, n):
    import numpy as np
    if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous and a.size == n):
        raise ValueError("expected a C-contiguous float32 numpy array of %d elements" % n)
    return a.ctypes.data_as(C.c_void_p)


def read_state(path, nx, ny, nz):
    """The reference's init file (Heterogeneous_MHD/C/init.c:33-66) -> (u, b) numpy."""
    import numpy as np
    n = nx * ny * nz
    u = np.empty(5 * n, dtype=np.float32)
    b = np.empty(3 * n, dtype=np.float32)
    _check(lib().mhdgpu_read_state(os.fsencode(path), _host_f32(u, 5 * n), _host_f32(b, 3 * n), nx, ny, nz))
    return u, b


def write_state(path, u, b, nx, ny, nz):
    n = nx * ny * nz
    _check(lib().mhdgpu_write_state(os.fsencode(path), _host_f32(u, 5 * n), _host_f32(b, 3 * n), nx, ny, nz))


def write_result(path_u, path_b, u, b, nx, ny, nz):
    n = nx * ny * nz
    _check(lib().mhdgpu_write_result(os.fsencode(path_u), os.fsencode(path_b), _host_f32(u, 5 * n),
                                     _host_f32(b, 3 * n), nx, ny, nz))


def write_check(prefix, u, b, nx, ny, nz):
    n = nx * ny * nz
    _check(lib().mhdgpu_write_check(os.fsencode(prefix), _host_f32(u, 5 * n), _host_f32(b, 3 * n), nx, ny, nz))


DIAG_NAMES = ("mass", "m_x", "m_y", "m_z", "energy", "max_div_b", "min_p", "cells_p_nonpositive")


def diagnostics(u, b, nx, ny, nz, stream=None) -> dict:
    """FP64 totals, max |div B|, min p and the count of p <= 0 cells of a device
    state (mhdgpu_diagnostics); synchronises the stream to return host values."""
    import torch
    out = torch.empty(8, dtype=torch.float64, device=u.device)
    scr = torch.empty(int(lib().mhdgpu_diagnostics_scratch_bytes(nx, ny, nz)), dtype=torch.uint8,
                      device=u.device)
    _check(lib().mhdgpu_diagnostics(_p(u), _p(b), nx, ny, nz, _p(out), _p(scr), _stream(stream)))
    vals = out.cpu().tolist()
    return dict(zip(DIAG_NAMES, vals))


def batch_workspace_bytes(dims) -> int:
    """Device bytes mhdgpu_batch_create allocates for boxes of these sizes (0 if invalid)."""
    flat = [int(v) for d in dims for v in d]
    arr = (C.c_int * len(flat))(*flat)
    return int(lib().mhdgpu_batch_workspace_bytes(len(dims), arr))


class Batch:
    """Batched ensemble (mhdgpu_batch_*): boxes[i] = (u, b, (nx, ny, nz)) with u, b
    flat float32 CUDA tensors in the reference layout, advanced in place.

    The tensors must outlive the handle; the handle keeps references to them."""

    def __init__(self, boxes, cfl_number=0.7, cfl_mode=MHD_CFL_C, tf=None):
        self.boxes = list(boxes)
        n = len(self.boxes)
        flat = [int(v) for _, _, d in self.boxes for v in d]
        dims = (C.c_int * len(flat))(*flat)
        us = (C.c_void_p * n)(*[u.data_ptr() for u, _, _ in self.boxes])
        bs = (C.c_void_p * n)(*[b.data_ptr() for _, b, _ in self.boxes])
        tfa = None if tf is None else (C.c_float * n)(*[float(x) for x in tf])
        self.h = C.c_void_p()
        _check(lib().mhdgpu_batch_create(C.byref(self.h), n, dims, us, bs, float(cfl_number),
                                         int(cfl_mode), tfa))

    def advance(self, nsteps=1, stream=None, resume=False):
        """resume: continue the previous advance of the unchanged boxes without
        the first step's CFL pass (mhdgpu_batch_resume)."""
        fn = lib().mhdgpu_batch_resume if resume else lib().mhdgpu_batch_advance
        _check(fn(self.h, int(nsteps), _stream(stream)))

    def run_host(self, host_u, host_b, nsteps=1, stream=None):
        """Uploads every box from host_u[i], host_b[i] (CPU float32 arrays or
        tensors, pinned for speed), advances nsteps steps, downloads into the
        same buffers and synchronises (mhdgpu_batch_run_host)."""
        n = len(self.boxes)
        hu = (C.c_void_p * n)(*[_host_ptr(x) for x in host_u])
        hb = (C.c_void_p * n)(*[_host_ptr(x) for x in host_b])
        _check(lib().mhdgpu_batch_run_host(self.h, hu, hb, int(nsteps), _stream(stream)))

    def clocks(self, stream=None, check=True):
        """Synchronises and returns the boxes' Clock records; with check, raises on
        a stall (MHD_ERR_TIMEOUT) or an unphysical box (MHD_ERR_UNPHYSICAL)."""
        out = (Clock * len(self.boxes))()
        st = lib().mhdgpu_batch_read_clocks(self.h, out, _stream(stream))
        if check:
            _check(st)
        return list(out)

    def set_schedule(self, axis, threads, ctas_per_sm):
        _check(lib().mhdgpu_batch_set_schedule(self.h, int(axis), int(threads), int(ctas_per_sm)))

    def get_schedule(self, axis):
        t, c = C.c_int(), C.c_int()
        _check(lib().mhdgpu_batch_get_schedule(self.h, int(axis), C.byref(t), C.byref(c)))
        return t.value, c.value

    def save_schedule(self, path):
        """Write the schedule with the batch's signature (mhdgpu_batch_schedule_save)."""
        _check(lib().mhdgpu_batch_schedule_save(self.h, os.fsencode(path)))

    def load_schedule(self, path) -> bool:
        """Apply a saved schedule if it was made for this batch on this device model."""
        ok = C.c_int()
        _check(lib().mhdgpu_batch_schedule_load(self.h, os.fsencode(path), C.byref(ok)))
        return bool(ok.value)

    def tune(self, stream=None):
        """Autotune the block schedule per axis; returns [(threads, ctas_per_sm)] * 3."""
        _check(lib().mhdgpu_batch_tune(self.h, _stream(stream)))
        return [self.get_schedule(a) for a in range(3)]

    def inject_stall(self):
        """Failure-path test hook (mhdgpu_batch_inject_stall)."""
        _check(lib().mhdgpu_batch_inject_stall(self.h))

    def close(self):
        if self.h:
            lib().mhdgpu_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
