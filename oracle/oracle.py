"""ctypes front end of the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Loads ``oracle/lib/liboracle.so`` (the restatement of the reference C path,
float and double builds) and, where it was built, ``oracle/_ref/libref_*.so``
(the reference's own C path compiled from its sources by ``make ref``).
Both expose the reference subroutine signatures
(Heterogeneous_MHD/C/spu_function.h:1-15), so :class:`CPath` drives either.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
use this module.  The product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_ORACLE = os.path.join(HERE, "lib", "liboracle.so")
LIB_REF = {"f32": os.path.join(HERE, "_ref", "libref_f32.so"),
           "f64": os.path.join(HERE, "_ref", "libref_f64.so")}

_cache: dict = {}


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and the reference libraries when ``ref``)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _load(path: str) -> C.CDLL:
    if path not in _cache:
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        _cache[path] = C.CDLL(path, mode=os.RTLD_LOCAL)
    return _cache[path]


def ref_available(kind: str = "f32") -> bool:
    return os.path.exists(LIB_REF[kind])


def _ptr(a: np.ndarray):
    assert a.flags.c_contiguous
    return a.ctypes.data_as(C.c_void_p)


class CPath:
    """One build of the C-path subroutines (reference or restatement).

    ``prefix`` is ``""`` for the reference, ``oracle_`` / ``oracle64_`` for
    the restatement.  Arrays are flat numpy arrays in the reference layout.
    """

    def __init__(self, lib: C.CDLL, prefix: str, dtype):
        self.lib = lib
        self.p = prefix
        self.dtype = np.dtype(dtype)
        self.ct = C.c_float if self.dtype == np.float32 else C.c_double
        f = getattr(lib, prefix + "calcfl")
        f.restype = self.ct
        if hasattr(lib, prefix + "calcfl_averaged"):
            getattr(lib, prefix + "calcfl_averaged").restype = self.ct
        if hasattr(lib, prefix + "dt_from_cfl"):
            g = getattr(lib, prefix + "dt_from_cfl")
            g.restype = self.ct
            g.argtypes = [self.ct, C.c_double, self.ct, self.ct]
        if hasattr(lib, prefix + "run"):
            getattr(lib, prefix + "run").restype = C.c_int

    def _f(self, name):
        return getattr(self.lib, self.p + name)

    def _chk(self, *arrs):
        for a in arrs:
            assert a.dtype == self.dtype and a.flags.c_contiguous, (a.dtype, self.dtype)

    @staticmethod
    def _dims(nx, ny, nz):
        return C.byref(C.c_int(nx)), C.byref(C.c_int(ny)), C.byref(C.c_int(nz))

    def fluidx(self, u, b, nx, ny, nz, dt, update_u, update_b):
        self._chk(u, b, update_u, update_b)
        d = self.ct(dt)
        self._f("fluidx")(_ptr(u), _ptr(b), *self._dims(nx, ny, nz), C.byref(d),
                          _ptr(update_u), _ptr(update_b), C.c_int(0))

    def advectbyzx(self, u, b, nx, ny, nz, dt, update_u, update_b):
        self._chk(u, b, update_u, update_b)
        d = self.ct(dt)
        self._f("advectbyzx")(_ptr(u), _ptr(b), *self._dims(nx, ny, nz), C.byref(d),
                              _ptr(update_u), _ptr(update_b))

    def transpose12(self, u, b, update_u, update_b, nx, ny, nz):
        self._chk(u, b, update_u, update_b)
        self._f("transpose12")(_ptr(u), _ptr(b), _ptr(update_u), _ptr(update_b),
                               *self._dims(nx, ny, nz), C.c_int(0))

    def transpose13(self, u, b, update_u, update_b, nx, ny, nz):
        self._chk(u, b, update_u, update_b)
        self._f("transpose13")(_ptr(u), _ptr(b), _ptr(update_u), _ptr(update_b),
                               *self._dims(nx, ny, nz))

    def calcfl(self, u, b, nx, ny, nz):
        self._chk(u, b)
        return self.dtype.type(self._f("calcfl")(_ptr(u), _ptr(b), *self._dims(nx, ny, nz)))

    def calcfl_averaged(self, u, b, nx, ny, nz):
        self._chk(u, b)
        return self.dtype.type(
            self._f("calcfl_averaged")(_ptr(u), _ptr(b), *self._dims(nx, ny, nz)))

    def copy_matrix(self, u, b, nx, ny, nz, update_u, update_b):
        self._chk(u, b, update_u, update_b)
        self._f("copy_matrix")(_ptr(u), _ptr(b), *self._dims(nx, ny, nz),
                               _ptr(update_u), _ptr(update_b))

    # ---- driver (mhd.c:60-125) -------------------------------------------
    def dt_from_cfl(self, inv_c, cfl_number, t, tf):
        """dt = cfl_number*(1/c) formed in double, clamped to (tf-t)/2 (mhd.c:63-64)."""
        if hasattr(self.lib, self.p + "dt_from_cfl"):
            return self.dtype.type(self._f("dt_from_cfl")(inv_c, cfl_number, t, tf))
        T = self.dtype.type
        dt = T(float(cfl_number) * float(inv_c))
        if tf > 0 and dt > T(T(tf) - T(t)) / T(2):
            dt = T(T(tf) - T(t)) / T(2)
        return dt

    def step(self, u, b, nx, ny, nz, dt, wu=None, wb=None):
        """One full x,y,z,z,y,x step in place, following mhd.c:72-119 call by call."""
        self._chk(u, b)
        wu = np.empty_like(u) if wu is None else wu
        wb = np.empty_like(b) if wb is None else wb
        if hasattr(self.lib, self.p + "step"):
            self._f("step")(_ptr(u), _ptr(b), C.c_int(nx), C.c_int(ny), C.c_int(nz),
                            self.ct(dt), _ptr(wu), _ptr(wb))
            return
        cp = self.copy_matrix
        cp(u, b, nx, ny, nz, wu, wb)
        self.fluidx(u, b, nx, ny, nz, dt, wu, wb); cp(u, b, nx, ny, nz, wu, wb)
        self.advectbyzx(u, b, nx, ny, nz, dt, wu, wb); cp(u, b, nx, ny, nz, wu, wb)
        self.transpose12(u, b, wu, wb, nx, ny, nz); cp(u, b, ny, nx, nz, wu, wb)
        self.fluidx(u, b, ny, nx, nz, dt, wu, wb); cp(u, b, ny, nx, nz, wu, wb)
        self.advectbyzx(u, b, ny, nx, nz, dt, wu, wb); cp(u, b, ny, nx, nz, wu, wb)
        self.transpose13(u, b, wu, wb, ny, nx, nz); cp(u, b, nz, nx, ny, wu, wb)
        self.fluidx(u, b, nz, nx, ny, dt, wu, wb); cp(u, b, nz, nx, ny, wu, wb)
        self.advectbyzx(u, b, nz, nx, ny, dt, wu, wb); cp(u, b, nz, nx, ny, wu, wb)
        self.advectbyzx(u, b, nz, nx, ny, dt, wu, wb); cp(u, b, nz, nx, ny, wu, wb)
        self.fluidx(u, b, nz, nx, ny, dt, wu, wb); cp(u, b, nz, nx, ny, wu, wb)
        self.transpose13(u, b, wu, wb, nz, nx, ny); cp(u, b, ny, nx, nz, wu, wb)
        self.advectbyzx(u, b, ny, nx, nz, dt, wu, wb); cp(u, b, ny, nx, nz, wu, wb)
        self.fluidx(u, b, ny, nx, nz, dt, wu, wb); cp(u, b, ny, nx, nz, wu, wb)
        self.transpose12(u, b, wu, wb, ny, nx, nz); cp(u, b, nx, ny, nz, wu, wb)
        self.advectbyzx(u, b, nx, ny, nz, dt, wu, wb); cp(u, b, nx, ny, nz, wu, wb)
        self.fluidx(u, b, nx, ny, nz, dt, wu, wb); cp(u, b, nx, ny, nz, wu, wb)

    def run(self, u, b, nx, ny, nz, cfl_number=0.9, cfl_mode=0, t=0.0, tf=0.0,
            max_steps=1):
        """Time loop of mhd.c:60-125 (tf>0: do-while t<tf; tf<=0: max_steps steps).

        Returns (steps, t, dts)."""
        T = self.dtype.type
        t = T(t)
        dts = []
        wu, wb = np.empty_like(u), np.empty_like(b)
        for s in range(max_steps):
            if tf > 0 and s > 0 and not (t < T(tf)):
                break
            inv = (self.calcfl_averaged if cfl_mode else self.calcfl)(u, b, nx, ny, nz)
            dt = self.dt_from_cfl(inv, cfl_number, t, T(tf))
            t = T(t + T(2) * dt)
            dts.append(dt)
            self.step(u, b, nx, ny, nz, dt, wu, wb)
        return len(dts), t, np.array(dts, dtype=self.dtype)


def oracle(kind: str = "f32") -> CPath:
    lib = _load(LIB_ORACLE)
    if kind == "f32":
        return CPath(lib, "oracle_", np.float32)
    return CPath(lib, "oracle64_", np.float64)


def reference(kind: str = "f32") -> CPath:
    """The reference's own C path (built here by ``make ref``); no driver of its own."""
    lib = _load(LIB_REF[kind])
    return CPath(lib, "", np.float32 if kind == "f32" else np.float64)


def set_threads(n: int) -> None:
    lib = _load(LIB_ORACLE)
    lib.oracle_set_threads(C.c_int(int(n)))
