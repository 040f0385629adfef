"""Build libmhdgpu.so (sm_103a) in-tree with nvcc.

    python mhd-gpu_gb300/build.py [--verbose-ptxas]

Each .cu (and host-only .cpp) in csrc/ is compiled in parallel to an object under _build/ and the
objects are linked into lib/libmhdgpu.so.  A file is rebuilt when it or any
header is newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libmhdgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                  "-I" + os.path.join(REPO, "include"), "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(REPO, "include", "*.h"))


def _stale(src: str, obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src, *deps])


# the debug build: every kernel index checked (csrc/mhd_debug.cuh); its
# record lives in one translation unit, so the objects are relocatable
BUILD_DEBUG = os.path.join(HERE, "_build_debug")
LIB_DEBUG = os.path.join(LIBDIR, "libmhdgpu_debug.so")
DEBUG_FLAGS = ["-DMHD_DEBUG", "-rdc=true"]


def _obj(src: str, bdir: str = BUILD) -> str:
    return os.path.join(bdir, os.path.splitext(os.path.basename(src))[0] + ".o")


def build(verbose_ptxas: bool = False, quiet: bool = True, debug: bool = False) -> str:
    bdir, lib = (BUILD_DEBUG, LIB_DEBUG) if debug else (BUILD, LIB)
    extra = DEBUG_FLAGS if debug else []
    os.makedirs(bdir, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    # the heaviest translation units first, so the parallel build ends sooner
    heavy = ("batch_", "fluidx", "advect")
    srcs.sort(key=lambda s: (not os.path.basename(s).startswith(heavy), s))
    deps = _headers()
    cc = nvcc()
    jobs = []
    for s in srcs:
        o = _obj(s, bdir)
        if verbose_ptxas or _stale(s, o, deps):
            cmd = [cc, *NVFLAGS, *extra, "-c", s, "-o", o]
            if verbose_ptxas:
                cmd += ["-Xptxas", "-v"]
            jobs.append((s, cmd))

    def run(job):
        s, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return s, r

    failed = []
    with cf.ThreadPoolExecutor(max_workers=min(os.cpu_count() or 8, 16, max(1, len(jobs)))) as ex:
        for s, r in ex.map(run, jobs):
            if r.returncode != 0:
                failed.append((s, r.stderr))
            elif verbose_ptxas or not quiet:
                sys.stderr.write(r.stderr)
    if failed:
        msg = "\n".join(f"--- {s}\n{e}" for s, e in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    objs = [_obj(s, bdir) for s in srcs]
    if jobs or not os.path.exists(lib) or any(os.path.getmtime(o) > os.path.getmtime(lib) for o in objs):
        cmd = [cc, *ARCH, *(["-rdc=true"] if debug else []), "-shared", "-o", lib, *objs, "-lcudart",
               "-Xlinker", "-Bsymbolic"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr)
    return lib


if __name__ == "__main__":
    print(build(verbose_ptxas="--verbose-ptxas" in sys.argv, quiet=False, debug="--debug" in sys.argv))
