"""Generate the golden vectors of tests/golden/ from the reference itself.

    make -C oracle ref            # compiles pandaPQY/MHD-GPU's C path from its sources
    python tests/golden/gen_golden.py [--ref /root/reference]

Every output here is computed by the reference's own C path
(Heterogeneous_MHD/C/*.c compiled unmodified into oracle/_ref/libref_*.so),
driven in the order of Heterogeneous_MHD/C/mhd.c:60-125.  The inputs are
  - the reference's shipped initial states data/source_init_alfvenlinear_16cube.dat
    and _32cube.dat (raw little-endian float32, 8 per cell, read into C index
    order i, j, k as Heterogeneous_MHD/C/init.c:33-54 does), and
  - seeded random physical states (mhd-gpu_gb300/ics.py random_state).
The fixtures carry their inputs, so checking them needs neither the
reference checkout nor the reference build.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "mhd-gpu_gb300"))
import ics  # noqa: E402
import oracle as O  # noqa: E402


def read_dat(path, n):
    a = np.fromfile(path, dtype="<f4").reshape(n, n, n, 8)   # file order i, j, k, field
    # C array element (ii, i, j, k) at ((k*ny + j)*nx + i)*nub + ii
    u = np.ascontiguousarray(a[..., :5].transpose(2, 1, 0, 3)).ravel()
    b = np.ascontiguousarray(a[..., 5:].transpose(2, 1, 0, 3)).ravel()
    return u, b


def subroutines(R, u, b, dims, dt):
    nx, ny, nz = dims
    out = {}
    uu = np.zeros_like(u)
    R.fluidx(uu, b.copy(), nx, ny, nz, dt, u.copy(), b.copy())
    out["fluidx_u"] = uu
    bb = b.copy()
    R.advectbyzx(u.copy(), bb, nx, ny, nz, dt, u.copy(), b.copy())
    out["advect_b"] = bb
    tu, tb = np.zeros_like(u), np.zeros_like(b)
    R.transpose12(tu, tb, u.copy(), b.copy(), nx, ny, nz)
    out["t12_u"], out["t12_b"] = tu, tb
    if nx == nz:
        tu, tb = np.zeros_like(u), np.zeros_like(b)
        R.transpose13(tu, tb, u.copy(), b.copy(), nx, ny, nz)
        out["t13_u"], out["t13_b"] = tu, tb
    out["calcfl"] = np.array([R.calcfl(u, b, nx, ny, nz)], dtype=u.dtype)
    return out


def write_digest(ref):
    """sha256 of the shipped init file: pins the state-file writer to the
    reference's own bytes without copying the file."""
    import hashlib
    path = os.path.join(ref, "data", "source_init_alfvenlinear_16cube.dat")
    raw = open(path, "rb").read()
    with open(os.path.join(HERE, "alfven16_dat_sha256.txt"), "w") as f:
        f.write(f"{hashlib.sha256(raw).hexdigest()} {len(raw)}\n")


def write_alfven32(ref, R):
    """The shipped 32^3 state run by the reference to tf = 4*nx = 128 at CFL
    0.9: the input, the dt sequence, sha256 digests of the final u and b, and
    every 97th value of them (the fixture stays small; the oracle must match
    the digests bit for bit)."""
    import hashlib
    u0, b0 = read_dat(os.path.join(ref, "data", "source_init_alfvenlinear_32cube.dat"), 32)
    uf, bf = u0.copy(), b0.copy()
    sf, tfin, dtsf = R.run(uf, bf, 32, 32, 32, cfl_number=0.9, tf=128.0, max_steps=100000)
    np.savez_compressed(os.path.join(HERE, "alfven32_dat.npz"), u0=u0, b0=b0, dtsf=dtsf,
                        steps=np.array([sf]), t=np.array([tfin], dtype=np.float32),
                        uf_sha=np.array([hashlib.sha256(uf.tobytes()).hexdigest()]),
                        bf_sha=np.array([hashlib.sha256(bf.tobytes()).hexdigest()]),
                        uf_sample=uf[::97].copy(), bf_sample=bf[::97].copy())
    print("alfven32_dat: steps", sf, "t", tfin)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("MHD_REFERENCE"),
                    help="pandaPQY/MHD-GPU checkout (or set MHD_REFERENCE)")
    ap.add_argument("--only-digest", action="store_true")
    ap.add_argument("--only-alfven32", action="store_true")
    args = ap.parse_args()
    if not args.ref:
        ap.error("give --ref <pandaPQY/MHD-GPU checkout> or set MHD_REFERENCE")
    write_digest(args.ref)
    if args.only_digest:
        return
    R = O.reference("f32")
    R64 = O.reference("f64")
    write_alfven32(args.ref, R)
    if args.only_alfven32:
        return

    # 1. shipped 16^3 Alfven state: 1 step and the reference's full run to tf = 4*nx
    u0, b0 = read_dat(os.path.join(args.ref, "data", "source_init_alfvenlinear_16cube.dat"), 16)
    u1, b1 = u0.copy(), b0.copy()
    s1, t1, dts1 = R.run(u1, b1, 16, 16, 16, cfl_number=0.9, tf=64.0, max_steps=1)
    uf, bf = u0.copy(), b0.copy()
    sf, tfin, dtsf = R.run(uf, bf, 16, 16, 16, cfl_number=0.9, tf=64.0, max_steps=100000)
    np.savez_compressed(os.path.join(HERE, "alfven16_dat.npz"), u0=u0, b0=b0,
                        u1=u1, b1=b1, dts1=dts1, uf=uf, bf=bf, dtsf=dtsf,
                        steps=np.array([sf]), t=np.array([tfin], dtype=np.float32))
    print("alfven16_dat: steps", sf, "t", tfin)

    # 2. per-subroutine outputs on random states (cubic and non-cubic)
    rec = {}
    for tag, dims, seed, dt in [("c8", (8, 8, 8), 11, 0.05), ("r12", (12, 6, 10), 12, 0.04),
                                ("r5", (5, 7, 9), 13, 0.03)]:
        u, b = ics.random_state(*dims, seed=seed)
        rec[f"{tag}_u"], rec[f"{tag}_b"] = u, b
        rec[f"{tag}_dims"] = np.array(dims)
        rec[f"{tag}_dt"] = np.array([dt], dtype=np.float32)
        for k, v in subroutines(R, u, b, dims, np.float32(dt)).items():
            rec[f"{tag}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, "subroutines_f32.npz"), **rec)
    print("subroutines_f32:", len(rec), "arrays")

    # 3. FP64 build of the reference: 3 steps of the 8^3 random state
    u, b = ics.random_state(8, 8, 8, seed=21, dtype=np.float64)
    u64, b64 = u.copy(), b.copy()
    s, t, dts = R64.run(u64, b64, 8, 8, 8, cfl_number=0.9, tf=0.0, max_steps=3)
    np.savez_compressed(os.path.join(HERE, "run8_f64.npz"), u0=u, b0=b, u=u64, b=b64, dts=dts)
    print("run8_f64: steps", s)

    # 4. FP32 whole-run golden of the x Alfven wave at 16^3 (CFL 0.7, 20 steps)
    u, b = ics.alfven_x(16)
    ua, ba = u.copy(), b.copy()
    s, t, dts = R.run(ua, ba, 16, 16, 16, cfl_number=0.7, tf=0.0, max_steps=20)
    np.savez_compressed(os.path.join(HERE, "alfvenx16_cfl07.npz"), u0=u, b0=b, u=ua, b=ba, dts=dts)
    print("alfvenx16_cfl07: steps", s)


if __name__ == "__main__":
    main()
