"""A fluid-sweep case whose total pressure lands on a double-precision tie.

    make -C oracle
    python tests/golden/gen_tie_pencil.py

Box 48 of the turbulent ensemble (mhd-gpu_gb300/ics.py ensemble(64, seed=0),
96 x 64 x 48), pencil j = 57, k = 26 of its first x sweep (dt = the C-path
CFL step at CFL 0.7).  In the half step of that pencil, cell 70's total
pressure (Heterogeneous_MHD/C/mhdflux.c:28) is exactly half a double ulp
above a float rounding midpoint.  The C path evaluates it as
RN_d(RN_d(A (gamma-1)) + M), which rounds away from the tie to the float
above; an FMA-contracted A (gamma-1) + M rounds once, onto the midpoint
itself, which then rounds to the even float below.  One ulp of pressure there
moves x momentum by 14 ulps in the cells beside it.

The fixture is a 96 x 2 x 2 box whose pencil (j, k) = (0, 0) reproduces that
pencil exactly: u of the pencil, its face b, b at j+1 and b at k+1 (the other
three pencils hold copies of the same rows).  It stores the input, dt and
the oracle's fluidx output.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "mhd-gpu_gb300"))
import ics  # noqa: E402
import oracle as O  # noqa: E402

BOX, J, K, CFL = 48, 57, 26, 0.7


def main() -> None:
    e = ics.ensemble(64, seed=0)[BOX]
    nx, ny, nz = e["dims"]
    P = O.oracle("f32")
    dt = P.dt_from_cfl(P.calcfl(e["u"], e["b"], nx, ny, nz), CFL, np.float32(0), np.float32(0))
    U = e["u"].reshape(nz, ny, nx, 5)
    B = e["b"].reshape(nz, ny, nx, 3)
    u = np.empty((2, 2, nx, 5), np.float32)
    b = np.empty((2, 2, nx, 3), np.float32)
    u[:] = U[K, J]
    b[0, 0] = B[K, J]
    b[0, 1] = B[K, (J + 1) % ny]
    b[1, 0] = B[(K + 1) % nz, J]
    b[1, 1] = B[(K + 1) % nz, (J + 1) % ny]
    u, b = u.ravel(), b.ravel()
    out = np.zeros_like(u)
    P.fluidx(out, b.copy(), nx, 2, 2, dt, u.copy(), b.copy())
    np.savez(os.path.join(HERE, "tie_pencil.npz"), u=u, b=b, dims=np.array([nx, 2, 2]),
             dt=np.array([dt], np.float32), out=out)
    print("dt", repr(dt), "saved", u.nbytes + b.nbytes + out.nbytes, "bytes")


if __name__ == "__main__":
    main()
