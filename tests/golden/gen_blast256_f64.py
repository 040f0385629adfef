"""Record of the FP64 oracle's run of the low-beta blast at 256^3 (golden fixture).

    make -C oracle
    python tests/golden/gen_blast256_f64.py        # ~40 min on 8 cores

The spherical MHD blast (mhd-gpu_gb300/ics.py blast: r0 = 0.1 L, p = 100
inside and 0.1 outside, rho = 1, B = 10 (1,1,0)/sqrt 2, beta = 0.002 in the
ambient gas) on a 256^3 periodic box, advanced 300 steps at CFL 0.7 with the
C path's CFL formula by the oracle's double build (the reference C path's
algorithm in FP64, Heterogeneous_MHD/C/mhd.c:60-125 with every float a
double), each step taking its own dt.  The record holds the run's
diagnostics (positivity of the gas pressure, FP64 totals, max |div B|), which
the GPU tests compare with their FP32 runs of the same configuration; the
state itself (1 GB) is not kept.
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "mhd-gpu_gb300"))
import ics  # noqa: E402
import oracle as O  # noqa: E402

N = 256
STEPS = 300
CFL = 0.7


def gas_pressure(u, b, n):
    """p = (gamma-1)(E - m^2/2rho - Bc^2/2) in float64, B face -> centre."""
    g = float(np.float32(5.0 / 3.0))
    uu = np.asarray(u, dtype=np.float64).reshape(n, n, n, 5)
    bb = np.asarray(b, dtype=np.float64).reshape(n, n, n, 3)
    cx = 0.5 * (bb[..., 0] + np.roll(bb[..., 0], -1, axis=2))
    cy = 0.5 * (bb[..., 1] + np.roll(bb[..., 1], -1, axis=1))
    cz = 0.5 * (bb[..., 2] + np.roll(bb[..., 2], -1, axis=0))
    q = (uu[..., 1] ** 2 + uu[..., 2] ** 2 + uu[..., 3] ** 2) / uu[..., 0]
    return (g - 1.0) * (uu[..., 4] - 0.5 * q - 0.5 * (cx ** 2 + cy ** 2 + cz ** 2))


def diagnostics(u, b, n):
    p = gas_pressure(u, b, n)
    tot = ics.totals(u, n, n, n)
    return {"mass": float(tot[0]), "energy": float(tot[4]), "min_p": float(p.min()),
            "cells_p_nonpositive": int((p <= 0).sum()), "max_div_b": ics.div_b(b, n, n, n),
            "min_rho": float(np.asarray(u, dtype=np.float64).reshape(-1, 5)[:, 0].min())}


def main():
    O.set_threads(os.cpu_count() or 1)
    u32, b32 = ics.blast(N)
    u, b = u32.astype(np.float64), b32.astype(np.float64)
    d0 = diagnostics(u, b, N)
    t0 = time.time()
    steps, t, dts = O.oracle("f64").run(u, b, N, N, N, cfl_number=CFL, cfl_mode=0, max_steps=STEPS)
    d1 = diagnostics(u, b, N)
    rec = {"config": {"workload": "blast", "n": N, "steps": steps, "cfl": CFL, "cfl_mode": "c_path",
                      "ic": "ics.blast(256): r0=0.1L, p_in=100, p_out=0.1, rho=1, B=10(1,1,0)/sqrt2"},
           "solver": "oracle FP64 build (oracle64_*), own dt per step",
           "t_end": float(t), "dt_first": float(dts[0]), "dt_last": float(dts[-1]),
           "initial": d0, "final": d1,
           "energy_drift": abs(d1["energy"] - d0["energy"]) / abs(d0["energy"]),
           "mass_drift": abs(d1["mass"] - d0["mass"]) / abs(d0["mass"]),
           "cpu_seconds": time.time() - t0}
    with open(os.path.join(HERE, "blast256_f64.json"), "w") as fh:
        json.dump(rec, fh, indent=1)
    print(json.dumps(rec))


if __name__ == "__main__":
    main()
