"""Benchmark of one full MHD step (x, y, z, z, y, x sweeps + CFL) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 128]

Workload: the 128^3 configuration of the reference's plain drop-in case, a
linear Alfven wave on the box diagonal k = (1,1,1) 2 pi/L, A = 1e-3, rho = p = 1,
CFL 0.7 (C-path CFL formula), synthetic inputs (mhd-gpu_gb300/ics.py).
A step is one full Strang-split step; one cell-update is one cell advanced by
one step.  value = cell-updates/s over K steps replayed from a CUDA graph with
the state resident in HBM; L2 is flushed (512 MB write) between timed steps,
outside the timed events.  e2e = the same metric through the host-buffer C-ABI
entry mhdgpu_run_host (pinned host state uploaded and downloaded every step).

With N > 1 (torchrun) every rank advances its own replica of the box: the
single-box step has no data-parallel split, so scaling is weak and the ranks
exchange nothing but the timing max.

--impl reference times the reference algorithm's CPU implementation on this
host's cores (the C restatement in oracle/, OpenMP over pencils, bit-identical
to the reference C path) on the same workload and prints the same JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "mhd-gpu_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

METRIC = "cell-updates/s per full MHD step, fused+batched vs plain; % of HBM roofline"
UNIT = "cell-updates/s"
FLUIDX_BYTES_PER_CELL = 52      # R u 20 + b 12, W u 20 (one read and write of the pencil data)
STEP_BYTES_64 = 64              # one read + one write of the 8-float state per cell-update
PLAIN_PASS_BYTES = 792          # minimal per-subroutine pass bytes per cell-update


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None
        self.marks = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "25"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), line.strip()))

    def mark(self, name):
        self.marks.append((name, time.time()))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)

    def summary(self, t0, t1):
        rows = []
        for ts, line in self.samples:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm, mx = float(parts[0]), float(parts[1])
            except ValueError:
                continue
            rows.append((ts, sm, mx, parts[2:6]))
        inside = [r for r in rows if t0 <= r[0] <= t1] or rows
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"],
                    "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in inside for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[1] for r in inside),
                "sm_max_mhz": max(r[2] for r in inside), "reasons": reasons,
                "samples": len(inside)}


def read_traffic():
    """dram bytes per fluidx launch from the committed ncu summary, if any."""
    p = os.path.join(REPO, "profiles", "fluidx_alfven128_ncu.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def dist_setup(n_gpus):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return rank, world, local


def dist_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_rate(n, seconds, threads, use_ref):
    """Cell-updates/s of the reference algorithm on the host: whole steps of the
    same workload until `seconds` of work have run (at least one step)."""
    import numpy as np
    import ics
    import oracle as O
    u, b = ics.alfven_oblique(n)
    if use_ref:
        P = O.reference("f32")
        kind = "reference"
        threads = 1
    else:
        O.set_threads(threads)
        P = O.oracle("f32")
        kind = "port"
    # one untimed step to page everything in
    inv = P.calcfl(u, b, n, n, n)
    dt = P.dt_from_cfl(inv, 0.7, np.float32(0), np.float32(0))
    P.step(u, b, n, n, n, dt)
    steps = 0
    t0 = time.perf_counter()
    while True:
        inv = P.calcfl(u, b, n, n, n)
        dt = P.dt_from_cfl(inv, 0.7, np.float32(0), np.float32(0))
        P.step(u, b, n, n, n, dt)
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    rate = n ** 3 * steps / el
    return rate, kind, threads, f"{steps} full steps of the {n}^3 workload ({el:.1f} s)"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--math", default="faithful", choices=["faithful", "fast"])
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (default tiles)")
    args = ap.parse_args()
    n, K, W = args.n, args.steps, max(3, args.warmup)
    ncell = n ** 3
    config = {"workload": f"alfven_diag_{n}", "box": [n, n, n], "cfl": 0.7, "cfl_mode": "c_path",
              "ic": "linear Alfven wave, k=(1,1,1)2pi/L, A=1e-3, rho=p=1, B0 along k",
              "path": "plain drop-in: per-subroutine kernels, one CUDA graph per step",
              "l2": "flushed between timed steps (512 MB write, outside the timed events)",
              "parallelism": f"replicas x{args.gpus}"}

    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        if rank != 0:
            return
        threads = os.cpu_count() or 1
        use_ref = os.path.exists(os.path.join(REPO, "oracle", "_ref", "libref_f32.so"))
        if not os.path.exists(os.path.join(REPO, "oracle", "lib", "liboracle.so")):
            subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle")], check=True)
        budget = min(120.0, max(10.0, 0.25 * (K + W)))
        rate, kind, cores, sample = cpu_rate(n, budget, threads, use_ref)
        print(json.dumps({
            "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus, "steps": K,
            "warmup": W, "ms_per_step": ncell / rate * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config, "impl": "reference",
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": sample},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }))
        return

    import numpy as np
    import torch

    import ics
    import mhdgpu

    rank, world, local = dist_setup(args.gpus)
    dev = torch.device("cuda", local if world > 1 else 0)
    math_mode = mhdgpu.MHD_MATH_FAST if args.math == "fast" else mhdgpu.MHD_MATH_FAITHFUL
    mhdgpu.set_math(math_mode)
    if not args.no_tune:
        picks = mhdgpu.autotune(n, n, n, math_mode)
    else:
        picks = {(k, n, r): mhdgpu.get_tile(k, n, rows=r) for k in ("fluidx", "advectbyzx")
                 for r in (False, True)}
    config["math"] = args.math
    config["tiles"] = {f"{k}@{m}{'/rows' if r else ''}": list(v) for (k, m, r), v in picks.items()}
    config["tiles_from"] = "defaults" if args.no_tune else "mhdgpu_autotune"
    u0, b0 = ics.alfven_oblique(n)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    vis = [x.strip() for x in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if x.strip()]
    sampler = ClockSampler(vis[local] if len(vis) > local else local)
    sampler.start()
    time.sleep(0.3)

    def measure(path):
        """K graph-replayed steps (L2 flushed between them, outside the
        events), then K directly launched steps under the event profiler."""
        du = torch.from_numpy(u0).to(dev)
        db = torch.from_numpy(b0).to(dev)
        work = torch.empty(mhdgpu.step_workspace_bytes(n, n, n, path), dtype=torch.uint8, device=dev)
        clock = mhdgpu.new_clock(device=dev)

        def one_step():
            mhdgpu.advance(du, db, n, n, n, 1, 0.7, mhdgpu.MHD_CFL_C, 0.0, clock, None, work, path)

        with torch.cuda.stream(stream):          # warm-up; sets kernel attributes before capture
            for _ in range(W):
                one_step()
        torch.cuda.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            one_step()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
        dist_barrier(world)
        torch.cuda.synchronize()
        tw0 = time.time()
        with torch.cuda.stream(stream):
            for i in range(K):
                flush.zero_()
                ev[i][0].record(stream)
                graph.replay()
                ev[i][1].record(stream)
        torch.cuda.synchronize()
        tw1 = time.time()
        dist_barrier(world)
        total_s = dist_max(sum(a.elapsed_time(b) for a, b in ev) / 1e3, world)
        prof = mhdgpu.Profiler(max_records=K * 40 + 100)
        with torch.cuda.stream(stream):
            with prof:
                for i in range(K):
                    flush.zero_()
                    one_step()
        torch.cuda.synchronize()
        summ = prof.summary()
        prof.close()
        health = mhdgpu.read_clock(clock).health
        del graph
        return total_s, summ, health, (tw0, tw1)

    total_s, summ, health, (t_wall0, t_wall1) = measure(mhdgpu.MHD_PATH_FUSED)
    value = world * ncell * K / total_s
    plain_s, plain_summ, plain_health, _ = measure(mhdgpu.MHD_PATH_PLAIN)
    value_plain = world * ncell * K / plain_s
    sampler.stop()
    clocks = sampler.summary(t_wall0, t_wall1)
    launches_per_step = sum(v[1] for v in summ.values()) / K
    tot_ms = sum(v[2] for v in summ.values())
    fl_rec, fl_launch, fl_ms = summ["fluidx"]
    fl_avg_s = fl_ms / 1e3 / max(fl_launch, 1)
    hbm, peak_kind = peaks()
    achieved = FLUIDX_BYTES_PER_CELL * ncell / fl_avg_s / 1e9
    traffic = read_traffic()

    # end to end through the host-buffer C-ABI entry: every step uploads the
    # state from pinned memory, advances one step and downloads it
    hu = torch.from_numpy(u0.copy()).pin_memory()
    hb = torch.from_numpy(b0.copy()).pin_memory()
    un, bn = hu.numpy(), hb.numpy()
    ke = max(3, min(K, 50))
    t = 0.0
    mhdgpu.run_host(un, bn, n, n, n, 0.7, 0, t, 0.0, 1, path=mhdgpu.MHD_PATH_FUSED)
    dist_barrier(world)
    t0 = time.perf_counter()
    for _ in range(ke):
        st, t, _done = mhdgpu.run_host(un, bn, n, n, n, 0.7, 0, t, 0.0, 1, path=mhdgpu.MHD_PATH_FUSED)
    e2e_s = dist_max(time.perf_counter() - t0, world)
    e2e = world * ncell * ke / e2e_s
    config["path"] = "transpose-free step (mhdgpu_step_fused), one CUDA graph per step"

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": total_s / K * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seedless analytic initial state, see config.ic)",
        "config": config,
        "gpu_launches": int(round(launches_per_step * K)),
        "roofline": {"bound": "hbm",
                     "kernel": "fluidx_kernel (x sweep %s, y/z sweeps %s [cpl,wpp,ppc], %s)" % (
                         list(mhdgpu.get_tile("fluidx", n)), list(mhdgpu.get_tile("fluidx", n, rows=True)),
                         args.math),
                     "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "traffic": traffic,
                     "algorithmic_bytes_per_launch": FLUIDX_BYTES_PER_CELL * ncell,
                     "avg_launch_us": fl_avg_s * 1e6,
                     "share_of_step": fl_ms / tot_ms if tot_ms else None},
        "roofline_step": {"bytes_per_cell_update_64B_basis": STEP_BYTES_64,
                          "frac_64B_basis": value * STEP_BYTES_64 / 1e9 / world / hbm,
                          "plain_pass_bytes_per_cell_update": PLAIN_PASS_BYTES,
                          "frac_plain_pass_bytes": value * PLAIN_PASS_BYTES / 1e9 / world / hbm},
        "kernel_time_ms_per_step": {k: v[2] / K for k, v in summ.items()},
        "kernel_launches_per_step": {k: v[1] / K for k, v in summ.items()},
        "plain_drop_in": {"value": value_plain, "unit": UNIT, "ms_per_step": plain_s / K * 1e3,
                          "path": "per-subroutine kernels + transposes (mhdgpu_step)",
                          "kernel_time_ms_per_step": {k: v[2] / K for k, v in plain_summ.items()},
                          "health": plain_health},
        "fused_over_plain": value / value_plain,
        "e2e": {"value": e2e, "unit": UNIT, "steps": ke,
                "h2d_bytes_per_step": 32 * ncell, "d2h_bytes_per_step": 32 * ncell,
                "api": "mhdgpu_run_host, 1 step per call"},
        "clocks": clocks, "health": health,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        use_ref = os.path.exists(os.path.join(REPO, "oracle", "_ref", "libref_f32.so"))
        try:
            rate, kind, cores, sample = cpu_rate(n, args.cpu_seconds, os.cpu_count() or 1, use_ref)
            out["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": kind,
                                   "sample": sample}
        except Exception as e:  # noqa: BLE001
            out["cpu_baseline"] = {"value": None, "unit": UNIT, "error": str(e)}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
