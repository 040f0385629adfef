"""Benchmark of full MHD steps (x, y, z, z, y, x sweeps + CFL) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload ensemble64|alfven_diag_128]

Workloads (synthetic inputs, mhd-gpu_gb300/ics.py):
  ensemble64 (default, the headline "fused+batched vs plain"): 64 independent
    periodic boxes, sizes along each axis drawn from {32,48,64,96,128} by seed 0
    (27.2 M cells, 0.87 GB of state), each a linear Alfven wave on the box
    diagonal or a turbulent start with an amplitude drawn log-uniformly from
    [1e-4, 1e-1]; CFL 0.7, C-path CFL formula.  The batched path
    (mhdgpu_batch_*) advances all boxes together: per sweep, one persistent
    launch per pencil-length class, the classes concurrent;
    the comparison loops the plain per-subroutine drop-in (mhdgpu_advance,
    path PLAIN) box by box, and the fused single-box step box by box.
  alfven_diag_128: the 128^3 plain drop-in configuration, a linear Alfven wave
    on the box diagonal k = (1,1,1) 2 pi/L, A = 1e-3, rho = p = 1, CFL 0.7.
    Its numbers are also reported inside the ensemble line.

A step is one full Strang-split step of every box; one cell-update is one
cell advanced by one step.  value = cell-updates/s over K steps replayed from
a CUDA graph with the state resident in HBM; L2 is flushed (512 MB write)
between timed steps, outside the timed events (the ensemble's state is also
larger than L2).  e2e = the same metric through the public API with host
buffers: every step uploads the state from pinned host memory, advances one
step and downloads it.

With N > 1 (torchrun): the ensemble's boxes are split across the ranks,
balanced by cells (mhd-gpu_gb300/shard.py), each rank advancing its share
with no exchange on the data path (strong scaling of the fixed 64-box
workload); the single-box workload runs one replica per rank (weak scaling).
Ranks exchange only the timing max.

--impl reference times the reference algorithm's CPU implementation on this
host's cores (the C restatement in oracle/, OpenMP over pencils, bit-identical
to the reference C path) on a bounded sample of the same workload and prints
the same JSON line.
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
# Algorithmic bytes of one sweep per cell: one read and one write of the 8-float
# state (32 R + 32 W), the basis the roofline fraction is quoted on.
SWEEP_BYTES_PER_CELL = 64
# The bytes the current sweep actually has to move per cell, as a diagnostic:
# fluid 52 (above); field 32 (R rho, m 8, R b2 b3 8, W b2 b3 8, W sA sB 8);
# b(1) 16 (R sA sB 8, R+W b1 8)
SWEEP_PASS_BYTES_PER_CELL = 100
STEP_BYTES_64 = 64              # one read + one write of the 8-float state per cell-update
# floating-point operations per cell-update of one full step (6 fluid and 6 field
# sweeps + the CFL reduction), counted on the oracle as the reference writes
# them (oracle/flopcount.cpp, 64^3: fluidx 579.7 and advectbyzx 60.0 per
# cell-sweep, CFL 40.0 per step)
FLOPS_PER_CELL_UPDATE = 3878
PLAIN_PASS_BYTES = 792          # minimal per-subroutine pass bytes per cell-update
ENSEMBLE = {"nbox": 64, "seed": 0, "sizes": (32, 48, 64, 96, 128), "amp_range": (1e-4, 1e-1)}
CFL = 0.7


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


def roofline_step(value, world, hbm, dev, clocks, pass_bytes):
    """The whole step against both roofs: HBM at the 64 B/cell-update basis and
    at the path's own pass bytes, and FP32 issue at the counted flops."""
    import torch
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = clocks.get("sm_max_mhz") or 2070.0
    fp32_peak = sms * 128 * 2 * mhz * 1e6 / 1e12        # FMA = 2 flops, 128 FP32 lanes per SM
    per_gpu = value / world
    return {"bytes_per_cell_update_64B_basis": STEP_BYTES_64,
            "frac_64B_basis": per_gpu * STEP_BYTES_64 / 1e9 / hbm,
            "pass_bytes_per_cell_update": pass_bytes,
            "frac_pass_bytes": per_gpu * pass_bytes / 1e9 / hbm,
            "flops_per_cell_update": FLOPS_PER_CELL_UPDATE,
            "flops_source": "oracle/flopcount.cpp (every +,-,*,/,sqrt of the restatement)",
            "tflops": per_gpu * FLOPS_PER_CELL_UPDATE / 1e12,
            "fp32_peak_tflops": fp32_peak,
            "fp32_peak_source": f"nominal: {sms} SMs x 128 lanes x 2 x {mhz:.0f} MHz",
            "frac_fp32_peak": per_gpu * FLOPS_PER_CELL_UPDATE / 1e12 / fp32_peak}


def read_traffic(name):
    """dram bytes per launch of a kernel from its committed ncu summary, if any."""
    p = os.path.join(REPO, "profiles", name)
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


# ---------------------------------------------------------------- CPU arms
def _cpu_path(threads, use_ref):
    import oracle as O
    if use_ref:
        return O.reference("f32"), "reference", 1
    O.set_threads(threads)
    return O.oracle("f32"), "port", threads


def cpu_rate(n, seconds, threads, use_ref):
    """Cell-updates/s of the reference algorithm on the host: whole steps of the
    n^3 Alfven workload until `seconds` of work have run (at least one step)."""
    import numpy as np
    import ics
    u, b = ics.alfven_oblique(n)
    P, kind, threads = _cpu_path(threads, use_ref)
    inv = P.calcfl(u, b, n, n, n)      # one untimed step pages everything in
    P.step(u, b, n, n, n, P.dt_from_cfl(inv, CFL, np.float32(0), np.float32(0)))
    steps = 0
    t0 = time.perf_counter()
    while True:
        inv = P.calcfl(u, b, n, n, n)
        P.step(u, b, n, n, n, P.dt_from_cfl(inv, CFL, np.float32(0), np.float32(0)))
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return n ** 3 * steps / el, kind, threads, f"{steps} full steps of the {n}^3 workload ({el:.1f} s)"


def cpu_rate_ensemble(ens, seconds, threads):
    """Cell-updates/s of the oracle port on the ensemble: full steps of its
    boxes in order (wrapping around) until `seconds` of work have run.  The
    reference's own C path cannot run these boxes (its transpose13 refuses
    nx != nz, Heterogeneous_MHD/C/transpose13.c:58-61), so this is the port."""
    import numpy as np
    P, kind, threads = _cpu_path(threads, False)
    states = [(e["u"].copy(), e["b"].copy(), e["dims"]) for e in ens]
    u, b, d = states[0]
    P.step(u, b, *d, P.dt_from_cfl(P.calcfl(u, b, *d), CFL, np.float32(0), np.float32(0)))
    cells = steps = 0
    t0 = time.perf_counter()
    i = 0
    while True:
        u, b, d = states[i % len(states)]
        P.step(u, b, *d, P.dt_from_cfl(P.calcfl(u, b, *d), CFL, np.float32(0), np.float32(0)))
        cells += d[0] * d[1] * d[2]
        steps += 1
        i += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return cells / el, kind, threads, (f"{steps} box-steps of the ensemble's boxes in order "
                                       f"({cells / 1e6:.1f} M cell-updates, {el:.1f} s)")


def host_cpu():
    """The host CPU's model name (lscpu), for the CPU-baseline record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return "unknown"


def reference_arm(args, config, ens_mode, n, K, W):
    """--impl reference: the reference algorithm's CPU implementation on this
    host's cores, on the same workload, metric and config as the GPU arm.
    The reference's own C path compiled from its sources (oracle/_ref) is timed
    where it was built and the workload is a cubic box; otherwise the oracle
    port (bit-identical to that C path, OpenMP over pencils).  Each timed step
    is one whole step of the workload (all 64 boxes of the ensemble); the
    number of timed steps is K capped so that the timed work stays near a
    minute, and the line reports the steps that ran.  A 1-core rate of the same
    code is reported beside it."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    import numpy as np
    import oracle as O
    import ics
    threads = os.cpu_count() or 1
    if not os.path.exists(O.LIB_ORACLE):
        subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle")], check=True)
    cap_s = 60.0
    if ens_mode:
        ens = ics.ensemble(**ENSEMBLE)
        cells = sum(e["dims"][0] * e["dims"][1] * e["dims"][2] for e in ens)
        P, kind, cores = _cpu_path(threads, False)
        states = [(e["u"].copy(), e["b"].copy(), e["dims"]) for e in ens]

        def one_step():
            for u, b, d in states:
                P.step(u, b, *d, P.dt_from_cfl(P.calcfl(u, b, *d), CFL, np.float32(0), np.float32(0)))

        for w in range(W):   # warm-up: W box-steps (the first pages everything in)
            u, b, d = states[w % len(states)]
            P.step(u, b, *d, P.dt_from_cfl(P.calcfl(u, b, *d), CFL, np.float32(0), np.float32(0)))
        what = "the 64 boxes of the ensemble"
    else:
        cells = n ** 3
        use_ref = O.ref_available("f32")
        P, kind, cores = _cpu_path(threads, use_ref)
        u, b = ics.alfven_oblique(n)

        def one_step():
            P.step(u, b, n, n, n, P.dt_from_cfl(P.calcfl(u, b, n, n, n), CFL, np.float32(0), np.float32(0)))

        for _ in range(W):
            one_step()
        what = f"the {n}^3 box"
    times = []
    t_all = time.perf_counter()
    while len(times) < K:
        t0 = time.perf_counter()
        one_step()
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all + times[-1] > cap_s:
            break
    secs = sum(times)
    rate = cells * len(times) / secs
    sample = (f"{len(times)} timed steps of {what} ({cells * len(times) / 1e6:.1f} M cell-updates, "
              f"{secs:.1f} s) after {W} warm-up {'box-steps' if ens_mode else 'steps'}; "
              f"{cores} threads on {host_cpu()}")
    one = None
    if ens_mode:
        r1, k1, c1, s1 = cpu_rate_ensemble(ens, 8.0, 1)
        one = {"value": r1, "unit": UNIT, "cores": c1, "kind": k1, "sample": s1}
    else:
        r1, k1, c1, s1 = cpu_rate(n, 8.0, 1, O.ref_available("f32"))
        one = {"value": r1, "unit": UNIT, "cores": c1, "kind": k1, "sample": s1}
    print(json.dumps({
        "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus, "steps": len(times),
        "steps_requested": K, "warmup": W, "ms_per_step": secs / len(times) * 1e3,
        "higher_is_better": True, "scaling": "strong" if ens_mode else "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic", "config": config, "impl": "reference",
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
        "cpu_baseline_1core": one,
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def spawn_ranks(n_gpus):
    """--gpus N without a launcher: re-run this command under torch.distributed.run
    with N ranks on this node (one per GPU), after checking that N GPUs are
    visible.  Under a launcher, WORLD_SIZE must equal N."""
    env_world = os.environ.get("WORLD_SIZE")
    if env_world is not None:
        if int(env_world) != n_gpus:
            sys.exit(f"bench.py: --gpus {n_gpus} but WORLD_SIZE={env_world}")
        return
    if n_gpus <= 1:
        return
    import torch
    have = torch.cuda.device_count()
    if have < n_gpus:
        sys.exit(f"bench.py: --gpus {n_gpus} asked for, {have} visible")
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n_gpus}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__),
           *sys.argv[1:]]
    os.execv(sys.executable, cmd)


# ---------------------------------------------------------------- GPU timing
def timed_replays(graph_fn, K, W, stream, flush, world):
    """K graph replays bracketed by CUDA events on `stream`, L2 flushed before
    each (outside the events), after W untimed replays; returns (seconds, wall)."""
    import torch
    with torch.cuda.stream(stream):
        for _ in range(W):
            flush.zero_()
            graph_fn()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    dist_barrier(world)
    torch.cuda.synchronize()
    tw0 = time.time()
    with torch.cuda.stream(stream):
        for i in range(K):
            flush.zero_()
            ev[i][0].record(stream)
            graph_fn()
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    tw1 = time.time()
    dist_barrier(world)
    return dist_max(sum(a.elapsed_time(b) for a, b in ev) / 1e3, world), (tw0, tw1)


def capture(fn, stream, warm=2):
    import torch
    with torch.cuda.stream(stream):          # sets kernel attributes before capture
        for _ in range(warm):
            fn()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        fn()
    torch.cuda.synchronize()
    return g


def profiled(fn, steps, stream, flush):
    import torch
    import mhdgpu
    prof = mhdgpu.Profiler(max_records=steps * 2000 + 100)
    with torch.cuda.stream(stream):
        with prof:
            for _ in range(steps):
                flush.zero_()
                fn()
    torch.cuda.synchronize()
    s = prof.summary()
    prof.close()
    return s


TUNE_CACHE = None   # --tune-cache


def tune_tiles(n, math_mode):
    """mhdgpu_autotune for an n^3 box, or its picks from --tune-cache when the
    cache holds them for this device (then saved there after tuning); returns
    where the shapes came from."""
    import mhdgpu
    path = os.path.join(TUNE_CACHE, f"tiles_{n}_math{math_mode}.json") if TUNE_CACHE else None
    if path and os.path.exists(path) and mhdgpu.tile_cache_load(path) > 0:
        return "tile cache (mhdgpu_tile_cache_load)"
    mhdgpu.autotune(n, n, n, math_mode)
    if path:
        os.makedirs(TUNE_CACHE, exist_ok=True)
        mhdgpu.tile_cache_save(path)
    return "mhdgpu_autotune"


def tune_batch(bt, stream):
    """mhdgpu_batch_tune, or the schedule from --tune-cache when it was saved
    for this batch on this device model (then saved there after tuning)."""
    path = os.path.join(TUNE_CACHE, "batch_schedule.json") if TUNE_CACHE else None
    if path and os.path.exists(path) and bt.load_schedule(path):
        return "schedule cache (mhdgpu_batch_schedule_load)"
    bt.tune(stream=stream)
    if path:
        os.makedirs(TUNE_CACHE, exist_ok=True)
        bt.save_schedule(path)
    return "mhdgpu_batch_tune"


def single_box(n, K, W, stream, flush, world, dev, tune, math_mode):
    """The 128^3 (n^3) single-box numbers: fused and plain steps, the fluidx
    roofline and the e2e host-buffer call."""
    import torch
    import ics
    import mhdgpu
    ncell = n ** 3
    tiles_from = tune_tiles(n, math_mode) if tune else "defaults"
    picks = {(k, n, r): mhdgpu.get_tile(k, n, rows=r) for k in ("fluidx", "advectbyzx") for r in (False, True)}
    u0, b0 = ics.alfven_oblique(n)
    res = {"workload": f"alfven_diag_{n}", "box": [n, n, n],
           "tiles": {f"{k}@{m}{'/rows' if r else ''}": list(v) for (k, m, r), v in picks.items()},
           "tiles_from": tiles_from}
    for path, name in ((mhdgpu.MHD_PATH_FUSED, "fused"), (mhdgpu.MHD_PATH_PLAIN, "plain")):
        du = torch.from_numpy(u0).to(dev)
        db = torch.from_numpy(b0).to(dev)
        work = torch.empty(mhdgpu.step_workspace_bytes(n, n, n, path), dtype=torch.uint8, device=dev)
        clock = mhdgpu.new_clock(device=dev)
        started = [False]

        def one_step():
            # one step per call; after the first, the step continues the
            # previous one and takes the CFL speed its last sweep folded in
            mhdgpu.advance(du, db, n, n, n, 1, CFL, mhdgpu.MHD_CFL_C, 0.0, clock, None, work, path,
                           resume=started[0])
            started[0] = True

        g = capture(one_step, stream, W)
        secs, wall = timed_replays(g.replay, K, 1, stream, flush, world)
        summ = profiled(one_step, K, stream, flush)
        del g
        res[name] = {"value": world * ncell * K / secs, "ms_per_step": secs / K * 1e3,
                     "kernel_time_ms_per_step": {k: v[2] / K for k, v in summ.items()},
                     "kernel_launches_per_step": {k: v[1] / K for k, v in summ.items()},
                     "health": mhdgpu.read_clock(clock).health,
                     "path": "transpose-free step (mhdgpu_step_fused)" if name == "fused"
                     else "per-subroutine kernels + transposes (mhdgpu_step)"}
        if name == "fused":
            fl_rec, fl_launch, fl_ms = summ["fluidx"]
            fl_avg_s = fl_ms / 1e3 / max(fl_launch, 1)
            hbm, kind = peaks()
            ach = FLUIDX_BYTES_PER_CELL * ncell / fl_avg_s / 1e9
            tot_ms = sum(v[2] for v in summ.values())
            res["fluidx_roofline"] = {
                "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                "peak_source": f"{kind} (MEASURED_PEAKS.json hbm_gbs)",
                # the committed capture is of the 128^3 launch
                "traffic": read_traffic("fluidx_alfven128_ncu.txt") if n == 128 else None,
                "algorithmic_bytes_per_launch": FLUIDX_BYTES_PER_CELL * ncell,
                "avg_launch_us": fl_avg_s * 1e6, "share_of_step": fl_ms / tot_ms if tot_ms else None}
    res["fused_over_plain"] = res["fused"]["value"] / res["plain"]["value"]
    # end to end through the host-buffer entry (upload, one step, download per call)
    hu = torch.from_numpy(u0.copy()).pin_memory()
    hb = torch.from_numpy(b0.copy()).pin_memory()
    un, bn = hu.numpy(), hb.numpy()
    ke = max(3, min(K, 50))
    t = 0.0
    mhdgpu.run_host(un, bn, n, n, n, CFL, 0, t, 0.0, 1, path=mhdgpu.MHD_PATH_FUSED)
    dist_barrier(world)
    t0 = time.perf_counter()
    for _ in range(ke):
        _st, t, _d = mhdgpu.run_host(un, bn, n, n, n, CFL, 0, t, 0.0, 1, path=mhdgpu.MHD_PATH_FUSED)
    secs = dist_max(time.perf_counter() - t0, world)
    res["e2e"] = {"value": world * ncell * ke / secs, "unit": UNIT, "steps": ke,
                  "h2d_bytes_per_step": 32 * ncell, "d2h_bytes_per_step": 32 * ncell,
                  "api": "mhdgpu_run_host, 1 step per call"}
    return res


def ensemble_bench(ens, K, W, stream, flush, world, dev, tune, total_cells):
    """Batched ensemble vs box-by-box loops; e2e through mhdgpu_batch_* with
    the state uploaded from and downloaded to pinned host memory every step.
    ens is this rank's share of the boxes; rates count total_cells (every
    rank's boxes) over the slowest rank's time."""
    import numpy as np
    import torch
    import mhdgpu
    dims = [e["dims"] for e in ens]
    cells = int(sum(int(np.prod(d)) for d in dims))
    boxes = [(torch.from_numpy(e["u"]).to(dev), torch.from_numpy(e["b"]).to(dev), e["dims"]) for e in ens]
    bt = mhdgpu.Batch(boxes, cfl_number=CFL, cfl_mode=mhdgpu.MHD_CFL_C)
    sched_from = tune_batch(bt, stream) if tune else "defaults"
    sched = [bt.get_schedule(a) for a in range(3)]

    def step():
        # one step per call, continuing the previous one (the CFL speed comes
        # from its last sweep; the handle runs the pass before its first step)
        bt.advance(1, stream=stream, resume=True)

    g = capture(step, stream, 2)
    secs, wall = timed_replays(g.replay, K, W, stream, flush, world)
    del g
    summ = profiled(step, max(3, min(K, 20)), stream, flush)
    ksteps = max(3, min(K, 20))
    clocks = bt.clocks(stream=None, check=False)
    health = 0
    for c in clocks:
        health |= c.health
    value = total_cells * K / secs
    # one profiler record spans one sweep: the concurrent class launches of
    # every box (the unit the algorithmic bytes are counted on)
    b_rec, b_launch, b_ms = summ["batch"]
    avg_s = b_ms / 1e3 / max(b_rec, 1)
    hbm, kind = peaks()
    ach = SWEEP_BYTES_PER_CELL * cells / avg_s / 1e9
    pass_ach = SWEEP_PASS_BYTES_PER_CELL * cells / avg_s / 1e9
    tot_ms = sum(v[2] for v in summ.values())
    res = {"value": value, "ms_per_step": secs / K * 1e3, "cells": cells, "schedule": sched,
           "schedule_from": sched_from, "wall": wall,
           "kernel_time_ms_per_step": {k: v[2] / ksteps for k, v in summ.items()},
           "kernel_launches_per_step": {k: v[1] / ksteps for k, v in summ.items()},
           "health": health,
           "roofline": {"bound": "hbm",
                        "kernel": "batch_class_kernel: one sweep of every box (concurrent persistent "
                                  "launches, one per pencil-length class)",
                        "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                        "peak_source": f"{kind} (MEASURED_PEAKS.json hbm_gbs)",
                        "traffic": read_traffic("batch_class_ensemble64_ncu.txt"),
                        "algorithmic_bytes_per_launch": SWEEP_BYTES_PER_CELL * cells,
                        "algorithmic_basis": "64 B/cell per sweep: one read and one write of the "
                                             "8-float state",
                        "pass_bytes_diagnostic": {"bytes_per_cell": SWEEP_PASS_BYTES_PER_CELL,
                                                  "what": "fluid 52 + field flux 32 + b(1) gather 16",
                                                  "achieved_gbs": pass_ach, "frac": pass_ach / hbm},
                        "launch_unit": "one sweep (its class launches together)",
                        "avg_launch_us": avg_s * 1e6,
                        "share_of_step": b_ms / tot_ms if tot_ms else None}}
    # box by box: the fused single-box step and the plain per-subroutine drop-in,
    # each one CUDA graph holding the loop over the 64 boxes
    kb = max(3, min(K, 30))
    for path, name in ((mhdgpu.MHD_PATH_FUSED, "boxwise_fused"), (mhdgpu.MHD_PATH_PLAIN, "boxwise_plain")):
        works = [torch.empty(mhdgpu.step_workspace_bytes(*d, path), dtype=torch.uint8, device=dev) for d in dims]
        cks = [mhdgpu.new_clock(device=dev) for _ in dims]
        started = [False]

        def loop():
            for (u, b, d), w, c in zip(boxes, works, cks):
                mhdgpu.advance(u, b, *d, 1, CFL, mhdgpu.MHD_CFL_C, 0.0, c, None, w, path, stream=stream,
                               resume=started[0])
            started[0] = True

        gl = capture(loop, stream, 1)
        s2, _ = timed_replays(gl.replay, kb, 1, stream, flush, world)
        del gl
        res[name] = {"value": total_cells * kb / s2, "ms_per_step": s2 / kb * 1e3, "steps": kb,
                     "path": ("mhdgpu_advance path FUSED" if path else "mhdgpu_advance path PLAIN (per-subroutine drop-in)")
                     + " looped over the boxes, one CUDA graph per step"}
        del works
    res["batched_over_boxwise_plain"] = value / res["boxwise_plain"]["value"]
    res["batched_over_boxwise_fused"] = value / res["boxwise_fused"]["value"]
    # e2e: pinned host state, upload all boxes, one batched step, download all boxes
    hu = [torch.from_numpy(e["u"].copy()).pin_memory() for e in ens]
    hb = [torch.from_numpy(e["b"].copy()).pin_memory() for e in ens]
    ke = max(3, min(K, 20))

    def e2e_step():
        # one C-ABI call: upload every box, one step, download every box
        bt.run_host(hu, hb, 1, stream=stream)

    e2e_step()
    dist_barrier(world)
    t0 = time.perf_counter()
    for _ in range(ke):
        e2e_step()
    s3 = dist_max(time.perf_counter() - t0, world)
    res["e2e"] = {"value": total_cells * ke / s3, "unit": UNIT, "steps": ke,
                  "h2d_bytes_per_step": 32 * cells, "d2h_bytes_per_step": 32 * cells,
                  "api": "mhdgpu_batch_run_host (1 step per call): pinned host -> device copies of every "
                         "box, the batched step, device -> host copies, synchronised; the library "
                         "pipelines four parts of the boxes (a part's copies overlap the other parts' steps)"}
    bt.close()
    return res


def large_boxes(stream, dev):
    """The single-box step at the sizes of the blast and turbulence
    configurations (256^3 and 512^3) on MHD_PATH_AUTO: the diagonal Alfven
    wave on the 256^3 box, tiled 2x2x2 on the device for the 512^3 box (still
    an exact periodic wave; the time per step does not depend on the values),
    one warm step, then k steps in one advance call timed with CUDA events;
    the states are larger than L2."""
    import torch
    import ics
    import mhdgpu
    out = {}
    u0, b0 = ics.alfven_oblique(256)
    for n, k in ((256, 10), (512, 5)):
        r = n // 256
        du = torch.from_numpy(u0).to(dev).view(256, 256, 256, 5).repeat(r, r, r, 1).reshape(-1)
        db = torch.from_numpy(b0).to(dev).view(256, 256, 256, 3).repeat(r, r, r, 1).reshape(-1)
        auto = mhdgpu.MHD_PATH_AUTO
        work = torch.empty(mhdgpu.step_workspace_bytes(n, n, n, auto), dtype=torch.uint8, device=dev)
        clock = mhdgpu.new_clock(device=dev)
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            mhdgpu.advance(du, db, n, n, n, 1, CFL, mhdgpu.MHD_CFL_C, 0.0, clock, None, work, auto, stream=stream)
            a.record(stream)
            mhdgpu.advance(du, db, n, n, n, k, CFL, mhdgpu.MHD_CFL_C, 0.0, clock, None, work, auto,
                           stream=stream, resume=True)
            e.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(e) / k
        fused = mhdgpu.resolve_path(n, n, n) == mhdgpu.MHD_PATH_FUSED
        out[f"{n}^3"] = {"value": n ** 3 / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "steps": k,
                         "path": "MHD_PATH_AUTO -> " + ("transpose-free step" if fused else "plain step"),
                         "health": mhdgpu.read_clock(clock).health}
        del du, db, work
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ensemble64", choices=["ensemble64", "alfven_diag_128"])
    ap.add_argument("--n", type=int, default=128, help="box size of the single-box workload")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--math", default="faithful", choices=["faithful", "fast"])
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuners (default tiles)")
    ap.add_argument("--tune-cache", default=None,
                    help="directory of the autotuners' JSON picks: reused when they match this device and "
                         "workload, written after tuning otherwise")
    ap.add_argument("--headline-only", action="store_true",
                    help="time the headline path only (no secondary paths, e2e or CPU baseline); "
                         "for profiler captures")
    args = ap.parse_args()
    global TUNE_CACHE
    TUNE_CACHE = args.tune_cache
    n, K, W = args.n, args.steps, max(3, args.warmup)
    ens_mode = args.workload == "ensemble64"
    if args.impl == "ours":
        spawn_ranks(args.gpus)
    world_hint = int(os.environ.get("WORLD_SIZE", args.gpus))
    if ens_mode:
        config = {"workload": "ensemble64", "boxes": ENSEMBLE["nbox"], "sizes": list(ENSEMBLE["sizes"]),
                  "seed": ENSEMBLE["seed"], "amp_range": list(ENSEMBLE["amp_range"]),
                  "ic": "per box: linear Alfven wave on the box diagonal or turbulent start "
                        "(k^-2 velocity, k^-3 vector potential), amplitude log-uniform in [1e-4,1e-1]",
                  "cfl": CFL, "cfl_mode": "c_path",
                  "path": "batched: per sweep one persistent launch per pencil-length class over all "
                          "boxes, the classes concurrent, one CUDA graph per step",
                  "l2": "flushed between timed steps (512 MB write, outside the timed events); state 0.87 GB > L2",
                  "parallelism": f"boxes sharded across {world_hint} rank(s), balanced by cells"}
        import ics
        import shard
        ens_dims = ics.ensemble_dims(**ENSEMBLE)
        parts = shard.partition_boxes(ens_dims, world_hint)
        config["shard"] = {"ranks": world_hint, "boxes_per_rank": [len(p) for p in parts],
                           "cells_per_rank": shard.shard_cells(ens_dims, parts)}
    else:
        config = {"workload": f"alfven_diag_{n}", "box": [n, n, n], "cfl": CFL, "cfl_mode": "c_path",
                  "ic": "linear Alfven wave, k=(1,1,1)2pi/L, A=1e-3, rho=p=1, B0 along k",
                  "path": "transpose-free step (mhdgpu_step_fused), one CUDA graph per step",
                  "l2": "flushed between timed steps (512 MB write, outside the timed events)",
                  "parallelism": f"replicas x{world_hint}"}
    # the arithmetic: the faithful policy reproduces the reference C path's
    # rounding (the CPU arm runs that path's restatement); "fast" is plain FP32
    config["math"] = args.math

    if args.impl == "reference":
        reference_arm(args, config, ens_mode, n, K, W)
        return

    import torch

    import ics
    import mhdgpu

    rank, world, local = dist_setup(args.gpus)
    dev = torch.device("cuda", local if world > 1 else 0)
    math_mode = mhdgpu.MHD_MATH_FAST if args.math == "fast" else mhdgpu.MHD_MATH_FAITHFUL
    mhdgpu.set_math(math_mode)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    vis = [x.strip() for x in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if x.strip()]
    sampler = ClockSampler(vis[local] if len(vis) > local else local)
    sampler.start()
    time.sleep(0.3)
    tune = not args.no_tune

    if args.headline_only:
        if ens_mode:
            import shard
            ens = ics.ensemble(**ENSEMBLE)
            total = sum(e["dims"][0] * e["dims"][1] * e["dims"][2] for e in ens)
            parts = shard.partition_boxes([e["dims"] for e in ens], world)
            ens = [ens[i] for i in parts[rank]]
            boxes = [(torch.from_numpy(e["u"]).to(dev), torch.from_numpy(e["b"]).to(dev), e["dims"]) for e in ens]
            bt = mhdgpu.Batch(boxes, cfl_number=CFL, cfl_mode=mhdgpu.MHD_CFL_C)
            if tune:
                tune_batch(bt, stream)
            g = capture(lambda: bt.advance(1, stream=stream, resume=True), stream, 2)
            cells = total
        else:
            u0, b0 = ics.alfven_oblique(n)
            du, db = torch.from_numpy(u0).to(dev), torch.from_numpy(b0).to(dev)
            work = torch.empty(mhdgpu.step_workspace_bytes(n, n, n, 1), dtype=torch.uint8, device=dev)
            clock = mhdgpu.new_clock(device=dev)
            if tune:
                tune_tiles(n, math_mode)
            started = [False]

            def one_step():
                mhdgpu.advance(du, db, n, n, n, 1, CFL, 0, 0.0, clock, None, work, 1, resume=started[0])
                started[0] = True

            g = capture(one_step, stream, 2)
            cells = world * n ** 3
        secs, wall = timed_replays(g.replay, K, W, stream, flush, world)
        sampler.stop()
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": cells * K / secs, "unit": UNIT,
                              "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": secs / K * 1e3,
                              "config": config, "note": "--headline-only: no secondary measurements"}))
        return

    sb = single_box(n, K, W, stream, flush, world, dev, tune, math_mode)
    if ens_mode:
        import shard
        ens = ics.ensemble(**ENSEMBLE)
        total_cells = sum(e["dims"][0] * e["dims"][1] * e["dims"][2] for e in ens)
        # the boxes are independent: with N ranks each advances its share
        # (balanced by cells), no exchange on the data path
        parts = shard.partition_boxes([e["dims"] for e in ens], world)
        mine = [ens[i] for i in parts[rank]]
        eb = ensemble_bench(mine, K, W, stream, flush, world, dev, tune, total_cells)
        sampler.stop()
        clocks = sampler.summary(*eb["wall"])
        value, ms_step = eb["value"], eb["ms_per_step"]
        launches = eb["kernel_launches_per_step"]
        out_roof = eb["roofline"]
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded ensemble, see config)", "config": config,
            "gpu_launches": int(round(sum(launches.values()) * K)),
            "roofline": out_roof,
            "roofline_step": roofline_step(value, world, out_roof["peak"], dev, clocks,
                                           SWEEP_PASS_BYTES_PER_CELL * 6),
            "plain_drop_in": {"value": eb["boxwise_plain"]["value"], "unit": UNIT,
                              "ms_per_step": eb["boxwise_plain"]["ms_per_step"],
                              "path": eb["boxwise_plain"]["path"]},
            "fused_over_plain": eb["batched_over_boxwise_plain"],
            "ensemble": {k: v for k, v in eb.items() if k not in ("roofline", "wall", "e2e")},
            sb["workload"]: sb,
            "e2e": eb["e2e"], "clocks": clocks, "health": eb["health"],
        }
    else:
        sampler.stop()
        fused = sb["fused"]
        clocks = sampler.summary(0, time.time())
        out = {
            "metric": METRIC, "value": fused["value"], "unit": UNIT, "n_gpus": world, "steps": K,
            "warmup": W, "ms_per_step": fused["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seedless analytic initial state, see config.ic)", "config": config,
            "gpu_launches": int(round(sum(fused["kernel_launches_per_step"].values()) * K)),
            "roofline": sb["fluidx_roofline"],
            "roofline_step": roofline_step(fused["value"], world, sb["fluidx_roofline"]["peak"], dev, clocks,
                                           SWEEP_PASS_BYTES_PER_CELL * 6),
            "plain_drop_in": {"value": sb["plain"]["value"], "unit": UNIT,
                              "ms_per_step": sb["plain"]["ms_per_step"], "path": sb["plain"]["path"]},
            "fused_over_plain": sb["fused_over_plain"],
            sb["workload"]: sb, "e2e": sb["e2e"], "clocks": clocks, "health": fused["health"],
        }
    if world == 1:
        out["large_boxes"] = large_boxes(stream, dev)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            if ens_mode:
                rate, kind, cores, sample = cpu_rate_ensemble(ens, args.cpu_seconds, os.cpu_count() or 1)
            else:
                use_ref = os.path.exists(os.path.join(REPO, "oracle", "_ref", "libref_f32.so"))
                rate, kind, cores, sample = cpu_rate(n, args.cpu_seconds, os.cpu_count() or 1, use_ref)
            out["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": kind,
                                   "sample": sample + f"; {host_cpu()}"}
            if ens_mode:
                r1, k1, c1, s1 = cpu_rate_ensemble(ens, 6.0, 1)
            else:
                r1, k1, c1, s1 = cpu_rate(n, 6.0, 1, use_ref)
            out["cpu_baseline_1core"] = {"value": r1, "unit": UNIT, "cores": c1, "kind": k1, "sample": s1}
        except Exception as e:  # noqa: BLE001
            out["cpu_baseline"] = {"value": None, "unit": UNIT, "error": str(e)}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
