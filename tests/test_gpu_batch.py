"""GPU tests of the batched ensemble (mhdgpu_batch_*), through the C ABI.

The batch runs each box through the same tile functions and rounding as the
transpose-free single-box step, so the bar is bit-for-bit equality with
mhdgpu_advance(path = MHD_PATH_FUSED) run box by box (whose own parity with the
oracle is covered in test_gpu_parity.py), for the state and for the clocks.
"""
import numpy as np
import pytest

from util import bits_equal

pytestmark = pytest.mark.gpu

# every team class of the batched kernel, along x (contiguous pencils) and
# along y or z (pencils across memory): n = 32, 48, 64, 96, 128, other n < 64,
# other n < 128, n <= 256, and degenerate boxes
CLASS_BOXES = [(8, 16, 24), (32, 48, 20), (64, 40, 12), (96, 8, 16), (130, 12, 8), (16, 200, 8),
               (8, 8, 128), (100, 16, 10), (5, 7, 9), (1, 4, 3), (16, 96, 8), (48, 32, 64),
               (12, 128, 6)]


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _states(dims_list, seed=5, amp=0.2):
    import ics
    return [ics.random_state(*d, seed=seed + i, amp=amp) for i, d in enumerate(dims_list)]


def _per_box(gpu, states, dims_list, nsteps, cfl, mode=0, tf=None):
    import torch
    out = []
    for i, ((u, b), d) in enumerate(zip(states, dims_list)):
        du, db = dev(u), dev(b)
        work = torch.empty(gpu.step_workspace_bytes(*d, gpu.MHD_PATH_FUSED), dtype=torch.uint8, device="cuda")
        clock = gpu.new_clock()
        log = torch.zeros(max(nsteps, 1), dtype=torch.float32, device="cuda")
        gpu.advance(du, db, *d, nsteps, cfl, mode, 0.0 if tf is None else tf[i], clock, log, work,
                    gpu.MHD_PATH_FUSED)
        out.append((host(du), host(db), gpu.read_clock(clock)))
    return out


def _batched(gpu, states, dims_list, nsteps, cfl, mode=0, tf=None, schedule=None):
    boxes = [(dev(u), dev(b), d) for (u, b), d in zip(states, dims_list)]
    bt = gpu.Batch(boxes, cfl_number=cfl, cfl_mode=mode, tf=tf)
    if schedule:
        for axis, (t, c) in enumerate(schedule):
            bt.set_schedule(axis, t, c)
    bt.advance(nsteps)
    clocks = bt.clocks()
    res = [(host(u), host(b), c) for (u, b, _), c in zip(boxes, clocks)]
    bt.close()
    return res


def _same(a, b):
    for (u1, b1, c1), (u2, b2, c2) in zip(a, b):
        assert bits_equal(u1, u2) and bits_equal(b1, b2)
        assert (c1.t, c1.dt, c1.iter, c1.health) == (c2.t, c2.dt, c2.iter, c2.health)


@pytest.mark.parametrize("mode", [0, 1])
def test_batch_equals_per_box_fused_bitwise(gpu, mode):
    """Every team class (all pencil-length classes along x, y and z), both CFL
    formulas: the batch ends where the boxes advanced one by one end."""
    states = _states(CLASS_BOXES)
    ref = _per_box(gpu, states, CLASS_BOXES, 4, 0.7, mode)
    got = _batched(gpu, states, CLASS_BOXES, 4, 0.7, mode)
    _same(got, ref)
    assert all(c.iter == 4 for _, _, c in got)


@pytest.mark.parametrize("schedule", [[(256, 1)] * 3, [(128, 2)] * 3, [(128, 4), (256, 2), (128, 1)],
                                      [(256, 8)] * 3])
def test_batch_schedules_agree(gpu, schedule):
    """The block schedule (pencils per CTA, CTAs per SM) changes no value."""
    dims = CLASS_BOXES
    states = _states(dims, seed=11)
    ref = _batched(gpu, states, dims, 2, 0.8)
    got = _batched(gpu, states, dims, 2, 0.8, schedule=schedule)
    _same(got, ref)


def test_batch_threads64_without_long_pencils(gpu):
    """64 threads per CTA serve pencils up to 127 cells; longer ones need a
    128-thread team and the schedule is refused."""
    dims = [(8, 16, 24), (100, 16, 10), (32, 48, 20)]
    states = _states(dims, seed=2)
    ref = _batched(gpu, states, dims, 2, 0.7)
    got = _batched(gpu, states, dims, 2, 0.7, schedule=[(64, 4)] * 3)
    _same(got, ref)
    boxes = [(dev(u), dev(b), d) for (u, b), d in zip(_states([(130, 4, 4)]), [(130, 4, 4)])]
    bt = gpu.Batch(boxes)
    with pytest.raises(gpu.MhdError) as ei:
        bt.set_schedule(0, 64, 2)
    assert ei.value.status == gpu.MHD_ERR_ARG
    bt.set_schedule(1, 64, 2)   # y and z pencils are 4 cells long: fine
    bt.close()


def test_batch_tf_clamp_and_stop(gpu):
    """Per-box end times: dt clamps to (tf - t)/2 and steps after the end are
    no-ops, as in mhdgpu_advance."""
    dims = [(16, 16, 16), (24, 8, 12), (32, 12, 8)]
    states = _states(dims, seed=9, amp=0.1)
    tf = [0.5, 1.0, 100.0]
    ref = _per_box(gpu, states, dims, 12, 0.9, tf=tf)
    got = _batched(gpu, states, dims, 12, 0.9, tf=tf)
    _same(got, ref)
    assert abs(got[0][2].t - 0.5) < 1e-6 and got[0][2].iter < 12


def test_batch_tune_restores_state(gpu):
    """The autotuner times schedules on the batch's own boxes and puts the
    state and clocks back: afterwards the run equals an untuned one."""
    dims = [(32, 48, 20), (64, 40, 12), (96, 8, 16), (16, 200, 8)]
    states = _states(dims, seed=3)
    ref = _batched(gpu, states, dims, 3, 0.7)
    boxes = [(dev(u), dev(b), d) for (u, b), d in zip(states, dims)]
    bt = gpu.Batch(boxes, cfl_number=0.7)
    sched = bt.tune()
    assert all(t in (64, 128, 256) and c in (2, 4, 8) for t, c in sched)
    for (u, b, _), (u0, b0) in zip(boxes, states):
        assert bits_equal(host(u), u0) and bits_equal(host(b), b0)
    assert all(c.iter == 0 and c.t == 0.0 for c in bt.clocks())
    bt.advance(3)
    clocks = bt.clocks()
    got = [(host(u), host(b), c) for (u, b, _), c in zip(boxes, clocks)]
    bt.close()
    _same(got, ref)


def test_schedule_change_waits_for_steps_in_flight(gpu):
    """A schedule change (mhdgpu_batch_set_schedule, mhdgpu_batch_tune) issued
    while steps of the handle still run on a non-blocking stream waits for them
    before it uploads the new work tables: no dependency wait gives up, and the
    run ends where one with a synchronisation before each change ends."""
    import torch
    dims = [(128, 128, 64), (96, 64, 64), (64, 64, 32), (32, 48, 128)]
    states = _states(dims, seed=41, amp=0.1)
    s = torch.cuda.Stream()
    runs = []
    for sync in (True, False):
        boxes = [(dev(u), dev(b), d) for (u, b), d in zip(states, dims)]
        torch.cuda.synchronize()
        bt = gpu.Batch(boxes, cfl_number=0.7)
        bt.advance(6, stream=s)
        if sync:
            torch.cuda.synchronize()
        for axis in range(3):
            bt.set_schedule(axis, 128, 2)
        bt.advance(4, stream=s, resume=True)
        if sync:
            torch.cuda.synchronize()
        bt.tune(stream=s)
        bt.advance(2, stream=s, resume=True)
        torch.cuda.synchronize()
        clocks = bt.clocks()            # raises MHD_ERR_TIMEOUT if a wait gave up
        runs.append([(host(u), host(b), c) for (u, b, _), c in zip(boxes, clocks)])
        bt.close()
    _same(runs[1], runs[0])


def test_batch_graph_replay(gpu):
    """A captured step replays to the same state as eager steps."""
    import torch
    dims = [(32, 16, 24), (48, 32, 16), (8, 64, 8)]
    states = _states(dims, seed=4)
    ref = _batched(gpu, states, dims, 3, 0.7)
    boxes = [(dev(u), dev(b), d) for (u, b), d in zip(states, dims)]
    bt = gpu.Batch(boxes, cfl_number=0.7)
    s = torch.cuda.Stream()
    # snapshot, warm the launch path once, restore, then capture one step
    snap = [(u.clone(), b.clone()) for u, b, _ in boxes]
    with torch.cuda.stream(s):
        bt.advance(1)
    torch.cuda.synchronize()
    bt.close()
    for (u, b, _), (u0, b0) in zip(boxes, snap):
        u.copy_(u0)
        b.copy_(b0)
    bt = gpu.Batch(boxes, cfl_number=0.7)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        bt.advance(1, stream=s)
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    clocks = bt.clocks()
    got = [(host(u), host(b), c) for (u, b, _), c in zip(boxes, clocks)]
    bt.close()
    _same(got, ref)


@pytest.mark.parametrize("path", [0, 1])
def test_advance_resume_equals_one_call(gpu, path):
    """One step per call with MHD_ADVANCE_RESUME after the first (the CFL speed
    taken from the previous step's fold instead of a pass) ends where one
    multi-step call ends, bit for bit, state and clock."""
    import torch
    d = (48, 32, 16)
    u0, b0 = _states([d], seed=21)[0]
    runs = []
    for resume in (False, True):
        du, db = dev(u0), dev(b0)
        work = torch.empty(gpu.step_workspace_bytes(*d, path), dtype=torch.uint8, device="cuda")
        clock = gpu.new_clock()
        if resume:
            gpu.advance(du, db, *d, 1, 0.7, 0, 0.0, clock, None, work, path)
            for _ in range(3):
                gpu.advance(du, db, *d, 1, 0.7, 0, 0.0, clock, None, work, path, resume=True)
        else:
            gpu.advance(du, db, *d, 4, 0.7, 0, 0.0, clock, None, work, path)
        runs.append((host(du), host(db), gpu.read_clock(clock)))
    _same([runs[1]], [runs[0]])
    assert runs[1][2].iter == 4


@pytest.mark.parametrize("path", [0, 1])
def test_new_state_after_steps_takes_its_own_cfl(gpu, path):
    """A step's last sweep folds the next CFL speed into the clock; a later
    call without resume on a state written in between (a slower one here)
    must take that state's own speed, as a fresh clock does: single box and
    batch (device and host-buffer entries)."""
    import torch
    d = (32, 24, 16)
    fast = _states([d], seed=3, amp=0.6)[0]
    slow = _states([d], seed=4, amp=0.01)[0]
    work = torch.empty(gpu.step_workspace_bytes(*d, path), dtype=torch.uint8, device="cuda")
    ref_u, ref_b = dev(slow[0]), dev(slow[1])
    ref_clk = gpu.new_clock()
    gpu.advance(ref_u, ref_b, *d, 1, 0.7, 0, 0.0, ref_clk, None, work, path)
    ref = gpu.read_clock(ref_clk)
    du, db = dev(fast[0]), dev(fast[1])
    clk = gpu.new_clock()
    gpu.advance(du, db, *d, 2, 0.7, 0, 0.0, clk, None, work, path)
    du.copy_(dev(slow[0]))
    db.copy_(dev(slow[1]))
    t0 = gpu.read_clock(clk).t
    gpu.advance(du, db, *d, 1, 0.7, 0, 0.0, clk, None, work, path)
    c = gpu.read_clock(clk)
    assert c.dt == ref.dt and c.t == np.float32(np.float32(t0) + np.float32(2) * np.float32(ref.dt))
    assert bits_equal(host(du), host(ref_u)) and bits_equal(host(db), host(ref_b))
    if path:
        return
    dims = [d, (16, 40, 8)]
    fasts = _states(dims, seed=7, amp=0.6)
    slows = _states(dims, seed=8, amp=0.01)
    ref_batch = _batched(gpu, slows, dims, 1, 0.7)
    boxes = [(dev(u), dev(b), dd) for (u, b), dd in zip(fasts, dims)]
    bt = gpu.Batch(boxes, cfl_number=0.7)
    bt.advance(2)
    for (u, b, _), (su, sb) in zip(boxes, slows):
        u.copy_(dev(su))
        b.copy_(dev(sb))
    bt.advance(1)
    got = [(host(u), host(b), c) for (u, b, _), c in zip(boxes, bt.clocks())]
    assert [g[2].dt for g in got] == [r[2].dt for r in ref_batch]
    assert all(bits_equal(g[0], r[0]) and bits_equal(g[1], r[1]) for g, r in zip(got, ref_batch))
    hu = [torch.from_numpy(u.copy()).pin_memory() for u, _ in slows]
    hb = [torch.from_numpy(b.copy()).pin_memory() for _, b in slows]
    bt.run_host(hu, hb, 1)               # a host state written over the stepped one
    got = [c.dt for c in bt.clocks()]
    assert got == [r[2].dt for r in ref_batch]
    bt.close()


def test_batch_resume_equals_one_call(gpu):
    """mhdgpu_batch_resume continues without the CFL pass and ends where one
    multi-step mhdgpu_batch_advance ends; on a handle that has not advanced
    yet it runs the pass (same result as advance)."""
    dims = CLASS_BOXES
    states = _states(dims, seed=17)
    ref = _batched(gpu, states, dims, 3, 0.7)
    boxes = [(dev(u), dev(b), d) for (u, b), d in zip(states, dims)]
    bt = gpu.Batch(boxes, cfl_number=0.7)
    bt.advance(1, resume=True)     # first call: no fold yet, the pass runs
    bt.advance(1, resume=True)
    bt.advance(1, resume=True)
    clocks = bt.clocks()
    got = [(host(u), host(b), c) for (u, b, _), c in zip(boxes, clocks)]
    bt.close()
    _same(got, ref)


def test_auto_path_resolves_and_matches(gpu):
    """MHD_PATH_AUTO takes the transpose-free step for boxes whose y and z
    pencils are at most 48 cells, the plain step otherwise, and ends where
    the path it resolves to ends (the two paths are bit-identical)."""
    import torch
    assert gpu.resolve_path(64, 48, 32) == gpu.MHD_PATH_FUSED
    assert gpu.resolve_path(256, 16, 48) == gpu.MHD_PATH_FUSED
    assert gpu.resolve_path(64, 128, 96) == gpu.MHD_PATH_PLAIN
    assert gpu.resolve_path(16, 256, 32) == gpu.MHD_PATH_PLAIN
    assert gpu.resolve_path(16, 8, 200) == gpu.MHD_PATH_PLAIN
    assert gpu.resolve_path(512, 512, 512) == gpu.MHD_PATH_PLAIN
    for d in [(24, 16, 20), (8, 4, 160)]:
        u0, b0 = _states([d], seed=29)[0]
        runs = []
        for path in (gpu.MHD_PATH_AUTO, gpu.resolve_path(*d)):
            du, db = dev(u0), dev(b0)
            work = torch.empty(gpu.step_workspace_bytes(*d, path), dtype=torch.uint8, device="cuda")
            clock = gpu.new_clock()
            gpu.advance(du, db, *d, 3, 0.7, 0, 0.0, clock, None, work, path)
            runs.append((host(du), host(db), gpu.read_clock(clock)))
        _same([runs[0]], [runs[1]])


def test_batch_run_host_equals_device_path(gpu):
    """mhdgpu_batch_run_host (upload, steps, download, from pinned and from
    pageable host buffers) ends where the device path ends, bit for bit."""
    import torch
    dims = CLASS_BOXES
    states = _states(dims, seed=23)
    ref = _batched(gpu, states, dims, 2, 0.7)
    for pinned in (True, False):
        boxes = [(dev(np.zeros_like(u)), dev(np.zeros_like(b)), d) for (u, b), d in zip(states, dims)]
        bt = gpu.Batch(boxes, cfl_number=0.7)
        hu = [torch.from_numpy(u.copy()) for u, _ in states]
        hb = [torch.from_numpy(b.copy()) for _, b in states]
        if pinned:
            hu = [x.pin_memory() for x in hu]
            hb = [x.pin_memory() for x in hb]
        bt.run_host(hu, hb, 1)
        bt.run_host(hu, hb, 1)
        clocks = bt.clocks()
        got = [(x.numpy(), y.numpy(), c) for x, y, c in zip(hu, hb, clocks)]
        bt.close()
        _same(got, ref)


def test_batch_run_host_pipeline_resume_and_reschedule(gpu):
    """The host entry's pipeline over parts leaves the folded CFL speeds in
    the handle's clocks (a resumed device step continues it), rebuilds its
    parts after a schedule change, and a single-box handle takes the direct
    path; every run ends where the device path ends, bit for bit."""
    import torch
    dims = CLASS_BOXES[:7]
    states = _states(dims, seed=31)
    ref = _batched(gpu, states, dims, 4, 0.7)
    boxes = [(dev(np.zeros_like(u)), dev(np.zeros_like(b)), d) for (u, b), d in zip(states, dims)]
    bt = gpu.Batch(boxes, cfl_number=0.7)
    hu = [torch.from_numpy(u.copy()).pin_memory() for u, _ in states]
    hb = [torch.from_numpy(b.copy()).pin_memory() for _, b in states]
    bt.run_host(hu, hb, 2)
    bt.advance(1, resume=True)
    for axis in range(3):
        bt.set_schedule(axis, 128, 4)
    hu = [u.cpu().pin_memory() for u, _, _ in boxes]
    hb = [b.cpu().pin_memory() for _, b, _ in boxes]
    bt.run_host(hu, hb, 1)
    clocks = bt.clocks()
    got = [(x.numpy(), y.numpy(), c) for x, y, c in zip(hu, hb, clocks)]
    bt.close()
    _same(got, ref)
    one = [dims[1]]
    ref1 = _batched(gpu, states[1:2], one, 2, 0.7)
    box1 = [(dev(np.zeros_like(states[1][0])), dev(np.zeros_like(states[1][1])), one[0])]
    b1 = gpu.Batch(box1, cfl_number=0.7)
    hu1 = [torch.from_numpy(states[1][0].copy())]
    hb1 = [torch.from_numpy(states[1][1].copy())]
    b1.run_host(hu1, hb1, 2)
    got1 = [(hu1[0].numpy(), hb1[0].numpy(), b1.clocks()[0])]
    b1.close()
    _same(got1, ref1)


def test_batch_fast_math_matches_per_box(gpu):
    """The fast policy lets the compiler contract multiply-adds, and the
    contraction can differ between the single-box and the batched kernels in
    the last bit; the faithful policy (the other tests) is bit-reproducible.
    Here: agreement within 1e-5 per field and in dt."""
    from util import field_errors
    dims = [(32, 48, 20), (100, 16, 10), (8, 8, 128)]
    states = _states(dims, seed=8)
    prev = gpu.set_math(gpu.MHD_MATH_FAST)
    try:
        ref = _per_box(gpu, states, dims, 3, 0.7)
        got = _batched(gpu, states, dims, 3, 0.7)
    finally:
        gpu.set_math(prev)
    for (u1, b1, c1), (u2, b2, c2) in zip(got, ref):
        assert max(field_errors(u1, u2, 5)) < 1e-5 and max(field_errors(b1, b2, 3)) < 1e-5
        assert c1.iter == c2.iter and abs(c1.dt - c2.dt) <= 1e-5 * abs(c2.dt)


def test_batch_fp64_pressure_equals_per_box(gpu):
    """The FP64 pressure-recovery policy on low-beta boxes: bit for bit."""
    import ics
    dims = [(32, 24, 16), (48, 32, 20)]
    states = [ics.blast(d[0], ny=d[1], nz=d[2]) for d in dims]
    prev = gpu.set_math(gpu.MHD_MATH_FP64P)
    try:
        ref = _per_box(gpu, states, dims, 3, 0.7)
        got = _batched(gpu, states, dims, 3, 0.7)
    finally:
        gpu.set_math(prev)
    _same(got, ref)


def test_batch_ensemble_workload_sample(gpu):
    """Twelve boxes of the ensemble workload (sizes {32,48,64,96,128} by
    seed, Alfven or turbulent starts): equal to box-by-box runs, finite, with
    div B held at round-off."""
    import ics
    ens = ics.ensemble(12, seed=1, sizes=(32, 48, 64))
    dims = [e["dims"] for e in ens]
    states = [(e["u"], e["b"]) for e in ens]
    ref = _per_box(gpu, states, dims, 5, 0.7)
    got = _batched(gpu, states, dims, 5, 0.7)
    _same(got, ref)
    for (u, b, c), e in zip(got, ens):
        assert np.isfinite(u).all() and c.health & (gpu.MHD_HEALTH_NONFINITE | gpu.MHD_HEALTH_DENSITY) == 0
        # round-off of the face updates: a few ulps of |B| per step
        bound = 2 * ics.div_b(e["b"], *e["dims"]) + 5 * 16 * 2.0 ** -24 * float(np.abs(b).max())
        assert ics.div_b(b, *e["dims"]) < bound


def test_batch_wait_timeout_is_reported_and_context_survives(gpu):
    """A dependency wait that cannot be satisfied (the test hook asks for one
    item more than exist) gives up after its bounded limit: the box's health
    carries MHD_HEALTH_STALL, the launch drains, the host reads
    MHD_ERR_TIMEOUT, and the CUDA context keeps working for a new batch."""
    import time
    import torch
    dims = [(16, 8, 8), (8, 16, 8)]
    states = _states(dims, seed=6)
    boxes = [(dev(u), dev(b), d) for (u, b), d in zip(states, dims)]
    bt = gpu.Batch(boxes, cfl_number=0.7)
    bt.inject_stall()
    t0 = time.time()
    bt.advance(1)
    torch.cuda.synchronize()
    el = time.time() - t0
    with pytest.raises(gpu.MhdError) as ei:
        bt.clocks()
    assert ei.value.status == gpu.MHD_ERR_TIMEOUT
    assert bt.clocks(check=False)[0].health & gpu.MHD_HEALTH_STALL
    assert 1.0 < el < 30.0
    bt.close()
    ref = _per_box(gpu, states, dims, 2, 0.7)
    got = _batched(gpu, states, dims, 2, 0.7)
    _same(got, ref)


def test_batch_schedule_cache(gpu, tmp_path):
    """mhdgpu_batch_schedule_save / _load: a saved schedule applies to a batch
    of the same boxes (same signature) and leaves a batch of other boxes as it
    is; the reloaded schedule steps bit for bit like the original."""
    import json
    dims = [(32, 48, 20), (16, 96, 8), (48, 32, 64)]
    states = _states(dims)
    boxes = [(dev(u), dev(b), d) for (u, b), d in zip(states, dims)]
    bt = gpu.Batch(boxes, cfl_number=0.7)
    bt.set_schedule(0, 128, 4)
    bt.set_schedule(2, 64, 2)
    p = tmp_path / "schedule.json"
    bt.save_schedule(str(p))
    rec = json.load(open(p))
    assert rec["format"] == "mhdgpu batch schedule 1" and rec["boxes"] == 3
    assert rec["schedule"][0] == {"axis": 0, "threads": 128, "ctas_per_sm": 4}
    bt.advance(2)
    ref = [(host(u), host(b)) for u, b, _ in boxes]
    bt.close()
    boxes2 = [(dev(u), dev(b), d) for (u, b), d in zip(states, dims)]
    bt2 = gpu.Batch(boxes2, cfl_number=0.7)
    assert bt2.get_schedule(0) != (128, 4) or bt2.get_schedule(2) != (64, 2)
    assert bt2.load_schedule(str(p))
    assert bt2.get_schedule(0) == (128, 4) and bt2.get_schedule(2) == (64, 2)
    assert bt2.get_schedule(1) == tuple((rec["schedule"][1]["threads"], rec["schedule"][1]["ctas_per_sm"]))
    bt2.advance(2)
    for (ru, rb), (u, b, _) in zip(ref, boxes2):
        assert bits_equal(host(u), ru) and bits_equal(host(b), rb)
    bt2.close()
    other = [(dev(u), dev(b), d) for (u, b), d in zip(_states(dims[:2]), dims[:2])]
    bt3 = gpu.Batch(other, cfl_number=0.7)
    before = [bt3.get_schedule(a) for a in range(3)]
    assert not bt3.load_schedule(str(p))
    assert [bt3.get_schedule(a) for a in range(3)] == before
    bt3.close()
