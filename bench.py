#!/usr/bin/env python
"""Benchmark of the streamParanumal streaming suite on GB300.

One step = one pass of the FP64 BS1-BS8 suite, each kernel called exactly as the
reference's drivers call it:
  BS1 copy, BS2 axpy, BS3 norm (bs3_1+bs3_2; stage 1 is the integer-pipe norm that
  the drivers run by default), BS4 dot (bs4_1+bs4_2), BS5 CG update
  (bs5_1+bs5_2; stage 1 with r.r on the integer pipe, the drivers' default) on
  vectors of N = 2^28 doubles (the top of the 2^10..2^28 sweep), and
  BS6 gather, BS7 scatter, BS8 gather+scatter on a 64x64x64 hex box at p=7 whose
  element slots are permuted from a seed (134,217,728 local / 90,518,849 global nodes).
value = sum of the reference's accounted bytes (bs{1..8}Run.cpp) / step time, GB/s.
Inputs are seeded synthetic data (no dataset is involved); every vector is larger
than the 129 MB L2, so no flush is needed between steps.

--impl reference times the CPU restatement of the same path (oracle/, OpenMP on all
host cores) on a bounded sample of the workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "BS1-8 HBM GB/s (reference byte accounting), FP64 suite"
UNIT = "GB/s"
E2E_REPEATS = 5


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nlog2", type=int, default=28, help="vector length 2^k for BS1-BS5")
    ap.add_argument("--mesh", type=int, default=64, help="box edge in elements for BS6-BS8")
    ap.add_argument("--p", type=int, default=7)
    ap.add_argument("--perm-seed", type=int, default=20240607)
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-nlog2", type=int, default=24)
    ap.add_argument("--cpu-mesh", type=int, default=32)
    ap.add_argument("--json-out", default=None)
    ap.add_argument("--batch", action="store_true",
                    help="the batched workload: 256 uneven instances (CG update + BS8 each), "
                         "one persistent launch vs per-instance launches, plain and graphed")
    ap.add_argument("--degree-sweep", default=None,
                    help="comma list of degrees (e.g. 1-15): per degree, autotune and time "
                         "BS6-BS8 on a box of ~1e8 local nodes, lexicographic and permuted")
    ap.add_argument("--sweep-nodes", type=float, default=1e8)
    ap.add_argument("--save-tuning", action="store_true",
                    help="write the winners of --degree-sweep to the tuning table")
    ap.add_argument("--batch-count", type=int, default=256)
    ap.add_argument("--batch-emax", type=int, default=40)
    ap.add_argument("--kernels-only", action="store_true",
                    help="time the suite only (no e2e, BS0, clock soak or CPU leg): for ncu")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip detail.batch and detail.degree_sample of the default run")
    ap.add_argument("--sample-degrees", default="1,3,7,15",
                    help="degrees of detail.degree_sample")
    return ap.parse_args()


# ---------------------------------------------------------------- byte accounting
def bytes_bs(N: int) -> dict:
    """bs1Run.cpp:82-84, bs2Run.cpp:85-87, bs3Run.cpp:90-92, bs4Run.cpp:90-92,
    bs5Run.cpp:94-96."""
    return {"BS1": 16 * N, "BS2": 24 * N, "BS3": 8 * N, "BS4": 16 * N, "BS5": 24 * N}


def bytes_ogs(Nt: int, Ng: int, val: int = 8) -> dict:
    """bs6Run.cpp:58-63, bs7Run.cpp:58-63, bs8Run.cpp:56-61 (dlong = 4 bytes)."""
    return {"BS6": (Ng + 1) * 4 + Nt * 4 + Nt * val + Ng * val,
            "BS7": (Ng + 1) * 4 + Nt * 4 + Ng * val + Nt * val,
            "BS8": (Ng + 1) * 4 + Nt * 4 + 2 * Nt * val}


# ---------------------------------------------------------------- replicas
def max_over_ranks(x: float, device) -> float:
    """The largest x over all ranks of the process group (the job's step time is its
    slowest replica's); x itself when no group is running."""
    import torch
    import torch.distributed as tdist

    if not (tdist.is_available() and tdist.is_initialized()) or tdist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world: int, bytes_per_step: int, ms_per_step: float) -> float:
    """Whole-job GB/s: every replica moves bytes_per_step per step (weak scaling)."""
    return world * bytes_per_step / 1e9 / (ms_per_step / 1e3)


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"sp_clocks_gpu{gpu}_{os.getpid()}.csv"

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.gpu), "-lms", "100"], stdout=self.fh, stderr=subprocess.DEVNULL)
            self.t0 = time.time()
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.fh.close()
        rows = []
        for line in self.path.read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[4:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for _, _, r in rows:
            for name, val in zip(names, r[1:]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": rows[0][1],
                "reasons": sorted(reasons), "samples": len(rows)}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic() -> dict:
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


# ---------------------------------------------------------------- CPU baseline
def cpu_sample(nlog2: int, mesh: int, p: int, perm_seed: int, seed: int, reps: int = 3):
    """Times the oracle (OpenMP, all host cores) on a bounded sample of the
    workload.  Returns (GB/s, description, cores)."""
    import numpy as np

    from oracle import oracle as orc

    N = 1 << nlog2
    a = orc.uniform(N, seed)
    b = orc.uniform(N, seed + 1)
    ids = orc.box_hex_ids(mesh, mesh, mesh, p, perm_seed)
    csr = orc.ogs_setup(ids, kind=1, unique=True)
    rs, ci = csr["rsT"], csr["ciT"]
    Nt, Ng = ids.size, rs.size - 1
    q = orc.uniform(Nt, seed + 2)
    gq = np.zeros(Ng)
    alpha, beta = 0.5, -0.25
    nb256 = max(1, min((N + 255) // 256, 256))
    nb1024 = max(1, min((N + 1023) // 1024, 1024))
    lib = orc.load()
    D = orc._d

    def one_pass():
        lib.or_bs1(N, D(a), D(b))
        lib.or_bs2(N, alpha, D(a), beta, D(b), 1)
        part = np.zeros(1024)
        out = np.zeros(1)
        lib.or_bs3_1(256, nb256, N, D(a), D(part), 1)
        lib.or_finish(256, nb256, D(part), D(out))
        lib.or_bs4_1(256, nb256, N, D(a), D(b), D(part), 1)
        lib.or_finish(256, nb256, D(part), D(out))
        lib.or_bs5_1(1024, nb1024, N, D(a), alpha, D(b), D(part), 1)
        lib.or_finish(1024, nb1024, D(part), D(out))
        lib.or_ogs_gather(1, 0, Ng, orc._i32(rs), orc._i32(ci), 1, gq.ctypes.data, q.ctypes.data)
        lib.or_ogs_scatter(1, Ng, orc._i32(rs), orc._i32(ci), 1, q.ctypes.data, gq.ctypes.data)
        lib.or_ogs_gather_scatter(1, 0, Ng, orc._i32(rs), orc._i32(ci), orc._i32(rs),
                                  orc._i32(ci), 1, q.ctypes.data)

    nbytes = sum(bytes_bs(N).values()) + sum(bytes_ogs(Nt, Ng).values())
    one_pass()
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        one_pass()
        times.append(time.perf_counter() - t0)
    gbs = nbytes / 1e9 / statistics.median(times)
    desc = (f"oracle restatement (OpenMP) of the same FP64 suite at N=2^{nlog2} and a "
            f"{mesh}^3 p={p} permuted box ({Nt} local nodes); median of {reps} passes")
    return gbs, desc, os.cpu_count(), nbytes, statistics.median(times)


def run_reference(args, rank: int):
    if rank != 0:
        return
    from streamparanumal_gb300 import _build

    _build.build_oracle()
    import numpy as np

    from oracle import oracle as orc

    N = 1 << args.cpu_nlog2
    seed = args.seed
    a = orc.uniform(N, seed)
    b = orc.uniform(N, seed + 1)
    mesh, p = args.cpu_mesh, args.p
    ids = orc.box_hex_ids(mesh, mesh, mesh, p, args.perm_seed)
    csr = orc.ogs_setup(ids, kind=1, unique=True)
    rs, ci = csr["rsT"], csr["ciT"]
    Nt, Ng = ids.size, rs.size - 1
    q = orc.uniform(Nt, seed + 2)
    gq = np.zeros(Ng)
    lib = orc.load()
    D = orc._d
    nb256 = max(1, min((N + 255) // 256, 256))
    nb1024 = max(1, min((N + 1023) // 1024, 1024))
    part = np.zeros(1024)
    out = np.zeros(1)

    def step():
        lib.or_bs1(N, D(a), D(b))
        lib.or_bs2(N, 0.5, D(a), -0.25, D(b), 1)
        lib.or_bs3_1(256, nb256, N, D(a), D(part), 1)
        lib.or_finish(256, nb256, D(part), D(out))
        lib.or_bs4_1(256, nb256, N, D(a), D(b), D(part), 1)
        lib.or_finish(256, nb256, D(part), D(out))
        lib.or_bs5_1(1024, nb1024, N, D(a), 0.5, D(b), D(part), 1)
        lib.or_finish(1024, nb1024, D(part), D(out))
        lib.or_ogs_gather(1, 0, Ng, orc._i32(rs), orc._i32(ci), 1, gq.ctypes.data, q.ctypes.data)
        lib.or_ogs_scatter(1, Ng, orc._i32(rs), orc._i32(ci), 1, q.ctypes.data, gq.ctypes.data)
        lib.or_ogs_gather_scatter(1, 0, Ng, orc._i32(rs), orc._i32(ci), orc._i32(rs),
                                  orc._i32(ci), 1, q.ctypes.data)

    nbytes = sum(bytes_bs(N).values()) + sum(bytes_ogs(Nt, Ng).values())
    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    el = time.perf_counter() - t0
    gbs = nbytes * args.steps / 1e9 / el
    desc = (f"each step: the FP64 suite at N=2^{args.cpu_nlog2} and a {mesh}^3 p={p} "
            f"permuted box ({Nt} local nodes), a bounded sample of the GPU workload")
    line = {"metric": METRIC, "value": round(gbs, 3), "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(el / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded uniform[-1,1])", "impl": "reference",
            "config": {"workload": "BS1-BS8 FP64 suite (CPU sample)", "n": N,
                       "mesh": f"{mesh}^3 p={p} permuted", "bytes_per_step": nbytes},
            "cpu_baseline": {"value": round(gbs, 3), "unit": UNIT, "cores": os.cpu_count(),
                             "kind": "port", "sample": desc},
            "e2e": {"value": round(gbs, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU arm
def run_ours(args, rank: int, world: int, local_rank: int):
    import numpy as np
    import torch

    from oracle import oracle as orc  # input generation only (seeded uniform values)
    from streamparanumal_gb300 import _build, autotune, capi, kernels
    from streamparanumal_gb300 import ogs as O

    _build.build_library()
    capi.load()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream

    N = 1 << args.nlog2
    mesh, p = args.mesh, args.p
    # ---- the batched workload and a degree sample (one GPU, outside the timed
    # region, before the suite's buffers exist; everything they allocate is freed)
    extras = {}
    if world == 1 and not args.kernels_only and not args.no_extras:
        peak0, _ = measured_peak()
        t_x = time.time()
        extras["degree_sample"] = degree_sample(dev, _degrees(args.sample_degrees),
                                                args.sweep_nodes, args.perm_seed, peak0)
        extras["batch"] = {"small": batch_measure(dev, args.batch_count, 6, args.seed, 20),
                           "full": batch_measure(dev, args.batch_count, args.batch_emax,
                                                 args.seed, 10)}
        extras["extras_s"] = round(time.time() - t_x, 1)
    # ---- inputs (host, pinned) and plans
    t_setup = time.time()
    h_a = torch.from_numpy(orc.uniform(N, args.seed)).pin_memory()
    h_b = torch.from_numpy(orc.uniform(N, args.seed + 1)).pin_memory()
    # mesh ids and the gather-scatter plan, both built on the device, with the
    # per-degree tuning of this layout (as the BS6-BS8 drivers apply it)
    t_plan = time.time()
    tuning = autotune.apply(p, args.perm_seed != 0)
    ids = O.box_hex_ids(mesh, mesh, mesh, p, args.perm_seed, device=dev, stream=stream)
    Nt = ids.numel()
    h = O.ogs_t()
    h.Setup(Nt, ids, kind=O.Signed, unique=True, stream=stream)
    Ng = h.NgatherGlobal
    del ids
    t_plan = time.time() - t_plan
    h_q = torch.from_numpy(orc.uniform(Nt, args.seed + 2)).pin_memory()
    a = h_a.to(dev)
    b = h_b.to(dev)
    q = h_q.to(dev)
    gq = torch.zeros(Ng, dtype=torch.float64, device=dev)
    tmp = torch.zeros(1024, dtype=torch.float64, device=dev)
    scal = torch.zeros(4, dtype=torch.float64, device=dev)
    red = kernels.ReduceScratch(dev)
    rng = np.random.default_rng(args.seed)
    alpha, beta = (float(x) for x in rng.uniform(-1, 1, size=2))
    nb256 = kernels.nblocks_for(N, 256)
    nb1024 = kernels.nblocks_for(N, 1024)
    torch.cuda.synchronize()
    t_setup = time.time() - t_setup

    names = ["BS1", "BS2", "BS3", "BS4", "BS5", "BS6", "BS7", "BS8"]
    nbytes = {**bytes_bs(N), **bytes_ogs(Nt, Ng)}
    step_bytes = sum(nbytes.values())
    call = capi.call

    def suite(a=a, b=b, q=q, scal=scal):
        call("sp_bs1_copy_f64", N, a.data_ptr(), b.data_ptr(), sptr)
        yield "BS1"
        call("sp_bs2_axpy_f64", N, alpha, a.data_ptr(), beta, b.data_ptr(), sptr)
        yield "BS2"
        # the drivers' default BS3: integer-pipe stage 1, the reference's stage 2
        call("sp_bs3_1_fast_f64", 256, nb256, N, a.data_ptr(), tmp.data_ptr(), red.ptr, sptr)
        call("sp_reduce_finish_f64", 256, nb256, tmp.data_ptr(), scal.data_ptr(), sptr)
        yield "BS3"
        call("sp_bs4_1_f64", 256, nb256, N, a.data_ptr(), b.data_ptr(), tmp.data_ptr(), sptr)
        call("sp_reduce_finish_f64", 256, nb256, tmp.data_ptr(), scal.data_ptr() + 8, sptr)
        yield "BS4"
        # the drivers' default BS5: r updated as the reference does, r.r on the integer
        # pipe, the reference's stage 2
        call("sp_bs5_1_fast_f64", 1024, nb1024, N, a.data_ptr(), alpha, b.data_ptr(),
             tmp.data_ptr(), red.ptr, sptr)
        call("sp_reduce_finish_f64", 1024, nb1024, tmp.data_ptr(), scal.data_ptr() + 16, sptr)
        yield "BS5"
        h.Gather(gq, q, 1, O.Add, O.Trans, stream=stream)
        yield "BS6"
        h.Scatter(q, gq, 1, O.NoTrans, stream=stream)
        yield "BS7"
        h.GatherScatter(q, 1, O.Add, O.Sym, stream=stream)
        yield "BS8"

    def run_steps(k, events=None):
        for s in range(k):
            if events is not None:
                events[s][0].record(stream)
            for i, _ in enumerate(suite()):
                if events is not None:
                    events[s][i + 1].record(stream)

    dist = world > 1
    if dist:
        import torch.distributed as tdist
    # ---- warm-up
    run_steps(args.warmup)
    torch.cuda.synchronize()
    sampler = ClockSampler(local_rank)
    sampler.start()
    # ---- timed region (device events on the launching stream)
    events = [[torch.cuda.Event(enable_timing=True) for _ in range(len(names) + 1)]
              for _ in range(args.steps)]
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    if dist:
        tdist.barrier()
    torch.cuda.synchronize()
    capi.load().sp_launch_count_reset()
    start.record(stream)
    run_steps(args.steps, events)
    end.record(stream)
    torch.cuda.synchronize()
    launches = int(capi.load().sp_launch_count())
    if dist:
        tdist.barrier()
    total_ms = start.elapsed_time(end)
    # keep the clock sampler running over a short soak of the same work so the
    # record covers at least ~1 s under load
    t_soak = time.time()
    while not args.kernels_only and time.time() - t_soak < 1.0:
        run_steps(5)
        torch.cuda.synchronize()
    clocks = sampler.stop()
    per = {n: 0.0 for n in names}
    for ev in events:
        for i, n in enumerate(names):
            per[n] += ev[i].elapsed_time(ev[i + 1])
    per = {n: v / args.steps for n, v in per.items()}  # ms per call
    total_ms = max_over_ranks(total_ms, dev)
    ms_per_step = total_ms / args.steps
    value = job_rate(world, step_bytes, ms_per_step)

    if args.kernels_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": round(value, 2), "unit": UNIT,
                              "ms_per_step": round(ms_per_step, 4), "gpu_launches": launches,
                              "per_kernel_ms": {n: round(per[n], 4) for n in names}}))
        return
    # ---- e2e: host buffers in, host buffers out, through the same public calls.
    # Double-buffered across steps: step k+1's inputs upload (copy engine, stream
    # s_in) into the second device set while step k computes, and step k's results
    # download (stream s_out) while step k+1 computes; a set is refilled only after
    # its previous results have left.  Every step moves all of its inputs in and its
    # results out inside the timed region.
    h_out_b = torch.empty_like(h_b).pin_memory()
    h_out_q = torch.empty_like(h_q).pin_memory()
    h_scal = torch.empty(4, dtype=torch.float64).pin_memory()
    e2e_steps = max(3, min(args.steps, 10))
    sets = [(a, b, q, scal), (torch.empty_like(a), torch.empty_like(b), torch.empty_like(q),
                              torch.zeros_like(scal))]
    s_in = torch.cuda.Stream(device=dev)
    s_out = torch.cuda.Stream(device=dev)
    uploaded = [None, None]
    drained = [None, None]

    def upload(k):
        da, db, dq, _ = sets[k % 2]
        if drained[k % 2] is not None:
            s_in.wait_event(drained[k % 2])  # this set's previous results have left
        with torch.cuda.stream(s_in):
            da.copy_(h_a, non_blocking=True)
            db.copy_(h_b, non_blocking=True)
            dq.copy_(h_q, non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(s_in)
        uploaded[k % 2] = ev

    def compute_and_download(k):
        da, db, dq, ds = sets[k % 2]
        stream.wait_event(uploaded[k % 2])
        for _ in suite(da, db, dq, ds):
            pass
        ev = torch.cuda.Event()
        ev.record(stream)
        s_out.wait_event(ev)
        with torch.cuda.stream(s_out):
            h_out_b.copy_(db, non_blocking=True)
            h_out_q.copy_(dq, non_blocking=True)
            h_scal.copy_(ds, non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(s_out)
        drained[k % 2] = ev

    def e2e_run(k_steps):
        ev = torch.cuda.Event()
        ev.record(stream)
        s_in.wait_event(ev)
        upload(0)
        for k in range(k_steps):
            if k + 1 < k_steps:
                upload(k + 1)
            compute_and_download(k)
        stream.wait_stream(s_out)  # the run ends when the last results are on the host

    e2e_run(2)
    torch.cuda.synchronize()
    # the host link is shared with the machine's other work, so the pipeline is
    # timed E2E_REPEATS times and the median run is reported (all runs are listed)
    e2e_runs = []
    for _ in range(E2E_REPEATS):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        if dist:
            tdist.barrier()
        e0.record(stream)
        e2e_run(e2e_steps)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_runs.append(max_over_ranks(e0.elapsed_time(e1) / e2e_steps, dev))
    e2e_ms = statistics.median(e2e_runs)
    h2d = (h_a.numel() + h_b.numel() + h_q.numel()) * 8
    d2h = (h_out_b.numel() + h_out_q.numel() + h_scal.numel()) * 8
    e2e_value = job_rate(world, step_bytes, e2e_ms)

    # ---- BS0 launch latency: 10,000 empty launches, plain and graph-captured
    bs0 = bs0_latency(stream, dev)
    # ---- FP32-storage forms and the full CG update (not part of `value`)
    forms = storage_forms(stream, dev, h_a, h_b, h_q, h, N, Nt, Ng, per, alpha, beta)

    if rank != 0:
        return
    peak, peak_kind = measured_peak()
    dom = max(names, key=lambda n: per[n])
    achieved = nbytes[dom] / 1e9 / (per[dom] / 1e3)
    # the kernel furthest below the roofline, beside the dominant one
    worst = min(names, key=lambda n: nbytes[n] / per[n])
    worst_gbs = nbytes[worst] / 1e9 / (per[worst] / 1e3)
    traffic = ncu_traffic().get(dom)
    detail = {n: {"ms": round(per[n], 4), "bytes": nbytes[n],
                  "GBps": round(nbytes[n] / 1e9 / (per[n] / 1e3), 1),
                  "frac_of_peak": round(nbytes[n] / 1e9 / (per[n] / 1e3) / peak, 4)}
              for n in names}
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded uniform[-1,1] FP64; seeded element permutation)",
        "config": {"workload": f"BS1-BS8 FP64 suite: BS1-BS5 at N=2^{args.nlog2}, BS6/BS7/BS8 "
                               f"on a {mesh}^3 hex box at p={p}, permuted elements",
                   "n": N, "local_nodes": Nt, "global_nodes": Ng, "bytes_per_step": step_bytes,
                   "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": peak_kind, "traffic": traffic,
                     "worst": {"kernel": worst, "achieved": round(worst_gbs, 1),
                               "frac": round(worst_gbs / peak, 4),
                               "traffic": ncu_traffic().get(worst)}},
        "e2e": {"value": round(e2e_value, 2), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": round(e2e_ms, 3),
                "steps": e2e_steps, "repeats": E2E_REPEATS,
                "runs_ms_per_step": [round(x, 3) for x in e2e_runs],
                "pipeline": "double-buffered: step k+1 uploads and step k-1 downloads "
                            "overlap step k's kernels (pinned host buffers, copy engines)"},
        "gpu_launches": launches,
        "clocks": clocks,
        "detail": {"per_kernel": detail, "bs0_us_per_launch": bs0,
                   "storage_forms": forms, "setup_s": round(t_setup, 2),
                   "mesh_and_plan_s": round(t_plan, 2), "ogs_tuning": tuning, **extras},
    }
    if not args.no_cpu_baseline:
        gbs, desc, cores, _, _ = cpu_sample(args.cpu_nlog2, args.cpu_mesh, p, args.perm_seed,
                                            args.seed)
        line["cpu_baseline"] = {"value": round(gbs, 3), "unit": UNIT, "cores": cores,
                                "kind": "port", "sample": desc}
    print(json.dumps(line), flush=True)
    if args.json_out:
        Path(args.json_out).write_text(json.dumps(line, indent=1))


def _time(fn, stream, reps=10, warm=3) -> float:
    """Mean device milliseconds of fn() over `reps` calls on `stream`."""
    import torch

    for _ in range(warm):
        fn()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def storage_forms(stream, dev, h_a, h_b, h_q, h, N, Nt, Ng, per, alpha, beta) -> dict:
    """FP32-storage forms of BS1-BS8 (BS5 as the single-launch reference update) and
    the full CG update (x += alpha p, r -= alpha Ap, r.r), each against its FP64 form: device time, useful GB/s (the
    FP64 byte accounting / time), bytes actually moved, and the error of every
    result against the FP64 computation on the same FP64 inputs."""
    import torch

    from streamparanumal_gb300 import capi, kernels
    from streamparanumal_gb300 import ogs as O

    call = capi.call
    sptr = stream.cuda_stream
    out = {}
    with torch.cuda.stream(stream):
        a = h_a.to(dev, non_blocking=True)
        b = h_b.to(dev, non_blocking=True)
        a32, b32 = a.float(), b.float()
        y32 = b32.clone()
        res = torch.zeros(8, dtype=torch.float64, device=dev)
        sc = kernels.ReduceScratch(dev)
        f64 = {"BS1": 16 * N, "BS2": 24 * N, "BS3": 8 * N, "BS4": 16 * N}

        def form(name, ms, actual, err=None):
            d = {"ms": round(ms, 4), "useful_GBps": round(f64[name] / 1e6 / ms, 1),
                 "actual_GBps": round(actual / 1e6 / ms, 1)}
            if name in per:
                d["speedup_vs_fp64"] = round(per[name] / ms, 3)
            if err is not None:
                d.update(err)
            out[name] = d

        form("BS1", _time(lambda: call("sp_bs1_copy_f32", N, a32.data_ptr(), y32.data_ptr(), sptr),
                          stream), 8 * N)
        form("BS2", _time(lambda: call("sp_bs2_axpy_f32", N, alpha, a32.data_ptr(), beta,
                                       y32.data_ptr(), sptr), stream), 12 * N)
        # BS3 / BS4: compensated FP32 lanes, FP64 finish
        call("sp_norm2_f64", N, a.data_ptr(), res.data_ptr(), sc.ptr, sptr)
        call("sp_dot_f64", N, a.data_ptr(), b.data_ptr(), res.data_ptr() + 8, sc.ptr, sptr)
        a32d, b32d = a32.double(), b32.double()
        call("sp_norm2_f64", N, a32d.data_ptr(), res.data_ptr() + 16, sc.ptr, sptr)
        call("sp_dot_f64", N, a32d.data_ptr(), b32d.data_ptr(), res.data_ptr() + 24, sc.ptr, sptr)
        del a32d, b32d
        ms3 = _time(lambda: call("sp_norm2_f32", N, a32.data_ptr(), res.data_ptr() + 32, sc.ptr,
                                 sptr), stream)
        ms4 = _time(lambda: call("sp_dot_f32", N, a32.data_ptr(), b32.data_ptr(),
                                 res.data_ptr() + 40, sc.ptr, sptr), stream)
        r = res.cpu().tolist()
        dot_scale = float((a * b).abs().sum())
        form("BS3", ms3, 4 * N, {"rel_err_vs_fp64": abs(r[4] - r[0]) / abs(r[0]),
                                 "rel_err_arith": abs(r[4] - r[2]) / abs(r[2])})
        form("BS4", ms4, 8 * N, {"rel_err_vs_fp64": abs(r[5] - r[1]) / abs(r[1]),
                                 "err_vs_fp64_over_sum_abs": abs(r[5] - r[1]) / dot_scale,
                                 "rel_err_arith": abs(r[5] - r[3]) / abs(r[3])})
        # full CG update: FP64 and FP32 storage
        f64["CG"] = 48 * N
        x, rr, p_, Ap = a.clone(), b.clone(), b.flip(0).contiguous(), a.flip(0).contiguous()
        cg_alpha = 0.25
        call("sp_cg_update_f64", N, cg_alpha, p_.data_ptr(), Ap.data_ptr(), x.data_ptr(),
             rr.data_ptr(), res.data_ptr() + 48, sc.ptr, sptr)
        x32, r32, p32, Ap32 = (t.float() for t in (a, b, p_, Ap))
        call("sp_cg_update_f32", N, cg_alpha, p32.data_ptr(), Ap32.data_ptr(), x32.data_ptr(),
             r32.data_ptr(), res.data_ptr() + 56, sc.ptr, sptr)
        r = res.cpu().tolist()
        xerr = float(((x32.double() - x).abs().max() / x.abs().max()))
        ms64 = _time(lambda: call("sp_cg_update_f64", N, 1e-12, p_.data_ptr(), Ap.data_ptr(),
                                  x.data_ptr(), rr.data_ptr(), res.data_ptr() + 48, sc.ptr, sptr),
                     stream)
        ms32 = _time(lambda: call("sp_cg_update_f32", N, 1e-12, p32.data_ptr(), Ap32.data_ptr(),
                                  x32.data_ptr(), r32.data_ptr(), res.data_ptr() + 56, sc.ptr,
                                  sptr), stream)
        out["CG_fp64"] = {"ms": round(ms64, 4), "GBps": round(48 * N / 1e6 / ms64, 1)}
        per["CG"] = ms64
        form("CG", ms32, 24 * N, {"rdotr_rel_err_vs_fp64": abs(r[7] - r[6]) / abs(r[6]),
                                  "x_max_rel_err_vs_fp64": xerr})
        # the reference's BS5 update (r += alpha Ap, r.r) stored in FP32, one launch,
        # against the FP64 BS5 of the suite
        f64["BS5"] = 24 * N
        r5, Ap5 = b.clone(), a.flip(0).contiguous()
        call("sp_cg_update_ref_f64", N, cg_alpha, Ap5.data_ptr(), r5.data_ptr(),
             res.data_ptr() + 48, sc.ptr, sptr)
        r5_32, Ap5_32 = b.float(), Ap5.float()
        call("sp_cg_update_ref_f32", N, cg_alpha, Ap5_32.data_ptr(), r5_32.data_ptr(),
             res.data_ptr() + 56, sc.ptr, sptr)
        r = res.cpu().tolist()
        r5err = float(((r5_32.double() - r5).abs().max() / r5.abs().max()))
        ms5 = _time(lambda: call("sp_cg_update_ref_f32", N, 1e-12, Ap5_32.data_ptr(),
                                 r5_32.data_ptr(), res.data_ptr() + 56, sc.ptr, sptr), stream)
        form("BS5", ms5, 12 * N, {"rdotr_rel_err_vs_fp64": abs(r[7] - r[6]) / abs(r[6]),
                                  "r_max_rel_err_vs_fp64": r5err})
        del r5, Ap5, r5_32, Ap5_32
        del x, rr, p_, Ap, x32, r32, p32, Ap32, a, b, a32, b32, y32
        # BS6-BS8 on FP32 node data (same plan)
        q = h_q.to(dev, non_blocking=True)
        q32 = q.float()
        g32 = torch.zeros(Ng, dtype=torch.float32, device=dev)
        g64 = torch.zeros(Ng, dtype=torch.float64, device=dev)
        f64.update({"BS6": (Ng + 1) * 4 + Nt * 4 + Nt * 8 + Ng * 8,
                    "BS7": (Ng + 1) * 4 + Nt * 4 + Ng * 8 + Nt * 8,
                    "BS8": (Ng + 1) * 4 + Nt * 4 + 2 * Nt * 8})
        act = {"BS6": (Ng + 1) * 4 + Nt * 4 + Nt * 4 + Ng * 4,
               "BS7": (Ng + 1) * 4 + Nt * 4 + Ng * 4 + Nt * 4,
               "BS8": (Ng + 1) * 4 + Nt * 4 + 2 * Nt * 4}
        h.Gather(g64, q, 1, O.Add, O.Trans, stream=stream)
        h.Gather(g32, q32, 1, O.Add, O.Trans, stream=stream)
        e6 = float((g32.double() - g64).abs().max() / g64.abs().max())
        q64gs, q32gs = q.clone(), q32.clone()
        h.GatherScatter(q64gs, 1, O.Add, O.Sym, stream=stream)
        h.GatherScatter(q32gs, 1, O.Add, O.Sym, stream=stream)
        e8 = float((q32gs.double() - q64gs).abs().max() / q64gs.abs().max())
        del q64gs, q32gs
        form("BS6", _time(lambda: h.Gather(g32, q32, 1, O.Add, O.Trans, stream=stream), stream),
             act["BS6"], {"max_err_vs_fp64_over_max": e6})
        form("BS7", _time(lambda: h.Scatter(q32, g32, 1, O.NoTrans, stream=stream), stream),
             act["BS7"], {"exact_copy_of_fp32_values": True})
        form("BS8", _time(lambda: h.GatherScatter(q32, 1, O.Add, O.Sym, stream=stream), stream),
             act["BS8"], {"max_err_vs_fp64_over_max": e8})
        del q, q32, g32, g64
    torch.cuda.synchronize()
    tot64 = sum(per[k] for k in ("BS1", "BS2", "BS3", "BS4", "BS6", "BS7", "BS8"))
    tot32 = sum(out[k]["ms"] for k in ("BS1", "BS2", "BS3", "BS4", "BS6", "BS7", "BS8"))
    out["suite_speedup_vs_fp64"] = round(tot64 / tot32, 3)
    return out


def bs0_latency(stream, dev) -> dict:
    """bs0Run.cpp:68-79: host time of n back-to-back empty launches plus one
    synchronisation, divided by n; and the same n launches replayed from one graph."""
    import torch

    from streamparanumal_gb300 import capi

    a = torch.zeros(1, dtype=torch.float64, device=dev)
    b = torch.zeros(1, dtype=torch.float64, device=dev)
    lib = capi.load()
    sptr = stream.cuda_stream
    n = 10000
    for _ in range(100):
        lib.sp_bs0(1, a.data_ptr(), b.data_ptr(), sptr)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(n):
        lib.sp_bs0(1, a.data_ptr(), b.data_ptr(), sptr)
    stream.synchronize()
    plain = (time.perf_counter() - t0) / n * 1e6
    g = capi.ctypes.c_void_p()
    capi.call("sp_bs0_graph_create", n, 1, a.data_ptr(), b.data_ptr(), sptr, capi.ctypes.byref(g))
    lib.sp_graph_launch(g, sptr)
    stream.synchronize()
    t0 = time.perf_counter()
    lib.sp_graph_launch(g, sptr)
    stream.synchronize()
    graph = (time.perf_counter() - t0) / n * 1e6
    lib.sp_graph_destroy(g)
    return {"plain": round(plain, 3), "graph": round(graph, 3), "launches": n}


def batch_measure(dev, count: int, emax: int, seed: int, reps: int) -> dict:
    """Batched uneven workload: instance i has an Ex*Ey*Ez hex box (each in
    [2, emax]) of degree p in [2, 9] (seeded), a CG update on its own x, r, p, Ap
    (n = its local nodes) and a BS8 gather+scatter on its own q.  Timed four ways:
    per-instance launches (2 per instance), the same launches replayed from one CUDA
    graph, one persistent batched launch, and that launch replayed from a graph; in
    FP64 and in FP32 storage.  Returns per-instance microseconds and rates."""
    import numpy as np
    import torch

    from streamparanumal_gb300 import batch, capi, kernels
    from streamparanumal_gb300 import ogs as O

    rng = np.random.default_rng(seed)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    stream = torch.cuda.Stream(device=dev)
    t0 = time.time()
    plans, vecs, alphas, sizes = [], [], [], []
    with torch.cuda.stream(stream):
        for i in range(count):
            ex, ey, ez = (int(v) for v in rng.integers(2, emax + 1, size=3))
            p = int(rng.integers(2, 10))
            ids = O.box_hex_ids(ex, ey, ez, p, int(rng.integers(1, 1 << 30)), device=dev,
                                stream=stream)
            n = ids.numel()
            h = O.ogs_t()
            h.Setup(n, ids, unique=True, stream=stream)
            del ids
            v = {k: torch.rand(n, dtype=torch.float64, device=dev, generator=gen) * 2 - 1
                 for k in ("x", "r", "p", "Ap", "q")}
            v["rr"] = torch.zeros(1, dtype=torch.float64, device=dev)
            plans.append(h)
            vecs.append(v)
            alphas.append(float(rng.uniform(-1, 1)) * 1e-3)
            sizes.append((ex, ey, ez, p, n, h.NgatherGlobal))
    torch.cuda.synchronize()
    setup_s = time.time() - t0
    sc = kernels.ReduceScratch(dev)
    sptr = stream.cuda_stream

    def time_forms(vs, f32: bool) -> dict:
        cg = "sp_cg_update_f32" if f32 else "sp_cg_update_f64"
        ty = capi.FLOAT if f32 else capi.DOUBLE

        def per_instance():
            for h, v, a in zip(plans, vs, alphas):
                capi.call(cg, v["x"].numel(), a, v["p"].data_ptr(), v["Ap"].data_ptr(),
                          v["x"].data_ptr(), v["r"].data_ptr(), v["rr"].data_ptr(), sc.ptr, sptr)
                capi.call("sp_ogs_gather_scatter", h._plan, ty, capi.ADD, capi.SYM, 1,
                          v["q"].data_ptr(), sptr)

        b = batch.Batch(plans, [v["x"] for v in vs], [v["r"] for v in vs], [v["p"] for v in vs],
                        [v["Ap"] for v in vs], [v["rr"] for v in vs], [v["q"] for v in vs],
                        alphas, stream=stream)
        with torch.cuda.stream(stream):
            g_inst = batch.Graph(stream)
            with g_inst:
                per_instance()
            g_batch = batch.Graph(stream)
            with g_batch:
                b.run(stream=stream)
        return {"per_instance_launches": _time(per_instance, stream, reps),
                "per_instance_graph": _time(lambda: g_inst.launch(), stream, reps),
                "batched_persistent": _time(lambda: b.run(stream=stream), stream, reps),
                "batched_graph": _time(lambda: g_batch.launch(), stream, reps)}

    res = time_forms(vecs, False)
    vecs32 = [{k: (t if k == "rr" else t.float()) for k, t in v.items()} for v in vecs]
    res32 = time_forms(vecs32, True)
    del vecs32
    nodes = sum(x[4] for x in sizes)
    ng = sum(x[5] for x in sizes)
    # CG: x, p, r, Ap read, x, r written; BS8: row starts, column ids, q read and written
    nbytes = 48 * nodes + (ng + len(sizes)) * 4 + nodes * 4 + 16 * nodes
    nbytes32 = 24 * nodes + (ng + len(sizes)) * 4 + nodes * 4 + 8 * nodes
    per = {k: round(v / len(sizes) * 1e3, 3) for k, v in res.items()}  # us per instance
    per32 = {k: round(v / len(sizes) * 1e3, 3) for k, v in res32.items()}
    out = {"instances": len(sizes), "Exyz_range": [2, emax], "p_range": [2, 9],
           "local_nodes": nodes, "global_nodes": ng, "reps": reps,
           "per_instance_us": per,
           "speedup_batched_graph_vs_launches": round(res["per_instance_launches"]
                                                      / res["batched_graph"], 3),
           "GBps_batched": round(nbytes / 1e6 / res["batched_persistent"], 1),
           "GBps_per_instance_launches": round(nbytes / 1e6 / res["per_instance_launches"], 1),
           "fp32_storage": {
               "per_instance_us": per32,
               "speedup_batched_graph_vs_launches": round(res32["per_instance_launches"]
                                                          / res32["batched_graph"], 3),
               "GBps_batched": round(nbytes32 / 1e6 / res32["batched_persistent"], 1),
               "useful_speedup_vs_fp64_batched": round(res["batched_persistent"]
                                                       / res32["batched_persistent"], 3)},
           "launches": {"per_instance": 2 * len(sizes), "batched": 1},
           "setup_s": round(setup_s, 1)}
    for h in plans:
        h.Free()
    del plans, vecs
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return out


def run_batch(args, local_rank: int) -> None:
    """--batch: batch_measure() at the command line's count and box range, one JSON line."""
    import torch

    from streamparanumal_gb300 import _build, capi

    _build.build_library()
    capi.load()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    d = batch_measure(dev, args.batch_count, args.batch_emax, args.seed,
                      max(3, min(args.steps, 20)))
    line = {"metric": "batched CG update + BS8 per-instance time", "unit": "us/instance",
            "value": d["per_instance_us"]["batched_graph"], "higher_is_better": False,
            "n_gpus": 1, "steps": d["reps"], "dtype": "f64", "data": "synthetic (seeded)",
            "config": {"workload": f"{d['instances']} instances, Ex,Ey,Ez in [2,{args.batch_emax}], "
                                   f"p in [2,9]", "local_nodes": d["local_nodes"],
                       "global_nodes": d["global_nodes"]}, **d}
    print(json.dumps(line), flush=True)
    if args.json_out:
        Path(args.json_out).write_text(json.dumps(line, indent=1))


def degree_sample(dev, degrees, nodes: float, perm_seed: int, peak: float, reps: int = 10) -> list:
    """BS6-BS8 per degree on a box of about `nodes` local nodes, lexicographic and
    permuted, FP64 and FP32, with the stored per-degree tuning (as the BS6-BS8
    drivers apply it).  GB/s by the reference accounting and the fraction of the
    HBM peak."""
    import torch

    from streamparanumal_gb300 import autotune
    from streamparanumal_gb300 import ogs as O

    stream = torch.cuda.current_stream(dev)
    rows = []
    for p in degrees:
        E = int(round((nodes / (p + 1) ** 3) ** (1.0 / 3.0)))
        for perm in (0, perm_seed):
            tuning = autotune.apply(p, bool(perm))
            ids = O.box_hex_ids(E, E, E, p, perm, device=dev)
            h = O.ogs_t()
            h.Setup(ids.numel(), ids, unique=True)
            Nt, Ng = ids.numel(), h.NgatherGlobal
            del ids
            row = {"p": p, "E": E, "layout": "permuted" if perm else "lexicographic",
                   "local_nodes": Nt, "global_nodes": Ng, "tuning": tuning}
            for dt, val in ((torch.float64, 8), (torch.float32, 4)):
                q = (torch.rand(Nt, dtype=torch.float64, device=dev) * 2 - 1).to(dt)
                gq = torch.zeros(Ng, dtype=dt, device=dev)
                by = bytes_ogs(Nt, Ng, val)
                by64 = bytes_ogs(Nt, Ng, 8)
                t6 = _time(lambda: h.Gather(gq, q, 1, O.Add, O.Trans), stream, reps)
                t7 = _time(lambda: h.Scatter(q, gq, 1, O.NoTrans), stream, reps)
                t8 = _time(lambda: h.GatherScatter(q, 1, O.Add, O.Sym), stream, reps)
                row["fp64" if val == 8 else "fp32"] = {
                    k: {"ms": round(t, 4), "GBps": round(by[k] / 1e6 / t, 1),
                        "useful_GBps": round(by64[k] / 1e6 / t, 1),
                        "frac": round(by[k] / 1e6 / t / peak, 4)}
                    for k, t in (("BS6", t6), ("BS7", t7), ("BS8", t8))}
                del q, gq
            h.Free()
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
            rows.append(row)
    return rows


def _degrees(spec: str) -> list[int]:
    out = []
    for part in spec.split(","):
        if "-" in part:
            a, b = part.split("-")
            out += list(range(int(a), int(b) + 1))
        else:
            out.append(int(part))
    return out


def run_degree_sweep(args, local_rank: int) -> None:
    """For each degree p the box edge is E = round((nodes / (p+1)^3)^(1/3)); the
    autotuner times every ogs variant (FP64) and the winner is then timed in FP64
    and FP32.  One JSON line per (p, layout)."""
    import torch

    from streamparanumal_gb300 import _build, autotune, capi
    from streamparanumal_gb300 import ogs as O

    _build.build_library()
    capi.load()
    torch.cuda.set_device(local_rank)
    torch.manual_seed(args.seed)
    peak, peak_kind = measured_peak()
    table = autotune.load_table()
    stream = torch.cuda.current_stream()
    for p in _degrees(args.degree_sweep):
        E = int(round((args.sweep_nodes / (p + 1) ** 3) ** (1.0 / 3.0)))
        for perm in (0, args.perm_seed):
            ids = O.box_hex_ids(E, E, E, p, perm, device="cuda")
            res = autotune.tune_ogs(E, p, perm, ids=ids)
            autotune.record(table, res)
            best = res["best"]
            autotune.apply(p, bool(perm), table)
            h = O.ogs_t()
            h.Setup(ids.numel(), ids, unique=True)
            Nt, Ng = ids.numel(), h.NgatherGlobal
            del ids
            line = {"metric": "BS6-BS8 GB/s per degree (reference byte accounting)", "p": p,
                    "E": E, "layout": "permuted" if perm else "lexicographic",
                    "local_nodes": Nt, "global_nodes": Ng, "tuned": best, "peak": peak,
                    "peak_source": peak_kind}
            for dt, val in ((torch.float64, 8), (torch.float32, 4)):
                q = (torch.rand(Nt, dtype=torch.float64, device="cuda") * 2 - 1).to(dt)
                gq = torch.zeros(Ng, dtype=dt, device="cuda")
                by = bytes_ogs(Nt, Ng, val)
                by64 = bytes_ogs(Nt, Ng, 8)
                t6 = _time(lambda: h.Gather(gq, q, 1, O.Add, O.Trans), stream, 10)
                t7 = _time(lambda: h.Scatter(q, gq, 1, O.NoTrans), stream, 10)
                t8 = _time(lambda: h.GatherScatter(q, 1, O.Add, O.Sym), stream, 10)
                key = "fp64" if val == 8 else "fp32"
                line[key] = {k: {"ms": round(t, 4), "GBps": round(by[k] / 1e6 / t, 1),
                                 "useful_GBps": round(by64[k] / 1e6 / t, 1),
                                 "frac": round(by[k] / 1e6 / t / peak, 4)}
                             for k, t in (("BS6", t6), ("BS7", t7), ("BS8", t8))}
                del q, gq
            h.Free()
            print(json.dumps(line), flush=True)
    if args.save_tuning:
        autotune.save_table(table)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.batch:
        if rank == 0:
            run_batch(args, local_rank)
        return
    if args.degree_sweep:
        if rank == 0:
            run_degree_sweep(args, local_rank)
        return
    if world > 1:
        import torch
        import torch.distributed as tdist

        torch.cuda.set_device(local_rank)
        tdist.init_process_group("nccl")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as tdist

        tdist.destroy_process_group()


if __name__ == "__main__":
    main()
