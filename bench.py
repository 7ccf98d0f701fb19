"""Benchmark: triangles/sec of the threeD 3PCF count on one GB300.

Workload (default): the clustered periodic box -- 2,000,000 Neyman-Scott
points (200,000 uniform parents x Poisson(10) children, sigma 2 Mpc/h,
wrapped) in L = 2000 Mpc/h, r_max = 100 Mpc/h, 20 linear bins per side,
unweighted, float32 xyz, seeded. One step = one full calculateD1D2D3(p, p, p):
GPU cell-list build, triangle kernel, histogram fold and read-back.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]

Prints one JSON line (rank 0). `value` is device-resident throughput
(inputs already in HBM, CUDA events on the launch stream, L2 flushed between
steps); `e2e` is the same metric through the reference-facing host call with
host->device copies of the catalogue from pinned memory and the histogram
read-back inside the timed region. `roofline` is the triangle kernel's FP32
issue rate against the nominal FFMA peak at the sampled SM clock;
`cpu_baseline` is the CPU oracle on the host cores over a bounded anchor
sample. With --impl reference the reference's own kernel (oracle/_ref,
compiled unmodified from its source/device.cu) runs behind its host flow on
a random anchor sample.

Under torchrun (N > 1) each rank counts its own independently seeded
catalogue (weak scaling, no data-path collective); value sums all ranks'
triangles over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "triangles/sec"
UNIT = "triangles/s"
N_SM = 152
FP32_LANES_PER_SM = 128
L2_FLUSH_BYTES = 256 << 20
# Triangle-kernel DRAM traffic per launch (dram__bytes_read.sum +
# dram__bytes_write.sum): 150.1 MB read + 1.5 MB written, measured with ncu
# on the 249,814-point box_clustered_L1000 workload, scaled by the anchor
# count to the 2,001,574-point box_clustered launch. The per-warp neighbour
# lists (about 33 KB per anchor) stay out of DRAM: each warp discards their
# L2 lines when its anchor is done.
TRIANGLE_KERNEL_DRAM_BYTES = {"box_clustered": int(151.65e6 * 2001574 / 249814),
                              "box_clustered_L1000": int(151.65e6)}


def workload(name: str, seed_offset: int):
    from cudancorr_gb300 import catalogs as C
    if name == "box_clustered":
        p, box, edges = C.config_box_clustered(seed=2 + seed_offset)
        desc = ("Neyman-Scott box: 200,000 parents x Poisson(10), sigma 2, L=2000 Mpc/h, "
                "r_max=100, 20 linear bins, unweighted")
    elif name == "box_clustered_L1000":
        # Same process and density as box_clustered in one eighth of the
        # volume (250,000 points): the per-anchor work is the same, so this is
        # the small case for full ncu captures of the triangle kernel.
        p, box, edges = C.neyman_scott(25000, 10.0, 2.0, 1000.0, 12 + seed_offset), 1000.0, C.linear_edges(100.0, 20)
        desc = ("Neyman-Scott box: 25,000 parents x Poisson(10), sigma 2, L=1000 Mpc/h, "
                "r_max=100, 20 linear bins, unweighted")
    elif name == "box_uniform":
        p, box, edges = C.config_box_uniform(seed=1 + seed_offset)
        desc = "uniform box: 20,000 points, L=1000 Mpc/h, r_max=50, 10 linear bins, unweighted"
    elif name == "soneira_peebles":
        p, box, edges = C.config_soneira_peebles(seed=5 + seed_offset)
        desc = ("Soneira-Peebles box: 5 levels, eta=4, lambda=1.9, R0=200, L=1500 Mpc/h, "
                "r_max=80, 16 linear bins, unweighted")
    else:
        raise SystemExit(f"unknown workload {name}")
    return p, box, edges, desc


class ClockSampler:
    """nvidia-smi clock and throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in pathlib.Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def cpu_baseline(p, box, edges, budget_s: float = 12.0) -> dict:
    """CPU oracle (OpenMP, all host threads) on a random anchor sample."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(7)
    n_try = 256
    sub = np.ascontiguousarray(p[rng.choice(len(p), n_try, replace=False)])
    t = time.perf_counter()
    O.count_threeD(box, edges, sub, p, p, nthreads=threads)
    dt = time.perf_counter() - t
    n = int(min(len(p), max(n_try, n_try * budget_s / max(dt, 1e-3))))
    sub = np.ascontiguousarray(p[rng.choice(len(p), n, replace=False)])
    t = time.perf_counter()
    h = O.count_threeD(box, edges, sub, p, p, nthreads=threads)
    dt = time.perf_counter() - t
    return {"value": float(h.sum() / dt), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{n} random anchors of the {len(p):,}-point catalogue (all points as p2/p3), "
                      f"{dt:.1f} s, oracle/ncorr_oracle.cpp neighbour-list form"}


def engine_launches(n_distinct: int, sym: bool, learned: bool = False, rppi: bool = False) -> int:
    """Kernels one calculateD1D2D3 launches: per distinct catalogue the cell
    list (assign, scan, scatter), the neighbourhood bound per list catalogue,
    then the triangle kernel with its exact pass and fold (threeD) or the
    rppi kernel with the fold of its histogram copies (a histogram under
    32 MiB has more than one); the learned schedule adds the features, the
    prediction and seven queue-building kernels."""
    n = 3 * n_distinct + (1 if sym else 2) + (2 if rppi else 3)
    return n + (9 if learned else 0)


def dist_setup():
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    return world, rank, local


def _reduce(value: float, world: int, op) -> float:
    """All-reduce of one number over the ranks: on the GPU under NCCL, on the
    host under gloo (the CPU tests)."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=op)
    return float(t.item())


def barrier_max(value: float, world: int) -> float:
    """Slowest rank's time: the whole job's clock."""
    import torch.distributed as dist
    return value if world == 1 else _reduce(value, world, dist.ReduceOp.MAX)


def barrier_sum(value: float, world: int) -> float:
    """Units (triangles) counted by all ranks together."""
    import torch.distributed as dist
    return value if world == 1 else _reduce(value, world, dist.ReduceOp.SUM)


def barrier(world: int):
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def training_catalogue(name: str, i: int):
    """Catalogue i of the work model's training set: the workload's process,
    smaller, with its own seed."""
    from cudancorr_gb300 import catalogs as C
    if name == "soneira_peebles":
        return C.training_soneira_peebles(i)
    if name in ("box_clustered", "box_clustered_L1000"):
        return C.neyman_scott(25000, 10.0, 2.0, 1000.0, 200 + i), 1000.0, C.linear_edges(100.0, 20)
    raise SystemExit(f"no training process for workload {name}")


def train_work_model(name: str, n_cat: int = 20):
    """Trains the scheduler's work model on cell work measured by plain runs
    (dynamic schedule) of n_cat training catalogues, on the GPU."""
    from cudancorr_gb300 import api
    t0 = time.perf_counter()
    xs, ys = [], []
    for i in range(n_cat):
        q, qbox, qedges = training_catalogue(name, i)
        with api.ncorr(np.full(3, qbox), api.threeD, qedges, False, (0.0, 0.0, 0.0)) as c:
            c.set_record_work(True)
            c.calculateD1D2D3(q, q, q)
            f, w = c.cell_work()
        keep = f[:, 0] > 0
        xs.append(f[keep])
        ys.append(np.log1p(w[keep]).astype(np.float32))
    t1 = time.perf_counter()
    x, y = np.concatenate(xs), np.concatenate(ys)
    model = api.WorkModel(seed=1)
    mse = model.train(x, y, epochs=200, batch=256, lr=3e-3, seed=2)
    t2 = time.perf_counter()
    return model, {"training_catalogues": n_cat, "training_cells": int(len(x)), "train_mse_log": mse,
                   "s_measure": round(t1 - t0, 2), "s_train": round(t2 - t1, 2)}


def run_engine(args) -> dict:
    import torch
    from cudancorr_gb300 import api

    world, rank, local = dist_setup()
    p, box, edges, desc = workload(args.workload, rank)
    dev = torch.device("cuda", local)
    t_cat = torch.from_numpy(p).to(dev)
    # Anchor catalogue: all points, or (profiling size) the slab x < W.
    p1 = p if args.anchor_slab is None else np.ascontiguousarray(p[p[:, 0] < args.anchor_slab])
    t_p1 = t_cat if p1 is p else torch.from_numpy(p1).to(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    corr = api.ncorr(np.full(3, box), api.threeD, edges, False, (0.0, 0.0, 0.0))
    model, train_info = None, None
    if args.schedule == "learned":
        model, train_info = train_work_model(args.workload)
        corr.set_schedule(api.SCHED_LEARNED, model)
    elif args.schedule == "static":
        corr.set_schedule(api.SCHED_STATIC)

    def device_step():
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        corr._calculate_device(t_p1, t_cat, t_cat, stream=stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), corr.stats()

    for _ in range(args.warmup):
        device_step()
    sampler = ClockSampler(local)
    sampler.start()
    barrier(world)
    step_ms, kernel_ms, tri, flops = [], [], [], []
    for _ in range(args.steps):
        ms, st = device_step()
        step_ms.append(ms)
        kernel_ms.append(st["ms_count"])
        tri.append(st["triangles"])
        flops.append(8.0 * (st["n_pairs"] + st["n_pair_evals"]))
    barrier(world)
    clocks = sampler.stop()
    st_last = corr.stats()
    total_ms = barrier_max(sum(step_ms), world)
    total_tri = barrier_sum(float(sum(tri)), world)

    # End to end through the host call: pinned host catalogue, H2D inside.
    pinned = torch.from_numpy(p).pin_memory()
    p_host = pinned.numpy()
    p1_host = p_host if p1 is p else torch.from_numpy(p1).pin_memory().numpy()
    for _ in range(1):
        corr.calculateD1D2D3(p1_host, p_host, p_host)
    barrier(world)
    e2e_ms = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        corr.calculateD1D2D3(p1_host, p_host, p_host)
        _ = corr.getTriCountsOut()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_total = barrier_max(sum(e2e_ms), world)
    h_main = corr.getTriCountsAll()

    sched_cmp = None
    if args.schedule == "learned":
        # The same count under the other schedules (device-resident, one step
        # each), the model's prediction error on this catalogue's cells, and
        # the check that the counts do not depend on the schedule.
        times, same = {"learned": statistics.mean(kernel_ms)}, True
        for name, mode in (("dynamic", api.SCHED_DYNAMIC), ("static", api.SCHED_STATIC)):
            corr.set_schedule(mode)
            corr.set_record_work(name == "dynamic")
            device_step()
            times[name] = corr.stats()["ms_count"]
            same = same and bool(np.array_equal(corr.getTriCountsAll(), h_main))
            if name == "dynamic":
                f, w = corr.cell_work()
        corr.set_record_work(False)
        keep = f[:, 0] > 0
        y = np.log1p(w[keep])
        pred = model.predict(f[keep]).astype(np.float64)
        sched_cmp = {"kernel_ms": times, "speedup_vs_static": times["static"] / times["learned"],
                     "speedup_vs_dynamic": times["dynamic"] / times["learned"], "counts_identical": same,
                     "prediction": {"cells": int(keep.sum()), "mse_log": float(np.mean((pred - y) ** 2)),
                                    "r2_log": float(1.0 - np.mean((pred - y) ** 2) / np.var(y)),
                                    "total_work_rel_err": float(np.expm1(pred).sum() / np.expm1(y).sum() - 1.0)},
                     "training": train_info}
    corr.close()

    sm_mhz = clocks.get("sm_mhz") or 1995.0
    peak_tflops = N_SM * FP32_LANES_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    achieved = statistics.mean(f / (k / 1e3) for f, k in zip(flops, kernel_ms)) / 1e12
    nb = len(edges) - 1
    out = {
        "metric": METRIC, "value": total_tri / (total_ms / 1e3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32+fp64-exact",
        "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "description": desc, "n_points": int(len(p)),
                   "n_anchors": int(len(p1)), "box": box, "r_max": float(edges[-1]), "bins_per_side": nb,
                   "triangles_per_step": int(tri[-1]), "l2": "flushed (256 MiB write) between steps",
                   "parallelism": f"{world} independent catalogue(s), one per GPU"},
        "e2e": {"value": total_tri / (e2e_total / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": int(p.nbytes + (0 if p1 is p else p1.nbytes)),
                "d2h_bytes_per_step": int(nb ** 3 * 8),
                "ms_per_step": e2e_total / args.steps},
        "roofline": {"bound": "fp32_issue", "achieved": achieved, "peak": peak_tflops,
                     "unit": "TFLOP/s", "frac": achieved / peak_tflops,
                     "traffic": (TRIANGLE_KERNEL_DRAM_BYTES.get(args.workload)
                                 if args.anchor_slab is None else None),
                     "kernel": "k_triangles", "kernel_ms": statistics.mean(kernel_ms),
                     "work": "8 flops x (candidate triangles W + pair-stage evaluations P) per launch",
                     "W": int(st_last["n_pairs"]), "P": int(st_last["n_pair_evals"]),
                     "peak_basis": "152 SMs x 128 FP32 lanes x 2 x median sampled SM clock "
                                   "(MEASURED_PEAKS.json has no FP32 entry)"},
        "gpu_launches": engine_launches(1 if p1 is p else 2, True, args.schedule == "learned") * args.steps,
        "clocks": clocks,
        "exact_path": {"pairs": int(st_last["n_exact_pairs"]), "triangles": int(st_last["n_exact_tris"]),
                       "flagged_rows": int(st_last["n_flagged_rows"]), "queued": int(st_last["n_queued"])},
        "schedule": args.schedule,
    }
    if sched_cmp is not None:
        out["schedules"] = sched_cmp
    if world == 1 and not args.no_cpu_baseline and args.anchor_slab is None:
        out["cpu_baseline"] = cpu_baseline(p, box, edges)
    if world == 1 and args.workload == "box_clustered" and not args.no_north_star and args.anchor_slab is None:
        out["north_star"] = north_star_block()
    return out if rank == 0 else None


def north_star_block() -> dict:
    """The two comparisons the project's target is stated in, measured in the
    same process on the same GPU (device-resident inputs, L2 flushed before
    every call, one call each after a warm-up call):
      * soneira_peebles: the 4M-point Soneira-Peebles box (L=1500, r_max=80,
        16 bins) under the learned, dynamic and static schedules: whole-call
        and triangle-kernel times, counts identical across schedules, and the
        work model's prediction quality on this catalogue's cells;
      * batch_mocks: the 64 Neyman-Scott mocks counted by one persistent
        launch in a CUDA graph (autotuned) against 64 separate calls, with
        per-mock identity of the counts."""
    import torch
    from cudancorr_gb300 import api
    from cudancorr_gb300 import catalogs as C

    dev = torch.device("cuda", torch.cuda.current_device())
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    out = {}

    def timed(corr, t1, t2, t3):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        corr._calculate_device(t1, t2, t3, stream=stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), corr.stats()

    # Learned scheduling on the 4M-point clustered box.
    t0 = time.perf_counter()
    p, box, edges = C.config_soneira_peebles()
    t_cat = torch.from_numpy(p).to(dev)
    model, train_info = train_work_model("soneira_peebles")
    corr = api.ncorr(np.full(3, box), api.threeD, edges, False, (0.0, 0.0, 0.0))
    sched = {}
    ref_counts = None
    same = True
    for name, mode in (("learned", api.SCHED_LEARNED), ("dynamic", api.SCHED_DYNAMIC), ("static", api.SCHED_STATIC)):
        corr.set_schedule(mode, model if mode == api.SCHED_LEARNED else None)
        corr.set_record_work(name == "dynamic")
        timed(corr, t_cat, t_cat, t_cat)  # warm-up (and, for dynamic, the recorded cell work)
        if name == "dynamic":
            f, w = corr.cell_work()
        corr.set_record_work(False)
        ms, st = timed(corr, t_cat, t_cat, t_cat)
        h = corr.getTriCountsAll()
        if ref_counts is None:
            ref_counts = h
        same = same and bool(np.array_equal(h, ref_counts))
        sched[name] = {"call_ms": ms, "kernel_ms": st["ms_count"], "triangles": int(st["triangles"]),
                       "tail_idle": st["tail_idle"]}
    corr.close()
    keep = f[:, 0] > 0
    y = np.log1p(w[keep])
    pred = model.predict(f[keep]).astype(np.float64)
    model.close()
    out["soneira_peebles"] = {
        "description": "4M-point Soneira-Peebles box (5 levels, eta=4, lambda=1.9, R0=200), L=1500, r_max=80, "
                       "16 bins, unweighted",
        "n_points": int(len(p)), "schedules": sched, "counts_identical": same,
        "speedup_learned_vs_static": sched["static"]["call_ms"] / sched["learned"]["call_ms"],
        "speedup_learned_vs_dynamic": sched["dynamic"]["call_ms"] / sched["learned"]["call_ms"],
        "prediction": {"cells": int(keep.sum()), "mse_log": float(np.mean((pred - y) ** 2)),
                       "r2_log": float(1.0 - np.mean((pred - y) ** 2) / np.var(y)),
                       "total_work_rel_err": float(np.expm1(pred).sum() / np.expm1(y).sum() - 1.0)},
        "training": train_info, "wall_s": round(time.perf_counter() - t0, 1)}
    del t_cat

    # Batched mocks: one graph replay against 64 separate calls.
    t0 = time.perf_counter()
    mocks, mbox, medges = C.config_batch_mocks()
    t_mocks = [torch.from_numpy(m).to(dev) for m in mocks]
    corr = api.ncorr(np.full(3, mbox), api.threeD, medges, False, (0.0, 0.0, 0.0))
    b = api.Batch(corr, [(t, t, t) for t in t_mocks], autotune=True)
    plan = b.stats()
    b.run()  # warm-up
    flush.fill_(1.0)
    torch.cuda.synchronize()
    b.run()
    bst = b.stats()
    counts_batch = [b.counts_all(i) for i in range(len(mocks))]
    b.close()
    for t in t_mocks[:2]:
        corr._calculate_device(t, t, t)  # warm-up
    plain_ms, plain_kernel_ms, same = 0.0, 0.0, True
    for i, t in enumerate(t_mocks):
        ms, st = timed(corr, t, t, t)
        plain_ms += ms
        plain_kernel_ms += st["ms_count"]
        same = same and bool(np.array_equal(corr.getTriCountsAll(), counts_batch[i]))
    corr.close()
    out["batch_mocks"] = {
        "description": "64 Neyman-Scott mocks, L=1000, sizes log-uniform in [50,000, 1,000,000], r_max=60, "
                       "12 bins, unweighted",
        "n_points": int(sum(len(m) for m in mocks)), "batched_replay_ms": bst["ms_run"],
        "batched_kernel_ms": bst["ms_count"], "plain_64_calls_ms": plain_ms,
        "plain_64_kernel_ms": plain_kernel_ms, "speedup_batched_vs_plain": plain_ms / bst["ms_run"],
        "counts_identical": same, "triangles": int(bst["triangles"]),
        "tuning": {"hist_copies": plan["hist_copies"], "ms_autotune": plan["ms_autotune"]},
        "wall_s": round(time.perf_counter() - t0, 1)}
    return out


def run_batch(args) -> dict:
    """Batched mocks: 64 Neyman-Scott catalogues counted by one persistent
    launch inside one CUDA graph (autotuned), against 64 separate
    calculateD1D2D3 calls. Each rank counts its own 64 mocks."""
    import torch
    from cudancorr_gb300 import api
    from cudancorr_gb300 import catalogs as C

    world, rank, local = dist_setup()
    mocks, box, edges = C.config_batch_mocks(seed=4 + rank)
    desc = ("64 Neyman-Scott mocks, L=1000 Mpc/h, sizes log-uniform in [50,000, 1,000,000], N/8 parents "
            "x Poisson(8), sigma 1.5, r_max=60 (17 cells, non-divisible), 12 linear bins, unweighted")
    dev = torch.device("cuda", local)
    t_mocks = [torch.from_numpy(m).to(dev) for m in mocks]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    corr = api.ncorr(np.full(3, box), api.threeD, edges, False, (0.0, 0.0, 0.0))
    sched = args.schedule
    model, train_info = None, None
    if sched == "learned":
        raise SystemExit("batch_mocks: the learned schedule has no training process here; use dynamic or static")
    if sched == "static":
        corr.set_schedule(api.SCHED_STATIC)
    b = api.Batch(corr, [(t, t, t) for t in t_mocks], autotune=not args.no_autotune)
    plan = b.stats()

    def step():
        flush.fill_(1.0)
        torch.cuda.synchronize()
        b.run()
        return b.stats()

    for _ in range(args.warmup):
        step()
    sampler = ClockSampler(local)
    sampler.start()
    barrier(world)
    run_ms, count_ms, tri = [], [], []
    for _ in range(args.steps):
        st = step()
        run_ms.append(st["ms_run"])
        count_ms.append(st["ms_count"])
        tri.append(st["triangles"])
    barrier(world)
    clocks = sampler.stop()
    st_last = b.stats()
    counts_batch = [b.counts_all(i) for i in range(len(mocks))]
    b.close()
    total_ms = barrier_max(sum(run_ms), world)
    total_tri = barrier_sum(float(sum(tri)), world)

    # 64 separate calls (device-resident), the plain method; counts must agree.
    plain_ms, same = 0.0, True
    for i, t in enumerate(t_mocks):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        corr._calculate_device(t, t, t)
        plain_ms += (time.perf_counter() - t0) * 1e3
        same = same and bool(np.array_equal(corr.getTriCountsAll(), counts_batch[i]))

    # End to end: host arrays bound to a batch, copies inside the graph.
    corr.set_tuning(plan["sub_j"], plan["hist_copies"])  # the device batch's autotuned choice
    hb = api.Batch(corr, [(m, m, m) for m in mocks], autotune=False)
    hb.run()
    barrier(world)
    e2e_ms = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hb.run()
        _ = [hb.counts_all(i) for i in range(len(mocks))]
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    hb.close()
    corr.close()
    e2e_total = barrier_max(sum(e2e_ms), world)

    sm_mhz = clocks.get("sm_mhz") or 1995.0
    peak_tflops = N_SM * FP32_LANES_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    flops = 8.0 * (st_last["n_pairs"] + st_last["n_pair_evals"])
    achieved = flops / (statistics.mean(count_ms) / 1e3) / 1e12
    nb = len(edges) - 1
    n_pts = int(sum(len(m) for m in mocks))
    out = {
        "metric": METRIC, "value": total_tri / (total_ms / 1e3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32+fp64-exact",
        "data": "synthetic (seeded)",
        "config": {"workload": "batch_mocks", "description": desc, "n_catalogues": len(mocks),
                   "n_points": n_pts, "box": box, "r_max": float(edges[-1]), "bins_per_side": nb,
                   "triangles_per_step": int(tri[-1]), "l2": "flushed (256 MiB write) between steps",
                   "parallelism": f"{world} x 64 independent catalogues, one batch per GPU"},
        "e2e": {"value": total_tri / (e2e_total / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": int(sum(m.nbytes for m in mocks)),
                "d2h_bytes_per_step": int(len(mocks) * nb ** 3 * 8), "ms_per_step": e2e_total / args.steps},
        "roofline": {"bound": "fp32_issue", "achieved": achieved, "peak": peak_tflops, "unit": "TFLOP/s",
                     "frac": achieved / peak_tflops, "traffic": None, "kernel": "k_triangles",
                     "kernel_ms": statistics.mean(count_ms),
                     "work": "8 flops x (candidate triangles W + pair-stage evaluations P) per launch",
                     "W": int(st_last["n_pairs"]), "P": int(st_last["n_pair_evals"]),
                     "peak_basis": "152 SMs x 128 FP32 lanes x 2 x median sampled SM clock"},
        "gpu_launches": int(plan["graph_nodes"]) * args.steps,
        "clocks": clocks,
        "batch": {"graph_nodes": plan["graph_nodes"], "ms_plan": plan["ms_plan"],
                  "ms_autotune": plan["ms_autotune"], "tuning": {"sub_j": plan["sub_j"],
                                                                 "hist_copies": plan["hist_copies"]},
                  "grid_ctas": plan["grid_ctas"], "schedule": sched,
                  "plain_64_calls_ms": plain_ms, "speedup_vs_plain": plain_ms / (total_ms / args.steps),
                  "counts_identical_to_plain": same},
    }
    return out if rank == 0 else None


SURVEY_COMBOS = (("DDD", 4), ("DDR", 32), ("DRR", 64), ("RRR", 256))  # (triple, anchor sampling 1/f)


def survey_catalogues(seed: int):
    """Data 500k (lognormal(0, 0.3) weights) and randoms 2.5M in the RA 0-90,
    Dec 0-60 wedge, r ~ N(1000, 150) in [600, 1400], jointly shifted by the
    engine's prep_cat_survey; 15 log bins in [5, 120)."""
    from cudancorr_gb300 import catalogs as C
    return C.config_survey(seed)


def run_survey(args) -> dict:
    """Survey mode with weights: DDD, DDR, DRR and RRR per step, each on a
    seeded anchor sample (fractions in SURVEY_COMBOS); weighted bins checked
    per bin against the FP64 oracle on a few anchors."""
    import torch
    from cudancorr_gb300 import api
    from oracle import oracle as O

    world, rank, local = dist_setup()
    d, r, box, ori, edges = survey_catalogues(7 + 10 * rank)
    dev = torch.device("cuda", local)
    cats = {"D": d, "R": r}
    tcat = {k: torch.from_numpy(v).to(dev) for k, v in cats.items()}
    rng = np.random.default_rng(3)
    runs = []
    triples = args.triples.split(",") if args.triples else [c for c, _ in SURVEY_COMBOS]
    for combo, frac in SURVEY_COMBOS:
        if combo not in triples:
            continue
        frac *= args.anchor_scale
        anc = cats[combo[0]]
        sub = np.ascontiguousarray(anc[np.sort(rng.choice(len(anc), len(anc) // frac, replace=False))])
        runs.append((combo, frac, sub, torch.from_numpy(sub).to(dev)))
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    corr = api.ncorr(box, api.threeD, edges, True, ori)

    def call(t1, combo):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        corr._calculate_device(t1, tcat[combo[1]], tcat[combo[2]], stream=stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), corr.stats()

    # Triangles of each sample: the same call with unit weights (the
    # geometry, not the weights, decides which triangles count).
    ones = {k: v.clone() for k, v in tcat.items()}
    for v in ones.values():
        v[:, 3] = 1.0
    tri = {}
    for combo, frac, sub, tsub in runs:
        t1 = tsub.clone()
        t1[:, 3] = 1.0
        corr._calculate_device(t1, ones[combo[1]], ones[combo[2]], stream=stream.cuda_stream)
        tri[combo] = corr.stats()["triangles"]
    del ones

    for _ in range(args.warmup):
        for combo, frac, sub, tsub in runs[:1]:
            call(tsub, combo)
    sampler = ClockSampler(local)
    sampler.start()
    barrier(world)
    step_ms, kernel_ms, per = [], [], {c: [] for c, _, _, _ in runs}
    flops = []
    for _ in range(args.steps):
        tot = 0.0
        for combo, frac, sub, tsub in runs:
            ms, st = call(tsub, combo)
            tot += ms
            per[combo].append(ms)
            kernel_ms.append(st["ms_count"])
            flops.append(8.0 * (st["n_pairs"] + st["n_pair_evals"]))
        step_ms.append(tot)
    barrier(world)
    clocks = sampler.stop()
    total_ms = barrier_max(sum(step_ms), world)
    tri_step = float(sum(tri.values()))

    # End to end: host arrays through the reference-facing call.
    e2e_ms = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for combo, frac, sub, tsub in runs:
            corr.calculateD1D2D3(sub, cats[combo[1]], cats[combo[2]])
            _ = corr.getTriCountsOut()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_total = barrier_max(sum(e2e_ms), world)

    # Precision: weighted bins against the FP64 oracle on a few anchors.
    precision = {}
    for combo, n_anc in (("DDD", 32), ("DDR", 8), ("DRR", 8)) if not args.no_cpu_baseline else ():
        sub = np.ascontiguousarray(cats[combo[0]][:n_anc])
        corr.calculateD1D2D3(sub, cats[combo[1]], cats[combo[2]])
        h = corr.getTriCountsAll()
        ref = O.count_threeD(box, edges, sub, cats[combo[1]], cats[combo[2]], survey=True,
                             nthreads=os.cpu_count() or 1)
        nz = ref != 0
        rel = np.abs(h[nz] - ref[nz]) / np.abs(ref[nz])
        precision[combo] = {"anchors": n_anc, "bins": int(nz.sum()), "max_rel_err": float(rel.max()),
                            "median_rel_err": float(np.median(rel)),
                            "nonzero_pattern_equal": bool(np.array_equal(h != 0, nz))}
    corr.close()

    sm_mhz = clocks.get("sm_mhz") or 1995.0
    peak_tflops = N_SM * FP32_LANES_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    achieved = sum(flops) / (sum(kernel_ms) / 1e3) / 1e12
    nb = len(edges) - 1
    out = {
        "metric": METRIC, "value": barrier_sum(tri_step * args.steps, world) / (total_ms / 1e3), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32+fp64-exact, int128 sums",
        "data": "synthetic (seeded)",
        "config": {"workload": "survey", "description": "survey wedge: data 500,000 (lognormal(0,0.3) weights), "
                                                       "randoms 2,500,000, 15 log bins in [5,120), weighted "
                                                       "DDD/DDR/DRR/RRR, anchors sampled per triple",
                   "anchor_fraction": {c: f"1/{f}" for c, f, _, _ in runs}, "box": [float(x) for x in box],
                   "bins_per_side": nb, "triangles_per_step": int(tri_step),
                   "triangles_per_triple": {c: int(v) for c, v in tri.items()},
                   "l2": "flushed (256 MiB write) before every call", "parallelism": "independent catalogues per GPU"},
        "e2e": {"value": barrier_sum(tri_step * args.steps, world) / (e2e_total / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": int(sum(sub.nbytes + cats[c[1]].nbytes + (0 if c[2] == c[1] else cats[c[2]].nbytes)
                                              for c, _, sub, _ in runs)),
                "d2h_bytes_per_step": int(len(runs) * nb ** 3 * 8), "ms_per_step": e2e_total / args.steps},
        "roofline": {"bound": "fp32_issue", "achieved": achieved, "peak": peak_tflops, "unit": "TFLOP/s",
                     "frac": achieved / peak_tflops, "traffic": None, "kernel": "k_triangles",
                     "kernel_ms": sum(kernel_ms) / args.steps,
                     "work": "8 flops x (candidate triangles W + pair-stage evaluations P), four calls",
                     "peak_basis": "152 SMs x 128 FP32 lanes x 2 x median sampled SM clock"},
        "gpu_launches": sum(engine_launches(2 if c[1] == c[2] else 3, c[1] == c[2]) for c, _, _, _ in runs)
        * args.steps,
        "clocks": clocks,
        "per_triple_ms": {c: statistics.mean(v) for c, v in per.items()},
        "precision_vs_fp64_oracle": precision,
    }
    return out if rank == 0 else None


RPPI_NPI = 30


def rppi_workload(seed_offset: int, logspace):
    """The clustered box of the default workload with the rppi binning: rp in
    12 log bins on [1, 30) Mpc/h, 30 unit pi bins (piMax = 30 Mpc/h), line of
    sight z. The reference quotes no rppi configuration; this is a typical
    projected 3PCF binning."""
    from cudancorr_gb300 import catalogs as C
    p, box, _ = C.config_box_clustered(seed=2 + seed_offset)
    edges = logspace(1.0, 30.0, 13)
    desc = ("Neyman-Scott box: 200,000 parents x Poisson(10), sigma 2, L=2000 Mpc/h; rppi: rp 12 log bins "
            "in [1,30), 30 unit pi bins, unweighted")
    return p, box, edges, RPPI_NPI, desc


def run_rppi(args) -> dict:
    """The rppi bin type (the reference's second constructor) on one GPU."""
    import torch
    from cudancorr_gb300 import api

    world, rank, local = dist_setup()
    p, box, edges, npi, desc = rppi_workload(rank, api.logspace)
    dev = torch.device("cuda", local)
    t_cat = torch.from_numpy(p).to(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    corr = api.ncorr(np.full(3, box), api.rppi, edges, npi, False, (0.0, 0.0, 0.0))

    def device_step():
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        corr._calculate_device(t_cat, t_cat, t_cat, stream=stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), corr.stats()

    for _ in range(args.warmup):
        device_step()
    sampler = ClockSampler(local)
    sampler.start()
    barrier(world)
    step_ms, kernel_ms, tri = [], [], []
    for _ in range(args.steps):
        ms, st = device_step()
        step_ms.append(ms)
        kernel_ms.append(st["ms_count"])
        tri.append(st["triangles"])
    barrier(world)
    clocks = sampler.stop()
    st_last = corr.stats()
    total_ms = barrier_max(sum(step_ms), world)
    total_tri = barrier_sum(float(sum(tri)), world)
    p_host = torch.from_numpy(p).pin_memory().numpy()
    corr.calculateD1D2D3(p_host, p_host, p_host)
    barrier(world)
    e2e_ms = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        corr.calculateD1D2D3(p_host, p_host, p_host)
        _ = corr.getTriCountsOut()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_total = barrier_max(sum(e2e_ms), world)
    n_out = len(corr.getTriCountsOut())
    corr.close()
    # FP32 issue roofline, as for the threeD kernel: 8 flops (the third
    # side's |d_j - d_l|^2) per candidate pair visited; the FP32 classifier
    # settles almost all of them and the rest go to FP64.
    sm_mhz = clocks.get("sm_mhz") or 1995.0
    peak_tflops = N_SM * FP32_LANES_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    achieved = 8.0 * st_last["n_pairs"] / (statistics.mean(kernel_ms) / 1e3) / 1e12
    nb = len(edges) - 1
    out = {
        "metric": METRIC, "value": total_tri / (total_ms / 1e3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32 classifier + fp64 exact",
        "data": "synthetic (seeded)",
        "config": {"workload": "rppi_box_clustered", "description": desc, "n_points": int(len(p)), "box": box,
                   "rp_max": float(edges[-1]), "rp_bins": nb, "pi_bins": npi, "triangles_per_step": int(tri[-1]),
                   "overflow_per_step": float(st_last["overflow"]),
                   "l2": "flushed (256 MiB write) between steps",
                   "parallelism": f"{world} independent catalogue(s), one per GPU"},
        "e2e": {"value": total_tri / (e2e_total / 1e3), "unit": UNIT, "h2d_bytes_per_step": int(p.nbytes),
                "d2h_bytes_per_step": int(nb ** 3 * npi * npi * 8), "ms_per_step": e2e_total / args.steps},
        "roofline": {"bound": "fp32_issue", "achieved": achieved, "peak": peak_tflops, "unit": "TFLOP/s",
                     "frac": achieved / peak_tflops, "traffic": None, "kernel": "k_rppi",
                     "kernel_ms": statistics.mean(kernel_ms),
                     "work": "8 flops x candidate pairs visited per launch",
                     "pairs_visited": int(st_last["n_pairs"]), "pairs_fp32_classifier": int(st_last["n_queued"]),
                     "pairs_fp64": int(st_last["n_exact_tris"]),
                     "peak_basis": "152 SMs x 128 FP32 lanes x 2 x median sampled SM clock"},
        "gpu_launches": engine_launches(1, True, rppi=True) * args.steps,
        "clocks": clocks,
        "n_out": n_out,
    }
    if world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        rng = np.random.default_rng(7)
        n = 4096
        sub = np.ascontiguousarray(p[rng.choice(len(p), n, replace=False)])
        t = time.perf_counter()
        h, _ = O.count_rppi(box, edges, npi, sub, p, p, nthreads=threads)
        dt = time.perf_counter() - t
        n2 = int(min(len(p), n * 10.0 / max(dt, 1e-3)))
        sub = np.ascontiguousarray(p[rng.choice(len(p), n2, replace=False)])
        t = time.perf_counter()
        h, _ = O.count_rppi(box, edges, npi, sub, p, p, nthreads=threads)
        dt = time.perf_counter() - t
        out["cpu_baseline"] = {"value": float(h.sum() / dt), "unit": UNIT, "cores": threads, "kind": "port",
                               "sample": f"{n2} random anchors of the {len(p):,}-point catalogue, {dt:.1f} s, "
                                         "oracle/ncorr_oracle.cpp rppi neighbour-list form"}
    return out if rank == 0 else None


def run_reference_rppi(args) -> dict:
    """The reference's own rppi kernel (countTrianglesRppiBox from the
    oracle/_ref cubin) behind its host flow, on a random anchor sample."""
    from oracle import oracle as O
    p, box, edges, npi, desc = rppi_workload(0, O.logspace)
    for _ in range(args.warmup):
        O.reference_count_rppi(box, edges, npi, p[:2048], p, p)
    rng = np.random.default_rng(11)
    n_sub = min(len(p), args.ref_anchors)
    tri, tot_ms, k_ms = [], [], []
    for _ in range(args.steps):
        sub = np.ascontiguousarray(p[rng.choice(len(p), n_sub, replace=False)])
        h, ov, kms, tms = O.reference_count_rppi(box, edges, npi, sub, p, p)
        tri.append(h.sum() + ov)
        tot_ms.append(tms)
        k_ms.append(kms)
    value = sum(tri) / (sum(tot_ms) / 1e3)
    sample = (f"{n_sub} random anchors per timed step of the {len(p):,}-point catalogue; reference "
              f"source/device.cu countTrianglesRppiBox, unmodified, on the GB300 via oracle/ref_runner.cu")
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sum(tot_ms) / len(tot_ms),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic (seeded)",
        "config": {"workload": "rppi_box_clustered", "description": desc, "n_points": int(len(p)),
                   "anchor_sample": n_sub, "l2": "inputs staged per call by the reference host flow"},
        "kernel_only": {"value": sum(tri) / (sum(k_ms) / 1e3), "unit": UNIT, "ms_per_step": sum(k_ms) / len(k_ms)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "reference",
                         "device": "GB300 (the reference's CUDA kernel; one host thread drives it)",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_rppi_survey(args) -> dict:
    """The rppi bin type in survey mode on one GPU: DDD of the survey wedge's
    data (unit weights, so that triangles are counted) on a seeded 1/8 anchor
    sample, all data as p2 and p3; rp in 12 log bins on [1, 30), 30 unit pi
    bins. An FP32 classifier with rigorous bands settles almost every pair
    (line-of-sight projections, order, bins); the rest are evaluated in FP64,
    32 lanes wide."""
    import torch
    from cudancorr_gb300 import api

    world, rank, local = dist_setup()
    d, _, box, ori, _ = survey_catalogues(7 + 10 * rank)
    d = np.ascontiguousarray(d)
    d[:, 3] = 1.0
    edges = api.logspace(1.0, 30.0, 13)
    rng = np.random.default_rng(3)
    sub = np.ascontiguousarray(d[np.sort(rng.choice(len(d), len(d) // 8, replace=False))])
    dev = torch.device("cuda", local)
    t_d, t_s = torch.from_numpy(d).to(dev), torch.from_numpy(sub).to(dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    corr = api.ncorr(box, api.rppi, edges, RPPI_NPI, True, ori)

    def device_step():
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        corr._calculate_device(t_s, t_d, t_d, stream=stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1), corr.stats()

    for _ in range(args.warmup):
        device_step()
    sampler = ClockSampler(local)
    sampler.start()
    barrier(world)
    step_ms, kernel_ms, tri = [], [], []
    for _ in range(args.steps):
        ms, st = device_step()
        step_ms.append(ms)
        kernel_ms.append(st["ms_count"])
        tri.append(st["triangles"])
    barrier(world)
    clocks = sampler.stop()
    st_last = corr.stats()
    total_ms = barrier_max(sum(step_ms), world)
    total_tri = barrier_sum(float(sum(tri)), world)
    s_host = torch.from_numpy(sub).pin_memory().numpy()
    d_host = torch.from_numpy(d).pin_memory().numpy()
    corr.calculateD1D2D3(s_host, d_host, d_host)
    barrier(world)
    e2e_ms = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t = time.perf_counter()
        corr.calculateD1D2D3(s_host, d_host, d_host)
        _ = corr.getTriCountsOut()
        e2e_ms.append((time.perf_counter() - t) * 1e3)
    e2e_total = barrier_max(sum(e2e_ms), world)
    n_out = len(corr.getTriCountsOut())
    corr.close()
    nb = len(edges) - 1
    sm_mhz = clocks.get("sm_mhz") or 1995.0
    peak_tflops = N_SM * FP32_LANES_PER_SM * 2 * sm_mhz * 1e6 / 1e12
    achieved = 8.0 * st_last["n_pairs"] / (statistics.mean(kernel_ms) / 1e3) / 1e12
    return {
        "metric": METRIC, "value": total_tri / (total_ms / 1e3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32 classifier + fp64 exact",
        "data": "synthetic (seeded)",
        "config": {"workload": "rppi_survey",
                   "description": "survey wedge data (500,000 points, unit weights), DDD on a 1/8 anchor sample; "
                                  "rppi: rp 12 log bins in [1,30), 30 unit pi bins",
                   "n_points": int(len(d)), "anchors": int(len(sub)), "rp_bins": nb, "pi_bins": RPPI_NPI,
                   "triangles_per_step": int(tri[-1]), "overflow_per_step": float(st_last["overflow"]),
                   "l2": "flushed (256 MiB write) between steps",
                   "parallelism": f"{world} independent catalogue(s), one per GPU"},
        "e2e": {"value": total_tri / (e2e_total / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": int(sub.nbytes + d.nbytes), "d2h_bytes_per_step": int(nb ** 3 * RPPI_NPI ** 2 * 8),
                "ms_per_step": e2e_total / args.steps},
        "roofline": {"bound": "fp32_issue", "achieved": achieved, "peak": peak_tflops, "unit": "TFLOP/s",
                     "frac": achieved / peak_tflops, "traffic": None, "kernel": "k_rppi",
                     "kernel_ms": statistics.mean(kernel_ms),
                     "work": "8 flops x candidate pairs visited per launch, as for the box",
                     "pairs_visited": int(st_last["n_pairs"]), "pairs_fp64": int(st_last["n_exact_tris"]),
                     "peak_basis": "152 SMs x 128 FP32 lanes x 2 x median sampled SM clock"},
        "gpu_launches": engine_launches(2, True, rppi=True) * args.steps,
        "clocks": clocks,
        "n_out": n_out,
    }


def run_reference(args) -> dict:
    """The reference's own kernel (oracle/_ref cubin, compiled unmodified from
    its source/device.cu) behind a restatement of its host flow, on an anchor
    sample of the same workload (all points as p2/p3).

    The reference runs one thread per anchor in 64-thread blocks, in FP64, so
    a step lasts as long as its most expensive anchor's thread. Measured on
    GB300 (2M-point clustered box, random anchors): 9,728 anchors (one block
    per SM) 58.6 s per step, 9.1e7 triangles/s; 19,456 (two) 59.2 s,
    1.8e8; 38,912 (four) 86 s, 2.5e8. No random sample fits twenty timed steps
    in the run's time limit, so every timed step draws 19,456 anchors at
    random from the 1% of anchors whose estimated cost for the reference's
    thread (oracle.reference_anchor_cost) is lowest: that bounds a step near
    36 s and, since it trims the slow tail that sets the reference's step
    time, it can only raise the reference's rate. Warm-up steps load the
    module and run 640 anchors of the small uniform box.
    """
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    from oracle import oracle as O
    try:
        O.runner()
    except Exception as e:  # the cubin is built where the reference sources are mounted
        return {"impl": "reference", "unavailable": f"reference kernel not loadable: {e}"}
    if args.workload == "rppi_box_clustered":
        return run_reference_rppi(args)
    if args.workload in ("batch_mocks", "survey", "rppi_survey"):
        return {"impl": "reference", "unavailable": "the reference arm times the single-catalogue box workloads; "
                                                    f"{args.workload} would take the reference kernel hours"}
    p, box, edges, desc = workload(args.workload, 0)
    from cudancorr_gb300 import catalogs as C
    wp, wbox, wedges = C.config_box_uniform()
    for _ in range(args.warmup):
        O.reference_count(wbox, wedges, wp[:640], wp, wp)
    cost, _ = O.reference_anchor_cost(p, p, p, box, edges[-1])
    pool = np.flatnonzero(cost <= np.quantile(cost, args.ref_pool))
    rng = np.random.default_rng(11)
    n_sub = min(len(pool), args.ref_anchors)
    tri, tot_ms, k_ms = [], [], []
    for _ in range(args.steps):
        sub = np.ascontiguousarray(p[np.sort(rng.choice(pool, n_sub, replace=False))])
        h, kms, tms = O.reference_count(box, edges, sub, p, p)
        tri.append(h.sum())
        tot_ms.append(tms)
        k_ms.append(kms)
    value = sum(tri) / (sum(tot_ms) / 1e3)
    sample = (f"{n_sub} anchors per timed step, drawn at random from the {len(pool):,} anchors "
              f"({100 * args.ref_pool:g}%) of the {len(p):,}-point catalogue with the lowest estimated cost for "
              f"the reference's one-thread-per-anchor kernel (a random sample's slowest anchor alone takes "
              f"about 59 s); all points as p2/p3; reference source/device.cu kernel, unmodified, on the GB300 "
              f"via oracle/ref_runner.cu (the reference has no CPU counting path); warm-up steps: 640 anchors "
              f"of the 20,000-point uniform box")
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sum(tot_ms) / len(tot_ms),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "description": desc, "n_points": int(len(p)),
                   "anchor_sample": n_sub, "anchor_pool": int(len(pool)),
                   "l2": "inputs staged per call by the reference host flow"},
        "kernel_only": {"value": sum(tri) / (sum(k_ms) / 1e3), "unit": UNIT,
                        "ms_per_step": sum(k_ms) / len(k_ms)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "reference",
                         "device": "GB300 (the reference's CUDA kernel; one host thread drives it)",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="box_clustered",
                    choices=["box_clustered", "box_clustered_L1000", "box_uniform", "soneira_peebles",
                             "batch_mocks", "survey", "rppi_box_clustered", "rppi_survey"])
    ap.add_argument("--schedule", default="dynamic", choices=["dynamic", "static", "learned"],
                    help="anchor order of the triangle kernel (learned: trains the work model first)")
    ap.add_argument("--no-autotune", action="store_true", help="batch_mocks: default tuning")
    ap.add_argument("--triples", default="", help="survey: comma-separated subset of DDD,DDR,DRR,RRR")
    ap.add_argument("--anchor-scale", type=int, default=1,
                    help="survey: divide each triple's anchor sample by this factor (profiling size)")
    ap.add_argument("--ref-anchors", type=int, default=152 * 2 * 64,
                    help="reference arm: anchors per timed step")
    ap.add_argument("--ref-pool", type=float, default=0.01,
                    help="reference arm: fraction of anchors, cheapest for the reference kernel, to draw from")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-north-star", action="store_true",
                    help="skip the learned-schedule and batched-mocks comparisons of the default line")
    ap.add_argument("--anchor-slab", type=float, default=None,
                    help="profiling size: anchors restricted to points with x < W (Mpc/h)")
    args = ap.parse_args()
    if args.impl == "reference":
        out = run_reference(args)
    elif args.workload == "batch_mocks":
        out = run_batch(args)
    elif args.workload == "survey":
        out = run_survey(args)
    elif args.workload == "rppi_box_clustered":
        out = run_rppi(args)
    elif args.workload == "rppi_survey":
        out = run_rppi_survey(args)
    else:
        out = run_engine(args)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
