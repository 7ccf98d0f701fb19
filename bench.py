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
# dram__bytes_write.sum): 27.37 MB measured with ncu on the 249,814-point
# box_clustered_L1000 workload, scaled by the anchor count to the
# 2,001,574-point box_clustered launch.
TRIANGLE_KERNEL_DRAM_BYTES = {"box_clustered": int(27.37e6 * 2001574 / 249814),
                              "box_clustered_L1000": int(27.37e6)}


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


def barrier_max(value: float, world: int) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], device="cuda", dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier_sum(value: float, world: int) -> float:
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], device="cuda", dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(world: int):
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()


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
        "gpu_launches": 6 * args.steps,
        "clocks": clocks,
        "exact_path": {"pairs": int(st_last["n_exact_pairs"]), "triangles": int(st_last["n_exact_tris"]),
                       "flagged_rows": int(st_last["n_flagged_rows"]), "queued": int(st_last["n_queued"])},
    }
    if world == 1 and not args.no_cpu_baseline and args.anchor_slab is None:
        out["cpu_baseline"] = cpu_baseline(p, box, edges)
    return out if rank == 0 else None


def run_reference(args) -> dict:
    """The reference's own kernel (oracle/_ref cubin, compiled unmodified from
    its source/device.cu) behind a restatement of its host flow, on a random
    anchor sample of the same workload.

    The reference runs one thread per anchor in 64-thread blocks, so its
    throughput depends on how many blocks each SM holds. Measured on GB300
    (2M-point clustered box): 7.7e7 triangles/s with 8192 anchors (about one
    block per SM), 2.47e8 with 38,912 (4 blocks per SM), 2.52e8 with 155,648
    (16 per SM). The default sample of 38,912 anchors (152 SMs x 4 x 64)
    reaches that plateau. A step takes about 86 s, which the slowest anchor
    thread sets. Warm-up steps load the module and run the small uniform box.
    """
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    from oracle import oracle as O
    try:
        O.runner()
    except Exception as e:  # the cubin is built where the reference sources are mounted
        return {"impl": "reference", "unavailable": f"reference kernel not loadable: {e}"}
    p, box, edges, desc = workload(args.workload, 0)
    from cudancorr_gb300 import catalogs as C
    wp, wbox, wedges = C.config_box_uniform()
    for _ in range(args.warmup):
        O.reference_count(wbox, wedges, wp[:4096], wp, wp)
    rng = np.random.default_rng(11)
    n_sub = min(len(p), args.ref_anchors)
    tri, tot_ms, k_ms = [], [], []
    for _ in range(args.steps):
        sub = p if n_sub == len(p) else np.ascontiguousarray(p[rng.choice(len(p), n_sub, replace=False)])
        h, kms, tms = O.reference_count(box, edges, sub, p, p)
        tri.append(h.sum())
        tot_ms.append(tms)
        k_ms.append(kms)
    value = sum(tri) / (sum(tot_ms) / 1e3)
    sample = (f"{n_sub} random anchors per timed step of the {len(p):,}-point catalogue (all points as "
              f"p2/p3); reference source/device.cu kernel, unmodified, on the GB300 via "
              f"oracle/ref_runner.cu (the reference has no CPU counting path); warm-up steps: "
              f"4096 anchors of the 20,000-point uniform box")
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sum(tot_ms) / len(tot_ms),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "description": desc, "n_points": int(len(p)),
                   "anchor_sample": n_sub, "l2": "inputs staged per call by the reference host flow"},
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
                    choices=["box_clustered", "box_clustered_L1000", "box_uniform", "soneira_peebles"])
    ap.add_argument("--ref-anchors", type=int, default=152 * 4 * 64)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--anchor-slab", type=float, default=None,
                    help="profiling size: anchors restricted to points with x < W (Mpc/h)")
    args = ap.parse_args()
    if args.impl == "reference":
        out = run_reference(args)
    else:
        out = run_engine(args)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
