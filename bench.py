"""Benchmark: the FMM-accelerated single-layer operator (one matvec per step).

Workload (N = 1,048,576): sources = targets uniform in the unit cube
(torch.rand, seed 0, generated in FP64 then cast to FP32), charges
2 rand - 1 (seed 1), panel areas 1, Laplace 1/r kernel, expansion order 8,
leaf size 64, MAC theta 0.5, adaptive tight-bbox octree built once (outside
the timed region, like the operator's constructor).  One step = one matvec.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`value` is throughput with inputs resident in HBM (device sigma, CUDA events
around each matvec on the launching stream, L2 flushed by a 256 MiB write
between steps); `e2e` goes through the public API
(LaplaceFmm3D.matvec with a host sigma: pinned H2D, compute, D2H inside the
timed region).  `--impl reference` times the CPU oracle's restatement of the
operator (FP64, all host cores) on a bounded sample of the same workload.
Under torchrun every rank runs its own replica (no data-path collective).
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "BEM solves/s to 1e-6 residual, mixed+learned vs plain FP64 GMRES; FMM Mpts/s"
N_DEFAULT = 1 << 20
WORKLOAD = "fmm_matvec_uniform_unit_cube_N1048576_p8_leaf64_theta0.5_fp32"
# algorithmic FP32 flops of one M2L pair at p = 8 in the azimuth-factored
# form the kernel evaluates: 45 x 81 real-by-complex multiply-adds (4 flops),
# two azimuthal rotations of 45 coefficients (complex multiply, 8 flops
# each) and 153 real harmonics by a 3-term recurrence (6 flops each)
M2L_FLOPS_PER_PAIR = 4 * 45 * 81 + 2 * 8 * 45 + 6 * 153
# DRAM bytes one M2L pass moves per pair (ncu --set full of k_m2l_fast<8, SET>
# at N = 262,144: 44.6 MB for 9,091,877 pairs; traffic grows with the pair
# count, so it is scaled to the benchmark's pair count)
M2L_DRAM_BYTES_PER_PAIR_PER_PASS = 44.6e6 / 9_091_877
# near field: 3 sub + 3 fma (r^2) + max + rsqrt + fma per interaction, counted
# as the reference FLOP model's 20 flops (autotune.py:622-667)
P2P_FLOPS_PER_INTERACTION = 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--cpu-sample", type=int, default=262144)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def gen_inputs(n):
    import torch

    pts = torch.rand(n, 3, generator=torch.Generator().manual_seed(0), dtype=torch.float64).float()
    q = (2 * torch.rand(n, generator=torch.Generator().manual_seed(1), dtype=torch.float64) - 1).float()
    return pts, q


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def cpu_baseline(n_sample: int):
    """The oracle's FP64 restatement of the operator on all host cores, one matvec."""
    import numpy as np

    from oracle import oracle as O

    O.lib()
    pts, q = gen_inputs(n_sample)
    p = pts.numpy()
    t = O.build_tree(p, 64, 32)
    lists = O.build_lists(t, 0.5)
    sig = q.double().numpy()
    ones = np.ones(n_sample)
    t0 = time.perf_counter()
    O.fmm_matvec(t, lists, p, sig, ones, None, p=8, ke=1.0)
    dt = time.perf_counter() - t0
    return {"value": n_sample / dt / 1e6, "unit": "Mpts/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"one FP64 FMM matvec (p=8, leaf 64, theta 0.5) on the first {n_sample} points of the "
                      f"same generator, tree and lists prebuilt; {dt:.2f} s"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    import numpy as np

    from oracle import oracle as O

    O.lib()
    n = min(args.n, args.cpu_sample)
    pts, q = gen_inputs(n)
    p = pts.numpy()
    t = O.build_tree(p, 64, 32)
    lists = O.build_lists(t, 0.5)
    sig = q.double().numpy()
    ones = np.ones(n)
    for _ in range(args.warmup):
        O.fmm_matvec(t, lists, p, sig, ones, None, p=8, ke=1.0)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.fmm_matvec(t, lists, p, sig, ones, None, p=8, ke=1.0)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    val = n / (ms * 1e-3) / 1e6
    out = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "Mpts/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_points": n},
        "cpu_baseline": {"value": val, "unit": "Mpts/s", "cores": O.num_threads(), "kind": "port",
                         "sample": f"FP64 FMM matvec of the CPU oracle on the first {n} points of the workload "
                                   "generator per step (tree and lists prebuilt)"},
        "e2e": {"value": val, "unit": "Mpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import numpy as np
    import torch

    from electrodrive_gb300 import _lib
    from electrodrive_gb300.fmm3d import make_laplace_fmm_backend

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    n = args.n
    pts, q = gen_inputs(n)
    areas = torch.ones(n, dtype=torch.float32)
    fmm = make_laplace_fmm_backend(pts, areas, max_leaf_size=64, theta=0.5, expansion_order=8)
    plan = fmm.plan
    info = plan.info
    sig_d = q.to(dev)
    areas_d = areas.to(dev)
    out_d = torch.empty_like(sig_d)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        plan.matvec(sig_d, areas_d, None, k_e=1.0, out=out_d)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize(dev)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(dev)
    l0 = _lib.launch_count()
    times = []
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            times.append((e0, e1))
        torch.cuda.synchronize(dev)
    launches = _lib.launch_count() - l0
    ms = sum(a.elapsed_time(b) for a, b in times) / args.steps
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    torch.cuda.synchronize(dev)
    value = n * world / (ms * 1e-3) / 1e6

    # end to end through the public API: host sigma -> device -> host result
    for _ in range(2):
        fmm.matvec(sigma=q, src_centroids=pts, areas=areas, tile_size=1024, self_integrals=None)
    e2e_times = []
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        v = fmm.matvec(sigma=q, src_centroids=pts, areas=areas, tile_size=1024, self_integrals=None)
        e2e_times.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * sum(e2e_times) / len(e2e_times)
    if dist:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e_val = n * world / (e2e_ms * 1e-3) / 1e6

    # per-stage timing (separate pass, same stream) for the roofline
    plan.set_charges(sig_d)
    stage_ms = {}
    reps = 3
    for name, fn in [("p2m", lambda: plan.stage("p2m")), ("m2m", lambda: plan.stage("m2m")),
                     ("m2l", lambda: plan.stage("m2l", 0)), ("l2l", lambda: plan.stage("l2l")),
                     ("p2p", lambda: plan.p2p())]:
        fn()
        acc = 0.0
        for _ in range(reps):
            flush.fill_(2)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize(dev)
            acc += a.elapsed_time(b)
        stage_ms[name] = acc / reps
    fp32_peak = _lib.measure_fp32_peak()
    m2l_flops = info.n_m2l_pairs * M2L_FLOPS_PER_PAIR
    achieved = m2l_flops / (stage_ms["m2l"] * 1e-3) / 1e12
    p2p_tflops = info.p2p_interactions * P2P_FLOPS_PER_INTERACTION / (stage_ms["p2p"] * 1e-3) / 1e12

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(min(args.cpu_sample, n))
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "error": str(e)[:200]}

    if rank == 0:
        # accuracy of this run's output on 256 sampled targets (FP64 direct sum)
        err = None
        try:
            from oracle import oracle as O

            idx = torch.randperm(n, generator=torch.Generator().manual_seed(3))[:256].numpy()
            d = O.direct(pts.numpy(), q.double().numpy(), idx)
            got = v.double().numpy()[idx] / O.K_E  # the public operator includes K_E
            err = float(np.linalg.norm(got - d) / np.linalg.norm(d))
        except Exception:
            pass
        out = {
            "metric": METRIC,
            "value": value,
            "unit": "Mpts/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": max(args.warmup, 3),
            "ms_per_step": ms,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "n_points": n, "expansion_order": 8, "leaf_size": 64,
                       "mac_theta": 0.5, "n_nodes": info.n_nodes, "n_p2p_pairs": info.n_p2p_pairs,
                       "n_m2l_pairs": info.n_m2l_pairs, "p2p_interactions": info.p2p_interactions,
                       "l2": "flushed by a 256 MiB write between steps", "parallelism": f"replicas x{world}",
                       "rel_l2_vs_fp64_direct_256_targets": err},
            "e2e": {"value": e2e_val, "unit": "Mpts/s", "h2d_bytes_per_step": 4 * n, "d2h_bytes_per_step": 4 * n,
                    "ms_per_step": e2e_ms},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "roofline": {"kernel": "k_m2l_fast (M2L stage: two passes over split output sets)", "bound": "fp32",
                         "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp32_peak if fp32_peak else None,
                         "traffic": 2 * M2L_DRAM_BYTES_PER_PAIR_PER_PASS * info.n_m2l_pairs,
                         "traffic_note": "DRAM bytes of the M2L stage, scaled from an ncu capture at N=262,144",
                         "peak_source": "FP32 FMA probe measured in this run (edfmm_measure_fp32_peak)",
                         "flops_per_pair": M2L_FLOPS_PER_PAIR},
            "stages_ms": stage_ms,
            "p2p_tflops": p2p_tflops,
            "cpu_baseline": cpu,
        }
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
