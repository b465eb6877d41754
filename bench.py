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

At N = 1 the same line also carries the solve workloads, each a complete
record of its own under ``workloads`` (``--matvec-only`` leaves them out):
``torus_solve`` (200,000-panel torus, FMM p = 8 + near correction, mixed
FP32/FP64 refinement with the learned warm start, solves/s to a 1e-6
relative true residual, beside plain FP64 GMRES on the same GPU, the sigma
error against the converged density, and the same solve run to 1e-7, whose
sigma is within 1e-5), ``sphere_solve`` (5,120-panel icosphere, dense FP64)
and ``batch_solve`` (256 sphere dimers of 2k-40k panels); ``torus_solve`` is
summarised at the top level.  ``--workload`` runs one of them alone.
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


def fmm_workload(n):
    """Workload name of the FMM matvec at n points (the default run is N = 1,048,576)."""
    return WORKLOAD.replace("N1048576", f"N{n}")


# non-zeros per degree of each of the four fixed quarter-turn tables
# (electrodrive_gb300/csrc/rotation_tables.h)
ROT_NNZ = [1, 3, 7, 13, 21, 31, 43, 57, 71]


def m2l_flops_per_pair(p):
    """Algorithmic flops of one M2L pair at order p in the rotation form the
    kernel evaluates (k_m2l_rot): the 4 fixed quarter-turn matrices (2 flops per
    non-zero), 4 azimuthal phase rotations of the m >= 1 coefficient pairs
    (6 flops each), the axial translation (real m = 0 terms, complex m >= 1
    terms), the scaling by the radius ratio, the phase and 1/rho powers and the
    accumulation.  4,116 at p = 8."""
    axial = 2 * (p + 1) ** 2 + 4 * sum(j * j for j in range(1, p + 1))
    return (2 * 4 * sum(ROT_NNZ[:p + 1]) + 4 * (p * (p + 1) // 2) * 6 + axial + ((p + 1) ** 2 + p) + 12 * p
            + 4 * p + (p + 1) ** 2)


M2L_FLOPS_PER_PAIR = m2l_flops_per_pair(8)
# DRAM bytes one M2L launch moves per pair: the source index (4 B) and one read
# of the source's multipole row (the rows stay in L2 across a target's pairs);
# taken from an ncu capture of k_m2l_rot<float, 8> at N = 262,144 (44.54 MB read
# for 9,091,877 pairs)
M2L_DRAM_BYTES_PER_PAIR = 44.54e6 / 9_091_877
# DRAM bytes (read + write) per M2L pair of k_m2l_rot<float, p> on the
# 200,000-panel torus (FP32 inner operator), from ncu captures of that kernel
# on that mesh (median over the profile run's launches)
M2L_DRAM_BYTES_PER_PAIR_TORUS = {(8, 64): 14_461_269 / 2_315_072, (6, 64): 12_600_576 / 2_315_072}  # (p, leaf)
# the same for the 256-dimer batch (FP32 inner operator, autotuned order)
M2L_DRAM_BYTES_PER_PAIR_BATCH = {(6, 64): (244_023_808 + 55_725_312) / 39_011_439}  # (p, leaf)
# DRAM bytes of one k_dense_partial<double> launch at n = 5,120 (ncu capture)
DENSE_DRAM_BYTES_PER_MATVEC_5120 = 293_120
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
    ap.add_argument("--workload", choices=["fmm_matvec", "sphere_solve", "torus_solve", "batch_solve", "warm_start"],
                    default="fmm_matvec",
                    help="fmm_matvec: the headline operator benchmark; sphere_solve: 5,120-panel icosphere dense "
                         "FP64 solve; torus_solve: 200,000-panel torus, FMM + near correction, mixed-precision solve; "
                         "batch_solve: 256 sphere dimers of 2k-40k panels solved together")
    ap.add_argument("--batch", type=int, default=256, help="instances of the batch_solve workload")
    ap.add_argument("--ws-geometries", type=int, default=500,
                    help="warm_start: held-out geometries (10k-50k panels each) to evaluate")
    ap.add_argument("--torus-grid", default="500x200", help="torus_solve mesh grid n_u x n_v (2 n_u n_v panels)")
    ap.add_argument("--plain-full-cycle", action="store_true",
                    help="torus_solve: also time plain FP64 GMRES with the reference's full 256-step cycles")
    ap.add_argument("--matvec-only", action="store_true",
                    help="default run: report the FMM matvec alone (no solve-workload sub-records)")
    ap.add_argument("--profile-run", action="store_true",
                    help="solve workloads: set-up and the timed steps only (for ncu captures; no comparisons)")
    ap.add_argument("--inner-tol-floor", type=float, default=3e-7,
                    help="batch_solve: floor of the per-instance inner GMRES tolerance")
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


SPHERE_WORKLOAD = "sphere_solve_icosphere5120_q1_at_0_0_2_grounded_dense_fp64_gmres50_tol1e-8"
TORUS_WORKLOAD = ("torus_solve_R1_r0.35_grid500x200_200000panels_V1_q1_at_1.6_0.3_0.2_fmm_p8_leaf64_theta0.5_"
                  "near1.5_depth3_self_depth4_mixed_fp32_gmres40_in_fp64_refinement_rtol1e-6")


def _solve_case(name, torus_grid="500x200"):
    """Mesh, conductor spec and solver settings of the two solve workloads."""
    from electrodrive_gb300.core.bem_mesh import icosphere, torus_mesh

    if name == "sphere_solve":
        spec = dict(conductors=[dict(type="sphere", radius=1.0, center=[0.0, 0.0, 0.0], potential=0.0)],
                    charges=[dict(type="point", q=1.0, pos=[0.0, 0.0, 2.0])])
        return icosphere(4), spec, dict(depth_self=3, near=False, kind="dense")
    spec = dict(conductors=[dict(type="torus", major_radius=1.0, minor_radius=0.35, potential=1.0)],
                charges=[dict(type="point", q=1.0, pos=[1.6, 0.3, 0.2])])
    nu, nv = (int(x) for x in torus_grid.split("x"))
    return torus_mesh(1.0, 0.35, nu, nv), spec, dict(depth_self=4, near=True, kind="fmm")


def _time_cuda(fn, dev, stream, flush, warmup, steps):
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize(dev)
    ms = []
    for i in range(steps):
        flush.fill_(i & 0xFF)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms.append(e0.elapsed_time(e1))
    return ms


def _oracle_operator(mesh, spec, near: bool, depth_self: int, kind: str = None):
    """The oracle's FP64 restatement of the operator on all host cores: the
    FMM (p = 8, leaf 64, theta 0.5; ``kind="fmm"``, the default with the near
    correction) or the dense sum (the default without it), plus the near
    correction when ``near``; returns (A, b, diag, x0, set-up seconds)."""
    import numpy as np

    from electrodrive_gb300.core.bem import bc_vector, point_charges
    from oracle import oracle as O

    O.lib()
    C, A = mesh.centroids, mesh.areas
    PV = mesh.vertices[mesh.triangles]
    t0 = time.perf_counter()
    si = O.self_integrals(PV, C, 2, depth_self)
    q = [(qq, np.asarray(pos)) for qq, pos in point_charges(spec)]
    vf = sum(qq * O.K_E / np.maximum(np.linalg.norm(C - pos, axis=1), 1e-12) for qq, pos in q)
    b = bc_vector(spec, mesh) - vf
    diag = np.maximum(si, 1e-18)
    kind = kind or ("fmm" if near else "dense")
    if kind == "fmm":
        t = O.build_tree(C, 64, 32)
        lists = O.build_lists(t, 0.5)
        if near:
            pairs = O.near_pairs(C, A, 1.5)
            w = O.near_weights(C, A, PV, pairs, 2, 3)

        def op(v):
            out = O.fmm_matvec(t, lists, C, v, A, si / A, p=8)
            if near:
                np.add.at(out, pairs[:, 0], w * v[pairs[:, 1]])
            return out
    else:
        def op(v):
            return O.dense_matvec(C, v, A, si / A)
    return op, b, diag, b / diag, time.perf_counter() - t0


def _oracle_plain_solve(mesh, spec, near: bool, depth_self: int, rtol: float = 1e-6, restart: int = 256,
                        kind: str = None):
    """One plain FP64 solve by the oracle on all host cores, with the
    reference's solver semantics (Jacobi GMRES from b / I_self, full
    ``restart``-step cycles, true-residual test per cycle), the tolerance
    set so that the stop means ``rtol`` relative true residual.  Returns the
    solve seconds (set-up excluded), iterations, the final relative residual
    and one operator application's seconds."""
    import numpy as np

    from oracle import gmres_ref

    op, b, diag, x0, _ = _oracle_operator(mesh, spec, near, depth_self, kind)
    t1 = time.perf_counter()
    r0 = float(np.linalg.norm(b - op(x0)))
    t_mv = time.perf_counter() - t1
    bn = float(np.linalg.norm(b))
    t0 = time.perf_counter()
    x, info = gmres_ref.gmres_restart(op, b, 1.0 / diag, restart=restart, tol=rtol * bn / r0, maxiter=4000, x0=x0)
    dt = time.perf_counter() - t0
    rel = float(np.linalg.norm(b - op(x)) / bn)
    return dict(seconds=dt, iters=int(info["iters"]), rel_resid=rel, matvec_s=t_mv, n=mesh.n_panels)


def _solve_cpu_baseline(name, mesh, spec, opts):
    """The oracle's FP64 restatement of the reference's plain solve on all
    host cores.  Sphere: the whole dense solve of the same system.  Torus: a
    whole solve of a down-scaled torus (same R, r, charge and near
    correction; 100 x 40 grid, 8,000 panels) to a 1e-6 relative true
    residual with the reference's 256-step cycles, scaled to the full mesh by
    the ratio of one oracle operator application on each mesh."""
    from electrodrive_gb300.core.bem_mesh import torus_mesh
    from oracle import oracle as O

    O.lib()
    if name == "sphere_solve":
        import numpy as np

        from oracle import gmres_ref

        op, b, diag, x0, t_setup = _oracle_operator(mesh, spec, False, opts["depth_self"])
        t0 = time.perf_counter()
        x, info = gmres_ref.gmres_restart(op, b, 1.0 / diag, restart=50, tol=1e-8, maxiter=2000, x0=x0)
        dt = time.perf_counter() - t0 + t_setup
        return {"value": 1.0 / dt, "unit": "solves/s", "cores": O.num_threads(), "kind": "port",
                "sample": f"one whole FP64 solve (self integrals, dense operator, MGS GMRES(50)) of the same "
                          f"{mesh.n_panels}-panel system: {info['iters']} iterations, {dt:.2f} s"}
    small = torus_mesh(1.0, 0.35, 100, 40)
    sol = _oracle_plain_solve(small, spec, True, opts["depth_self"])
    op, b, _, x0, _ = _oracle_operator(mesh, spec, True, opts["depth_self"])
    t0 = time.perf_counter()
    op(x0)
    t_full = time.perf_counter() - t0
    est = sol["seconds"] * t_full / sol["matvec_s"]
    return {"value": 1.0 / est, "unit": "solves/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"timed oracle solve of a {small.n_panels}-panel torus (same R, r, charge, near correction) "
                      f"to {sol['rel_resid']:.2e} relative true residual with 256-step cycles: {sol['iters']} "
                      f"iterations, {sol['seconds']:.2f} s; scaled to {mesh.n_panels} panels by one operator "
                      f"application on each ({sol['matvec_s']:.3f} s vs {t_full:.2f} s)",
            "solve_seconds_sample": sol["seconds"], "solve_seconds_scaled": est}


def _reference_near_module(mesh, sysd, dev, stream, flush):
    """The reference's own CUDA near-field module (electrodrive/core/
    bem_near_cuda_kernel.cu, one thread per pair with atomic adds; built
    unmodified from the reference's sources by oracle/ref_near.py) timed
    beside this library's on-the-fly module (edfmm_near_quadrature_matvec:
    one thread per pair in CSR order, rows summed in shared memory in pair
    order, no atomics) on the same near set, order-2 rule, FP64: the
    reference's API call, this library's API call (which groups the pairs
    into rows by target once per pair tensor; the reference's API receives
    them in any order) and its kernel alone on prebuilt rows."""
    import numpy as np
    import torch

    from electrodrive_gb300 import _lib
    from electrodrive_gb300.core.bem_near import apply_near_quadrature_matvec_cuda
    from electrodrive_gb300.utils.config import K_E

    try:
        from oracle import ref_near

        mod = ref_near.load()
    except Exception as e:  # sources absent or the build failed
        return {"unavailable": f"{type(e).__name__}: {str(e)[:200]}"}
    near = sysd["ops"][torch.float64].near
    pairs, _ = near.export()
    n = sysd["n"]
    C = sysd["centroids"].to(dev).contiguous()
    A = sysd["areas"].contiguous()
    PV = torch.as_tensor(np.ascontiguousarray(mesh.vertices[mesh.triangles]), dtype=torch.float64, device=dev)
    sig = sysd["x0"].contiguous()
    vfar = torch.zeros(n, dtype=torch.float64, device=dev)
    ref_out = {}

    def ref_call():
        ref_out["v"] = mod.near_quadrature_matvec(vfar, sig, C, A, PV, pairs, float(K_E), 2)

    ours_out = {}

    def ours_call():
        ours_out["v"] = apply_near_quadrature_matvec_cuda(vfar, sig, centroids=C, areas=A, panel_vertices=PV,
                                                         near_pairs=pairs, quad_order=2)
    # this library's kernel alone on rows built once
    key = pairs[:, 0] * n + pairs[:, 1]
    pr = pairs[torch.argsort(key, stable=True)]
    counts = torch.bincount(pr[:, 0], minlength=n)
    row_off = torch.cat([counts.new_zeros(1), torch.cumsum(counts, 0)]).to(torch.int32)
    cols = pr[:, 1].to(torch.int32).contiguous()
    kout = torch.empty_like(vfar)
    L = _lib.load_library()
    pv9 = PV.reshape(-1, 9)

    def ours_kernel():
        _lib.check(L.edfmm_near_quadrature_matvec(_lib.ptr(vfar), _lib.ptr(sig), _lib.ptr(C), _lib.ptr(A),
                                                  _lib.ptr(pv9), _lib.ptr(row_off), _lib.ptr(cols), n, float(K_E), 2,
                                                  _lib.EDFMM_F64, _lib.ptr(kout), _lib.stream_handle(dev)),
                   "edfmm_near_quadrature_matvec")
    t_ref = statistics.median(_time_cuda(ref_call, dev, stream, flush, 3, 10))
    t_api = statistics.median(_time_cuda(ours_call, dev, stream, flush, 3, 10))
    t_k = statistics.median(_time_cuda(ours_kernel, dev, stream, flush, 3, 10))
    ref_v, our_v = ref_out["v"], ours_out["v"]
    i, j = pairs[:, 0], pairs[:, 1]
    r = torch.linalg.norm(C[i] - C[j], dim=1)
    scale = torch.zeros(n, dtype=torch.float64, device=dev).index_add_(0, i, K_E * A[j] * sig[j].abs() / r)
    err = float(((ref_v - our_v).abs() / scale.clamp_min(1e-300)).max())
    return {"pairs": int(pairs.shape[0]), "quad_order": 2, "dtype": "f64",
            "reference_api_ms": t_ref, "ours_api_ms": t_api, "ours_kernel_ms": t_k,
            "speedup_api": t_ref / t_api, "speedup_kernel_vs_reference_api": t_ref / t_k,
            "max_diff_over_term_scale": err, "kernel_equals_api": bool(torch.equal(kout, our_v))}


def run_solve_workload(args, rank, world, local, emit=True):
    """sphere_solve / torus_solve: one BEM solve per step (solves/s).
    Returns the JSON record (printed by rank 0 when ``emit``)."""
    import numpy as np

    name = args.workload
    workload = SPHERE_WORKLOAD if name == "sphere_solve" else TORUS_WORKLOAD
    mesh, spec, opts = _solve_case(name, args.torus_grid)
    if args.impl == "reference":
        if rank != 0:
            return None
        vals = [_solve_cpu_baseline(name, mesh, spec, opts)["value"] for _ in range(max(1, args.steps))]
        cpu = _solve_cpu_baseline(name, mesh, spec, opts)
        val = float(np.mean(vals))
        out = {"impl": "reference", "metric": METRIC, "value": val, "unit": "solves/s",
               "n_gpus": args.gpus, "steps": args.steps, "warmup": 0, "ms_per_step": 1e3 / val,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
               "data": "synthetic", "config": {"workload": workload, "n_panels": mesh.n_panels},
               "cpu_baseline": dict(cpu, value=val),
               "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        if emit:
            print(json.dumps(out), flush=True)
        return out

    import torch

    from electrodrive_gb300 import _lib
    from electrodrive_gb300.core.bem import assemble_system, bem_solve, solve_mixed
    from electrodrive_gb300.core.bem_solver import gmres_restart
    from electrodrive_gb300.utils.config import BEMConfig

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    t_setup = time.perf_counter()
    sysd = assemble_system(mesh, spec, kind=opts["kind"], dtypes=(torch.float64, torch.float32), near=opts["near"],
                           device=dev)
    torch.cuda.synchronize(dev)
    t_setup = time.perf_counter() - t_setup
    op64 = sysd["ops"][torch.float64]
    b, diag, x0, n = sysd["b"], sysd["diag"], sysd["x0"], sysd["n"]
    bn = float(torch.linalg.norm(b))
    result = {}

    if name == "sphere_solve":
        def step():
            result["x"], result["info"] = gmres_restart(op64, b, restart=50, tol=1e-8, maxiter=2000, precond="jacobi",
                                                        areas=sysd["areas"], A_diag=diag, x0=x0, use_graph=True)
    else:
        # the FP32 inner operator: the fastest expansion order within 3e-7 of the FP64 operator
        from electrodrive_gb300.core.bem import autotune_inner_operator

        op32, inner_trials = autotune_inner_operator(op64, sysd["centroids"], sysd["areas"], sysd["self_corr"],
                                                     near=sysd["ops"][torch.float32].near, device=dev,
                                                     leaf_sizes=(64, 128))
        sysd["ops"][torch.float32] = op32
        # the refinement's FP64 residuals and stopping test: the FP64 FMM
        # operator with M2L and near field in two-float arithmetic (every
        # residual and sigma error reported below is taken in IEEE FP64)
        plan64 = op64.base.plan
        plan64.set_arithmetic("two_float")
        net = geom = None
        weights = os.path.join(ROOT, "electrodrive_gb300", "data", "pcn_weights.npz")
        if os.path.exists(weights):
            from electrodrive_gb300.core.warm_start import PointCloudNet, panel_geometry, warm_start

            net = PointCloudNet.load(weights, device=dev)
            geom = panel_geometry(mesh, dev)

        def mixed_step(rtol):
            # the learned warm start (features, network, one FP32 operator application) is part of the step
            xs = warm_start(net, geom, b, op32) if net is not None else x0
            result["x0"] = xs
            result["x"], result["info"] = solve_mixed(op64, op32, b, A_diag=diag, x0=xs, rtol=rtol, inner_restart=40)

        def step():
            mixed_step(1e-6)

    warm = max(args.warmup, 3)
    for _ in range(warm):
        step()
    torch.cuda.synchronize(dev)
    l0 = _lib.launch_count()
    with ClockSampler(local) as clk:
        times = _time_cuda(step, dev, stream, flush, 0, args.steps)
    launches = _lib.launch_count() - l0
    ms = sum(times) / len(times)
    value = world * 1e3 / ms
    if args.profile_run:
        out = {"metric": METRIC, "value": value, "unit": "solves/s", "ms_per_step": ms, "profile_run": True,
               "config": {"workload": workload}}
        if name == "torus_solve":
            p32 = sysd["ops"][torch.float32].base.plan
            out["config"].update({"n_m2l_pairs_fp32": int(p32.info.n_m2l_pairs),
                                  "expansion_order_fp32": int(p32.info.expansion_order)})
        if rank == 0 and emit:
            print(json.dumps(out), flush=True)
        return out
    x, info = result["x"], result["info"]
    plan64 = getattr(getattr(op64, "base", None), "plan", None) if name != "sphere_solve" else None

    def native64(fn):
        """fn() evaluated with the FP64 operator in IEEE FP64 arithmetic"""
        if plan64 is None:
            return fn()
        plan64.set_arithmetic("native")
        try:
            return fn()
        finally:
            plan64.set_arithmetic("two_float")
    true_rel = native64(lambda: float(torch.linalg.norm(b - op64(x.to(torch.float64))) / bn))

    # operator application timing and roofline of the dominant kernel
    sig = x0.clone()
    mv = {}
    for dt, op in sysd["ops"].items():
        s_dt = sig.to(dt)
        key = str(dt).replace("torch.", "")
        if dt == torch.float64 and plan64 is not None:
            mv[key + "_two_float"] = statistics.median(_time_cuda(lambda: op(s_dt), dev, stream, flush, 3, 10))
            mv[key] = native64(lambda: statistics.median(_time_cuda(lambda: op(s_dt), dev, stream, flush, 3, 10)))
        else:
            mv[key] = statistics.median(_time_cuda(lambda: op(s_dt), dev, stream, flush, 3, 10))
    extra = {}
    if name == "sphere_solve":
        peak = _lib.measure_fp64_peak()
        flops = 20.0 * n * n
        achieved = flops / (mv["float64"] * 1e-3) / 1e12
        roof = {"kernel": "k_dense_partial<double> (dense FP64 operator)", "bound": "fp64", "achieved": achieved,
                "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                "traffic": DENSE_DRAM_BYTES_PER_MATVEC_5120,
                "traffic_note": "DRAM bytes of one k_dense_partial<double> launch at n = 5,120 (ncu)",
                "peak_source": "FP64 FMA probe measured in this run (edfmm_measure_fp64_peak)",
                "flops_per_matvec": flops}
        # Kelvin image and exterior potential
        from electrodrive_gb300.core.bem import BEMSolution

        xs = x.double().cpu().numpy()
        c = mesh.centroids
        d = np.linalg.norm(c - np.array([0.0, 0.0, 2.0]), axis=1)
        sig_k = -(4.0 - 1.0) / (4 * np.pi * d ** 3)
        g = torch.Generator().manual_seed(2)
        u = torch.randn(1000, 3, generator=g, dtype=torch.float64)
        u = u / u.norm(dim=1, keepdim=True)
        r = 1.2 + 1.8 * torch.rand(1000, 1, generator=g, dtype=torch.float64)
        pts = (u * r).numpy()
        sol = BEMSolution(centroids=sysd["centroids"].to(dev), areas=sysd["areas"], sigma=x.double(),
                          charges=[(1.0, (0, 0, 2.0))])
        v = sol.eval(torch.as_tensor(pts, device=dev)).cpu().numpy()
        from electrodrive_gb300.utils.config import K_E

        vk = K_E * (1.0 / np.linalg.norm(pts - [0, 0, 2.0], axis=1) - 0.5 / np.linalg.norm(pts - [0, 0, 0.5], axis=1))
        extra = {"sigma_rel_l2_vs_kelvin": float(np.linalg.norm(xs - sig_k) / np.linalg.norm(sig_k)),
                 "exterior_potential_rel_l2_vs_kelvin_1000pts": float(np.linalg.norm(v - vk) / np.linalg.norm(vk))}
        # the same solve by mixed refinement: FP32 dense GMRES corrections, FP64
        # dense residuals, stopped at the same absolute tolerance 1e-8 |r0|
        op32 = sysd["ops"][torch.float32]
        r0 = float(torch.linalg.norm(b - op64(x0)))
        mixed = {}

        def mixed_solve():
            mixed["x"], mixed["info"] = solve_mixed(op64, op32, b, A_diag=diag, x0=x0, rtol=1e-8 * r0 / bn,
                                                    inner_restart=50)
        t_mixed = statistics.median(_time_cuda(mixed_solve, dev, stream, flush, 3, 3))
        mi = mixed["info"]
        extra["mixed_fp32_fp64"] = {
            "solves_per_s": 1e3 / t_mixed, "ms": t_mixed, "outer_iters": mi["outer"], "inner_iters": mi["inner_iters"],
            "fp64_matvecs": mi["matvec64"],
            "true_rel_resid": float(torch.linalg.norm(b - op64(mixed["x"])) / bn),
            "sigma_rel_l2_vs_plain": float(torch.linalg.norm(mixed["x"].double() - x.double()) /
                                           torch.linalg.norm(x.double()))}
        cfg = BEMConfig(fp64=True, gmres_restart=50, gmres_tol=1e-8, gmres_maxiter=2000)
        e2e_call = lambda: bem_solve(spec, cfg, mesh=mesh, operator="dense", self_integral="quadrature")
        h2d = n * 8 * (3 + 1 + 9 + 3 + 1)
    else:
        r0 = native64(lambda: float(torch.linalg.norm(b - op64(x0))))

        def plain(tol, early_exit, arith="native"):
            """plain FP64 cold-start Jacobi GMRES (the operator in IEEE FP64,
            or with ``arith="two_float"`` its two-float form)"""
            out = {}

            def run():
                out["x"], out["info"] = gmres_restart(op64, b, restart=256, tol=tol * bn / r0, maxiter=4000,
                                                      precond="jacobi", areas=sysd["areas"], A_diag=diag, x0=x0,
                                                      use_graph=True, early_exit=early_exit)
            plan64.set_arithmetic(arith)
            try:
                t = statistics.median(_time_cuda(run, dev, stream, flush, 0, 1 if early_exit is None else 2))
            finally:
                plan64.set_arithmetic("two_float")
            xo, io = out["x"], out["info"]
            return t, xo, {"ms": t, "solves_per_s": 1e3 / t, "iters": io["iters"], "code": io["code"],
                           "true_rel_resid": native64(lambda: float(torch.linalg.norm(b - op64(xo)) / bn)),
                           "restart": 256, "early_exit_every": early_exit, "fp64_arithmetic": arith}

        # the converged density every sigma error below is measured against:
        # plain FP64 GMRES to a 1e-11 relative true residual
        _, x_ref, ref_rec = plain(1e-11, 8)

        def sig_err(v):
            return float(torch.linalg.norm(v.to(torch.float64) - x_ref) / torch.linalg.norm(x_ref))

        # plain FP64 cold-start GMRES with an early exit (cycles end once the
        # preconditioned residual meets the tolerance, checked every 8 steps;
        # the reference's solver always completes its 256-step cycle)
        t_plain_ee, x_pee, plain_ee = plain(1e-6, 8)
        plain_ee["sigma_rel_l2_vs_converged"] = sig_err(x_pee)
        t_plain_ee7, x_pee7, plain_ee7 = plain(1e-7, 8)
        plain_ee7["sigma_rel_l2_vs_converged"] = sig_err(x_pee7)
        # the same plain solve on the two-float form of the FP64 operator
        t_plain_tf, x_ptf, plain_tf = plain(1e-6, 8, "two_float")
        plain_tf["sigma_rel_l2_vs_converged"] = sig_err(x_ptf)
        plain_full = None
        if args.plain_full_cycle:
            t_pf, x_pf, plain_full = plain(1e-6, None)
            plain_full["sigma_rel_l2_vs_converged"] = sig_err(x_pf)
        # the mixed + learned solve run to 1e-7: its sigma is within 1e-5 of
        # the converged density (a 1e-6 residual leaves about 1e-4 on this
        # system, for plain FP64 GMRES as well)
        t7 = statistics.median(_time_cuda(lambda: mixed_step(1e-7), dev, stream, flush, 1, 3))
        x7, i7 = result["x"], result["info"]
        accurate = {"rtol": 1e-7, "ms": t7, "solves_per_s": world * 1e3 / t7, "outer_iters": i7["outer"],
                    "inner_iters": i7["inner_iters"], "fp64_matvecs": i7["matvec64"],
                    "true_rel_resid": native64(lambda: float(torch.linalg.norm(b - op64(x7)) / bn)),
                    "sigma_rel_l2_vs_converged": sig_err(x7),
                    "speedup_vs_plain_fp64_early_exit_rtol1e-7": t_plain_ee7 / t7}
        mixed_step(1e-6)  # restore the headline run's result
        p64 = op64.base.plan
        p32 = op32.base.plan
        fp32_peak = _lib.measure_fp32_peak()
        p32.set_charges(sig.float() * sysd["areas"].float())
        m2l_ms = statistics.median(_time_cuda(lambda: p32.stage("m2l", 0), dev, stream, flush, 2, 5))
        order32 = int(p32.info.expansion_order)
        achieved = p32.info.n_m2l_pairs * m2l_flops_per_pair(order32) / (m2l_ms * 1e-3) / 1e12
        per_pair = M2L_DRAM_BYTES_PER_PAIR_TORUS.get((order32, int(p32.info.leaf_size)))
        roof = {"kernel": f"k_m2l_rot<float, {order32}> (M2L of the FP32 inner operator)", "bound": "fp32",
                "achieved": achieved,
                "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak if fp32_peak else None,
                "traffic": per_pair * p32.info.n_m2l_pairs if per_pair else None,
                "traffic_note": "DRAM bytes per pair of this kernel from an ncu capture on this torus (ncu summary "
                                "under profiles/), times this run's pairs",
                "peak_source": "FP32 FMA probe measured in this run (edfmm_measure_fp32_peak)",
                "flops_per_pair": m2l_flops_per_pair(order32)}
        extra = {"plain_fp64_gmres_early_exit": plain_ee,
                 "mixed_speedup_vs_plain_fp64_early_exit": t_plain_ee / ms,
                 "plain_fp64_gmres_early_exit_two_float_operator": plain_tf,
                 "mixed_speedup_vs_plain_two_float_early_exit": t_plain_tf / ms,
                 "fp64_operator_arithmetic": "two_float (M2L and near field on the FP32 pipe, ~48 bits)",
                 "plain_fp64_gmres_early_exit_rtol1e-7": plain_ee7,
                 "plain_fp64_gmres_full_cycles": plain_full,
                 "mixed_speedup_vs_plain_fp64_full_cycles": (plain_full["ms"] / ms) if plain_full else None,
                 "converged_reference": ref_rec,
                 "sigma_rel_l2_vs_converged": sig_err(x),
                 "accurate_rtol1e-7": accurate,
                 "outer_iters": info["outer"], "inner_iters": info["inner_iters"], "fp64_matvecs": info["matvec64"],
                 "n_nodes_fp32": p32.info.n_nodes, "n_m2l_pairs_fp32": p32.info.n_m2l_pairs,
                 "n_p2p_pairs_fp32": p32.info.n_p2p_pairs, "p2p_interactions_fp32": p32.info.p2p_interactions,
                 "n_m2l_pairs_fp64": p64.info.n_m2l_pairs, "m2l_fp32_ms": m2l_ms,
                 "inner_operator": {"expansion_order": order32, "leaf_size": int(p32.info.leaf_size),
                                    "trials": inner_trials}}
        # the same mixed solver from the cold start (x0 = b / I_self)
        cold = {}

        def cold_solve():
            cold["x"], cold["info"] = solve_mixed(op64, op32, b, A_diag=diag, x0=x0, rtol=1e-6, inner_restart=40)
        t_cold = statistics.median(_time_cuda(cold_solve, dev, stream, flush, 1, 2))
        extra["mixed_cold_start"] = {"ms": t_cold, "solves_per_s": 1e3 / t_cold, "outer_iters": cold["info"]["outer"],
                                     "inner_iters": cold["info"]["inner_iters"]}
        extra["warm_start"] = "learned (electrodrive_gb300/data/pcn_weights.npz)" if net is not None else "none"
        extra["reference_near_module"] = _reference_near_module(mesh, sysd, dev, stream, flush)
        if net is not None:
            from electrodrive_gb300.core.warm_start import relative_error

            extra["start_rel_error"] = {"learned": relative_error(result["x0"], x_ref, sysd["areas"]),
                                        "cold": relative_error(x0, x_ref, sysd["areas"])}
        cfg = BEMConfig(use_near_quadrature_matvec=True)
        e2e_call = lambda: bem_solve(spec, cfg, mesh=mesh, operator="fmm", self_integral="quadrature", mixed=True,
                                     mixed_rtol=1e-6, inner_restart=40, inner_expansion_order=order32,
                                     fp64_arithmetic="two_float", warm_start=net)
        h2d = n * 8 * (3 + 1 + 9 + 3 + 1) * 2

    # end to end through the public API: host mesh -> solve -> host sigma
    e2e_ms = []
    for i in range(1 + args.steps):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        res = e2e_call()
        sig_host = res["surface_charge_density"]  # host array
        if i:
            e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_val = world * 1e3 / (sum(e2e_ms) / len(e2e_ms))

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = _solve_cpu_baseline(name, mesh, spec, opts)
        except Exception as e:
            cpu = {"value": None, "error": str(e)[:200]}
    out = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
           "warmup": warm, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64" if name == "sphere_solve" else "f32+f64", "data": "synthetic",
           "config": {"workload": workload, "n_panels": n, "near_pairs": sysd["near_pairs"],
                      "l2": "flushed by a 256 MiB write between steps", "parallelism": f"replicas x{world}",
                      "setup_s": t_setup},
           "solve": {"iters": info.get("iters", info.get("inner_iters")), "code": info["code"],
                     "true_rel_resid": true_rel, **extra},
           "matvec_ms": mv,
           "e2e": {"value": e2e_val, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 8 * n,
                   "ms_per_step": sum(e2e_ms) / len(e2e_ms),
                   "includes": "set-up from the host mesh (self integrals, near pairs and weights, trees and "
                               "lists), the solve and the sigma read-back"},
           "gpu_launches": int(launches), "clocks": clk.summary(), "roofline": roof, "cpu_baseline": cpu}
    if rank == 0 and emit:
        print(json.dumps(out), flush=True)
    return out


def _batch_cpu_baseline(cases, n_total: int, budget_s: float = 12.0):
    """The oracle's plain solve (FP64 FMM p = 8 on all host cores, the
    reference's 256-step Jacobi GMRES cycles, 1e-6 relative true residual)
    timed on the smallest instances until ``budget_s`` of solve time, then
    scaled to every instance's panels (the FMM's cost grows in proportion to
    the panels)."""
    from oracle import oracle as O

    O.lib()
    done, secs, pans, its = 0, 0.0, 0, []
    for mesh, spec in sorted(cases, key=lambda c: c[0].n_panels):
        sol = _oracle_plain_solve(mesh, spec, False, 3, kind="fmm")
        done += 1
        secs += sol["seconds"]
        pans += mesh.n_panels
        its.append(sol["iters"])
        if secs >= budget_s:
            break
    est = secs * n_total / pans
    return {"value": len(cases) / est, "unit": "solves/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"timed oracle solves of the {done} smallest instances ({pans} panels, {secs:.2f} s, "
                      f"{sum(its) / len(its):.0f} iterations each on average) scaled by panels to all "
                      f"{len(cases)} instances ({n_total} panels)",
            "solve_seconds_sample": secs, "solve_seconds_scaled": est}


def run_batch_workload(args, rank, world, local, emit=True):
    """batch_solve: K sphere dimers (seeds 10 + i, 2k-40k panels each, grounded,
    one point charge each) solved together to a 1e-6 relative true residual
    per instance; one step = one batched solve of all K (solves/s = K / t).
    Returns the JSON record (printed by rank 0 when ``emit``)."""
    import numpy as np

    from electrodrive_gb300.core.batch import dimer_case

    K = args.batch
    cases = [dimer_case(10 + i) for i in range(K)]
    n_total = sum(m.n_panels for m, _ in cases)
    workload = (f"batch_solve_{K}_sphere_dimers_seeds10+i_2k-40k_panels_{n_total}_total_fmm_p8_"
                "mixed_fp32_inner_autotuned_fp64_refinement_rtol1e-6_per_instance")
    if args.impl == "reference":
        if rank != 0:
            return None
        cpu = _batch_cpu_baseline(cases, n_total)
        val = cpu["value"]
        out = {"impl": "reference", "metric": METRIC, "value": val, "unit": "solves/s",
               "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": 1e3 * K / val,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
               "data": "synthetic", "config": {"workload": workload, "n_panels": n_total},
               "cpu_baseline": cpu,
               "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        if emit:
            print(json.dumps(out), flush=True)
        return out

    import torch

    from electrodrive_gb300 import _lib
    from electrodrive_gb300.core.batch import BatchSystem, autotune_inner, plain_fp64_solve

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    t0 = time.perf_counter()
    system = BatchSystem(cases, device=dev)
    torch.cuda.synchronize(dev)
    t_setup = time.perf_counter() - t0
    tune = autotune_inner(system, inner_tol=args.inner_tol_floor)
    # the refinement's FP64 residuals and stopping test in two-float arithmetic
    system.op64.plan.set_arithmetic("two_float")
    result = {}
    net = None
    weights = os.path.join(ROOT, "electrodrive_gb300", "data", "pcn_weights.npz")
    if os.path.exists(weights):
        from electrodrive_gb300.core.warm_start import PointCloudNet

        net = PointCloudNet.load(weights, device=dev)

    def step():
        # zero start: the first residual is b itself (no operator application)
        result["x"], result["info"] = system.solve(inner_tol_floor=args.inner_tol_floor)

    warm = max(args.warmup, 3)
    for _ in range(warm):
        step()
    torch.cuda.synchronize(dev)
    l0 = _lib.launch_count()
    with ClockSampler(local) as clk:
        times = _time_cuda(step, dev, stream, flush, 0, args.steps)
    launches = _lib.launch_count() - l0
    ms = sum(times) / len(times)
    value = world * K * 1e3 / ms
    if args.profile_run:
        out = {"metric": METRIC, "value": value, "unit": "solves/s", "ms_per_step": ms, "profile_run": True,
               "config": {"workload": workload, "inner_operator": {k: tune[k] for k in ("leaf_size",
                                                                                        "expansion_order")},
                          "n_m2l_pairs_fp32": int(system.op32.plan.info.n_m2l_pairs)}}
        if rank == 0 and emit:
            print(json.dumps(out), flush=True)
        return out
    info = result["info"]
    system.op64.plan.set_arithmetic("native")  # residuals reported in IEEE FP64
    per = system.residuals(result["x"]).cpu().numpy()
    system.op64.plan.set_arithmetic("two_float")
    learned = {}

    def learned_step():
        # per-instance learned warm start (network + one FP32 application) inside the timing
        learned["x"], learned["info"] = system.solve(x0=system.learned_start(net), inner_tol_floor=args.inner_tol_floor)
    t_learned = _time_cuda(learned_step, dev, stream, flush, 1, 1)[0] if net is not None else None
    mv = {"float64_two_float": statistics.median(_time_cuda(lambda: system.op64(system.x0_cold), dev, stream, flush,
                                                            1, 3))}
    system.op64.plan.set_arithmetic("native")
    mv.update({"float64": statistics.median(_time_cuda(lambda: system.op64(system.x0_cold), dev, stream, flush, 1, 3)),
          "float32": statistics.median(_time_cuda(lambda: system.op32(system.x0_cold.float()), dev, stream, flush,
                                                  1, 3))})
    system.op64.plan.set_arithmetic("two_float")
    p32 = system.op32.plan
    p32.set_charges(system.x0_cold.float() * system.areas.float())
    m2l_ms = statistics.median(_time_cuda(lambda: p32.stage("m2l", 0), dev, stream, flush, 1, 3))
    fp32_peak = _lib.measure_fp32_peak()
    from electrodrive_gb300.core.batch import plain_fp64_solve as _plain

    sub = min(8, K)
    plain = [_plain(*cases[i], device=dev) for i in range(sub)]
    plain_ee = [_plain(*cases[i], device=dev, early_exit=8) for i in range(sub)]
    n_sub = sum(p["n"] for p in plain)
    t_plain_all = sum(p["seconds"] for p in plain) * n_total / n_sub
    t_plain_ee_all = sum(p["seconds"] for p in plain_ee) * n_total / n_sub
    # end to end: host meshes -> batched set-up -> solve -> sigma on the host
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    sys2 = BatchSystem(cases, device=dev, inner_leaf_size=tune["leaf_size"],
                       inner_expansion_order=tune["expansion_order"])
    sys2.op64.plan.set_arithmetic("two_float")
    x2, _ = sys2.solve(inner_tol_floor=args.inner_tol_floor)
    x2.cpu()
    e2e_ms = 1e3 * (time.perf_counter() - t0)
    e2e_h2d = sys2.h2d_bytes
    del sys2
    # the same set-up once more, synchronised at each phase end, for its breakdown
    setup_phases = {}
    sys3 = BatchSystem(cases, device=dev, inner_leaf_size=tune["leaf_size"],
                       inner_expansion_order=tune["expansion_order"], timings=setup_phases)
    del sys3
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = _batch_cpu_baseline(cases, n_total)
        except Exception as e:
            cpu = {"value": None, "error": str(e)[:200]}
    if True:
        order = tune["expansion_order"]
        flops_pair = m2l_flops_per_pair(order) if 1 <= order <= 8 else None
        ach = p32.info.n_m2l_pairs * flops_pair / (m2l_ms * 1e-3) / 1e12 if flops_pair else None
        per_pair = M2L_DRAM_BYTES_PER_PAIR_BATCH.get((order, int(tune["leaf_size"])))
        out = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
               "warmup": warm, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f32+f64", "data": "synthetic",
               "config": {"workload": workload, "instances": K, "n_panels": n_total, "setup_s": t_setup,
                          "l2": "flushed by a 256 MiB write between steps", "parallelism": f"replicas x{world}",
                          "inner_operator": {k: tune[k] for k in ("leaf_size", "expansion_order", "ms")},
                          "inner_solver": "batched GMRES (one Krylov space per instance), restart 100",
                          "inner_tol_floor": args.inner_tol_floor,
                          "n_m2l_pairs_fp32": int(p32.info.n_m2l_pairs), "m2l_fp32_ms": m2l_ms,
                          "start": "zero (first residual = b)"},
               "solve": {"code": info["code"], "outer_iters": info["outer"], "inner_iters": info["inner_iters"],
                         "instance_inner_iters": ({"mean": float(np.mean(info["instance_inner_iters"])),
                                                   "max": int(max(info["instance_inner_iters"]))}
                                                  if info.get("instance_inner_iters") else None),
                         "fp64_matvecs": info["matvec64"], "max_instance_rel_resid": float(per.max()),
                         "instances_converged": int((per <= 1e-6 * (1 + 1e-9)).sum()),
                         "plain_fp64_per_instance": {"instances_timed": sub, "panels_timed": n_sub,
                                                     "mean_iters": float(np.mean([p["iters"] for p in plain])),
                                                     "seconds_timed": sum(p["seconds"] for p in plain),
                                                     "seconds_all_extrapolated_by_panels": t_plain_all,
                                                     "solves_per_s": K / t_plain_all},
                         "speedup_vs_plain_fp64": t_plain_all / (ms * 1e-3),
                         "plain_fp64_early_exit_per_instance": {
                             "instances_timed": sub, "early_exit_every": 8,
                             "mean_iters": float(np.mean([p["iters"] for p in plain_ee])),
                             "max_rel_resid": float(max(p["rel_resid"] for p in plain_ee)),
                             "seconds_timed": sum(p["seconds"] for p in plain_ee),
                             "seconds_all_extrapolated_by_panels": t_plain_ee_all,
                             "solves_per_s": K / t_plain_ee_all},
                         "speedup_vs_plain_fp64_early_exit": t_plain_ee_all / (ms * 1e-3),
                         "learned_start": None if t_learned is None else {
                             "ms": t_learned, "solves_per_s": world * K * 1e3 / t_learned,
                             "outer_iters": learned["info"]["outer"], "inner_iters": learned["info"]["inner_iters"],
                             "fp64_matvecs": learned["info"]["matvec64"],
                             "instance_inner_iters_mean": float(np.mean(learned["info"]["instance_inner_iters"]))}},
               "autotune_trials": tune["trials"], "matvec_ms": mv,
               "e2e": {"value": world * K * 1e3 / e2e_ms, "unit": "solves/s",
                       "h2d_bytes_per_step": e2e_h2d, "d2h_bytes_per_step": int(8 * n_total),
                       "ms_per_step": e2e_ms, "includes": "batched set-up from the host meshes (trees, lists, "
                                                           "self integrals, rhs), the solve and the read-back",
                       "setup_phases_ms": setup_phases},
               "gpu_launches": int(launches), "clocks": clk.summary(),
               "roofline": {"kernel": f"k_m2l_rot<float, {order}> (M2L of the FP32 inner operator)", "bound": "fp32",
                            "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s",
                            "frac": ach / fp32_peak if ach else None,
                            "traffic": per_pair * p32.info.n_m2l_pairs if per_pair else None,
                            "traffic_note": "DRAM bytes per pair of this kernel from an ncu capture on this batch "
                                            "(ncu summary under profiles/), times this run's pairs",
                            "peak_source": "FP32 FMA probe measured in this run"},
               "cpu_baseline": cpu}
        if rank == 0 and emit:
            print(json.dumps(out), flush=True)
        return out


WS_FLOPS_PER_PANEL = 2 * (16 * 128 + 3 * 128 * 128 + 128)  # network forward, per panel (dense layers)


def _ws_cpu_baseline(sample_cases, mean_panels: float, budget_s: float = 10.0):
    """The oracle's plain cold-start solve (FP64 FMM p = 8, all host cores,
    the reference's 256-step cycles, 1e-6) on the smallest of the sampled
    geometries until ``budget_s``, as solves/s of a geometry of
    ``mean_panels`` panels (the FMM's cost grows in proportion)."""
    cpu = _batch_cpu_baseline(sample_cases, int(sum(m.n_panels for m, _ in sample_cases)), budget_s=budget_s)
    secs, est = cpu["solve_seconds_sample"], cpu["solve_seconds_scaled"]
    per_panel = est / sum(m.n_panels for m, _ in sample_cases)
    return dict(cpu, value=1.0 / (per_panel * mean_panels),
                sample=cpu["sample"] + f"; expressed per geometry of {mean_panels:.0f} panels (the held-out mean)")


def run_warm_start_workload(args, rank, world, local, emit=True):
    """warm_start: the learned warm start on held-out geometries (random
    spheres, ellipsoids, tori and dimers of 10k-50k panels, seeds 7000+,
    disjoint from the training and test seeds).  Per geometry: its converged
    density (the FP64 FMM operator in two-float arithmetic, refined to
    1e-10), then from the cold start (b / I_self), the base guess (b / A(1))
    and the learned start, the Jacobi GMRES iterations and time to a 1e-6
    true residual with the FP64 operator and the mixed FP32/FP64 solve to
    1e-6 (start included).  value = held-out solves/s of the learned mixed
    solve (mean time per geometry)."""
    import numpy as np

    from electrodrive_gb300.core.warm_start import KINDS, random_case

    K = max(1, int(args.ws_geometries))
    workload = (f"warm_start_heldout_{K}_geometries_sphere_ellipsoid_torus_dimer_10k-50k_panels_seeds7000+_"
                "fmm_p8_mixed_fp32_fp64_rtol1e-6")

    def cases():
        rng = np.random.default_rng(7000)
        for i in range(K):
            yield random_case(rng, KINDS[i % len(KINDS)], int(rng.integers(10000, 50001)))

    if args.impl == "reference":
        if rank != 0:
            return None
        allc = list(cases())
        cpu = _ws_cpu_baseline(allc[:8], float(np.mean([m.n_panels for m, _ in allc])))
        out = {"impl": "reference", "metric": METRIC, "value": cpu["value"], "unit": "solves/s",
               "n_gpus": args.gpus, "steps": 1, "warmup": 0, "ms_per_step": 1e3 / cpu["value"],
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
               "data": "synthetic", "config": {"workload": workload}, "cpu_baseline": cpu,
               "e2e": {"value": cpu["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        if emit:
            print(json.dumps(out), flush=True)
        return out

    import torch

    from electrodrive_gb300 import _lib
    from electrodrive_gb300.core.warm_start import PointCloudNet, compare_starts, make_sample
    from electrodrive_gb300.train_warm_start import summarize

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    net = PointCloudNet.load(os.path.join(ROOT, "electrodrive_gb300", "data", "pcn_weights.npz"), device=dev)
    evals, panels, kinds, largest = [], [], [], None
    l0 = _lib.launch_count()
    t_all = time.perf_counter()
    with ClockSampler(local) as clk:
        for i, (mesh, spec) in enumerate(cases()):
            s = make_sample(mesh, spec, device=dev, operator="fmm")
            evals.append(compare_starts(net, s))
            panels.append(mesh.n_panels)
            kinds.append(KINDS[i % len(KINDS)])
            if largest is None or mesh.n_panels > largest[0]:
                largest = (mesh.n_panels, s["centroids"], s["normals"], s["areas"], s["b"])
            del s
    t_all = time.perf_counter() - t_all
    launches = _lib.launch_count() - l0
    # end to end through the public API on the first geometries: host mesh ->
    # bem_solve(mixed, learned start) -> host sigma, set-up included
    from electrodrive_gb300.core.bem import bem_solve
    from electrodrive_gb300.utils.config import BEMConfig

    e2e_n = min(K, 16)
    e2e_s, e2e_h2d, e2e_d2h = [], [], []
    for i, (mesh, spec) in enumerate(cases()):
        if i >= e2e_n:
            break
        call = lambda: bem_solve(spec, BEMConfig(), mesh=mesh, operator="fmm", self_integral="quadrature",
                                 mixed=True, mixed_rtol=1e-6, warm_start=net)
        if i == 0:
            call()  # warm (graph capture, workspaces)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        res = call()
        sig_host = res["surface_charge_density"]
        e2e_s.append(time.perf_counter() - t0)
        e2e_h2d.append(8 * (3 + 1 + 9 + 3 + 1) * mesh.n_panels)
        e2e_d2h.append(int(np.asarray(sig_host).nbytes))
    summ = summarize(evals)
    learned_s = [e["learned"]["mixed"]["seconds"] for e in evals]
    cold_s = [e["cold"]["mixed"]["seconds"] for e in evals]
    base_s = [e["base"]["mixed"]["seconds"] for e in evals]
    ms = 1e3 * float(np.mean(learned_s))
    value = world * 1e3 / ms
    # roofline of the network's forward pass (BF16 tensor-core GEMMs) on the largest geometry
    n_l, c_l, nr_l, a_l, b_l = largest
    f = net.features(c_l, nr_l, a_l, b_l)
    stream = torch.cuda.current_stream(dev)
    net.forward(f)
    torch.cuda.synchronize(dev)
    tt = []
    for _ in range(10):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        net.forward(f)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        tt.append(e0.elapsed_time(e1))
    t_fwd = statistics.median(tt)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except Exception:
        pass
    ach = WS_FLOPS_PER_PANEL * n_l / (t_fwd * 1e-3) / 1e12
    peak = peaks.get("bf16_tflops") or 1900.0
    roof = {"kernel": "k_pcn_linear (network forward, BF16 mma.sync, largest held-out geometry)", "bound": "tensor",
            "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak, "traffic": None,
            "peak_source": "MEASURED_PEAKS.json bf16_tflops" if peaks.get("bf16_tflops") else "fallback 1.9 PFLOP/s",
            "panels": n_l, "forward_ms": t_fwd}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = _ws_cpu_baseline([c for c, _ in zip(cases(), range(8))], float(np.mean(panels)))
        except Exception as e:
            cpu = {"value": None, "error": str(e)[:200]}
    per_kind = {}
    for k in KINDS:
        idx = [j for j, kk in enumerate(kinds) if kk == k]
        if idx:
            per_kind[k] = {"geometries": len(idx),
                           "mixed_ms": {st: 1e3 * float(np.mean([evals[j][st]["mixed"]["seconds"] for j in idx]))
                                        for st in ("cold", "base", "learned")},
                           "mixed_outer": {st: float(np.mean([evals[j][st]["mixed"]["outer"] for j in idx]))
                                           for st in ("cold", "base", "learned")},
                           "gmres_iters": {st: float(np.mean([evals[j][st]["iters"] for j in idx]))
                                           for st in ("cold", "base", "learned")}}
    out = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": K, "warmup": 1,
           "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
           "data": "synthetic",
           "config": {"workload": workload, "geometries": K, "panels_mean": float(np.mean(panels)),
                      "panels_min": int(min(panels)), "panels_max": int(max(panels)),
                      "weights": "electrodrive_gb300/data/pcn_weights.npz", "wall_s": t_all},
           "held_out": summ,
           "mixed_speedup_learned_vs_cold": float(np.mean(cold_s) / np.mean(learned_s)),
           "mixed_speedup_learned_vs_base": float(np.mean(base_s) / np.mean(learned_s)),
           "fraction_learned_faster_than_cold": float(np.mean([a < b for a, b in zip(learned_s, cold_s)])),
           "per_kind": per_kind,
           "e2e": {"value": world / float(np.mean(e2e_s)), "unit": "solves/s",
                   "h2d_bytes_per_step": int(np.mean(e2e_h2d)), "d2h_bytes_per_step": int(np.mean(e2e_d2h)),
                   "ms_per_step": 1e3 * float(np.mean(e2e_s)), "geometries": e2e_n,
                   "includes": "bem_solve(mixed=True, warm_start=net) from the host mesh: self integrals, trees "
                               "and lists, the learned start, the solve and the sigma read-back"},
           "gpu_launches": int(launches), "clocks": clk.summary(), "roofline": roof, "cpu_baseline": cpu}
    if rank == 0 and emit:
        print(json.dumps(out), flush=True)
    return out


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload == "batch_solve":
        run_batch_workload(args, rank, world, local)
        return
    if args.workload == "warm_start":
        run_warm_start_workload(args, rank, world, local)
        return
    if args.workload != "fmm_matvec":
        run_solve_workload(args, rank, world, local)
        return
    out = None
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
            "config": {"workload": fmm_workload(n), "n_points": n, "expansion_order": 8, "leaf_size": 64,
                       "mac_theta": 0.5, "n_nodes": info.n_nodes, "n_p2p_pairs": info.n_p2p_pairs,
                       "n_m2l_pairs": info.n_m2l_pairs, "p2p_interactions": info.p2p_interactions,
                       "l2": "flushed by a 256 MiB write between steps", "parallelism": f"replicas x{world}",
                       "rel_l2_vs_fp64_direct_256_targets": err},
            "e2e": {"value": e2e_val, "unit": "Mpts/s", "h2d_bytes_per_step": 4 * n, "d2h_bytes_per_step": 4 * n,
                    "ms_per_step": e2e_ms},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "roofline": {"kernel": "k_m2l_rot<float, 8> (rotation-based M2L stage)", "bound": "fp32",
                         "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp32_peak if fp32_peak else None,
                         "traffic": M2L_DRAM_BYTES_PER_PAIR * info.n_m2l_pairs,
                         "traffic_note": "DRAM bytes of the M2L stage, scaled from an ncu capture at N=262,144",
                         "peak_source": "FP32 FMA probe measured in this run (edfmm_measure_fp32_peak)",
                         "flops_per_pair": M2L_FLOPS_PER_PAIR},
            "stages_ms": stage_ms,
            "p2p_tflops": p2p_tflops,
            "cpu_baseline": cpu,
        }
    if world == 1 and not args.matvec_only:
        # the solve workloads, each a full record of its own, timed after the
        # matvec on the same GPU (N = 1 only: the scaling runs time the matvec)
        del fmm, plan, sig_d, areas_d, out_d, flush
        torch.cuda.empty_cache()
        out["workloads"] = {}
        for sub, steps in (("torus_solve", min(args.steps, 5)), ("sphere_solve", min(args.steps, 5)),
                           ("batch_solve", min(args.steps, 3)), ("warm_start", None)):
            sargs = argparse.Namespace(**vars(args))
            sargs.workload = sub
            if steps is not None:
                sargs.steps = steps
            else:
                sargs.ws_geometries = min(args.ws_geometries, 48)  # held-out sample in the default run
            t0 = time.perf_counter()
            try:
                fn = {"batch_solve": run_batch_workload, "warm_start": run_warm_start_workload}.get(
                    sub, run_solve_workload)
                rec = fn(sargs, rank, world, local, emit=False)
                rec["wall_s"] = time.perf_counter() - t0
            except Exception as e:  # a failing sub-record must not lose the headline line
                rec = {"error": f"{type(e).__name__}: {str(e)[:300]}", "wall_s": time.perf_counter() - t0}
            out["workloads"][sub] = rec
            torch.cuda.empty_cache()
        tor = out["workloads"].get("torus_solve", {})
        if "solve" in tor:
            ts = tor["solve"]
            out["torus_solve"] = {
                "solves_per_s_rtol1e-6": tor["value"], "ms": tor["ms_per_step"],
                "true_rel_resid": ts["true_rel_resid"], "sigma_rel_l2_vs_converged": ts["sigma_rel_l2_vs_converged"],
                "plain_fp64_early_exit_solves_per_s": ts["plain_fp64_gmres_early_exit"]["solves_per_s"],
                "speedup_vs_plain_fp64_early_exit": ts["mixed_speedup_vs_plain_fp64_early_exit"],
                "accurate_rtol1e-7": ts["accurate_rtol1e-7"], "roofline": tor["roofline"], "e2e": tor["e2e"],
                "cpu_baseline": tor["cpu_baseline"]}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
