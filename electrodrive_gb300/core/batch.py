"""Batched uneven BEM solves (no counterpart in the reference, which solves
one geometry per call).

Many independent conductor geometries, each with its own right-hand side,
are solved together:

* one batched FMM plan per precision (libedfmm ``edfmm_plan_create_batch``):
  every instance keeps its own octree and interaction lists, and each FMM
  stage is one launch over the whole batch, so the operator is block
  diagonal;
* one FP64 iterative refinement around FP32 GMRES on the concatenated
  system, stopped when every instance's own relative true residual meets
  the tolerance (``solve_mixed(segments=...)``);
* an autotuner that picks the inner (FP32) operator's leaf size and
  expansion order by timing, subject to an accuracy bound against the FP64
  operator.

``dimer_case`` builds the sphere-dimer instances of the batched workload:
radii U[0.5, 1.5], surface gap U[0.1, 1.0], random orientation, panel count
split between the spheres by area, and a grounded pair with a point charge
U[-1, 1] at distance U[0.3, 2] outside the nearer sphere.
"""
from __future__ import annotations

import math
import statistics
import time
from typing import Any, Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch
from torch import Tensor

from .. import _lib
from .bem import point_charges, segment_norms, solve_mixed
from .bem_mesh import TriMesh, _finish, _mesh_sphere
from .bem_near import point_charge_potential, self_integrals
from .operators import FmmOperator


def _uv_sphere_shape(n_panels: int) -> Tuple[int, int]:
    """(n_theta, n_phi) of the tensor-grid sphere with about n_panels panels (n_phi = 2 n_theta)."""
    nt = max(4, int(round(1.0 + math.sqrt(1.0 + n_panels / 4.0))))
    return nt, 2 * nt


def _uv_sphere(center, radius: float, n_panels: int, cid: int) -> TriMesh:
    """The reference's tensor-grid sphere with about n_panels panels (n_phi = 2 n_theta)."""
    nt, nph = _uv_sphere_shape(n_panels)
    v, t = _mesh_sphere(np.asarray(center, float), float(radius), nt, nph)
    return _finish(v, t, np.full(t.shape[0], cid, np.int32))


def _join(a: TriMesh, b: TriMesh) -> TriMesh:
    v = np.concatenate([a.vertices, b.vertices])
    t = np.concatenate([a.triangles, b.triangles + a.vertices.shape[0]]).astype(np.int32)
    return _finish(v, t, np.concatenate([a.conductor_ids, b.conductor_ids]))


def _dimer_recipe(seed: int, n_panels: Optional[int]):
    """The random draws of one dimer instance: the two spheres (center,
    radius, panels) and the conductor spec with its point charge."""
    rng = np.random.default_rng(seed)
    if n_panels is None:
        n_panels = int(rng.integers(2000, 40001))
    r1, r2 = rng.uniform(0.5, 1.5, 2)
    gap = rng.uniform(0.1, 1.0)
    u = rng.normal(size=3)
    u /= np.linalg.norm(u)
    c1, c2 = -u * (r1 + gap / 2), u * (r2 + gap / 2)
    n1 = int(round(n_panels * r1 * r1 / (r1 * r1 + r2 * r2)))
    near, rn, far, rf = (c1, r1, c2, r2) if rng.random() < 0.5 else (c2, r2, c1, r1)
    d = rng.uniform(0.3, 2.0)
    for _ in range(100):
        w = rng.normal(size=3)
        w /= np.linalg.norm(w)
        pos = near + w * (rn + d)
        if np.linalg.norm(pos - far) > rf + 0.05:
            break
    spec = dict(conductors=[dict(type="sphere", potential=0.0, id=0), dict(type="sphere", potential=0.0, id=1)],
                charges=[dict(type="point", q=float(rng.uniform(-1, 1)), pos=pos.tolist())])
    return (c1, float(r1), n1), (c2, float(r2), n_panels - n1), spec


def dimer_case(seed: int, n_panels: Optional[int] = None) -> Tuple[TriMesh, Dict[str, Any]]:
    (c1, r1, n1), (c2, r2, n2), spec = _dimer_recipe(seed, n_panels)
    return _join(_uv_sphere(c1, r1, n1, 0), _uv_sphere(c2, r2, n2, 1)), spec


def dimer_case_device(seed: int, n_panels: Optional[int] = None, device=None):
    """dimer_case with the mesh generated on the GPU (bit-identical arrays)."""
    from .mesh_device import mesh_grids

    (c1, r1, n1), (c2, r2, n2), spec = _dimer_recipe(seed, n_panels)
    grids = [("sphere", (np.asarray(c1, float), r1) + _uv_sphere_shape(n1), 0),
             ("sphere", (np.asarray(c2, float), r2) + _uv_sphere_shape(n2), 1)]
    return mesh_grids(grids, device), spec


class BatchSystem:
    """Device-resident batched system: FP64 and FP32 batched FMM operators,
    right-hand side, Jacobi diagonal and instance offsets.  The cases' meshes
    are host TriMesh arrays or DeviceTriMesh tensors (generated on the GPU:
    then nothing of the geometry crosses from the host)."""

    def __init__(self, cases: Sequence[Tuple[TriMesh, Dict[str, Any]]], *, leaf_size: int = 64,
                 expansion_order: int = 8, inner_leaf_size: Optional[int] = None,
                 inner_expansion_order: Optional[int] = None, device=None,
                 timings: Optional[Dict[str, float]] = None):
        """``timings``, when given, receives the wall time in ms of each set-up
        phase (the device is synchronised at every phase end, so pass it only
        to measure)."""
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        clock = [time.perf_counter()]

        def mark(name):
            if timings is not None:
                torch.cuda.synchronize(dev)
                now = time.perf_counter()
                timings[name] = 1e3 * (now - clock[0])
                clock[0] = now
        self.cases = list(cases)
        sizes = [m.n_panels for m, _ in self.cases]
        self.offsets = [0] + list(np.cumsum(sizes).astype(int))
        self.n = int(self.offsets[-1])
        if self.cases and isinstance(self.cases[0][0].vertices, Tensor):
            # meshes generated on the device (core.mesh_device): concatenated there
            ms = [m for m, _ in self.cases]
            vbase = np.concatenate([[0], np.cumsum([m.vertices.shape[0] for m in ms])])
            V = torch.cat([m.vertices.to(dev) for m in ms])
            tri = torch.cat([m.triangles.to(dev).long() + int(vbase[k]) for k, m in enumerate(ms)])
            self.normals = torch.cat([m.normals.to(dev) for m in ms])
            self.C64 = torch.cat([m.centroids.to(dev) for m in ms])
            self.areas = torch.cat([m.areas.to(dev) for m in ms])
            self.h2d_bytes = 0
        else:
            C = np.concatenate([m.centroids for m, _ in self.cases])
            A = np.concatenate([m.areas for m, _ in self.cases])
            self.normals = torch.as_tensor(np.concatenate([m.normals for m, _ in self.cases]), dtype=torch.float64,
                                           device=dev)
            # panel vertex triples gathered on the device from the (smaller)
            # vertex and triangle arrays
            vbase = np.concatenate([[0], np.cumsum([m.vertices.shape[0] for m, _ in self.cases])])
            V = torch.as_tensor(np.concatenate([m.vertices for m, _ in self.cases]), dtype=torch.float64, device=dev)
            tri = torch.as_tensor(np.concatenate([np.asarray(m.triangles, dtype=np.int64) + vbase[k]
                                                  for k, (m, _) in enumerate(self.cases)]), device=dev)
            # host -> device bytes of the set-up (centroids, areas, normals, vertices, triangles)
            self.h2d_bytes = int(8 * (3 + 1 + 3) * self.n + V.numel() * 8 + tri.numel() * 8)
            self.C64 = torch.as_tensor(C, dtype=torch.float64, device=dev)
            self.areas = torch.as_tensor(A, dtype=torch.float64, device=dev)
        PV = V[tri]
        mark("host_concat_and_copy")
        I_self = self_integrals(PV, self.C64, order=2, depth=3, device=dev)
        self.self_corr = I_self / self.areas.clamp_min(torch.finfo(torch.float64).tiny)
        self.diag = I_self.clamp_min(1e-18)
        mark("self_integrals")
        b = torch.zeros(self.n, dtype=torch.float64, device=dev)
        for k, (m, spec) in enumerate(self.cases):
            a, e = self.offsets[k], self.offsets[k + 1]
            ch = point_charges(spec)
            if ch:
                b[a:e] = -point_charge_potential(self.C64[a:e], ch)
        self.b = b
        self.x0_cold = b / self.diag
        mark("rhs")
        self.op64 = self.make_operator(torch.float64, leaf_size, expansion_order)
        mark("fp64_plan")
        self.op32 = self.make_operator(torch.float32, inner_leaf_size or leaf_size,
                                       inner_expansion_order or expansion_order)
        mark("fp32_plan")

    def make_operator(self, dtype, leaf_size: int, expansion_order: int) -> FmmOperator:
        """A batched operator; with the FP64 operator's leaf size it shares
        that operator's partition (plan converted, no second tree build)."""
        op64 = getattr(self, "op64", None)
        if op64 is not None and leaf_size == int(op64.plan.info.leaf_size):
            plan = op64.plan.convert(dtype, expansion_order)
        else:
            plan = _lib.Plan(self.C64.to(dtype).contiguous(), leaf_size=leaf_size, expansion_order=expansion_order,
                             instance_offsets=self.offsets)
        return FmmOperator(plan, self.areas.to(dtype), self.self_corr.to(dtype))

    def solve(self, x0: Optional[Tensor] = None, rtol: float = 1e-6, inner_restart: int = 100,
              inner_tol_floor: float = 3e-7, **kw) -> Tuple[Tensor, Dict[str, Any]]:
        """Mixed FP32/FP64 solve of all instances to ``rtol`` each.  Without
        ``x0`` the solve starts from zero, whose residual is b itself (one FP64
        operator application fewer than the cold start b / I_self, which the
        Jacobi-preconditioned inner solve reaches in its first step anyway).
        The inner tolerance may go down to 3e-7: the FP32 batched operator is
        within about 2e-7 of the FP64 one on these geometries, so one
        refinement step usually reaches 1e-6 (on the 256 dimers: one FP64
        application instead of two, 1.9 s instead of 2.8 s)."""
        return solve_mixed(self.op64, self.op32, self.b, A_diag=self.diag, x0=x0, rtol=rtol,
                           segments=self.offsets, inner_restart=inner_restart, inner_tol_floor=inner_tol_floor,
                           **kw)

    def learned_start(self, net) -> Tensor:
        """Per-instance learned warm start x0 = s (1 + y) (core.warm_start):
        s = b / A(1) from one FP32 application of the batched operator (block
        diagonal, so every instance gets its own), y from the network run on
        each instance's panels (its context is pooled over that instance)."""
        from .warm_start import base_guess

        s = base_guess(self.op32, self.b)
        y = torch.empty(self.n, dtype=torch.float64, device=self.device)
        for k in range(len(self.cases)):
            a, e = self.offsets[k], self.offsets[k + 1]
            f = net.features(self.C64[a:e], self.normals[a:e], self.areas[a:e], self.b[a:e])
            y[a:e] = net.forward(f).to(torch.float64)
        return s * (1.0 + y)

    def residuals(self, x: Tensor) -> Tensor:
        """Each instance's relative FP64 true residual."""
        r = self.b - self.op64(x.to(torch.float64)).to(torch.float64)
        return segment_norms(r, self.offsets) / segment_norms(self.b, self.offsets).clamp_min(1e-300)


def _time_op(op, x: Tensor, reps: int) -> Tuple[float, Tensor]:
    dev = x.device
    stream = torch.cuda.current_stream(dev)
    op(x)
    times = []
    y = None
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        y = op(x)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        times.append(e0.elapsed_time(e1))
    return statistics.median(times), y


def autotune_inner(system: BatchSystem, leaf_sizes=(32, 64, 128), orders=(6, 7, 8), max_rel_error: float = 3e-7,
                   reps: int = 3, use_cache: bool = True, inner_tol: Optional[float] = 3e-7) -> Dict[str, Any]:
    """Pick the FP32 inner operator (leaf size, expansion order and launch
    shape: near field beside the far field or fused after it) with the
    shortest matvec whose output is within ``max_rel_error`` of the FP64
    operator's on a fixed random density, weighing its speed against its
    error relative to ``inner_tol``, the floor of the batched solve's inner
    tolerance (``fmm3d.autotune.select_trial``); installs it as
    system.op32.  The
    bound matches the inner tolerance floor of the batched solve (3e-7), so
    that one refinement step can reach 1e-6.  The choice is kept in the
    autotune cache (electrodrive_gb300.fmm3d.autotune) under this machine,
    the panel-count bucket and the batch's signature; a cached choice is
    rebuilt and its accuracy checked once instead of searching again."""
    from ..fmm3d import autotune as at

    dev = system.device
    g = torch.Generator(device="cpu").manual_seed(0)
    probe = torch.rand(system.n, generator=g, dtype=torch.float64).to(dev)
    ref = system.op64(probe).to(torch.float64).clone()
    x = probe.float()
    fingerprint = at.hardware_fingerprint(dev)
    bucket = at.bucket_problem_size(system.n)
    signature = f"batch:{len(system.offsets) - 1}:{system.n}"
    if use_cache:
        rec = at.load_best(fingerprint, bucket, max_rel_error, kind="inner_fp32", signature=signature)
        if rec is not None:
            c = rec["config"]
            op = system.make_operator(torch.float32, int(c["leaf_size"]), int(c["expansion_order"]))
            at.apply_launch(op.plan, rec.get("launch", {}))
            t, y = _time_op(op, x, reps)
            err = float(torch.linalg.norm(y.double() - ref) / torch.linalg.norm(ref))
            if err <= max_rel_error:
                system.op32 = op
                return dict(leaf_size=int(c["leaf_size"]), expansion_order=int(c["expansion_order"]), ms=t,
                            launch=dict(rec.get("launch", {})), trials=[], from_cache=True)
    trials = []
    for leaf in leaf_sizes:
        for p in orders:
            op = system.make_operator(torch.float32, leaf, p)
            for launch in at.LAUNCH_CHOICES:
                op.plan.set_launch(**launch)
                t, y = _time_op(op, x, reps)
                err = float(torch.linalg.norm(y.double() - ref) / torch.linalg.norm(ref))
                trials.append(dict(leaf_size=leaf, expansion_order=p, launch=dict(launch), ms=t, rel_error=err))
            del op
    choice = at.select_trial(trials, max_rel_error, inner_tol=inner_tol)
    if choice is None:
        raise RuntimeError("no inner operator met the accuracy bound")
    t, leaf, p, launch = choice["ms"], choice["leaf_size"], choice["expansion_order"], choice["launch"]
    op = system.make_operator(torch.float32, leaf, p)
    at.apply_launch(op.plan, launch)
    system.op32 = op
    if use_cache:
        at.append_record({"fingerprint": fingerprint, "problem_size_bucket": bucket, "kind": "inner_fp32",
                          "signature": signature, "config": {"leaf_size": leaf, "expansion_order": p,
                                                             "precision": "single"},
                          "launch": launch, "metrics": {"wall_time_s": t * 1e-3, "rel_l2_error": min(
                              tr["rel_error"] for tr in trials if tr["leaf_size"] == leaf and
                              tr["expansion_order"] == p)}})
    return dict(leaf_size=leaf, expansion_order=p, ms=t, launch=launch, trials=trials, from_cache=False)


def plain_fp64_solve(mesh: TriMesh, spec: Dict[str, Any], *, rtol: float = 1e-6, restart: int = 256,
                     device=None, early_exit: Optional[int] = None) -> Dict[str, Any]:
    """The plain method on one instance: FP64 FMM operator, Jacobi GMRES from
    the cold start (b / I_self) to the same relative true residual.  With
    ``early_exit=c`` a cycle ends once the preconditioned residual meets the
    tolerance (checked every c steps); without it every cycle runs its full
    ``restart`` steps, as the reference's solver does."""
    from .bem import assemble_system
    from .bem_solver import gmres_restart

    sysd = assemble_system(mesh, spec, kind="fmm", dtypes=(torch.float64,), device=device)
    op = sysd["ops"][torch.float64]
    b, x0 = sysd["b"], sysd["x0"]
    r0 = float(torch.linalg.norm(b - op(x0)))
    bn = float(torch.linalg.norm(b))
    torch.cuda.synchronize(b.device)
    t0 = time.perf_counter()
    x, info = gmres_restart(op, b, restart=restart, tol=rtol * bn / r0, maxiter=4000, precond="jacobi",
                            A_diag=sysd["diag"], x0=x0, use_graph=True, early_exit=early_exit)
    torch.cuda.synchronize(b.device)
    dt = time.perf_counter() - t0
    rel = float(torch.linalg.norm(b - op(x))) / bn
    return dict(seconds=dt, iters=info["iters"], code=info["code"], rel_resid=rel, n=mesh.n_panels)


__all__ = ["BatchSystem", "autotune_inner", "dimer_case", "dimer_case_device", "plain_fp64_solve"]
