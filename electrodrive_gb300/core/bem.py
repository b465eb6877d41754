"""BEM solve on the GPU (electrodrive/core/bem.py:1550-2695).

``bem_solve(spec, cfg)`` runs the reference's h-refinement loop; each pass:
mesh -> self integrals (adaptive near-singular quadrature, depth 3 for
spheres / two planes, else 4) -> optional near-pair corrections
(``cfg.use_near_quadrature_matvec``) -> single-layer operator (dense below
``fmm_threshold`` panels, FMM above) -> ``b = bc - V_free``,
``x0 = b / I_self`` -> Jacobi-preconditioned restarted GMRES (retried without
the preconditioner, then damped Jacobi, when it fails) -> surface charge
density, boundary residual and capacitive energy.  Control-file polling,
telemetry and run manifests are not part of this operator path.

``solve_mixed`` is the FP32-inner / FP64-outer iterative refinement solver:
the FP64 operator computes the true residual, an FP32 GMRES solves the
correction equation, and the loop stops on the FP64 relative true residual.
"""
from __future__ import annotations

import math
import threading
import time
from dataclasses import dataclass, field
from typing import Any, Callable, Dict, List, Optional, Tuple

import numpy as np
import torch
from torch import Tensor

from .. import _lib
from ..utils.config import K_E, BEMConfig
from .bem_mesh import TriMesh, generate_mesh
from .bem_near import (NearCorrection, field_at_targets, near_potential_correction, point_charge_field,
                       point_charge_potential, potential_at_targets, self_integrals)
from .bem_solver import gmres_batched, gmres_restart
from .operators import DenseOperator, FmmOperator


def _cget(c: Any, key: str, default=None):
    return c.get(key, default) if isinstance(c, dict) else getattr(c, key, default)


def quad_depths(spec: Any) -> Tuple[int, int]:
    """(self-integral depth, near-matvec depth) as chosen in bem.py:1764-1776."""
    types = [_cget(c, "type") for c in (_cget(spec, "conductors", []) or [])]
    if any(t == "sphere" for t in types) or types.count("plane") >= 2:
        return 3, 3
    return 4, 3


def bc_vector(spec: Any, mesh: TriMesh) -> np.ndarray:
    """Per-panel Dirichlet value of its conductor (bem.py:373-403)."""
    id_to_v: Dict[int, float] = {}
    for i, c in enumerate(_cget(spec, "conductors", []) or []):
        try:
            v = float(_cget(c, "potential", 0.0))
        except Exception:
            v = 0.0
        id_to_v[int(_cget(c, "id", i))] = v
    ids = np.asarray(mesh.conductor_ids).astype(np.int64, copy=False)
    out = np.zeros(ids.shape[0], dtype=np.float64)  # panels of unknown conductors: 0
    for cid, v in id_to_v.items():
        out[ids == cid] = v
    return out


def point_charges(spec: Any) -> List[Tuple[float, Tuple[float, float, float]]]:
    out = []
    for ch in _cget(spec, "charges", []) or []:
        if _cget(ch, "type") != "point":
            continue
        try:
            out.append((float(_cget(ch, "q")), tuple(float(x) for x in _cget(ch, "pos"))))
        except Exception:
            continue
    return out


class BEMOperator:
    """A(sigma) = single-layer operator (+ near correction); capturable."""

    capturable = True

    def __init__(self, base, near: Optional[NearCorrection] = None):
        self.base = base
        self.near = near
        self.n = base.n
        self.device, self.dtype = base.device, base.dtype

    def __call__(self, sigma: Tensor, out: Optional[Tensor] = None) -> Tensor:
        v = self.base(sigma, out)
        if self.near is not None and self.near.n_pairs > 0:
            self.near.apply(sigma, v, v)
        return v

    def graph_state(self) -> tuple:
        """Forwarded to the base operator (captured graphs depend on it)."""
        fn = getattr(self.base, "graph_state", None)
        return fn() if fn is not None else ()

    def set_active_mask(self, flags: Optional[Tensor], stride: int = 1) -> bool:
        """Forwarded to the FMM base operator (batched plans only)."""
        fn = getattr(self.base, "set_active_mask", None)
        return bool(fn(flags, stride)) if fn is not None else False


def converted_operator(op, areas, self_corr: Tensor, *, dtype: torch.dtype, expansion_order: int,
                       near: Optional[NearCorrection] = None) -> Optional[BEMOperator]:
    """``op``'s FMM partition in another dtype and expansion order (its plan
    converted: no second tree or list build), or None when ``op`` is not an
    FMM operator."""
    base = getattr(op, "base", op)
    if not isinstance(base, FmmOperator):
        return None
    dev = base.plan.device
    a = areas if isinstance(areas, Tensor) else torch.as_tensor(np.asarray(areas))
    plan = base.plan.convert(dtype, expansion_order)
    return BEMOperator(FmmOperator(plan, a.to(dev, dtype), self_corr.to(dev, dtype)), near)


def build_operator(centroids, areas, self_corr: Tensor, *, dtype: torch.dtype, kind: str = "auto",
                   fmm_threshold: int = 20000, near: Optional[NearCorrection] = None, leaf_size: int = 64,
                   theta: float = 0.5, expansion_order: int = 8, device=None) -> BEMOperator:
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    n = int(np.asarray(areas).shape[0]) if not isinstance(areas, Tensor) else int(areas.shape[0])
    use_fmm = kind == "fmm" or (kind == "auto" and n >= fmm_threshold)
    c = torch.as_tensor(np.asarray(centroids) if not isinstance(centroids, Tensor) else centroids)
    a = torch.as_tensor(np.asarray(areas) if not isinstance(areas, Tensor) else areas)
    if use_fmm:
        plan = _lib.Plan(c.to(dev, dtype).contiguous(), leaf_size=leaf_size, mac_theta=theta,
                         expansion_order=expansion_order)
        base = FmmOperator(plan, a.to(dev, dtype), self_corr.to(dev, dtype))
    else:
        base = DenseOperator(c, a, self_corr, dtype=dtype, device=dev)
    return BEMOperator(base, near)


@dataclass
class BEMSolution:
    """Panel solution with the reference's evaluation entry points (bem.py:1367-1542)."""

    centroids: Tensor
    areas: Tensor
    sigma: Tensor
    charges: List[Tuple[float, Tuple[float, float, float]]] = field(default_factory=list)
    # target-side near quadrature of the induced potential (bem.py:1404-1417)
    panel_vertices: Optional[Tensor] = None
    near_quadrature: bool = False
    near_quad_order: int = 2
    near_quad_dist_factor: float = 1.5
    near_quad_max_depth: Optional[int] = None
    # diagnostics of the pass that produced the solution (energy_A)
    meta: Dict[str, Any] = field(default_factory=dict)

    def eval(self, points: Tensor) -> Tensor:
        """Total potential V_free + V_induced at points (N, 3): the dense induced
        part, corrected near the surface by the panels' quadrature when
        ``near_quadrature`` is on and panel vertices are known (bem.py:1461-1499)."""
        pts = torch.as_tensor(points).to(self.sigma.device, self.sigma.dtype).reshape(-1, 3).contiguous()
        v = potential_at_targets(pts, self.centroids, self.sigma, self.areas)
        if self.near_quadrature and self.panel_vertices is not None and self.panel_vertices.numel() > 0:
            v = near_potential_correction(v, pts, self.centroids, self.areas, self.sigma, self.panel_vertices,
                                          distance_factor=self.near_quad_dist_factor,
                                          quad_order=self.near_quad_order, max_depth=self.near_quad_max_depth)
        if self.charges:
            v = v + point_charge_potential(pts, self.charges)
        return v

    def eval_V_E_batched(self, points: Tensor) -> Tuple[Tensor, Tensor]:
        """Total potential (N,) and field (N, 3) at points: free-space point
        charges plus the panels' induced part (bem.py:1533-1542 with
        bem_E_field_targets, bem_kernel.py:914, for the field)."""
        pts = torch.as_tensor(points).to(self.sigma.device, self.sigma.dtype).reshape(-1, 3).contiguous()
        v = self.eval(pts)
        e = field_at_targets(pts, self.centroids, self.sigma, self.areas)
        if self.charges:
            e = e + point_charge_field(pts, self.charges)
        return v, e


def jacobi_fallback_solve(A, b: Tensor, diag: Tensor, *, maxiter: int = 1024, tol: float = 1e-6,
                          omega: float = 0.8) -> Tuple[Tensor, Dict[str, Any]]:
    """Damped Jacobi iteration x <- x + omega D^-1 (b - A x) from x = 0, the
    reference's last resort after GMRES fails (bem.py:1156-1251): stops when
    ||b - A x|| <= tol max(||b||, 1), on a non-finite residual, or after
    ``maxiter`` sweeps; returns (x, info) with the reference's info keys."""
    x = torch.zeros_like(b)
    dinv = 1.0 / diag.to(b.dtype).clamp_min(1e-18)
    r = b - A(x)
    r0 = float(torch.linalg.norm(r))
    if not math.isfinite(r0):
        return x, {"iters": 0, "resid": r0, "success": False, "solver": "jacobi_fallback"}
    target = tol * max(r0, 1.0)
    it, rn = 0, r0
    for k in range(maxiter):
        it = k + 1
        x = x + omega * dinv * r
        r = b - A(x)
        rn = float(torch.linalg.norm(r))
        if not math.isfinite(rn):
            return x, {"iters": it, "resid": rn, "success": False, "solver": "jacobi_fallback"}
        if rn <= target:
            return x, {"iters": it, "resid": rn, "success": True, "solver": "jacobi_fallback"}
    return x, {"iters": it, "resid": rn, "success": False, "solver": "jacobi_fallback"}


def _info_ok(info: Dict[str, Any]) -> Tuple[bool, float, int]:
    try:
        resid = float(info.get("resid", float("inf")))
    except Exception:
        resid = float("inf")
    return bool(info.get("success", True)), resid, int(info.get("code", 0) or 0)


def _near_in_background(C: Tensor, A: Tensor, PV: Tensor, dev, **kw) -> Callable[[], NearCorrection]:
    """Start building NearCorrection(C, A, PV, **kw) on a side stream in a
    worker thread (the library call releases the GIL) and return a function
    that waits for it and orders the caller's stream after it."""
    main = torch.cuda.current_stream(dev)
    side = torch.cuda.Stream(device=dev)
    side.wait_stream(main)  # C, A and PV were written on the caller's stream
    box: Dict[str, Any] = {}

    def run():
        try:
            with torch.cuda.device(dev), torch.cuda.stream(side):
                box["near"] = NearCorrection(C, A, PV, device=dev, **kw)
        except BaseException as e:  # re-raised in the caller's thread
            box["error"] = e

    worker = threading.Thread(target=run, name="near-correction", daemon=True)
    worker.start()

    def result() -> NearCorrection:
        worker.join()
        if "error" in box:
            raise box["error"]
        main.wait_stream(side)
        return box["near"]

    return result


def panel_vertices_on(mesh: TriMesh, dev) -> Tensor:
    """(N, 3, 3) FP64 panel vertices vertices[triangles], gathered on the device."""
    V = torch.as_tensor(mesh.vertices, dtype=torch.float64).to(dev)
    T = torch.as_tensor(np.asarray(mesh.triangles, dtype=np.int64)).to(dev)
    return V[T].contiguous()


def _solve_pass(spec: Any, cfg: BEMConfig, mesh: TriMesh, h: float, *, dev, dtype, mixed: bool, mixed_rtol: float,
                inner_restart: int, inner_expansion_order: Optional[int], operator: str, fmm_threshold: int,
                use_graph: bool, self_integral: str, logger, fp64_arithmetic: str = "native",
                warm_start: Optional[Any] = None) -> Dict[str, Any]:
    """One refinement pass of bem.py:1629-2404 on a given mesh: set-up, the
    linear solve with its retry and fallback chain, and the pass results.
    Returns {"error": msg} on a failure the reference reports as an error."""
    N = mesh.n_panels
    # the mesh goes to the device once: centroids, areas, and the panels'
    # vertices gathered there from the vertex and triangle arrays
    C64 = torch.as_tensor(mesh.centroids, dtype=torch.float64).to(dev)
    A64 = torch.as_tensor(mesh.areas, dtype=torch.float64).to(dev)
    PV = panel_vertices_on(mesh, dev)
    depth_self, depth_near = quad_depths(spec)
    order = int(getattr(cfg, "near_quadrature_order", 2))
    use_quad = self_integral == "quadrature" or (self_integral == "auto" and (
        bool(getattr(cfg, "use_near_quadrature_matvec", False)) or bool(getattr(cfg, "use_near_quadrature", False))))
    if use_quad:
        I_self = self_integrals(PV, C64, order=order, depth=depth_self, device=dev)
    else:
        a = np.clip(mesh.areas, 0.0, None)
        I_self = torch.as_tensor(np.where(mesh.areas > 0, 2.0 * np.pi * K_E * np.sqrt(a / np.pi), 0.0),
                                 dtype=torch.float64, device=dev)
    A_dev = A64.to(dev)
    tiny = torch.finfo(dtype).tiny
    self_corr = (I_self / A_dev.clamp_min(tiny)).to(dtype)
    want_near = bool(getattr(cfg, "use_near_quadrature_matvec", False)) and N > 1
    near = None
    near_job = None
    if want_near:
        # the pair search and weights overlap the operator's tree and lists
        near_job = _near_in_background(C64, A64, PV, dev,
                                       distance_factor=float(getattr(cfg, "near_quadrature_distance_factor", 1.5)),
                                       order=order, depth=depth_near, dtype=dtype)
    op = build_operator(C64, A64, self_corr, dtype=dtype, kind=operator, fmm_threshold=fmm_threshold, device=dev)
    if near_job is not None:
        near = op.near = near_job()
    op32 = None
    if mixed:
        if isinstance(op.base, FmmOperator) and fp64_arithmetic != "native":
            op.base.plan.set_arithmetic(fp64_arithmetic)
        near32 = None if near is None else near.astype(torch.float32)
        op32 = converted_operator(op, A64, self_corr, dtype=torch.float32, expansion_order=inner_expansion_order or 8,
                                  near=near32)
        if op32 is None:
            op32 = build_operator(C64, A64, self_corr.to(torch.float32), dtype=torch.float32, kind=operator,
                                  fmm_threshold=fmm_threshold, near=near32, device=dev,
                                  expansion_order=inner_expansion_order or 8)
    charges = point_charges(spec)
    C_dev = C64.to(dev, dtype)
    V_free = point_charge_potential(C_dev, charges) if charges else torch.zeros(N, dtype=dtype, device=dev)
    bc = torch.as_tensor(bc_vector(spec, mesh), dtype=dtype, device=dev)
    if not bool(torch.isfinite(bc).all()):
        return {"error": "BEM BC vector contains NaN/Inf."}
    if not bool(torch.isfinite(V_free).all()):
        return {"error": "Free-space potential on centroids contains NaN/Inf."}
    b = bc - V_free
    diag = I_self.to(dtype).clamp_min(1e-18)
    x0 = b / diag
    if not bool(torch.isfinite(b).all()):
        return {"error": "BEM RHS contains NaN/Inf."}
    if not bool(torch.isfinite(diag).all()):
        return {"error": "BEM diagonal (self-integrals) contains NaN/Inf."}
    if not bool(torch.isfinite(x0).all()):
        x0 = torch.zeros_like(b)
    use_precond = bool(getattr(cfg, "use_precond", True))
    restart = int(getattr(cfg, "gmres_restart", 256))
    tol = float(getattr(cfg, "gmres_tol", 5e-8))
    maxiter = int(getattr(cfg, "gmres_maxiter", 2000))

    def plain(precond):
        return gmres_restart(op, b, restart=restart, tol=tol, maxiter=maxiter, precond=precond,
                             areas=A_dev.to(dtype), A_diag=diag, x0=x0, logger=logger, use_graph=use_graph)

    sigma = info = None
    r_sigma = None  # the mixed solve's FP64 residual b - A sigma at its sigma
    N64 = None
    if mixed:
        xm0 = x0
        if warm_start is not None:
            # the learned start (features, network, one FP32 operator
            # application); the reference's chain below keeps x0 = b / I_self
            from .warm_start import warm_start as learned_start

            # the network's panel data: the device copies this pass already holds
            N64 = torch.as_tensor(mesh.normals, dtype=torch.float64).to(dev).contiguous()
            geom = dict(centroids=C64.contiguous(), normals=N64, areas=A64.contiguous())
            xs = learned_start(warm_start, geom, b, op32)
            if bool(torch.isfinite(xs).all()):
                xm0 = xs.to(dtype)
        x, minfo = solve_mixed(op, op32, b, A_diag=diag if use_precond else None, x0=xm0, rtol=mixed_rtol,
                               inner_restart=inner_restart, use_graph=use_graph)
        bn = float(torch.linalg.norm(b))
        if minfo["success"]:
            sigma = x.to(dtype)
            r_sigma = minfo["residual"]
            info = dict(iters=minfo["inner_iters"], resid=minfo["rel_resid"] * bn, success=True, code=0,
                        tol_abs=mixed_rtol * bn, used_preconditioner=use_precond, outer=minfo["outer"],
                        matvec64=minfo["matvec64"], history=minfo["history"], precision="mixed")
    if sigma is None:
        # the reference's chain (bem.py:2172-2302): preconditioned GMRES, a
        # retry without the preconditioner, then damped Jacobi
        precond = "jacobi" if use_precond else None
        sigma, info = plain(precond)
        ok, resid, code = _info_ok(info)
        if precond is not None and (not ok or not math.isfinite(resid)):
            sigma, info = plain(None)
            ok, resid, code = _info_ok(info)
        if not ok or not math.isfinite(resid):
            if not bool(getattr(cfg, "allow_jacobi_fallback", True)):
                return {"error": f"BEM linear solve failed: GMRES(code={code}, resid={resid})",
                        "gmres_resid": resid, "gmres_code": code}
            sj, ij = jacobi_fallback_solve(op, b, diag, maxiter=int(getattr(cfg, "jacobi_maxiter", 256)),
                                           tol=float(getattr(cfg, "jacobi_tol", 1e-5)),
                                           omega=float(getattr(cfg, "jacobi_omega", 0.8)))
            rj = float(ij.get("resid", float("inf")))
            if not (ij.get("success", False) and math.isfinite(rj)):
                return {"error": f"BEM linear solve failed: GMRES(code={code}, resid={resid}) and Jacobi(resid={rj})",
                        "gmres_resid": resid, "gmres_code": code, "jacobi_resid": rj, "jacobi_iters": ij.get("iters")}
            sigma, info = sj, ij
    if not bool(torch.isfinite(sigma).all()):
        return {"error": "BEM sigma contains NaN/Inf after linear solve."}
    if r_sigma is not None:
        # V_free + A sigma = bc - (b - A sigma): the solve's last FP64
        # residual already holds the operator application at sigma
        V_tot = torch.nan_to_num(bc - r_sigma.to(dtype), nan=0.0, posinf=0.0, neginf=0.0)
    else:
        V_tot = torch.nan_to_num(V_free + op(sigma).clone(), nan=0.0, posinf=0.0, neginf=0.0)
    bc_resid = float(torch.max(torch.abs(V_tot - bc)))
    energy = float(0.5 * torch.sum(V_tot.double() * torch.nan_to_num(sigma).double() * A_dev))
    Nrm = N64.to(dtype) if N64 is not None else torch.as_tensor(mesh.normals, dtype=dtype, device=dev)
    return {"pass_payload": {"h": h, "dof": N, "bc_resid_linf": bc_resid, "energy_A": energy, "gmres_info": dict(info),
                             "tile_size": int(getattr(cfg, "tile_size", 0) or 0),
                             "artifacts": (spec, C_dev, A_dev.to(dtype), Nrm, sigma, V_tot, mesh)},
            "operator": "fmm" if isinstance(op.base, FmmOperator) else "dense",
            "near_pairs": 0 if near is None else near.n_pairs, "charges": charges, "PV": PV}


def bem_solve(spec: Any, cfg: Optional[BEMConfig] = None, logger: Optional[Any] = None, differentiable: bool = False,
              *, mesh: Optional[TriMesh] = None, operator: str = "auto", fmm_threshold: int = 20000,
              use_graph: bool = True, self_integral: str = "auto", mixed: bool = False, mixed_rtol: float = 1e-6,
              inner_restart: int = 40, inner_expansion_order: Optional[int] = None,
              fp64_arithmetic: str = "two_float", warm_start: Optional[Any] = None) -> Dict[str, Any]:
    """The reference's bem_solve (bem.py:1550-2695) on the GPU operator.

    h-refinement (bem.py:1667-2495): pass k meshes at h = initial_h *
    refine_factor^k and solves; the loop stops once the pass's boundary
    residual max |V_free + A sigma - bc| is at most ``target_bc_inf_norm``
    (after ``min_refine_passes`` and ``min_panels``), on a plateau when
    ``plateau_max`` is set, or after ``max_refine_passes``.  The best pass
    (smallest boundary residual; a finer mesh wins within a band of 1e-3 of
    the target) is returned.  Each solve is Jacobi-preconditioned restarted
    GMRES from x0 = b / I_self; if it fails it is retried without the
    preconditioner and then by damped Jacobi (``allow_jacobi_fallback``,
    ``jacobi_maxiter``, ``jacobi_tol``, ``jacobi_omega``), as the reference
    does.  Keys of the result are the reference's (``surface_charge_density``
    as a host array, ``solution``, ``mesh_stats``, ``gmres_stats``,
    ``refinement_history``, ``boundary_samples``, ``sample_points``) or
    {"error": ...}.  Control-file polling, telemetry and manifests are not
    part of this operator path; ``tile_size`` entries report 0 (no tiling).

    Additions: ``mesh`` solves one pass on a given mesh; ``operator``
    ("auto": dense below ``fmm_threshold`` panels, FMM above);
    ``self_integral`` "auto" follows the reference (quadrature self terms only
    when a near-quadrature option is on, else the equal-area disk value
    2 pi K_E sqrt(A / pi), bem.py:1747-1816) or forces "quadrature" / "disk";
    ``mixed=True`` builds the operator in FP64 and FP32 and solves with
    :func:`solve_mixed` to an FP64 relative true residual of ``mixed_rtol``
    (``cfg.fp64`` is then ignored; a failed mixed solve falls back to the
    reference's chain in FP64); ``fp64_arithmetic`` ("two_float", the
    default, or "native") is the arithmetic of that FP64 FMM operator's M2L
    and near field (two-float: about 48 significant bits on the FP32 pipe,
    within about 1e-13 of IEEE FP64); ``warm_start`` (a trained
    :class:`~electrodrive_gb300.core.warm_start.PointCloudNet`) starts the
    mixed solve from the network's prediction instead of b / I_self.
    """
    if differentiable:
        raise NotImplementedError("the differentiable (xitorch) path is not part of electrodrive_gb300")
    cfg = cfg or BEMConfig()
    if float(getattr(cfg, "near_alpha", 0.0) or 0.0) > 0.0:
        raise NotImplementedError("near_alpha neighbour smoothing of the operator is not part of electrodrive_gb300")
    _lib.load_library()
    dev = torch.device("cuda", torch.cuda.current_device())
    dtype = torch.float64 if (getattr(cfg, "fp64", False) or mixed) else torch.float32
    t0 = time.perf_counter()
    current_h = float(getattr(cfg, "initial_h", 0.3))
    refine_factor = float(getattr(cfg, "refine_factor", 0.5))
    target_bc = float(getattr(cfg, "target_bc_inf_norm", 1e-7))
    tiny_band = max(target_bc * 1e-3, 1e-12)
    max_passes = 1 if mesh is not None else int(getattr(cfg, "max_refine_passes", 3))
    plateau_raw = getattr(cfg, "plateau_max", None)
    try:
        max_plateau = None if plateau_raw is None else int(plateau_raw)
    except Exception:
        max_plateau = None
    plateau_rel = float(getattr(cfg, "plateau_rel_improvement", 0.05))
    history: List[Dict[str, Any]] = []
    best: Optional[Dict[str, Any]] = None
    best_extra: Dict[str, Any] = {}
    extras: List[Dict[str, Any]] = []
    best_bc = float("inf")
    plateau = 0

    def error_result(msg: str, **extra: Any) -> Dict[str, Any]:
        out: Dict[str, Any] = {"error": msg}
        if history:
            out["refinement_history"] = history
        if best is not None:
            out["best_bc_resid_linf"] = best.get("bc_resid_linf")
            out["best_dof"] = best.get("dof")
        out.update(extra)
        return out

    for rp in range(max_passes):
        try:
            m = mesh if mesh is not None else generate_mesh(spec, current_h)
        except Exception:
            break
        if m.n_panels == 0:
            break
        res = _solve_pass(spec, cfg, m, current_h, dev=dev, dtype=dtype, mixed=mixed, mixed_rtol=mixed_rtol,
                          inner_restart=inner_restart, inner_expansion_order=inner_expansion_order, operator=operator,
                          fmm_threshold=fmm_threshold, use_graph=use_graph, self_integral=self_integral,
                          logger=logger, fp64_arithmetic=fp64_arithmetic, warm_start=warm_start)
        if "error" in res:
            msg = res.pop("error")
            return error_result(msg, **res)
        payload = dict(res["pass_payload"], **{"pass": rp + 1})
        history.append(payload)
        extras.append(res)
        bc_r, N = payload["bc_resid_linf"], payload["dof"]
        if bc_r < best_bc:
            improvement = best_bc - bc_r if math.isfinite(best_bc) else float("inf")
            best, best_extra, best_bc = payload, res, bc_r
            plateau = 0 if improvement > max(1e-16, plateau_rel * max(best_bc, 1e-16)) else plateau + 1
        elif best is not None and abs(bc_r - best_bc) <= tiny_band and N > int(best.get("dof", 0)):
            best, best_extra, best_bc = payload, res, bc_r
            plateau = 0
        else:
            plateau += 1
        have_min_panels = N >= int(getattr(cfg, "min_panels", 0))
        have_min_passes = (rp + 1) >= int(getattr(cfg, "min_refine_passes", 1))
        if bc_r <= target_bc and have_min_panels and have_min_passes:
            break
        if max_plateau is not None and plateau >= max_plateau and have_min_panels and have_min_passes:
            break
        current_h *= refine_factor
    if best is None:
        if not history:
            return error_result("BEM solve failed (no passes)")
        good = [p for p in history if _info_ok(p.get("gmres_info") or {})[0]
                and math.isfinite(_info_ok(p.get("gmres_info") or {})[1])]
        if not good:
            return error_result("BEM solve failed (no successful linear solves)",
                                gmres_last=history[-1].get("gmres_info", {}))
        best = min(good, key=lambda p: p.get("bc_resid_linf", float("inf")))
        best_extra = extras[history.index(best)]
    spec_b, C_b, A_b, Nrm_b, sigma_b, Vtot_b, mesh_b = best["artifacts"]
    N_b = int(best["dof"])
    torch.cuda.synchronize(dev)
    t_total = time.perf_counter() - t0
    # evaluation near quadrature as bem.py:2560-2600 configures it
    eval_factor = float(getattr(cfg, "near_quadrature_distance_factor", 1.5))
    ctypes_ = {_cget(c, "type") for c in (_cget(spec, "conductors", []) or [])}
    if "sphere" in ctypes_:
        eval_factor = max(eval_factor, 6.0)
    elif "plane" in ctypes_:
        eval_factor = max(eval_factor, 3.0)
    use_near_eval = bool(getattr(cfg, "use_near_quadrature", False)) and N_b > 0
    sol = BEMSolution(centroids=C_b, areas=A_b, sigma=sigma_b, charges=best_extra["charges"],
                      panel_vertices=torch.as_tensor(best_extra["PV"], dtype=torch.float64, device=dev)
                      if use_near_eval else None,
                      near_quadrature=use_near_eval,
                      near_quad_order=int(getattr(cfg, "near_quadrature_order", 2)),
                      near_quad_dist_factor=eval_factor, near_quad_max_depth=quad_depths(spec)[0])
    n_samples = min(1024, max(1, N_b))
    step = max(1, N_b // n_samples)
    idx = torch.arange(0, N_b, step, device=C_b.device)[:n_samples]
    mesh_stats = dict(n_panels=N_b, total_area=float(A_b.sum()), bc_residual_linf=float(best["bc_resid_linf"]),
                      h_final=float(best["h"]), tile_size_final=int(best["tile_size"]),
                      operator=best_extra["operator"], near_pairs=best_extra["near_pairs"])
    if any(_cget(c, "type") == "plane" for c in (_cget(spec, "conductors", []) or [])) and mesh_stats["total_area"] > 0:
        mesh_stats["patch_L"] = math.sqrt(mesh_stats["total_area"])
    gmres_stats = dict(best.get("gmres_info", {}))
    gmres_stats.update(total_seconds=t_total)
    sol.meta["energy_A"] = best["energy_A"]
    return dict(solution=sol, surface_charge_density=sigma_b.detach().cpu().numpy(), mesh_stats=mesh_stats,
                gmres_stats=gmres_stats, refinement_history=history,
                boundary_samples=Vtot_b[idx].detach().cpu().numpy().tolist(),
                sample_points=C_b[idx].detach().cpu().numpy().tolist())


def assemble_system(mesh: TriMesh, spec: Any, *, kind: str = "dense", dtypes=(torch.float64,), near: bool = False,
                    self_integral: str = "quadrature", device=None) -> Dict[str, Any]:
    """The pieces bem_solve assembles, on the device: one operator per dtype
    (with the near correction when ``near``), the FP64 right-hand side
    b = bc - V_free, the Jacobi diagonal I_self and the reference's x0 = b / I_self."""
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    PV = mesh.vertices[mesh.triangles]
    C64 = torch.as_tensor(mesh.centroids, dtype=torch.float64)
    A64 = torch.as_tensor(mesh.areas, dtype=torch.float64)
    depth_self, depth_near = quad_depths(spec)
    if self_integral == "quadrature":
        I_self = self_integrals(PV, mesh.centroids, order=2, depth=depth_self, device=dev)
    else:
        a = np.clip(mesh.areas, 0.0, None)
        I_self = torch.as_tensor(np.where(mesh.areas > 0, 2.0 * np.pi * K_E * np.sqrt(a / np.pi), 0.0),
                                 dtype=torch.float64, device=dev)
    A_dev = A64.to(dev)
    self_corr = I_self / A_dev.clamp_min(torch.finfo(torch.float64).tiny)
    ops = {}
    nc0 = None
    for dt in dtypes:
        nc = None
        if near and mesh.n_panels > 1:
            # one pair search and quadrature; the other dtypes cast its weights
            if nc0 is None:
                nc0 = NearCorrection(mesh.centroids, mesh.areas, PV, distance_factor=1.5, order=2, depth=depth_near,
                                     dtype=dt, device=dev)
            nc = nc0.astype(dt)
        ops[dt] = build_operator(C64, A64, self_corr.to(dt), dtype=dt, kind=kind, near=nc, device=dev)
    charges = point_charges(spec)
    V_free = point_charge_potential(C64.to(dev), charges) if charges else torch.zeros(mesh.n_panels, dtype=torch.float64,
                                                                                       device=dev)
    b = torch.as_tensor(bc_vector(spec, mesh), dtype=torch.float64, device=dev) - V_free
    diag = I_self.clamp_min(1e-18)
    return dict(ops=ops, b=b, diag=diag, x0=b / diag, areas=A_dev, centroids=C64, n=mesh.n_panels,
                near_pairs=0 if not near else next(iter(ops.values())).near.n_pairs, charges=charges,
                self_corr=self_corr)


def autotune_inner_operator(op64, centroids: Tensor, areas: Tensor, self_corr: Tensor, near=None, *,
                            orders=(8, 7, 6), leaf_sizes=(64,), max_rel_error: float = 3e-7, reps: int = 5,
                            device=None, use_cache: bool = True,
                            signature: Optional[str] = None) -> Tuple[Any, List[Dict[str, Any]]]:
    """The FP32 FMM operator for the inner solves of iterative refinement:
    among expansion orders, leaf sizes and launch shapes (near field beside
    the far field or fused after it), the fastest whose output on a fixed
    random density is within ``max_rel_error`` of ``op64``'s (of candidates
    within 5% of the fastest, the most accurate; the FP32
    operator at p = 8 is about 2e-7 away; looser operators make the first
    refinement step fall short of 1e-6).  ``near`` is the FP32 near
    correction the operator adds.  The choice is kept in the autotune cache
    (electrodrive_gb300.fmm3d.autotune) under this machine, the panel-count
    bucket and ``signature`` (default: the panel count); a cached choice is
    rebuilt and checked once instead of searching again.  Returns
    (operator, trials)."""
    from ..fmm3d import autotune as at

    dev = torch.device(device) if device is not None else op64.device if hasattr(op64, "device") else \
        torch.device("cuda", torch.cuda.current_device())
    g = torch.Generator(device="cpu").manual_seed(0)
    probe = torch.rand(int(areas.shape[0]), generator=g, dtype=torch.float64).to(dev)
    ref = op64(probe).to(torch.float64).clone()
    stream = torch.cuda.current_stream(dev)
    base64 = getattr(op64, "base", op64)
    leaf64 = int(base64.plan.info.leaf_size) if isinstance(base64, FmmOperator) else None

    def make(leaf, p):
        op = (converted_operator(op64, areas, self_corr, dtype=torch.float32, expansion_order=p, near=near)
              if leaf == leaf64 else None)
        if op is None:
            op = build_operator(centroids, areas, self_corr.to(torch.float32), dtype=torch.float32, kind="fmm",
                                near=near, leaf_size=leaf, expansion_order=p, device=dev)
        return op

    def timed(op):
        x = probe.float()
        op(x)
        times = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            y = op(x)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            times.append(e0.elapsed_time(e1))
        return sorted(times)[len(times) // 2], float(torch.linalg.norm(y.double() - ref) / torch.linalg.norm(ref))

    n = int(areas.shape[0])
    fingerprint = at.hardware_fingerprint(dev)
    bucket = at.bucket_problem_size(n)
    sig = signature or f"single:{n}"
    if use_cache:
        rec = at.load_best(fingerprint, bucket, max_rel_error, kind="inner_fp32", signature=sig)
        if rec is not None:
            c = rec["config"]
            op = make(int(c["leaf_size"]), int(c["expansion_order"]))
            at.apply_launch(op.base.plan, rec.get("launch", {}))
            t, err = timed(op)
            if err <= max_rel_error:
                return op, [dict(leaf_size=int(c["leaf_size"]), expansion_order=int(c["expansion_order"]),
                                 launch=dict(rec.get("launch", {})), ms=t, rel_error=err, from_cache=True)]
    trials, ops = [], {}
    for leaf in leaf_sizes:
        for p in orders:
            op = make(leaf, p)
            for launch in at.LAUNCH_CHOICES:
                op.base.plan.set_launch(**launch)
                t, err = timed(op)
                trials.append(dict(leaf_size=leaf, expansion_order=p, launch=dict(launch), ms=t, rel_error=err))
            ops[(leaf, p)] = op
    choice = at.select_trial(trials, max_rel_error)
    if choice is None:
        raise RuntimeError("no inner operator met the accuracy bound")
    t, leaf, p, launch, err = choice["ms"], choice["leaf_size"], choice["expansion_order"], choice["launch"], \
        choice["rel_error"]
    op = ops.pop((leaf, p))
    ops.clear()
    at.apply_launch(op.base.plan, launch)
    if use_cache:
        at.append_record({"fingerprint": fingerprint, "problem_size_bucket": bucket, "kind": "inner_fp32",
                          "signature": sig, "config": {"leaf_size": leaf, "expansion_order": p, "precision": "single"},
                          "launch": launch, "metrics": {"wall_time_s": t * 1e-3, "rel_l2_error": err}})
    return op, trials


def segment_norms(v: Tensor, offsets: Optional[List[int]]) -> Tensor:
    """2-norm of each slice [offsets[k], offsets[k+1]) of v (FP64)."""
    v2 = v.to(torch.float64) ** 2
    if offsets is None:
        return torch.sqrt(v2.sum()).reshape(1)
    o = torch.as_tensor(offsets, dtype=torch.int64)
    lengths = (o[1:] - o[:-1]).to(v.device)
    return torch.sqrt(torch.segment_reduce(v2, "sum", lengths=lengths))


def solve_mixed(op64, op32, b: Tensor, *, A_diag: Optional[Tensor] = None, x0: Optional[Tensor] = None,
                rtol: float = 1e-6, inner_restart: int = 40, inner_tol: Optional[float] = None,
                inner_tol_floor: float = 1e-5, inner_maxiter: int = 400, max_outer: int = 30, use_graph: bool = True,
                inner_early_exit: Optional[int] = 8, segments: Optional[List[int]] = None,
                batched: bool = True, first_residual: str = "fp32") -> Tuple[Tensor, Dict[str, Any]]:
    """FP32 GMRES corrections inside FP64 iterative refinement.

    Stops when ||b - A64 x|| / ||b|| <= rtol (FP64 true residual; with
    ``segments``, the row offsets of independent instances, every instance's
    own relative residual must meet rtol).  The FP32 inner solve is
    left-preconditioned by Jacobi with ``A_diag``; its cycles may end early on
    the inner estimate (checked every ``inner_early_exit`` steps; None runs
    full cycles).  Each inner solve aims at the reduction the outer target
    still needs, 0.3 rtol / (current relative residual), but at most
    ``inner_tol_floor`` (about what the FP32 operator can deliver against the
    FP64 one); a fixed ``inner_tol`` overrides that.  With ``segments`` and
    ``batched`` the inner solve is ``gmres_batched``: every instance gets its
    own Krylov space and its own inner tolerance (instances already at rtol
    sit out), and the steps share one operator application.

    ``first_residual="fp32"`` takes the residual of a given ``x0`` from the
    FP32 operator: x0 is an estimate whose error is far above the FP32
    operator's (about 2e-7 of |A x0|), so the first correction needs no FP64
    application; every later residual, and the stopping test, is FP64.

    On success the returned dict also holds ``residual``, the FP64 residual
    b - A64 x at the returned x (the stopping test's own vector).
    """
    dev = b.device
    b64 = b.to(torch.float64)
    x = torch.zeros_like(b64) if x0 is None else x0.to(torch.float64).clone()
    bseg = segment_norms(b64, segments)
    bseg = torch.where(bseg > 0, bseg, torch.ones_like(bseg))
    d32 = None if A_diag is None else A_diag.to(dev, torch.float32)
    hist = []
    inner_total = 0
    inst_iters = None  # per-instance inner steps (batched inner solves)
    matvec64 = 0
    r_is_fp64 = True
    if x0 is None:
        r = b64.clone()  # x = 0: the residual needs no operator application
    elif first_residual == "fp32":
        r = b64 - op32(x.to(torch.float32)).to(torch.float64)
        r_is_fp64 = False
    else:
        r = b64 - op64(x)
        matvec64 += 1
    for it in range(max_outer + 1):
        rel = float((segment_norms(r, segments) / bseg).max())
        hist.append(rel)
        if not math.isfinite(rel):
            return x, dict(success=False, code=6, outer=it, inner_iters=inner_total, rel_resid=rel, history=hist,
                           matvec64=matvec64)
        if rel <= rtol and not r_is_fp64:
            r = b64 - op64(x)  # only an FP64 residual may stop the solve
            matvec64 += 1
            r_is_fp64 = True
            rel = float((segment_norms(r, segments) / bseg).max())
            hist[-1] = rel
        if rel <= rtol:
            # r is the FP64 residual b - A64 x of the returned x
            return x, dict(success=True, code=0, outer=it, inner_iters=inner_total, rel_resid=rel, history=hist,
                           matvec64=matvec64, instance_inner_iters=inst_iters, residual=r)
        if it == max_outer:
            break
        r32 = r.to(torch.float32)
        if segments is not None and batched:
            rel_i = segment_norms(r, segments) / bseg
            if inner_tol is not None:
                tol_i = torch.full_like(rel_i, float(inner_tol))
            else:
                tol_i = (0.3 * rtol / rel_i).clamp(min=inner_tol_floor, max=0.1)
            tol_i = torch.where(rel_i > rtol, tol_i, torch.full_like(tol_i, -1.0))
            d, info = gmres_batched(op32, r32, segments, restart=inner_restart, tol=tol_i, maxiter=inner_maxiter,
                                    A_diag=d32, use_graph=use_graph, check_every=inner_early_exit or 8)
            per = info["instance_iters"]
            inst_iters = per if inst_iters is None else [u + v for u, v in zip(inst_iters, per)]
        else:
            tol_k = inner_tol if inner_tol is not None else min(0.1, max(inner_tol_floor, 0.3 * rtol / rel))
            d, info = gmres_restart(op32, r32, restart=inner_restart, tol=tol_k, maxiter=inner_maxiter,
                                    precond="jacobi" if d32 is not None else None, A_diag=d32, use_graph=use_graph,
                                    early_exit=inner_early_exit, final_check=False)
        inner_total += info["iters"]
        x = x + d.to(torch.float64)
        r = b64 - op64(x)
        matvec64 += 1
        r_is_fp64 = True
    return x, dict(success=False, code=1, outer=max_outer, inner_iters=inner_total, rel_resid=hist[-1], history=hist,
                   matvec64=matvec64, instance_inner_iters=inst_iters)


__all__ = ["BEMOperator", "BEMSolution", "assemble_system", "autotune_inner_operator", "bem_solve", "build_operator",
           "bc_vector", "jacobi_fallback_solve", "point_charges",
           "quad_depths", "segment_norms", "solve_mixed"]
