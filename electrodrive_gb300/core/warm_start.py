"""Learned warm start for the BEM solve (no counterpart in the reference).

A small point-cloud network maps per-panel data (centroid, normal, area and
the right-hand side b) to an initial surface charge density x0 for GMRES:

    x0_i = s_i (1 + y_i),   s = b / A(1),   y = net(features)

``s`` is a base guess: b divided by the potential that a unit density
produces.  One operator application gives it, and it is exact for a single
conductor at constant potential.  The network learns the correction y from
solves of the plain method.  The network (libedfmm ``edfmm_pcn_*``): width
128, 16 input features, a mean-pooled global context, BF16 weights and
activations on the tensor cores, FP32 accumulation, trained with the
library's own forward / backward / Adam kernels.

Cold start (x0 = b / I_self, the reference's guess) stays the fallback, and
GMRES judges every warm start: the solve runs to the same true residual
whatever x0 is.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from typing import Any, Dict, List, Optional, Tuple

import numpy as np
import torch
from torch import Tensor

from .. import _lib
from .bem_mesh import TriMesh, _finish, icosphere, torus_mesh

WIDTH = 128
INPUTS = 16


def init_params(seed: int = 0) -> np.ndarray:
    """He-normal weights, zero biases and a near-zero output layer (y ~ 0:
    the network starts at the base guess)."""
    rng = np.random.default_rng(seed)
    parts = [rng.normal(0, math.sqrt(2.0 / 8), (WIDTH, INPUTS)) * (np.arange(INPUTS) < 8)[None, :],
             np.zeros(WIDTH), rng.normal(0, math.sqrt(2.0 / WIDTH), (WIDTH, WIDTH)),
             rng.normal(0, math.sqrt(1.0 / WIDTH), (WIDTH, WIDTH)), np.zeros(WIDTH),
             rng.normal(0, math.sqrt(2.0 / WIDTH), (WIDTH, WIDTH)), np.zeros(WIDTH), rng.normal(0, 1e-3, WIDTH),
             np.zeros(1)]
    return np.concatenate([p.reshape(-1) for p in parts]).astype(np.float32)


class PointCloudNet:
    """Parameters on the device plus the library calls that use them."""

    def __init__(self, params=None, *, seed: int = 0, device=None):
        self.L = _lib.load_library()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.n_params = int(self.L.edfmm_pcn_num_params())
        p = init_params(seed) if params is None else np.asarray(params, np.float32).reshape(-1)
        if p.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {p.size}")
        self.params = torch.as_tensor(p, device=self.device).contiguous()
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.grads = torch.zeros_like(self.params)
        self.step = 0
        self._ws: Optional[Tensor] = None
        self._ws_n = 0

    # -- workspace ---------------------------------------------------------
    def _workspace(self, n: int) -> Tuple[Tensor, int]:
        nbytes = int(self.L.edfmm_pcn_workspace_bytes(n))
        if self._ws is None or self._ws.numel() < nbytes:
            self._ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        self._ws_n = n
        return self._ws, nbytes

    def _s(self):
        return _lib.stream_handle(self.device)

    # -- kernels -----------------------------------------------------------
    def features(self, centroids: Tensor, normals: Tensor, areas: Tensor, rhs: Tensor) -> Tensor:
        n = int(areas.shape[0])
        T = lambda x: torch.as_tensor(x).to(self.device, torch.float64).contiguous()
        c, nr, a, b = T(centroids).reshape(-1, 3), T(normals).reshape(-1, 3), T(areas), T(rhs)
        out = torch.empty(n, INPUTS, dtype=torch.float32, device=self.device)
        ws, nb = self._workspace(n)
        with torch.cuda.device(self.device):
            _lib.check(self.L.edfmm_pcn_features(_lib.ptr(c), _lib.ptr(nr), _lib.ptr(a), _lib.ptr(b), n, _lib.ptr(out),
                                                 _lib.ptr(ws), nb, self._s()), "edfmm_pcn_features")
        return out

    def forward(self, feats: Tensor) -> Tensor:
        n = int(feats.shape[0])
        y = torch.empty(n, dtype=torch.float32, device=self.device)
        ws, nb = self._workspace(n)
        with torch.cuda.device(self.device):
            _lib.check(self.L.edfmm_pcn_forward(_lib.ptr(self.params), _lib.ptr(feats.contiguous()), n, _lib.ptr(y),
                                                _lib.ptr(ws), nb, self._s()), "edfmm_pcn_forward")
        return y

    def backward(self, dy: Tensor) -> Tensor:
        """Gradients of the last forward pass (same workspace) for dL/dy."""
        n = self._ws_n
        ws, nb = self._workspace(n)
        with torch.cuda.device(self.device):
            _lib.check(self.L.edfmm_pcn_backward(_lib.ptr(self.params), n, _lib.ptr(dy.contiguous()),
                                                 _lib.ptr(self.grads), _lib.ptr(ws), nb, self._s()),
                       "edfmm_pcn_backward")
        return self.grads

    def loss(self, y: Tensor, scale: Tensor, sigma: Tensor, areas: Tensor) -> Tuple[Tensor, Tensor]:
        n = int(y.shape[0])
        dy = torch.empty(n, dtype=torch.float32, device=self.device)
        out = torch.empty(1, dtype=torch.float64, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self.L.edfmm_pcn_loss(_lib.ptr(y), _lib.ptr(scale), _lib.ptr(sigma), _lib.ptr(areas), n,
                                             _lib.ptr(dy), _lib.ptr(out), self._s()), "edfmm_pcn_loss")
        return out, dy

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8):
        self.step += 1
        with torch.cuda.device(self.device):
            _lib.check(self.L.edfmm_pcn_adam(_lib.ptr(self.params), _lib.ptr(self.grads), _lib.ptr(self.m),
                                             _lib.ptr(self.v), self.n_params, float(lr), float(beta1), float(beta2),
                                             float(eps), self.step, self._s()), "edfmm_pcn_adam")

    # -- persistence ---------------------------------------------------------
    def save(self, path: str, **meta):
        np.savez_compressed(path, params=self.params.cpu().numpy(), step=self.step, **meta)

    @classmethod
    def load(cls, path: str, device=None) -> "PointCloudNet":
        z = np.load(path)
        net = cls(z["params"], device=device)
        net.step = int(z["step"]) if "step" in z.files else 0
        return net

    # -- use -----------------------------------------------------------------
    def correction(self, mesh: TriMesh, rhs: Tensor) -> Tensor:
        """y for a mesh and its right-hand side."""
        f = self.features(torch.as_tensor(mesh.centroids), torch.as_tensor(mesh.normals), torch.as_tensor(mesh.areas),
                          rhs)
        return self.forward(f)


def base_guess(op, b: Tensor) -> Tensor:
    """s = b / A(1): b over the potential of a unit density (FP64)."""
    ones = torch.ones(b.shape[0], dtype=op.dtype, device=b.device)
    u = op(ones).to(torch.float64).clone()
    return b / torch.where(u.abs() > 1e-300, u, torch.ones_like(u))


def panel_geometry(mesh: TriMesh, device) -> Dict[str, Tensor]:
    """Device copies of the panel data the network reads (reuse across solves)."""
    T = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64).to(device)
    return dict(centroids=T(mesh.centroids), normals=T(mesh.normals), areas=T(mesh.areas))


def warm_start(net: PointCloudNet, geometry, b: Tensor, op) -> Tensor:
    """x0 = s (1 + y) in FP64; ``geometry`` is a TriMesh or panel_geometry()."""
    g = geometry if isinstance(geometry, dict) else panel_geometry(geometry, b.device)
    s = base_guess(op, b)
    y = net.forward(net.features(g["centroids"], g["normals"], g["areas"], b)).to(torch.float64)
    return s * (1.0 + y)


# ---------------------------------------------------------------------------
# synthetic geometries for training and evaluation
# ---------------------------------------------------------------------------
def _rotation(rng) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


_ICO_CACHE: Dict[int, TriMesh] = {}


def _ico(sub: int) -> TriMesh:
    """The unit icosphere of ``sub`` subdivisions (built once per process)."""
    if sub not in _ICO_CACHE:
        _ICO_CACHE[sub] = icosphere(sub)
    return _ICO_CACHE[sub]


def _transform(mesh: TriMesh, R: np.ndarray, scale=(1.0, 1.0, 1.0), shift=(0.0, 0.0, 0.0), cid: int = 0) -> TriMesh:
    v = (mesh.vertices * np.asarray(scale)[None, :]) @ R.T + np.asarray(shift)[None, :]
    return _finish(v, mesh.triangles.copy(), np.full(mesh.triangles.shape[0], cid, np.int32))


def _join(a: TriMesh, b: TriMesh) -> TriMesh:
    v = np.concatenate([a.vertices, b.vertices])
    t = np.concatenate([a.triangles, b.triangles + a.vertices.shape[0]]).astype(np.int32)
    return _finish(v, t, np.concatenate([a.conductor_ids, b.conductor_ids]))


def _ico_sub(panels: float) -> int:
    """Icosphere subdivisions (20 * 4^k panels) closest to ``panels``, 3..6."""
    return int(min(6, max(3, round(math.log(max(panels, 20.0) / 20.0, 4)))))


def random_case(rng: np.random.Generator, kind: str, panels: int = 4000) -> Tuple[TriMesh, Dict[str, Any]]:
    """A random conductor geometry of about ``panels`` panels (icospheres come
    in 20 * 4^k panels: 1,280 to 81,920), a random potential per conductor
    and a unit-scale point charge outside it."""
    R = _rotation(rng)
    if kind in ("sphere", "ellipsoid"):
        sub = _ico_sub(panels)
        axes = (rng.uniform(0.5, 1.5),) * 3 if kind == "sphere" else tuple(rng.uniform(0.5, 2.0, 3))
        mesh = _transform(_ico(sub), R, axes)
        conds = [dict(type=kind, potential=float(rng.uniform(-1, 1)), id=0)]
    elif kind == "torus":
        Rt = rng.uniform(0.8, 1.5)
        rt = Rt * rng.uniform(0.15, 0.45)
        nv = max(8, int(round(math.sqrt(panels * rt / (2 * Rt)))))
        nu = max(8, int(round(panels / (2 * nv))))
        mesh = _transform(torus_mesh(Rt, rt, nu, nv), R)
        conds = [dict(type="torus", potential=float(rng.uniform(-1, 1)), id=0)]
    elif kind == "dimer":
        r1, r2 = rng.uniform(0.5, 1.5, 2)
        gap = rng.uniform(0.1, 1.0)
        axis = R[:, 0]
        sub = _ico_sub(panels / 2.0)
        a = _transform(_ico(sub), np.eye(3), (r1, r1, r1), -axis * (r1 + gap / 2), 0)
        b = _transform(_ico(sub), np.eye(3), (r2, r2, r2), axis * (r2 + gap / 2), 1)
        mesh = _join(a, b)
        conds = [dict(type="sphere", potential=float(rng.uniform(-1, 1)), id=0),
                 dict(type="sphere", potential=float(rng.uniform(-1, 1)), id=1)]
    else:
        raise ValueError(f"unknown geometry kind {kind!r}")
    ctr = mesh.vertices.mean(axis=0)
    rmax = float(np.linalg.norm(mesh.vertices - ctr, axis=1).max())
    u = rng.normal(size=3)
    u /= np.linalg.norm(u)
    pos = ctr + u * (rmax + rng.uniform(0.3, 2.0))
    spec = dict(conductors=conds, charges=[dict(type="point", q=float(rng.uniform(-1, 1)), pos=pos.tolist())])
    return mesh, spec


KINDS = ("sphere", "ellipsoid", "torus", "dimer")


def make_sample(mesh: TriMesh, spec: Dict[str, Any], *, device=None, tol: float = 1e-10, operator: str = "auto",
                keep_ops: bool = True) -> Dict[str, Any]:
    """Solve one case to ``tol`` and keep what training and evaluation need,
    on the device.  ``operator``: "dense" (FP64 dense operator, Jacobi GMRES;
    the default up to 8,000 panels) or "fmm" (FP64 FMM operator with M2L and
    near field in two-float arithmetic, refined around FP32 FMM GMRES; the
    default above).  ``keep_ops=False`` drops the operators (training needs
    only the panel data, b, the base guess and the converged density)."""
    from .bem import assemble_system, solve_mixed
    from .bem_solver import gmres_restart

    kind = "dense" if operator == "dense" or (operator == "auto" and mesh.n_panels <= 8000) else "fmm"
    if kind == "dense":
        sysd = assemble_system(mesh, spec, kind="dense", dtypes=(torch.float64,), device=device)
        op, op32 = sysd["ops"][torch.float64], None
        b, diag = sysd["b"], sysd["diag"]
        sigma, info = gmres_restart(op, b, restart=100, tol=tol, maxiter=2000, precond="jacobi", A_diag=diag,
                                    x0=sysd["x0"], use_graph=True, early_exit=10)
    else:
        sysd = assemble_system(mesh, spec, kind="fmm", dtypes=(torch.float64, torch.float32), device=device)
        op, op32 = sysd["ops"][torch.float64], sysd["ops"][torch.float32]
        op.base.plan.set_arithmetic("two_float")
        b, diag = sysd["b"], sysd["diag"]
        sigma, info = solve_mixed(op, op32, b, A_diag=diag, x0=sysd["x0"], rtol=tol, inner_restart=100)
    dev = b.device
    out = dict(mesh=mesh, spec=spec, op=op, op32=op32, b=b, diag=diag, sigma=sigma.to(torch.float64),
               areas=sysd["areas"], scale=base_guess(op, b), normals=torch.as_tensor(mesh.normals, device=dev),
               centroids=torch.as_tensor(mesh.centroids, device=dev), solve_info=info, operator=kind)
    if not keep_ops:
        out["op"] = out["op32"] = None
    return out


def train(net: PointCloudNet, samples: List[Dict[str, Any]], *, epochs: int = 100, lr: float = 1e-3,
          seed: int = 0, lr_min: float = 1e-5, log_every: int = 0) -> List[float]:
    """One geometry per step, Adam with a cosine learning-rate decay; returns
    the mean loss of each epoch."""
    rng = np.random.default_rng(seed)
    feats = [net.features(s["centroids"], s["normals"], s["areas"], s["b"]) for s in samples]
    hist = []
    total = epochs * len(samples)
    k = 0
    for ep in range(epochs):
        acc = []
        for i in rng.permutation(len(samples)):
            s = samples[i]
            y = net.forward(feats[i])
            l, dy = net.loss(y, s["scale"], s["sigma"], s["areas"])
            net.backward(dy)
            rate = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * k / max(total - 1, 1)))
            net.adam(rate)
            acc.append(l)
            k += 1
        hist.append(float(torch.cat(acc).mean()))
        if log_every and (ep % log_every == 0 or ep == epochs - 1):
            print(f"epoch {ep}: loss {hist[-1]:.4e}", flush=True)
    return hist


def relative_error(x0: Tensor, sigma: Tensor, areas: Tensor) -> float:
    return float(torch.sqrt((areas * (x0 - sigma) ** 2).sum() / (areas * sigma ** 2).sum()))


def iterations_to(op, b: Tensor, diag: Tensor, x0: Tensor, rtol: float = 1e-6, restart: int = 50) -> Dict[str, Any]:
    """Jacobi GMRES from x0 until |b - A x| <= rtol |b| (cycles may end early
    on the inner estimate, so the count measures the start's quality)."""
    from .bem_solver import gmres_restart

    r0 = float(torch.linalg.norm(b - op(x0.to(op.dtype)).to(torch.float64)))
    bn = float(torch.linalg.norm(b))
    torch.cuda.synchronize(b.device)
    t0 = time.perf_counter()
    if r0 <= rtol * bn:
        return dict(iters=0, seconds=0.0, code=0, rel_resid=r0 / bn, r0=r0 / bn)
    x, info = gmres_restart(op, b, restart=restart, tol=rtol * bn / r0, maxiter=4000, precond="jacobi", A_diag=diag,
                            x0=x0, use_graph=True, early_exit=1)
    torch.cuda.synchronize(b.device)
    dt = time.perf_counter() - t0
    rel = float(torch.linalg.norm(b - op(x.to(op.dtype)).to(torch.float64))) / bn
    return dict(iters=info["iters"], seconds=dt, code=info["code"], rel_resid=rel, r0=r0 / bn)


def _timed_start(fn) -> Tuple[Tensor, float]:
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    x0 = fn()
    torch.cuda.synchronize()
    return x0, time.perf_counter() - t0


def compare_starts(net: Optional[PointCloudNet], sample: Dict[str, Any], rtol: float = 1e-6,
                   mixed: bool = True) -> Dict[str, Any]:
    """For the cold start (b / I_self, the reference's x0), the base guess
    (b / A(1)) and the learned start: each start's relative error against the
    converged density, the Jacobi GMRES iterations and time to ``rtol`` with
    the FP64 operator, and (``mixed`` and an FP32 operator in the sample) the
    mixed FP32/FP64 refinement solve to ``rtol``: refinement steps, inner
    iterations, FP64 operator applications and time, the time to compute the
    start included."""
    from .bem import solve_mixed

    op, b, diag, sigma, areas = sample["op"], sample["b"], sample["diag"], sample["sigma"], sample["areas"]
    geom = panel_geometry(sample["mesh"], b.device)
    makers = {"cold": lambda: b / diag, "base": lambda: base_guess(op, b)}
    if net is not None:
        makers["learned"] = lambda: warm_start(net, geom, b, op)
    op32 = sample.get("op32")
    out = {}
    for name, make in makers.items():
        x0, t_start = _timed_start(make)
        r = iterations_to(op, b, diag, x0, rtol)
        r["start_error"] = relative_error(x0, sigma, areas)
        r["start_seconds"] = t_start
        if mixed and op32 is not None:
            solve_mixed(op, op32, b, A_diag=diag, x0=make(), rtol=rtol)  # warm (graphs, workspaces)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            xm, info = solve_mixed(op, op32, b, A_diag=diag, x0=make(), rtol=rtol)
            torch.cuda.synchronize()
            r["mixed"] = dict(seconds=time.perf_counter() - t0, outer=info["outer"], inner_iters=info["inner_iters"],
                              fp64_matvecs=info["matvec64"], code=info["code"], rel_resid=info["rel_resid"])
        out[name] = r
    return out


__all__ = ["PointCloudNet", "init_params", "base_guess", "panel_geometry", "warm_start", "random_case", "make_sample",
           "train", "iterations_to", "compare_starts", "relative_error", "KINDS"]
