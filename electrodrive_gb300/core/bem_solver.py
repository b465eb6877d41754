"""Restarted left-preconditioned GMRES on the GPU
(electrodrive/core/bem_solver.py:36-920).

``gmres_restart`` keeps the reference's signature, defaults, stopping rule and
``info`` dictionary:

* tol_abs = max(tol * |b - A x0|, tol * 1e-12, 1e-12) (|b - A x0| replaced by 1
  when below 1e-16);
* every restart cycle runs ``restart`` Arnoldi steps (the reference does not
  leave a cycle early on the inner estimate), then x += V y and the TRUE
  residual |b - A x| decides convergence;
* codes 0 converged, 1 maxiter, 2 terminate/stagnation, 3 non-finite initial
  residual, 5 non-finite inner residual, 6 non-finite post-update residual,
  7 non-finite initial preconditioned residual; for N <= 512 a failed
  preconditioned run is retried once without the preconditioner;
* the Krylov dtype is b's dtype (FP64 for FP32 systems with N <= 64).

The Krylov arithmetic runs in libedfmm (``edfmm_gmres_*``): CGS2
orthogonalisation with FP64 inner products, Hessenberg / Givens / triangular
solve in FP64 on the device.  The host reads the device status once per
cycle.  When the operator advertises ``capturable = True`` (the operators of
``electrodrive_gb300.core.operators``) a cycle's step sequence (or each
early-exit chunk of it) is captured as a CUDA graph the second time it is
asked for and replayed from then on; its first run launches the kernels
directly.
"""
from __future__ import annotations

import math
import time
import weakref
from typing import Any, Callable, Dict, List, Optional, Sequence, Tuple, Union

import torch
from torch import Tensor

from .. import _lib


class DiagonalPreconditioner:
    """x -> pinv * x (the form setup_preconditioner builds; pinv is read by the kernels)."""

    def __init__(self, pinv: Tensor):
        self.pinv = pinv

    def __call__(self, x: Tensor) -> Tensor:
        return self.pinv.to(x.device, x.dtype) * x


def setup_preconditioner(method: Optional[str], A_diag: Optional[Tensor] = None, areas: Optional[Tensor] = None,
                         logger: Optional[Any] = None) -> Optional[DiagonalPreconditioner]:
    """Same rules as bem_solver.py:36-117 (non-finite / |d| < 1e-18 entries act as identity)."""
    if method is None or method == "none":
        return None
    if method in ("diag", "jacobi"):
        if A_diag is None:
            if areas is None:
                return None
            method = "mass"
        else:
            d = A_diag.clone()
            bad = (~torch.isfinite(d)) | (d.abs() < 1e-18)
            d[bad] = 1.0
            return DiagonalPreconditioner(1.0 / d)
    if method == "mass":
        if areas is None:
            return None
        d = areas.clone()
        bad = (~torch.isfinite(d)) | (d.abs() < 1e-18)
        if not torch.any(~bad):
            return None
        d[bad] = 1.0
        return DiagonalPreconditioner(1.0 / d)
    return None


def _info(iters, resid, success, code, resid_true0, tol_abs, used_precond, **extra):
    d = dict(iters=int(iters), resid=float(resid), success=bool(success), code=int(code),
             resid_true0=float(resid_true0), tol_abs=float(tol_abs), used_preconditioner=bool(used_precond))
    d.update(extra)
    return d


class _Krylov:
    """Device buffers of one GMRES run."""

    def __init__(self, n: int, restart: int, dtype: torch.dtype, device: torch.device):
        L = _lib.load_library()
        self.n, self.restart, self.dtype, self.device = n, restart, dtype, device
        self.code = _lib.dtype_code(dtype)
        self.V = torch.zeros(restart + 1, n, dtype=dtype, device=device)
        self.H = torch.zeros(restart + 1, restart, dtype=torch.float64, device=device)
        self.g = torch.zeros(restart + 1, dtype=torch.float64, device=device)
        self.cs = torch.zeros(restart, dtype=torch.float64, device=device)
        self.sn = torch.zeros(restart, dtype=torch.float64, device=device)
        self.scal = torch.zeros(5 + restart, dtype=torch.float64, device=device)
        self.w = torch.zeros(n, dtype=dtype, device=device)
        nbytes = int(L.edfmm_gmres_work_bytes(n, restart))
        self.work = torch.zeros((nbytes + 7) // 8, dtype=torch.float64, device=device)
        self.L = L

    def start(self, b: Tensor, ax: Tensor, pinv: Optional[Tensor]):
        P = _lib.ptr
        _lib.check(self.L.edfmm_gmres_start(self.n, self.code, self.restart, P(b), P(ax), P(pinv), P(self.V[0]),
                                            P(self.g), P(self.scal), P(self.work), _lib.stream_handle(self.device)),
                   "edfmm_gmres_start")

    def arnoldi(self, j: int, av: Tensor, pinv: Optional[Tensor]):
        P = _lib.ptr
        _lib.check(self.L.edfmm_gmres_arnoldi(self.n, self.code, self.restart, j, P(self.V), P(av), P(pinv), P(self.H),
                                              P(self.g), P(self.cs), P(self.sn), P(self.scal), P(self.w),
                                              P(self.work), _lib.stream_handle(self.device)), "edfmm_gmres_arnoldi")

    def update(self, m: int, x: Tensor):
        P = _lib.ptr
        _lib.check(self.L.edfmm_gmres_update(self.n, self.code, self.restart, m, P(self.V), P(self.H), P(self.g), P(x),
                                             P(self.work), _lib.stream_handle(self.device)), "edfmm_gmres_update")


# Krylov buffers and captured step graphs kept with the operator object:
# repeated solves with the same operator replay the graphs instead of
# capturing them again (a graph bakes in the buffer addresses it was captured
# with, so the buffers live as long as the graphs).
_GRAPH_CACHE: "weakref.WeakKeyDictionary[Any, Dict[tuple, Dict[str, Any]]]" = weakref.WeakKeyDictionary()


def _graph_workspace(A: Any, key: tuple, make: Callable[[], Dict[str, Any]]) -> Dict[str, Any]:
    try:
        per = _GRAPH_CACHE.setdefault(A, {})
    except TypeError:  # the operator cannot be weakly referenced: no reuse
        return make()
    # graphs captured while the operator launched other kernels (an FP64
    # plan switched between IEEE and two-float arithmetic) are not reused
    state = getattr(A, "graph_state", None)
    if state is not None:
        key = key + (state(),)
    ws = per.get(key)
    if ws is None:
        ws = per[key] = make()
    return ws


@torch.no_grad()
def gmres_restart(A: Callable[[Tensor], Tensor], b: Tensor, M: Optional[Callable[[Tensor], Tensor]] = None,
                  restart: int = 80, tol: float = 1e-8, maxiter: int = 500, logger: Optional[Any] = None,
                  x0: Optional[Tensor] = None, telemetry: Optional[Any] = None, pass_index: int = 0,
                  live_control_poll_fn: Optional[Callable[[], Dict[str, Any]]] = None, log_every: int = 1, *,
                  callback: Optional[Callable[[int, float, Dict[str, Any]], None]] = None,
                  callback_context: Optional[Dict[str, Any]] = None,
                  precond: Optional[Union[str, Callable[[Tensor], Tensor]]] = None, areas: Optional[Tensor] = None,
                  A_diag: Optional[Tensor] = None, validate_operators: bool = False, use_graph: Union[bool, str] = "auto",
                  early_exit: Optional[int] = None, final_check: bool = True,
                  _retry_without_precond: bool = False) -> Tuple[Tensor, Dict[str, Any]]:
    """Restarted GMRES with the reference's semantics (see the module docstring).

    ``early_exit=c`` (not in the reference) lets a cycle end before ``restart``
    steps: every ``c`` steps the device's inner residual estimate is read, and
    the cycle ends once it is below ``tol`` times the first cycle's
    preconditioned residual norm; the true-residual test then decides as usual.
    With ``final_check=False`` (also not in the reference) a cycle that ends
    on that estimate returns at once (code 0, ``converged_on="estimate"``)
    instead of applying the operator once more for the true residual: for
    callers that compute the residual themselves (iterative refinement);
    such a solve from x0 = None also takes the zero start's residual as b
    without applying the operator.
    """
    if restart <= 0:
        raise ValueError("restart must be positive")
    if maxiter <= 0:
        raise ValueError("maxiter must be positive")
    if restart > 256:
        raise ValueError("restart must be <= 256")
    _lib.load_library()
    orig_dtype, orig_device = b.dtype, b.device
    dev = orig_device if orig_device.type == "cuda" else torch.device("cuda", torch.cuda.current_device())
    N = int(b.numel())
    work_dtype = torch.float64 if (N <= 64 and orig_dtype in (torch.float16, torch.bfloat16, torch.float32)) \
        else orig_dtype
    if work_dtype not in (torch.float32, torch.float64):
        work_dtype = torch.float32

    def A_apply(v: Tensor) -> Tensor:
        if work_dtype == orig_dtype and orig_device.type == "cuda":
            return A(v)
        out = A(v.to(dtype=orig_dtype, device=orig_device))
        return out.to(dtype=work_dtype, device=dev)

    # preconditioner: diagonal forms run inside the kernels, others in Python
    if M is None and precond is not None:
        M_local = setup_preconditioner(precond, A_diag=A_diag, areas=areas, logger=logger) if isinstance(precond, str) \
            else (precond if callable(precond) else None)
    else:
        M_local = M
    if M_local is not None:
        probe = torch.ones(N, dtype=work_dtype, device=dev)
        try:
            Mp = M_local(probe.to(orig_dtype).to(orig_device)).to(dev, work_dtype)
            if Mp.shape != b.shape or not torch.isfinite(Mp).all():
                M_local = None
        except Exception:
            M_local = None
    pinv = None
    M_python = None
    if isinstance(M_local, DiagonalPreconditioner):
        pinv = M_local.pinv.to(dev, work_dtype).contiguous()
    elif M_local is not None:
        M_python = M_local
    used_pc = M_local is not None

    if validate_operators:
        probe = torch.randn(N, dtype=work_dtype, device=dev)
        probe = probe / probe.norm()
        try:
            Ap = A_apply(probe)
        except Exception:
            return b.to(dtype=orig_dtype), _info(0, float("nan"), False, 4, float("nan"), float("nan"), False)
        if Ap.shape != b.shape or not torch.isfinite(Ap).all():
            return b.to(dtype=orig_dtype), _info(0, float("nan"), False, 4, float("nan"), float("nan"), False)

    def retry():
        return gmres_restart(A=A, b=b, M=None, restart=restart, tol=tol, maxiter=maxiter, logger=logger, x0=x0,
                             telemetry=telemetry, pass_index=pass_index, live_control_poll_fn=live_control_poll_fn,
                             log_every=log_every, callback=callback, callback_context=callback_context, precond=None,
                             areas=None, validate_operators=False, use_graph=use_graph, early_exit=early_exit,
                             _retry_without_precond=True)

    can_retry = used_pc and not _retry_without_precond and N <= 512
    x = torch.zeros(N, dtype=work_dtype, device=dev) if x0 is None else x0.to(dev, work_dtype).clone()
    b_work = b.to(dev, work_dtype).contiguous()
    want_graph = (use_graph is True) or (use_graph == "auto" and bool(getattr(A, "capturable", False))
                                          and M_python is None and work_dtype == orig_dtype
                                          and orig_device.type == "cuda")
    if want_graph and M_python is None:
        ws = _graph_workspace(A, ("gmres", N, restart, work_dtype, dev, pinv is not None), lambda: dict(
            K=_Krylov(N, restart, work_dtype, dev), av=torch.empty(N, dtype=work_dtype, device=dev),
            pinv=None if pinv is None else torch.empty_like(pinv), graphs={}))
        if pinv is not None:
            ws["pinv"].copy_(pinv)
            pinv = ws["pinv"]
    else:
        ws = dict(K=_Krylov(N, restart, work_dtype, dev), av=torch.empty(N, dtype=work_dtype, device=dev),
                  graphs={})
    K, av = ws["K"], ws["av"]

    # refinement callers (final_check=False) skip A(0) at a zero start; the
    # default keeps the reference's r = b - A(0), which also screens the
    # operator for non-finite output
    x_is_zero = [x0 is None and not final_check]

    def start_cycle():
        ax = torch.zeros_like(b_work) if x_is_zero[0] else A_apply(x)
        if M_python is None:
            K.start(b_work, ax, pinv)
        else:  # generic preconditioner: precondition on the host side of the call
            rt = b_work - ax
            K.start(M_python(rt).to(dev, work_dtype).contiguous(), torch.zeros_like(rt), None)
            K.scal[0] = torch.linalg.norm(rt.double())

    def inner_steps(steps: int, j0: int = 0):
        for j in range(j0, j0 + steps):
            y = A_apply(K.V[j])
            if M_python is not None:
                y = M_python(y).to(dev, work_dtype)
            av.copy_(y)
            K.arnoldi(j, av, pinv if M_python is None else None)

    graphs: Dict[Tuple[int, int], Any] = ws["graphs"]
    seen = ws.setdefault("seen", set())

    def run_steps(j0: int, count: int):
        """Arnoldi steps j0 .. j0+count-1, as a captured graph when allowed.
        A step sequence is captured the second time it is asked for (a later
        cycle, or a later solve with the same operator) and replayed from
        then on; its first run launches the kernels directly, since a graph
        that is never replayed costs more to capture and instantiate than
        it saves (a one-cycle solve on a fresh operator)."""
        if not want_graph:
            inner_steps(count, j0)
            return
        key = (j0, count)
        if key not in graphs and key not in seen:
            seen.add(key)
            inner_steps(count, j0)
            return
        if key not in graphs:
            # the eager first run has set up the operator's lazy state
            g = torch.cuda.CUDAGraph()
            l0 = _lib.launch_count()
            with torch.cuda.graph(g):
                inner_steps(count, j0)
            n_k = _lib.launch_count() - l0
            _lib.note_graph_replay(-n_k)  # captured, not executed
            graphs[key] = (g, n_k)
        g, n_k = graphs[key]
        g.replay()
        _lib.note_graph_replay(n_k)

    total_iters = 0
    beta_first = float("nan")
    tol_abs = float("nan")
    r_true_norm = float("nan")
    r_norm = float("nan")
    max_cycles = max(1, (maxiter + restart - 1) // restart)
    for cycle in range(max_cycles + 1):
        start_cycle()
        scal = K.scal[:2].cpu()
        r_true_norm, beta = float(scal[0]), float(scal[1])
        if cycle == 0:
            if not math.isfinite(r_true_norm):
                return x.to(orig_dtype).to(orig_device), _info(0, r_true_norm, False, 3, r_true_norm, float("nan"),
                                                               used_pc)
            if not math.isfinite(beta):
                if can_retry or (used_pc and not _retry_without_precond):
                    return retry()
                return x.to(orig_dtype).to(orig_device), _info(0, r_true_norm, False, 7, r_true_norm, float("nan"),
                                                               used_pc)
            init_true = r_true_norm if r_true_norm > 1e-16 else 1.0
            tol_abs = max(tol * init_true, tol * 1e-12, 1e-12)
            beta_first = beta
        else:
            if not math.isfinite(r_true_norm):
                if can_retry:
                    return retry()
                return x.to(orig_dtype).to(orig_device), _info(total_iters, r_true_norm, False, 6, r_true_norm, tol_abs,
                                                               used_pc)
            r_norm = beta
            if r_true_norm <= tol_abs:
                return x.to(orig_dtype).to(orig_device), _info(total_iters, r_true_norm, True, 0, r_true_norm, tol_abs,
                                                               used_pc, converged_on="true")
            if total_iters >= maxiter:
                break
        if live_control_poll_fn is not None:
            try:
                state = live_control_poll_fn() or {}
            except Exception:
                state = {}
            if state.get("terminate"):
                return x.to(orig_dtype).to(orig_device), _info(total_iters, float("nan"), False, 2, r_true_norm,
                                                               tol_abs, used_pc)
        steps = min(restart, maxiter - total_iters)
        met_estimate = False
        if early_exit:
            chunk = max(1, int(early_exit))
            j0 = 0
            while j0 < steps:
                cnt = min(chunk, steps - j0)
                run_steps(j0, cnt)
                j0 += cnt
                tail = K.scal[2:5 + restart].cpu()
                est = float(tail[2 + j0 - 1])
                if tail[0] >= 0 or tail[1] != 0 or not math.isfinite(est) or est <= tol * beta_first:
                    met_estimate = tail[0] < 0 and tail[1] == 0 and math.isfinite(est) and est <= tol * beta_first
                    break
            steps = j0
        elif want_graph and steps == restart:
            run_steps(0, steps)
        else:
            inner_steps(steps)
        total_iters += steps
        scal = K.scal.cpu()
        breakdown = int(scal[2]) if scal[2] >= 0 else -1
        nonfinite = bool(scal[3] != 0)
        ests = scal[4:4 + steps].tolist()
        if callback is not None:
            ctx = dict(callback_context or {})
            ctx.setdefault("pass_index", int(pass_index))
            for k, e in enumerate(ests if breakdown < 0 else ests[:breakdown]):
                try:
                    callback(total_iters - steps + k + 1, float(e), dict(ctx, arnoldi_dim=k + 1))
                except Exception:
                    pass
        m_use = breakdown if breakdown >= 0 else steps
        if breakdown >= 0 and can_retry:
            return retry()
        if nonfinite:
            bad = next((k for k, e in enumerate(ests) if not math.isfinite(e)), steps)
            if bad < m_use:
                if can_retry:
                    return retry()
                return x.to(orig_dtype).to(orig_device), _info(total_iters, float("nan"), False, 5, r_true_norm,
                                                               tol_abs, used_pc)
        if m_use == 0:
            if can_retry:
                return retry()
            return x.to(orig_dtype).to(orig_device), _info(total_iters, r_norm, False, 2, r_true_norm, tol_abs, used_pc)
        K.update(m_use, x)
        x_is_zero[0] = False
        if met_estimate and not final_check:
            return x.to(orig_dtype).to(orig_device), _info(total_iters, est, True, 0, r_true_norm, tol_abs, used_pc,
                                                           converged_on="estimate")
    if can_retry:
        return retry()
    return x.to(orig_dtype).to(orig_device), _info(total_iters, r_norm, False, 1, r_true_norm, tol_abs, used_pc)


class _BatchKrylov:
    """Device buffers of one batched GMRES run (K instances back to back)."""

    ACTIVE, TOTAL, RTRUE, TOLABS, NONFIN = 8, 9, 0, 6, 3

    def __init__(self, segments: List[int], restart: int, dtype: torch.dtype, device: torch.device):
        L = _lib.load_library()
        self.L = L
        self.n = int(segments[-1])
        self.K = len(segments) - 1
        lens = [segments[i + 1] - segments[i] for i in range(self.K)]
        if min(lens) <= 0:
            raise ValueError("every instance must own at least one row")
        self.max_seg = max(lens)
        self.restart, self.dtype, self.device = restart, dtype, device
        self.code = _lib.dtype_code(dtype)
        self.soff = torch.tensor(segments, dtype=torch.int64, device=device)
        self.V = torch.zeros(restart + 1, self.n, dtype=dtype, device=device)
        self.w = torch.zeros(self.n, dtype=dtype, device=device)
        cols = int(L.edfmm_bgmres_state_cols(restart))
        self.state = torch.zeros(self.K, cols, dtype=torch.float64, device=device)
        nbytes = int(L.edfmm_bgmres_work_bytes(self.K, self.max_seg, restart))
        self.work = torch.zeros((nbytes + 7) // 8, dtype=torch.float64, device=device)

    def _head(self):
        return (self.n, self.code, self.K, _lib.ptr(self.soff), self.max_seg, self.restart)

    def start(self, b: Tensor, ax: Tensor, pinv: Optional[Tensor], tol: Tensor, first: bool):
        P = _lib.ptr
        _lib.check(self.L.edfmm_bgmres_start(*self._head(), P(b), P(ax), P(pinv), P(self.V[0]), P(tol),
                                             1 if first else 0, P(self.state), P(self.work),
                                             _lib.stream_handle(self.device)), "edfmm_bgmres_start")

    def arnoldi(self, j: int, av: Tensor, pinv: Optional[Tensor]):
        P = _lib.ptr
        _lib.check(self.L.edfmm_bgmres_arnoldi(*self._head(), j, P(self.V), P(av), P(pinv), P(self.w),
                                               P(self.state), P(self.work), _lib.stream_handle(self.device)),
                   "edfmm_bgmres_arnoldi")

    def update(self, m: int, x: Tensor):
        P = _lib.ptr
        _lib.check(self.L.edfmm_bgmres_update(*self._head(), m, P(self.V), P(x), P(self.state), P(self.work),
                                              _lib.stream_handle(self.device)), "edfmm_bgmres_update")


@torch.no_grad()
def gmres_batched(A: Callable[[Tensor], Tensor], b: Tensor, segments: List[int], *, restart: int = 40,
                  tol: Union[float, Sequence[float], Tensor] = 1e-8, maxiter: int = 500,
                  A_diag: Optional[Tensor] = None, x0: Optional[Tensor] = None, use_graph: bool = True,
                  check_every: int = 8) -> Tuple[Tensor, Dict[str, Any]]:
    """Restarted GMRES on K independent systems at once (not in the reference).

    ``segments`` are the K+1 row offsets of the instances in ``b``; ``A`` must
    be block diagonal over them (a batched plan's operator).  Every instance
    runs the algorithm of ``gmres_restart`` with Jacobi preconditioning by
    ``A_diag`` in its own Krylov space: its cycle ends at the step where its
    residual estimate meets ``tol_k`` times its first preconditioned residual,
    and it is done when its true residual at a cycle start is within
    ``tol_k`` of its initial one.  One operator application per step serves
    all instances still iterating; finished ones contribute zero rows.  A
    negative ``tol_k`` leaves instance k untouched.  The host reads the active
    flags every ``check_every`` steps (one captured graph per chunk).

    Returns x and a dict with ``iters`` (operator applications), per-instance
    ``instance_iters``, ``converged`` (bool per instance), ``rel_resid`` (true
    residual at the last cycle start over the initial one) and ``code``
    (0 all converged, 1 iteration limit, 5 non-finite values).
    """
    if restart <= 0 or restart > 256:
        raise ValueError("restart must be in [1, 256]")
    if maxiter <= 0:
        raise ValueError("maxiter must be positive")
    segments = [int(v) for v in segments]
    if segments[0] != 0 or segments[-1] != b.numel() or any(segments[i + 1] < segments[i]
                                                             for i in range(len(segments) - 1)):
        raise ValueError("segments must be non-decreasing offsets from 0 to len(b)")
    dev = b.device
    if dev.type != "cuda":
        raise RuntimeError("gmres_batched needs CUDA tensors")
    dtype = b.dtype
    if dtype not in (torch.float32, torch.float64):
        raise ValueError("b must be float32 or float64")
    K = len(segments) - 1
    tolv = torch.as_tensor(tol, dtype=torch.float64).reshape(-1).to(dev)
    if tolv.numel() == 1:
        tolv = tolv.expand(K).contiguous()
    if tolv.numel() != K:
        raise ValueError("tol must be a scalar or one value per instance")
    pinv = None
    if A_diag is not None:
        pinv = setup_preconditioner("jacobi", A_diag=A_diag).pinv.to(dev, dtype).contiguous()
    if use_graph:
        ws = _graph_workspace(A, ("batched", tuple(segments), restart, dtype, dev, pinv is not None), lambda: dict(
            Kr=_BatchKrylov(segments, restart, dtype, dev), av=torch.empty_like(b),
            pinv=None if pinv is None else torch.empty_like(pinv), graphs={}))
        if pinv is not None:
            ws["pinv"].copy_(pinv)
            pinv = ws["pinv"]
    else:
        ws = dict(Kr=_BatchKrylov(segments, restart, dtype, dev), av=torch.empty_like(b), graphs={})
    Kr, av = ws["Kr"], ws["av"]
    x = torch.zeros_like(b) if x0 is None else x0.to(dev, dtype).clone()
    b = b.contiguous()

    def steps_eager(j0: int, count: int):
        for j in range(j0, j0 + count):
            av.copy_(A(Kr.V[j]))
            Kr.arnoldi(j, av, pinv)

    graphs: Dict[Tuple[int, int], Any] = ws["graphs"]
    seen = ws.setdefault("seen", set())

    def run_steps(j0: int, count: int):
        # captured the second time a step sequence is asked for (as in
        # gmres_restart): its first run launches the kernels directly
        if not use_graph:
            steps_eager(j0, count)
            return
        key = (j0, count)
        if key not in graphs and key not in seen:
            seen.add(key)
            steps_eager(j0, count)
            return
        if key not in graphs:
            # the eager first run has set up the operator's lazy state
            g = torch.cuda.CUDAGraph()
            l0 = _lib.launch_count()
            with torch.cuda.graph(g):
                steps_eager(j0, count)
            n_k = _lib.launch_count() - l0
            _lib.note_graph_replay(-n_k)  # captured, not executed
            graphs[key] = (g, n_k)
        g, n_k = graphs[key]
        g.replay()
        _lib.note_graph_replay(n_k)

    # Operators of batched plans skip the rows of instances that have left
    # their cycle (the active column of the state) during the Arnoldi steps;
    # the cycle starts apply the whole operator.
    set_mask = getattr(A, "set_active_mask", None)
    active_col = Kr.state[:, Kr.ACTIVE]  # a strided view: flags[k * cols]

    def mask(on: bool):
        if set_mask is not None:
            set_mask(active_col if on else None, Kr.state.shape[1])

    chunk = max(1, int(check_every))
    total = 0
    r0 = None
    code = 1
    max_cycles = max(1, (maxiter + restart - 1) // restart)
    try:
        for cycle in range(max_cycles + 1):
            mask(False)
            Kr.start(b, A(x), pinv, tolv, cycle == 0)
            st = Kr.state[:, :10].cpu()
            if cycle == 0:
                r0 = st[:, Kr.RTRUE].clone()
            if bool((st[:, Kr.NONFIN] != 0).any()):
                code = 5
                break
            if not bool((st[:, Kr.ACTIVE] != 0).any()):
                code = 0
                break
            if total >= maxiter:
                code = 1
                break
            steps = min(restart, maxiter - total)
            j0 = 0
            mask(True)
            while j0 < steps:
                cnt = min(chunk, steps - j0)
                run_steps(j0, cnt)
                j0 += cnt
                if not bool((Kr.state[:, Kr.ACTIVE] != 0).any()):
                    break
            mask(False)
            total += j0
            Kr.update(j0, x)
    finally:
        mask(False)
    st = Kr.state[:, :10].cpu()
    r0s = torch.where(r0 > 0, r0, torch.ones_like(r0))
    converged = (st[:, Kr.RTRUE] <= st[:, Kr.TOLABS])
    return x, dict(iters=total, instance_iters=st[:, Kr.TOTAL].to(torch.int64).tolist(),
                   converged=converged.tolist(), rel_resid=(st[:, Kr.RTRUE] / r0s).tolist(), code=code,
                   success=code == 0)


__all__ = ["DiagonalPreconditioner", "setup_preconditioner", "gmres_restart", "gmres_batched"]
