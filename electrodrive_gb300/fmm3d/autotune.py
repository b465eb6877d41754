"""FMM autotuner with a persisted cache (electrodrive/fmm3d/autotune.py:66-849).

``autotune_for_problem(base_cfg, problem_size, ...)`` keeps the reference's
signature, dry-run default, candidate grid (expansion order {p-2, p, p+2,
p+4}, MAC theta {0.6, 1, 1.25} x theta, leaf size {leaf/2, leaf, 2 leaf}),
selection rule (fastest candidate within ``target_rel_error`` of the direct
sum, ties to the smaller order) and JSON cache (records of hardware
fingerprint, problem-size bucket = next power of two, config and metrics,
at ``$ELECTRODRIVE_FMM3D_AUTOTUNE_CACHE`` or the user cache directory).
On the GPU every candidate is a libedfmm plan timed with CUDA events, and
the search also covers the launch shapes of the matvec
(``Plan.set_launch``: the near field on a second stream beside the far field
or fused after it); the chosen shapes are stored with the config
(``TuningResult.launch``) and reapplied by :func:`apply_launch`.  The
accuracy check is the FP64 direct sum at up to 1,024 sampled targets (the
reference compares all points of a 4,096-point cloud on the CPU).
"""
from __future__ import annotations

import json
import math
import os
import platform
import statistics
from dataclasses import dataclass, field
from pathlib import Path
from typing import Any, Dict, Iterable, List, Optional, Tuple

import torch

from .. import _lib
from .config import FmmConfig

AUTOTUNE_CACHE_ENV_VAR = "ELECTRODRIVE_FMM3D_AUTOTUNE_CACHE"
AUTOTUNE_CACHE_FILENAME = "fmm3d_autotune.json"


@dataclass
class TuningResult:
    """The selected configuration, its metrics and the launch shapes chosen
    with it (``launch``: keyword arguments of ``Plan.set_launch``)."""

    config: FmmConfig
    metrics: Dict[str, float]
    launch: Dict[str, int] = field(default_factory=dict)


def bucket_problem_size(n: int) -> int:
    """Problem sizes rounded up to the next power of two (the reference's buckets)."""
    if n <= 0:
        return 1
    return 1 << int(math.ceil(math.log2(n)))


def hardware_fingerprint(device: Optional[torch.device] = None) -> str:
    """Host name, OS, architecture and the GPU's name, SM count and memory."""
    parts: List[str] = [platform.node() or "unknown-host", platform.system() or "unknown-os",
                        platform.machine() or "unknown-arch"]
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    if dev.type == "cuda" and torch.cuda.is_available():
        props = torch.cuda.get_device_properties(dev.index or 0)
        parts += ["cuda", props.name.replace(" ", "_"), str(props.multi_processor_count), str(props.total_memory)]
    else:
        parts.append("cpu")
    return "|".join(parts)


def cache_path() -> Path:
    env = os.environ.get(AUTOTUNE_CACHE_ENV_VAR)
    if env:
        return Path(env)
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return Path(base) / "electrodrive_gb300" / AUTOTUNE_CACHE_FILENAME


def _read_cache() -> Dict[str, Any]:
    path = cache_path()
    try:
        with path.open("r", encoding="utf8") as f:
            raw = json.load(f)
        return raw if isinstance(raw, dict) else {"records": []}
    except Exception:
        return {"records": []}


def load_best(fingerprint: str, bucket: int, target_rel_error: float, *, kind: str = "fmm",
              precision: Optional[str] = None, signature: Optional[str] = None) -> Optional[Dict[str, Any]]:
    """The fastest cached record of this machine, bucket and kind (and
    problem ``signature``, when given) that meets ``target_rel_error``
    (None if there is none)."""
    best, best_t = None, float("inf")
    for rec in _read_cache().get("records", []):
        if rec.get("fingerprint") != fingerprint or int(rec.get("problem_size_bucket", -1)) != int(bucket):
            continue
        if rec.get("kind", "fmm") != kind:
            continue
        if signature is not None and rec.get("signature") != signature:
            continue
        if precision is not None and rec.get("config", {}).get("precision") != precision:
            continue
        m = rec.get("metrics", {})
        if float(m.get("rel_l2_error", float("inf"))) > target_rel_error:
            continue
        t = float(m.get("wall_time_s", float("inf")))
        if t < best_t:
            best, best_t = rec, t
    return best


def append_record(record: Dict[str, Any]) -> None:
    """Append one record to the cache file (failures are never fatal)."""
    path = cache_path()
    raw = _read_cache()
    raw.setdefault("records", []).append(record)
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(path.suffix + f".{os.getpid()}.tmp")
        with tmp.open("w", encoding="utf8") as f:
            json.dump(raw, f, indent=2, sort_keys=True)
        os.replace(tmp, path)
    except Exception:
        return


def cfg_to_dict(cfg: FmmConfig) -> Dict[str, Any]:
    return {"kernel": cfg.kernel, "expansion_order": int(cfg.expansion_order), "mac_theta": float(cfg.mac_theta),
            "leaf_size": int(cfg.leaf_size), "backend": cfg.backend, "precision": cfg.precision,
            "use_fft_m2l": bool(cfg.use_fft_m2l), "use_gpu": bool(cfg.use_gpu),
            "use_multi_gpu": bool(cfg.use_multi_gpu), "use_mpi": bool(cfg.use_mpi),
            "p2p_batch_size": None if cfg.p2p_batch_size is None else int(cfg.p2p_batch_size)}


def cfg_from_dict(base: FmmConfig, d: Dict[str, Any]) -> FmmConfig:
    return FmmConfig(kernel=d.get("kernel", base.kernel),
                     expansion_order=int(d.get("expansion_order", base.expansion_order)),
                     mac_theta=float(d.get("mac_theta", base.mac_theta)),
                     leaf_size=int(d.get("leaf_size", base.leaf_size)), backend=d.get("backend", base.backend),
                     precision=d.get("precision", base.precision), use_fft_m2l=bool(d.get("use_fft_m2l", base.use_fft_m2l)),
                     use_gpu=bool(d.get("use_gpu", base.use_gpu)), use_multi_gpu=bool(d.get("use_multi_gpu", base.use_multi_gpu)),
                     use_mpi=bool(d.get("use_mpi", base.use_mpi)), dtype=base.dtype,
                     p2p_batch_size=d.get("p2p_batch_size", base.p2p_batch_size))


def apply_launch(plan: _lib.Plan, launch: Dict[str, int]) -> None:
    """Set a plan's launch shapes from a tuning result."""
    if launch:
        plan.set_launch(**launch)


def candidate_configs(base: FmmConfig, benchmark_size: int) -> Iterable[FmmConfig]:
    """The reference's candidate grid around ``base`` (orders capped at 10,
    the largest this library's kernels take)."""
    p0 = base.expansion_order
    ps = sorted({max(2, p0 - 2), p0, min(p0 + 2, 10), min(p0 + 4, 10)})
    t0 = base.mac_theta
    ts = sorted({float(max(0.15, min(0.85, f * t0))) for f in (0.6, 1.0, 1.25)})
    l0 = base.leaf_size
    lmax = max(16, benchmark_size)
    ls = sorted({max(16, min(l0 // 2, lmax)), max(16, min(l0, lmax)), max(16, min(2 * l0, lmax))})
    for p in ps:
        for t in ts:
            for leaf in ls:
                cfg = FmmConfig(kernel=base.kernel, expansion_order=p, mac_theta=t, leaf_size=leaf,
                                backend=base.backend, precision=base.precision, use_fft_m2l=base.use_fft_m2l,
                                use_gpu=True, use_multi_gpu=base.use_multi_gpu, use_mpi=base.use_mpi,
                                dtype=base.dtype, p2p_batch_size=base.p2p_batch_size)
                try:
                    cfg.validate()
                except Exception:
                    continue
                yield cfg


def time_matvec(plan: _lib.Plan, sigma: torch.Tensor, areas: torch.Tensor, reps: int = 5) -> float:
    """Median matvec time (seconds, CUDA events on the current stream)."""
    stream = torch.cuda.current_stream(plan.device)
    plan.matvec(sigma, areas, None, k_e=1.0)
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.matvec(sigma, areas, None, k_e=1.0)
        e1.record(stream)
        torch.cuda.synchronize(plan.device)
        times.append(e0.elapsed_time(e1) * 1e-3)
    return statistics.median(times)


LAUNCH_CHOICES: Tuple[Dict[str, int], ...] = ({"near_overlap": 1}, {"near_overlap": 0})

# candidates this close to the fastest count as equally fast
TIME_SLACK = 0.05


def select_trial(trials: List[Dict[str, Any]], max_rel_error: float, time_slack: float = TIME_SLACK,
                 inner_tol: Optional[float] = None) -> Optional[Dict[str, Any]]:
    """The inner operator to use among trials (dicts with ``ms`` and
    ``rel_error``) within the accuracy bound.  An operator whose error is a
    fraction e of the tolerance the inner solves must reach (``inner_tol``)
    slows their convergence as e approaches 1, so with ``inner_tol`` the
    choice minimises ms / (1 - e); without it, the most accurate of the
    trials no more than ``time_slack`` slower than the fastest.  None if no
    trial meets the bound."""
    ok = [t for t in trials if t["rel_error"] <= max_rel_error]
    if not ok:
        return None
    if inner_tol is not None:
        return min(ok, key=lambda t: (t["ms"] / max(1.0 - t["rel_error"] / inner_tol, 1e-3), t["rel_error"]))
    fastest = min(t["ms"] for t in ok)
    pool = [t for t in ok if t["ms"] <= (1.0 + time_slack) * fastest]
    return min(pool, key=lambda t: (t["rel_error"], t["ms"]))


def autotune_for_problem(base_cfg: FmmConfig, problem_size: int, *, dry_run: bool = True,
                         target_rel_error: float = 1e-2, max_trials: int = 24, device: Optional[torch.device] = None,
                         use_cache: bool = True, points: Optional[torch.Tensor] = None) -> TuningResult:
    """Autotune the FMM configuration and launch shapes for a problem of
    ``problem_size`` points on this GPU (reference signature; ``points``,
    an addition, benchmarks on the caller's point set instead of a uniform
    cloud).  ``dry_run=True`` returns ``base_cfg`` untouched, as the
    reference does."""
    if problem_size <= 0:
        raise ValueError("problem_size must be positive")
    base_cfg.validate()
    if dry_run:
        return TuningResult(config=base_cfg, metrics={"mode": 0.0, "problem_size": float(problem_size)})
    _lib.load_library()
    dev = torch.device(device) if device is not None and torch.device(device).type == "cuda" else \
        torch.device("cuda", torch.cuda.current_device())
    fingerprint = hardware_fingerprint(dev)
    bucket = bucket_problem_size(problem_size)
    if use_cache:
        rec = load_best(fingerprint, bucket, target_rel_error, precision=base_cfg.precision)
        if rec is not None:
            cfg = cfg_from_dict(base_cfg, rec.get("config", {}))
            cfg.validate()
            metrics = {k: float(v) for k, v in rec.get("metrics", {}).items()}
            metrics.setdefault("problem_size", float(problem_size))
            metrics["from_cache"] = 1.0
            return TuningResult(config=cfg, metrics=metrics, launch=dict(rec.get("launch", {})))
    dt = torch.float64 if base_cfg.precision == "double" else torch.float32
    if points is not None:
        pts = points.to(dev, torch.float64).reshape(-1, 3)
    else:
        n_b = min(int(problem_size), 1 << 18)
        g = torch.Generator().manual_seed(12345)
        pts = torch.rand(n_b, 3, generator=g, dtype=torch.float64).to(dev)
    n = int(pts.shape[0])
    g = torch.Generator().manual_seed(54321)
    sigma64 = torch.randn(n, generator=g, dtype=torch.float64).to(dev)
    areas64 = torch.ones(n, dtype=torch.float64, device=dev)
    idx = torch.randperm(n, generator=g)[:min(n, 1024)].to(dev)
    ref = _direct_at(pts[idx], pts, sigma64, idx)
    best: Optional[Tuple[float, FmmConfig, Dict[str, float], Dict[str, int]]] = None
    for k, cfg in enumerate(candidate_configs(base_cfg, n)):
        if k >= max_trials:
            break
        try:
            plan = _lib.Plan(pts.to(dt).contiguous(), leaf_size=cfg.leaf_size, mac_theta=cfg.mac_theta,
                             expansion_order=cfg.expansion_order)
        except Exception:
            continue
        s, a = sigma64.to(dt), areas64.to(dt)
        v = plan.matvec(s, a, None, k_e=1.0).to(torch.float64)
        err = float(torch.linalg.norm(v[idx] - ref) / torch.linalg.norm(ref))
        if not err <= target_rel_error:
            plan.close()
            continue
        for launch in LAUNCH_CHOICES:
            plan.set_launch(**launch)
            t = time_matvec(plan, s, a)
            metrics = {"problem_size": float(problem_size), "benchmark_size": float(n),
                       "expansion_order": float(cfg.expansion_order), "mac_theta": float(cfg.mac_theta),
                       "leaf_size": float(cfg.leaf_size), "wall_time_s": t, "rel_l2_error": err,
                       "mpts_per_s": n / t / 1e6, "m2l_pairs": float(plan.info.n_m2l_pairs),
                       "p2p_pairs": float(plan.info.n_p2p_pairs)}
            if best is None or t < best[0] * (1 - 1e-3) or (
                    abs(t - best[0]) <= 1e-3 * best[0] and cfg.expansion_order < best[1].expansion_order):
                best = (t, cfg, metrics, dict(launch))
        plan.close()
    if best is None:
        return TuningResult(config=base_cfg, metrics={"mode": 1.0, "problem_size": float(problem_size)})
    _, cfg, metrics, launch = best
    if use_cache:
        append_record({"fingerprint": fingerprint, "problem_size_bucket": bucket, "kind": "fmm",
                       "config": cfg_to_dict(cfg), "launch": launch, "metrics": metrics})
    return TuningResult(config=cfg, metrics=metrics, launch=launch)


def _direct_at(targets: torch.Tensor, sources: torch.Tensor, charges: torch.Tensor, idx: torch.Tensor) -> torch.Tensor:
    """FP64 direct sum sum_j q_j / |x_i - y_j| at the sampled targets x_i =
    sources[idx_i], self terms excluded (exact coordinate differences)."""
    out = torch.zeros(targets.shape[0], dtype=torch.float64, device=targets.device)
    for j0 in range(0, sources.shape[0], 1 << 14):
        src = sources[j0:j0 + (1 << 14)]
        d = torch.cdist(targets, src, compute_mode="donot_use_mm_for_euclid_dist")
        inv = torch.where(d > 0, 1.0 / d, torch.zeros_like(d))
        out += inv @ charges[j0:j0 + (1 << 14)]
    return out


__all__ = ["AUTOTUNE_CACHE_ENV_VAR", "AUTOTUNE_CACHE_FILENAME", "LAUNCH_CHOICES", "TuningResult", "append_record",
           "apply_launch", "autotune_for_problem", "bucket_problem_size", "cache_path", "candidate_configs",
           "cfg_from_dict", "cfg_to_dict", "hardware_fingerprint", "load_best", "time_matvec"]
