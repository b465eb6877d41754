"""ctypes binding of libedfmm.so (declared in include/edfmm.h).

The library is the only compute path of this package: if it is missing, or
no CUDA device is visible, every entry point raises instead of falling back
to a CPU implementation.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional
import os
import re
import threading

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libedfmm.so")
HEADER_PATH = os.path.join(os.path.dirname(_HERE), "include", "edfmm.h")

EDFMM_OK = 0
EDFMM_ERR_ARG = -1
EDFMM_ERR_CUDA = -2
EDFMM_ERR_ALLOC = -3
EDFMM_ERR_UNSUPPORTED = -4
EDFMM_ERR_STATE = -5
EDFMM_F32 = 0
EDFMM_F64 = 1
EDFMM_REFERENCE_PAIR_ORDER = 1
EDFMM_NO_FARFIELD = 2
EDFMM_NO_NEARFIELD = 4
EDFMM_ARITH_NATIVE = 0
EDFMM_ARITH_TWO_FLOAT = 1
EDFMM_LAUNCH_M2L_TF_BLOCK = 1
EDFMM_LAUNCH_NEAR_OVERLAP = 2
EDFMM_LAUNCH_M2L_PACKED = 3
EDFMM_MESH_SPHERE = 1
EDFMM_MESH_TORUS = 2
EDFMM_MESH_PLANE = 3
EDFMM_TARGETS_M2L = 1
EDFMM_TARGETS_L2L = 2
EDFMM_TARGETS_L2P = 3
EDFMM_TARGETS_P2P = 4
EDFMM_TARGETS_LOCALS = 5


class EdfmmError(RuntimeError):
    """A libedfmm call returned a non-zero status."""

    def __init__(self, code: int, where: str, message: str):
        super().__init__(f"{where} failed with status {code}: {message}")
        self.code = code


class PlanInfo(C.Structure):
    _fields_ = [
        ("n_points", C.c_int64),
        ("n_nodes", C.c_int64),
        ("n_leaves", C.c_int64),
        ("n_p2p_pairs", C.c_int64),
        ("n_m2l_pairs", C.c_int64),
        ("p2p_interactions", C.c_int64),
        ("max_level", C.c_int32),
        ("depth_warnings", C.c_int32),
        ("dtype", C.c_int32),
        ("expansion_order", C.c_int32),
        ("leaf_size", C.c_int32),
        ("max_depth", C.c_int32),
        ("mac_theta", C.c_double),
    ]


_lib = None
_lock = threading.Lock()
_vp = C.c_void_p


def _declare(L):
    i32, i64, dbl = C.c_int, C.c_int64, C.c_double
    sig = {
        "edfmm_last_error": (C.c_char_p, []),
        "edfmm_version": (C.c_char_p, []),
        "edfmm_launch_count": (i64, []),
        "edfmm_block_cache_selfcheck": (i32, [C.POINTER(i64)]),
        "edfmm_plan_create": (i32, [_vp, i64, i32, i32, i32, dbl, i32, _vp, C.POINTER(_vp)]),
        "edfmm_plan_create_batch": (i32, [_vp, C.POINTER(i64), i32, i32, i32, i32, dbl, i32, _vp, C.POINTER(_vp)]),
        "edfmm_plan_convert": (i32, [_vp, i32, i32, _vp, C.POINTER(_vp)]),
        "edfmm_plan_destroy": (i32, [_vp]),
        "edfmm_targets_create": (i32, [_vp, _vp, i64, _vp, C.POINTER(_vp)]),
        "edfmm_targets_destroy": (i32, [_vp]),
        "edfmm_targets_info": (i32, [_vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)]),
        "edfmm_targets_export_lists": (i32, [_vp, _vp, _vp, _vp]),
        "edfmm_targets_potential": (i32, [_vp, _vp, _vp, dbl, _vp, i32, _vp]),
        "edfmm_targets_field": (i32, [_vp, _vp, _vp, dbl, _vp, i32, _vp]),
        "edfmm_targets_create_from_plan": (i32, [_vp, _vp, dbl, _vp, C.POINTER(_vp)]),
        "edfmm_targets_stage": (i32, [_vp, i32, _vp, _vp]),
        "edfmm_plan_rebuild_lists": (i32, [_vp, dbl, _vp]),
        "edfmm_plan_set_order": (i32, [_vp, i32, _vp]),
        "edfmm_plan_set_arithmetic": (i32, [_vp, i32, _vp]),
        "edfmm_plan_set_launch": (i32, [_vp, i32, i32]),
        "edfmm_plan_get_launch": (i32, [_vp, i32, C.POINTER(i32)]),
        "edfmm_plan_set_instance_mask": (i32, [_vp, _vp, i32]),
        "edfmm_plan_get_info": (i32, [_vp, C.POINTER(PlanInfo)]),
        "edfmm_plan_export_tree": (i32, [_vp] * 11),
        "edfmm_plan_export_lists": (i32, [_vp, _vp, _vp, _vp]),
        "edfmm_plan_matvec": (i32, [_vp, _vp, _vp, _vp, dbl, _vp, i32, _vp]),
        "edfmm_plan_set_charges": (i32, [_vp, _vp, _vp]),
        "edfmm_plan_p2m": (i32, [_vp, _vp]),
        "edfmm_plan_m2m": (i32, [_vp, _vp]),
        "edfmm_plan_m2l": (i32, [_vp, i32, _vp]),
        "edfmm_plan_l2l": (i32, [_vp, _vp]),
        "edfmm_plan_l2p": (i32, [_vp, _vp, _vp]),
        "edfmm_plan_p2p": (i32, [_vp, _vp, _vp]),
        "edfmm_plan_get_expansions": (i32, [_vp, _vp, _vp, _vp]),
        "edfmm_measure_fp32_peak": (i32, [i32, _vp, C.POINTER(C.c_double)]),
        "edfmm_measure_fp64_peak": (i32, [i32, _vp, C.POINTER(C.c_double)]),
        "edfmm_mesh_grid": (i32, [i32, C.POINTER(C.c_double), _vp, i64, _vp, i64, i64, C.c_int32, _vp, _vp, _vp, _vp]),
        "edfmm_mesh_finish": (i32, [_vp, i64, _vp, _vp, i64, _vp, _vp, _vp, _vp, _vp, C.POINTER(i64), _vp]),
        "edfmm_pcn_num_params": (i64, []),
        "edfmm_pcn_workspace_bytes": (C.c_size_t, [i64]),
        "edfmm_pcn_features": (i32, [_vp, _vp, _vp, _vp, i64, _vp, _vp, C.c_size_t, _vp]),
        "edfmm_pcn_forward": (i32, [_vp, _vp, i64, _vp, _vp, C.c_size_t, _vp]),
        "edfmm_pcn_backward": (i32, [_vp, i64, _vp, _vp, _vp, C.c_size_t, _vp]),
        "edfmm_pcn_loss": (i32, [_vp, _vp, _vp, _vp, i64, _vp, _vp, _vp]),
        "edfmm_pcn_adam": (i32, [_vp, _vp, _vp, _vp, i64, C.c_float, C.c_float, C.c_float, C.c_float, i32, _vp]),
        "edfmm_dense_matvec": (i32, [_vp, _vp, _vp, _vp, i64, i32, dbl, _vp, _vp]),
        "edfmm_dense_matvec_noalloc": (i32, [_vp, _vp, _vp, _vp, i64, i32, dbl, _vp, _vp]),
        "edfmm_dense_workspace_bytes": (C.c_size_t, [i64, i32]),
        "edfmm_dense_matvec_ws": (i32, [_vp, _vp, _vp, _vp, i64, i32, dbl, _vp, _vp, C.c_size_t, _vp]),
        "edfmm_dense_potential_targets": (i32, [_vp, i64, _vp, _vp, _vp, i64, i32, dbl, _vp, _vp]),
        "edfmm_dense_field_targets": (i32, [_vp, i64, _vp, _vp, _vp, i64, i32, dbl, _vp, _vp]),
        "edfmm_self_integrals": (i32, [_vp, _vp, i64, i32, i32, dbl, _vp, _vp]),
        "edfmm_near_targets_correct": (i32, [_vp, i64, _vp, _vp, _vp, _vp, i64, dbl, i32, i32, dbl, _vp, _vp]),
        "edfmm_near_create": (i32, [_vp, _vp, _vp, i64, dbl, i32, i32, dbl, i32, _vp, C.POINTER(_vp)]),
        "edfmm_near_convert": (i32, [_vp, i32, _vp, C.POINTER(_vp)]),
        "edfmm_near_destroy": (i32, [_vp]),
        "edfmm_near_num_pairs": (i64, [_vp]),
        "edfmm_near_export": (i32, [_vp, _vp, _vp, _vp]),
        "edfmm_near_apply": (i32, [_vp, _vp, _vp, _vp, _vp]),
        "edfmm_near_rows": (i32, [_vp, C.POINTER(_vp), C.POINTER(_vp)]),
        "edfmm_near_quadrature_matvec": (i32, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, i64, dbl, i32, i32, _vp, _vp]),
        "edfmm_point_charge_potential": (i32, [_vp, i64, _vp, i32, dbl, i32, _vp, _vp]),
        "edfmm_gmres_work_bytes": (C.c_size_t, [i64, i32]),
        "edfmm_gmres_start": (i32, [i64, i32, i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
        "edfmm_gmres_arnoldi": (i32, [i64, i32, i32, i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
        "edfmm_gmres_update": (i32, [i64, i32, i32, i32, _vp, _vp, _vp, _vp, _vp, _vp]),
        "edfmm_bgmres_state_cols": (C.c_size_t, [i32]),
        "edfmm_bgmres_work_bytes": (C.c_size_t, [i32, i32, i32]),
        "edfmm_bgmres_start": (i32, [i64, i32, i32, _vp, i32, i32, _vp, _vp, _vp, _vp, _vp, i32, _vp, _vp, _vp]),
        "edfmm_bgmres_arnoldi": (i32, [i64, i32, i32, _vp, i32, i32, i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
        "edfmm_bgmres_update": (i32, [i64, i32, i32, _vp, i32, i32, i32, _vp, _vp, _vp, _vp, _vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args


def load_library(require_cuda: bool = True):
    """Load libedfmm.so; raise if it is missing or (by default) CUDA is absent."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"libedfmm.so not found at {LIB_PATH}; build it with "
                    "`python -c 'import __graft_entry__ as g; g.build()'` (nvcc, sm_103a)"
                )
            L = C.CDLL(LIB_PATH)
            _declare(L)
            _lib = L
    if require_cuda and not torch.cuda.is_available():
        raise RuntimeError("electrodrive_gb300 requires a CUDA device (no CPU fallback)")
    return _lib


def header_symbols() -> list[str]:
    """Function names declared in include/edfmm.h."""
    with open(HEADER_PATH) as f:
        txt = f.read()
    return sorted(set(re.findall(r"\b(edfmm_[a-z0-9_]+)\s*\(", txt)))


def check(rc: int, where: str):
    if rc != EDFMM_OK:
        msg = _lib.edfmm_last_error().decode() if _lib is not None else ""
        raise EdfmmError(rc, where, msg)


def ptr(t: torch.Tensor | None):
    return None if t is None else _vp(t.data_ptr())


def stream_handle(device=None):
    return _vp(torch.cuda.current_stream(device).cuda_stream)


def dtype_code(dt: torch.dtype) -> int:
    if dt == torch.float32:
        return EDFMM_F32
    if dt == torch.float64:
        return EDFMM_F64
    raise ValueError(f"unsupported dtype {dt}; expected float32 or float64")


_replayed_launches = 0


def note_graph_replay(kernels_per_replay: int) -> None:
    """Account the library kernels a CUDA-graph replay re-launches (the C
    counter sees them once, when they are captured)."""
    global _replayed_launches
    _replayed_launches += int(kernels_per_replay)


def launch_count() -> int:
    """Library kernel launches so far, graph replays included."""
    return int(load_library(require_cuda=False).edfmm_launch_count()) + _replayed_launches


def measure_fp32_peak(iters: int = 20000) -> float:
    """FP32 FMA throughput of the current device, TFLOP/s."""
    L = load_library()
    out = C.c_double()
    check(L.edfmm_measure_fp32_peak(int(iters), stream_handle(), C.byref(out)), "edfmm_measure_fp32_peak")
    return float(out.value)


def measure_fp64_peak(iters: int = 4000) -> float:
    """FP64 FMA throughput of the current device, TFLOP/s."""
    L = load_library()
    out = C.c_double()
    check(L.edfmm_measure_fp64_peak(int(iters), stream_handle(), C.byref(out)), "edfmm_measure_fp64_peak")
    return float(out.value)


def dense_matvec(centroids, sigma, areas, self_integrals=None, *, k_e: float = 1.0, out=None):
    """Dense single-layer operator on CUDA tensors (edfmm_dense_matvec)."""
    L = load_library()
    n = int(sigma.shape[0])
    dev, dt = sigma.device, sigma.dtype
    for name, t in (("centroids", centroids), ("areas", areas), ("self_integrals", self_integrals)):
        if t is None:
            continue
        if t.device != dev or t.dtype != dt or not t.is_contiguous():
            raise ValueError(f"{name} must be a contiguous {dt} tensor on {dev}")
    if centroids.shape != (n, 3) or areas.shape != (n,) or (self_integrals is not None and self_integrals.shape != (n,)):
        raise ValueError("centroids must be (N, 3) and areas / self_integrals (N,) matching sigma")
    sigma = sigma.contiguous()
    if out is None:
        out = torch.empty_like(sigma)
    with torch.cuda.device(dev):
        check(L.edfmm_dense_matvec(ptr(centroids), ptr(sigma), ptr(areas), ptr(self_integrals), n, dtype_code(dt),
                                   float(k_e), ptr(out), stream_handle(dev)), "edfmm_dense_matvec")
    return out


class Plan:
    """Owns an edfmm_plan: device octree + interaction lists + expansion buffers."""

    def __init__(self, points: torch.Tensor, *, leaf_size: int = 64, max_depth: int = 32,
                 mac_theta: float = 0.5, expansion_order: int = 8, instance_offsets=None):
        """``instance_offsets`` (K + 1 row offsets) makes a batched plan: K
        independent point sets, each with its own tree and lists, applied as
        one block-diagonal operator."""
        L = load_library()
        if points.ndim != 2 or points.shape[-1] != 3:
            raise ValueError(f"points must have shape (N, 3), got {tuple(points.shape)}")
        if not points.is_cuda:
            raise ValueError("Plan expects CUDA points")
        pts = points.contiguous()
        self.device = pts.device
        self.dtype = pts.dtype
        h = _vp()
        self.instance_offsets = None
        with torch.cuda.device(self.device):
            if instance_offsets is None:
                rc = L.edfmm_plan_create(ptr(pts), pts.shape[0], dtype_code(pts.dtype), int(leaf_size),
                                         int(max_depth), float(mac_theta), int(expansion_order),
                                         stream_handle(self.device), C.byref(h))
            else:
                off = [int(x) for x in instance_offsets]
                if off[-1] != pts.shape[0]:
                    raise ValueError("instance_offsets must end at the number of points")
                arr = (C.c_int64 * len(off))(*off)
                rc = L.edfmm_plan_create_batch(ptr(pts), arr, len(off) - 1, dtype_code(pts.dtype), int(leaf_size),
                                               int(max_depth), float(mac_theta), int(expansion_order),
                                               stream_handle(self.device), C.byref(h))
                self.instance_offsets = off
        check(rc, "edfmm_plan_create")
        self._h = h
        self._lib = L
        info = PlanInfo()
        check(L.edfmm_plan_get_info(h, C.byref(info)), "edfmm_plan_get_info")
        self.info = info

    def convert(self, dtype: torch.dtype, expansion_order: Optional[int] = None) -> "Plan":
        """A plan in ``dtype`` (and ``expansion_order``, default this plan's)
        over this plan's partition: tree, lists and instances copied, point
        and node geometry cast, no new tree or list build."""
        order = int(self.info.expansion_order if expansion_order is None else expansion_order)
        h = _vp()
        with torch.cuda.device(self.device):
            check(self._lib.edfmm_plan_convert(self._h, dtype_code(dtype), order, stream_handle(self.device),
                                               C.byref(h)), "edfmm_plan_convert")
        out = Plan.__new__(Plan)
        out.device, out.dtype, out.instance_offsets = self.device, dtype, self.instance_offsets
        out._h, out._lib = h, self._lib
        out._refresh_info()
        return out

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.edfmm_plan_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _refresh_info(self):
        info = PlanInfo()
        check(self._lib.edfmm_plan_get_info(self._h, C.byref(info)), "edfmm_plan_get_info")
        self.info = info

    def rebuild_lists(self, mac_theta: float):
        with torch.cuda.device(self.device):
            check(self._lib.edfmm_plan_rebuild_lists(self._h, float(mac_theta), stream_handle(self.device)),
                  "edfmm_plan_rebuild_lists")
        self._refresh_info()

    def set_arithmetic(self, mode: str):
        """FP64 plans: "two_float" runs M2L and the near field in two-float
        arithmetic on the FP32 pipe (about 48 significant bits); "native"
        restores IEEE FP64."""
        code = {"native": EDFMM_ARITH_NATIVE, "two_float": EDFMM_ARITH_TWO_FLOAT}.get(mode)
        if code is None:
            raise ValueError(f"arithmetic must be 'native' or 'two_float', got {mode!r}")
        with torch.cuda.device(self.device):
            check(self._lib.edfmm_plan_set_arithmetic(self._h, code, stream_handle(self.device)),
                  "edfmm_plan_set_arithmetic")
        self.arithmetic = mode

    _KNOBS = {"m2l_tf_block": EDFMM_LAUNCH_M2L_TF_BLOCK, "near_overlap": EDFMM_LAUNCH_NEAR_OVERLAP,
              "m2l_packed": EDFMM_LAUNCH_M2L_PACKED}

    def set_launch(self, **knobs):
        """Launch shapes: m2l_tf_block (128 or 256), near_overlap (0 or 1)."""
        for k, v in knobs.items():
            if k not in self._KNOBS:
                raise ValueError(f"unknown launch knob {k!r}")
            check(self._lib.edfmm_plan_set_launch(self._h, self._KNOBS[k], int(v)), "edfmm_plan_set_launch")

    def get_launch(self) -> dict:
        out = {}
        for k, code in self._KNOBS.items():
            v = C.c_int()
            check(self._lib.edfmm_plan_get_launch(self._h, code, C.byref(v)), "edfmm_plan_get_launch")
            out[k] = int(v.value)
        return out

    def set_order(self, p: int):
        with torch.cuda.device(self.device):
            check(self._lib.edfmm_plan_set_order(self._h, int(p), stream_handle(self.device)), "edfmm_plan_set_order")
        self._refresh_info()

    # ---------------------------------------------------------------- exports
    def export_tree(self):
        i = self.info
        dev, dt = self.device, self.dtype
        M, N = i.n_nodes, i.n_points
        out = dict(
            index_map=torch.empty(N, dtype=torch.int64, device=dev),
            node_centers=torch.empty(M, 3, dtype=dt, device=dev),
            node_half_extents=torch.empty(M, 3, dtype=dt, device=dev),
            node_radii=torch.empty(M, dtype=dt, device=dev),
            node_levels=torch.empty(M, dtype=torch.int32, device=dev),
            node_parents=torch.empty(M, dtype=torch.int64, device=dev),
            node_children=torch.empty(M, 8, dtype=torch.int64, device=dev),
            node_ranges=torch.empty(M, 2, dtype=torch.int64, device=dev),
            node_is_leaf=torch.empty(M, dtype=torch.bool, device=dev),
        )
        with torch.cuda.device(dev):
            check(self._lib.edfmm_plan_export_tree(
                self._h, ptr(out["index_map"]), ptr(out["node_centers"]), ptr(out["node_half_extents"]),
                ptr(out["node_radii"]), ptr(out["node_levels"]), ptr(out["node_parents"]), ptr(out["node_children"]),
                ptr(out["node_ranges"]), ptr(out["node_is_leaf"]), stream_handle(dev)), "edfmm_plan_export_tree")
        return out

    def targets(self, points: torch.Tensor) -> "Targets":
        """FMM evaluation at arbitrary points (a tree of the points plus the
        interaction lists between this plan's tree and it)."""
        return Targets(self, points)

    def export_lists(self):
        dev = self.device
        p2p = torch.empty(self.info.n_p2p_pairs, 2, dtype=torch.int64, device=dev)
        m2l = torch.empty(self.info.n_m2l_pairs, 2, dtype=torch.int64, device=dev)
        with torch.cuda.device(dev):
            check(self._lib.edfmm_plan_export_lists(self._h, ptr(p2p), ptr(m2l), stream_handle(dev)),
                  "edfmm_plan_export_lists")
        return p2p, m2l

    def expansions(self):
        nc = (self.info.expansion_order + 1) * (self.info.expansion_order + 2) // 2
        cdt = torch.complex64 if self.dtype == torch.float32 else torch.complex128
        Mx = torch.empty(self.info.n_nodes, nc, dtype=cdt, device=self.device)
        Lx = torch.empty(self.info.n_nodes, nc, dtype=cdt, device=self.device)
        with torch.cuda.device(self.device):
            check(self._lib.edfmm_plan_get_expansions(self._h, ptr(Mx), ptr(Lx), stream_handle(self.device)),
                  "edfmm_plan_get_expansions")
        return Mx, Lx

    # ---------------------------------------------------------------- compute
    def _check_vec(self, t: torch.Tensor, name: str):
        if t.device != self.device or t.dtype != self.dtype or t.shape != (self.info.n_points,):
            raise ValueError(f"{name} must be a ({self.info.n_points},) {self.dtype} tensor on {self.device}, "
                             f"got {tuple(t.shape)} {t.dtype} on {t.device}")
        if not t.is_contiguous():
            raise ValueError(f"{name} must be contiguous")

    def matvec(self, sigma, areas, self_integrals=None, *, k_e: float = 1.0, out=None, flags: int = 0):
        self._check_vec(sigma, "sigma")
        self._check_vec(areas, "areas")
        if self_integrals is not None:
            self._check_vec(self_integrals, "self_integrals")
        if out is None:
            out = torch.empty_like(sigma)
        else:
            self._check_vec(out, "out")
        with torch.cuda.device(self.device):
            check(self._lib.edfmm_plan_matvec(self._h, ptr(sigma), ptr(areas), ptr(self_integrals), float(k_e),
                                              ptr(out), int(flags), stream_handle(self.device)), "edfmm_plan_matvec")
        return out

    def set_charges(self, charges):
        self._check_vec(charges, "charges")
        with torch.cuda.device(self.device):
            check(self._lib.edfmm_plan_set_charges(self._h, ptr(charges), stream_handle(self.device)),
                  "edfmm_plan_set_charges")

    @property
    def n_instances(self) -> int:
        return 1 if self.instance_offsets is None else len(self.instance_offsets) - 1

    def set_instance_mask(self, flags: Optional[torch.Tensor], stride: int = 1):
        """Batched plans: skip the M2L rows and near-field leaves of instances
        whose flags[k * stride] is 0 (an FP64 device tensor kept alive by the
        caller); None removes the mask."""
        check(self._lib.edfmm_plan_set_instance_mask(self._h, None if flags is None else ptr(flags), int(stride)),
              "edfmm_plan_set_instance_mask")

    def stage(self, name: str, *args):
        fn = getattr(self._lib, f"edfmm_plan_{name}")
        with torch.cuda.device(self.device):
            check(fn(self._h, *args, stream_handle(self.device)), f"edfmm_plan_{name}")

    def p2p(self):
        out = torch.empty(self.info.n_points, dtype=self.dtype, device=self.device)
        self.stage("p2p", ptr(out))
        return out

    def l2p(self):
        out = torch.empty(self.info.n_points, dtype=self.dtype, device=self.device)
        self.stage("l2p", ptr(out))
        return out


class Targets:
    """Owns an edfmm_targets: evaluation points of a plan's charges."""

    def __init__(self, plan: "Plan", points: torch.Tensor):
        if points.ndim != 2 or points.shape[-1] != 3 or not points.is_cuda:
            raise ValueError("targets must be CUDA points of shape (M, 3)")
        pts = points.to(plan.dtype).contiguous()
        self.plan = plan  # keeps the source plan alive
        self.device = plan.device
        self.n = int(pts.shape[0])
        L = plan._lib
        self._lib = L
        h = _vp()
        with torch.cuda.device(self.device):
            check(L.edfmm_targets_create(plan.handle, ptr(pts), self.n, stream_handle(self.device), C.byref(h)),
                  "edfmm_targets_create")
        self._h = h
        v = [C.c_int64() for _ in range(4)]
        check(L.edfmm_targets_info(h, *[C.byref(x) for x in v]), "edfmm_targets_info")
        self.n_nodes, self.n_p2p_pairs, self.n_m2l_pairs, self.p2p_interactions = (int(x.value) for x in v)

    @classmethod
    def from_plan(cls, plan: "Plan", target_plan: "Plan", mac_theta: float) -> "Targets":
        """Two-tree lists between ``plan``'s tree and the tree ``target_plan``
        already holds (copied), built with ``mac_theta``."""
        if target_plan.dtype != plan.dtype or target_plan.device != plan.device:
            raise ValueError("source and target trees must share a device and dtype")
        self = cls.__new__(cls)
        self.plan = plan
        self.device = plan.device
        self.n = int(target_plan.info.n_points)
        self.order = int(plan.info.expansion_order)
        self._lib = plan._lib
        h = _vp()
        with torch.cuda.device(self.device):
            check(self._lib.edfmm_targets_create_from_plan(plan.handle, target_plan.handle, float(mac_theta),
                                                           stream_handle(self.device), C.byref(h)),
                  "edfmm_targets_create_from_plan")
        self._h = h
        v = [C.c_int64() for _ in range(4)]
        check(self._lib.edfmm_targets_info(h, *[C.byref(x) for x in v]), "edfmm_targets_info")
        self.n_nodes, self.n_p2p_pairs, self.n_m2l_pairs, self.p2p_interactions = (int(x.value) for x in v)
        return self

    def stage(self, stage: int, out: Optional[torch.Tensor] = None) -> Optional[torch.Tensor]:
        """One two-tree stage (EDFMM_TARGETS_*) on the source plan's current
        multipoles / charges; L2P and P2P return tree-order potentials of the
        target points, LOCALS the target local expansions."""
        dt = self.plan.dtype
        if stage in (EDFMM_TARGETS_L2P, EDFMM_TARGETS_P2P) and out is None:
            out = torch.empty(self.n, dtype=dt, device=self.device)
        elif stage == EDFMM_TARGETS_LOCALS and out is None:
            p = int(self.plan.info.expansion_order)
            cdt = torch.complex64 if dt == torch.float32 else torch.complex128
            out = torch.empty(self.n_nodes, (p + 1) * (p + 2) // 2, dtype=cdt, device=self.device)
        with torch.cuda.device(self.device):
            check(self._lib.edfmm_targets_stage(self._h, int(stage), ptr(out), stream_handle(self.device)),
                  "edfmm_targets_stage")
        return out

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.edfmm_targets_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def export_lists(self):
        p2p = torch.empty(self.n_p2p_pairs, 2, dtype=torch.int64, device=self.device)
        m2l = torch.empty(self.n_m2l_pairs, 2, dtype=torch.int64, device=self.device)
        with torch.cuda.device(self.device):
            check(self._lib.edfmm_targets_export_lists(self._h, ptr(p2p), ptr(m2l), stream_handle(self.device)),
                  "edfmm_targets_export_lists")
        return p2p, m2l

    def potential(self, sigma: torch.Tensor, areas: torch.Tensor, *, k_e: float = 1.0, out=None, flags: int = 0):
        dt = self.plan.dtype
        s = sigma.to(self.device, dt).contiguous()
        a = areas.to(self.device, dt).contiguous()
        o = torch.empty(self.n, dtype=dt, device=self.device) if out is None else out
        with torch.cuda.device(self.device):
            check(self._lib.edfmm_targets_potential(self._h, ptr(s), ptr(a), float(k_e), ptr(o), int(flags),
                                                    stream_handle(self.device)), "edfmm_targets_potential")
        return o

    def field(self, sigma: torch.Tensor, areas: torch.Tensor, *, k_e: float = 1.0, out=None, flags: int = 0):
        """Field k_e sum_j sigma_j A_j (x - c_j) / |x - c_j|^3 at the targets, (m, 3), by FMM."""
        dt = self.plan.dtype
        s = sigma.to(self.device, dt).contiguous()
        a = areas.to(self.device, dt).contiguous()
        o = torch.empty(self.n, 3, dtype=dt, device=self.device) if out is None else out
        with torch.cuda.device(self.device):
            check(self._lib.edfmm_targets_field(self._h, ptr(s), ptr(a), float(k_e), ptr(o), int(flags),
                                                stream_handle(self.device)), "edfmm_targets_field")
        return o
