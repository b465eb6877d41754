"""Write the golden fixtures in this folder by running the reference itself.

Run with REFERENCE_ROOT set to a checkout of the reference project::

    REFERENCE_ROOT=<path of the reference checkout> python tests/golden/make_golden.py

Nothing at test time imports the reference; the tests read only the .npz
files written here.  Each fixture records which reference routine produced
it (paths inside the reference project):

* ``tree_*.npz``   -- ``electrodrive/fmm3d/tree.py:968`` ``build_fmm_tree`` SoA
  and ``electrodrive/fmm3d/interaction_lists.py:531`` ``build_interaction_lists``
  pairs, plus ``electrodrive/fmm3d/kernels_cpu.py:183`` ``apply_p2p_cpu_tiled``
  potentials for seeded charges.
* ``nearpot_cases.npz`` -- ``electrodrive/core/bem.py:940``
  ``_apply_near_quadrature_potentials``.
* ``efield_cases.npz`` -- ``electrodrive/core/bem_kernel.py:914``
  ``bem_E_field_targets`` and ``electrodrive/core/bem.py:340``
  ``_free_space_E_field_at_points``.
* ``fmm_*.npz``    -- ``electrodrive/fmm3d/bem_fmm.py:888``
  ``make_laplace_fmm_backend(...).matvec`` (CPU) next to
  ``electrodrive/core/bem_kernel.py:558`` ``bem_matvec_gpu(backend="torch_tiled")``.
"""
from __future__ import annotations

import os
import sys
import time

from types import SimpleNamespace

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("REFERENCE_ROOT")
if not REF:
    sys.exit("set REFERENCE_ROOT to the reference checkout (the project that provides the electrodrive package)")
sys.path.insert(0, REF)
os.environ.setdefault("PYTHONDONTWRITEBYTECODE", "1")
sys.dont_write_bytecode = True

import torch  # noqa: E402

from electrodrive.fmm3d.tree import build_fmm_tree  # noqa: E402
from electrodrive.fmm3d.interaction_lists import build_interaction_lists  # noqa: E402
from electrodrive.fmm3d.kernels_cpu import apply_p2p_cpu_tiled  # noqa: E402


def gen_points(kind: str, n: int, seed: int, dtype) -> torch.Tensor:
    g = torch.Generator().manual_seed(seed)
    if kind == "uniform":
        p = torch.rand(n, 3, generator=g, dtype=torch.float64)
    elif kind == "clusters":
        # two tight Gaussian clusters plus a sparse uniform background
        a = 0.02 * torch.randn(n // 2, 3, generator=g, dtype=torch.float64) + 0.25
        b = 0.05 * torch.randn(n // 3, 3, generator=g, dtype=torch.float64) + torch.tensor([0.8, 0.7, 0.3], dtype=torch.float64)
        c = torch.rand(n - a.shape[0] - b.shape[0], 3, generator=g, dtype=torch.float64)
        p = torch.cat([a, b, c])
    elif kind == "lattice":
        # many points exactly on splitting planes and duplicated coordinates
        k = int(round(n ** (1.0 / 3.0))) + 1
        ix = torch.randint(0, k, (n, 3), generator=g)
        p = ix.to(torch.float64) / (k - 1)
    elif kind == "coincident":
        # blocks of exactly coincident points (degenerate boxes)
        base = torch.rand(n // 40 + 1, 3, generator=g, dtype=torch.float64)
        p = base.repeat_interleave(40, dim=0)[:n].clone()
        p[::7] += 1e-9  # some nearly coincident
    elif kind == "sphere":
        v = torch.randn(n, 3, generator=g, dtype=torch.float64)
        p = v / v.norm(dim=1, keepdim=True)
    else:
        raise ValueError(kind)
    return p.to(dtype)


def save_tree_case(name, kind, n, seed, dtype, leaf, theta, max_depth=32):
    pts = gen_points(kind, n, seed, dtype)
    t0 = time.time()
    tree = build_fmm_tree(pts, leaf_size=leaf, max_depth=max_depth)
    lists = build_interaction_lists(tree, tree, mac_theta=theta)
    g = torch.Generator().manual_seed(seed + 100)
    q = (2 * torch.rand(n, generator=g, dtype=torch.float64) - 1).to(dtype)
    q_tree = tree.map_to_tree_order(q)
    res = apply_p2p_cpu_tiled(tree, tree, q_tree, lists)
    p2p = np.asarray(lists.p2p_pairs, dtype=np.int32).reshape(-1, 2)
    m2l = np.asarray(lists.m2l_pairs, dtype=np.int32).reshape(-1, 2)
    np.savez_compressed(
        os.path.join(HERE, f"tree_{name}.npz"),
        kind=kind, n=n, seed=seed, leaf_size=leaf, max_depth=max_depth, theta=theta,
        dtype=str(dtype).replace("torch.", ""),
        points=pts.numpy(),
        charges=q.numpy(),
        index_map=tree.index_map.numpy().astype(np.int32),
        node_centers=tree.node_centers.numpy(),
        node_half_extents=tree.node_half_extents.numpy(),
        node_radii=tree.node_radii.numpy(),
        node_levels=tree.node_levels.numpy(),
        node_parents=tree.node_parents.numpy().astype(np.int32),
        node_children=tree.node_children.numpy().astype(np.int32),
        node_ranges=tree.node_ranges.numpy().astype(np.int32),
        node_is_leaf=tree.node_is_leaf.numpy(),
        p2p_pairs=p2p,
        m2l_pairs=m2l,
        p2p_potential_tree=res.potential.numpy(),
        p2p_n_interactions=res.n_interactions,
    )
    print(f"tree_{name}: N={n} nodes={tree.n_nodes} p2p={len(p2p)} m2l={len(m2l)} ({time.time() - t0:.1f}s)")


def save_fmm_case(name, n, seed, dtype, leaf, theta, p, kind="uniform"):
    from electrodrive.fmm3d.bem_fmm import make_laplace_fmm_backend
    from electrodrive.core.bem_kernel import bem_matvec_gpu

    pts = gen_points(kind, n, seed, dtype)
    g = torch.Generator().manual_seed(seed + 200)
    sigma = (2 * torch.rand(n, generator=g, dtype=torch.float64) - 1).to(dtype)
    areas = (0.5 + torch.rand(n, generator=g, dtype=torch.float64)).to(dtype) * 1e-3
    self_int = (torch.rand(n, generator=g, dtype=torch.float64) * 1e10).to(dtype)
    t0 = time.time()
    fmm = make_laplace_fmm_backend(pts, areas, max_leaf_size=leaf, theta=theta, expansion_order=p, backend="cpu")
    v_fmm = fmm.matvec(sigma=sigma, src_centroids=pts, areas=areas, tile_size=1024, self_integrals=self_int)
    t1 = time.time()
    v_dense = bem_matvec_gpu(sigma, pts, areas, tile_size=1024, self_integrals=self_int, backend="torch_tiled")
    np.savez_compressed(
        os.path.join(HERE, f"fmm_{name}.npz"),
        n=n, seed=seed, leaf_size=leaf, theta=theta, p=p, dtype=str(dtype).replace("torch.", ""), kind=kind,
        points=pts.numpy(), sigma=sigma.numpy(), areas=areas.numpy(), self_integrals=self_int.numpy(),
        v_fmm_reference=v_fmm.numpy(), v_dense_reference=v_dense.numpy(),
        reference_seconds_per_matvec=t1 - t0,
    )
    rel = float((v_fmm - v_dense).norm() / v_dense.norm())
    print(f"fmm_{name}: N={n} ref-FMM vs dense rel-L2 {rel:.3e} ({t1 - t0:.1f}s per matvec incl. setup)")


def save_gmres_cases():
    """electrodrive/core/bem_solver.py:125 gmres_restart on seeded dense systems."""
    from electrodrive.core.bem_solver import gmres_restart, setup_preconditioner

    cases = {}
    g = torch.Generator().manual_seed(40)
    # SPD 8x8 (as in the reference's tests/test_gmres.py), restart 8
    Q = torch.randn(8, 8, generator=g, dtype=torch.float64)
    cases["spd8"] = (Q @ Q.T + 8 * torch.eye(8, dtype=torch.float64), 8, 1e-8, 200, None)
    # nonsymmetric, diagonally weighted, 120x120, restart 10, Jacobi
    B = torch.randn(120, 120, generator=g, dtype=torch.float64) / 12 + torch.diag(1 + torch.rand(120, generator=g,
                                                                                                  dtype=torch.float64) * 5)
    cases["nonsym120_jacobi"] = (B, 10, 1e-10, 400, "jacobi")
    # single-layer-like matrix on 300 random points, restart 20, Jacobi:
    # A_ij = 1 / (300 |p_i - p_j|) (i != j), A_ii = 2 + u_i; the test rebuilds
    # it from the stored points and diagonal
    p = torch.rand(300, 3, generator=g, dtype=torch.float64)
    diag = 2.0 + torch.rand(300, generator=g, dtype=torch.float64)
    d = torch.sqrt(((p[:, None, :] - p[None, :, :]) ** 2).sum(-1))
    K = 1.0 / (300.0 * (d + torch.eye(300, dtype=torch.float64)))
    K.fill_diagonal_(0.0)
    K += torch.diag(diag)
    cases["bemlike300_jacobi"] = (K, 20, 1e-10, 600, "jacobi")
    # maxiter reached
    cases["nonsym120_maxiter"] = (B, 4, 1e-14, 7, None)
    out = {}
    for name, (Amat, restart, tol, maxiter, pc) in cases.items():
        n = Amat.shape[0]
        b = torch.randn(n, generator=g, dtype=torch.float64)
        M = setup_preconditioner(pc, A_diag=torch.diag(Amat)) if pc else None
        x, info = gmres_restart(A=lambda v, Am=Amat: Am @ v, b=b, M=M, restart=restart, tol=tol, maxiter=maxiter)
        if name.startswith("bemlike"):
            out[f"{name}__points"] = p.numpy()
            out[f"{name}__diag"] = diag.numpy()
        else:
            out[f"{name}__A"] = Amat.numpy()
        out[f"{name}__b"] = b.numpy()
        out[f"{name}__x"] = x.numpy()
        out[f"{name}__meta"] = np.array([restart, tol, maxiter, 1.0 if pc else 0.0, info["iters"], info["code"],
                                         float(info["resid"])])
        print(f"gmres {name}: iters={info['iters']} code={info['code']} resid={info['resid']:.3e}")
    np.savez_compressed(os.path.join(HERE, "gmres_cases.npz"), **out)


def _ref_self_integrals(C, PV, depth, order=2):
    """The per-panel loop of electrodrive/core/bem.py:1781-1805."""
    from electrodrive.core.bem_quadrature import near_singular_quadrature
    from electrodrive.utils.config import K_E

    vals = np.empty(C.shape[0])
    for i in range(C.shape[0]):
        pts, w = near_singular_quadrature(target=C[i], panel_vertices=PV[i], method="telles", order=order,
                                          max_depth=depth)
        r = np.maximum(np.linalg.norm(pts - C[i][None, :], axis=1), 1e-12)
        vals[i] = float(np.sum((K_E / r) * w))
    return vals


def _spec(conductors, charges):
    from electrodrive.orchestration.parser import CanonicalSpec

    return CanonicalSpec.from_json(dict(domain="free", conductors=conductors, charges=charges, dielectrics=[]))


def save_near_cases():
    """Self integrals, near pairs, correction weights and their application
    (electrodrive/core/bem.py:475-734, core/bem_quadrature.py:217-308)."""
    from electrodrive.core.bem import (_apply_near_quadrature_matvec_torch, _build_near_pairs_for_panels,
                                       _precompute_near_correction_weights)
    from electrodrive.core.bem_mesh import generate_mesh

    cases = {
        "sphere": (dict(type="sphere", radius=1.0, center=[0.0, 0.0, 0.0], potential=0.0), 0.5, 3),
        "torus": (dict(type="torus", major_radius=1.0, minor_radius=0.35, potential=1.0), 0.45, 4),
        "plane": (dict(type="plane", z=0.0, potential=0.0), 1.2, 4),
    }
    out = {}
    g = torch.Generator().manual_seed(77)
    for name, (cond, h, depth) in cases.items():
        mesh = generate_mesh(_spec([cond], [dict(type="point", q=1.0, pos=[0.2, 0.1, 1.7])]), h)
        C, A = mesh.centroids, mesh.areas
        PV = np.asarray(mesh.vertices)[np.asarray(mesh.triangles)]
        si = _ref_self_integrals(C, PV, depth)
        pairs = _build_near_pairs_for_panels(C, A, distance_factor=1.5, n_panels=C.shape[0])
        w = _precompute_near_correction_weights(C, A, PV, pairs, 2, max_depth=max(1, depth - 1))
        sig = torch.randn(C.shape[0], generator=g, dtype=torch.float64)
        v = _apply_near_quadrature_matvec_torch(torch.zeros_like(sig), sig, near_pairs=torch.as_tensor(pairs),
                                                weights=torch.as_tensor(w))
        for k, val in dict(centroids=C, areas=A, panel_vertices=PV, self_integrals=si, near_pairs=pairs,
                           near_weights=w, sigma=sig.numpy(), v_corr=v.numpy(),
                           meta=np.array([h, depth, max(1, depth - 1)])).items():
            out[f"{name}__{k}"] = val
        print(f"near {name}: N={C.shape[0]} pairs={pairs.shape[0]}")
    np.savez_compressed(os.path.join(HERE, "near_cases.npz"), **out)


def save_solve_cases():
    """electrodrive/core/bem.py:1550 bem_solve, one pass, FP64, CPU."""
    import tempfile

    from electrodrive.core.bem import bem_solve
    from electrodrive.utils.config import BEMConfig
    from electrodrive.utils.logging import JsonlLogger

    cases = {
        "sphere_h05": ([dict(type="sphere", radius=1.0, center=[0.0, 0.0, 0.0], potential=0.0)],
                       [dict(type="point", q=1.0, pos=[0.0, 0.0, 2.0])], 0.5, False),
        "torus_h045_near": ([dict(type="torus", major_radius=1.0, minor_radius=0.35, potential=1.0)],
                            [dict(type="point", q=1.0, pos=[1.6, 0.3, 0.2])], 0.45, True),
    }
    out = {}
    for name, (conds, charges, h, near) in cases.items():
        cfg = BEMConfig()
        cfg.fp64 = True
        cfg.use_gpu = False
        cfg.max_refine_passes = 1
        cfg.min_refine_passes = 1
        cfg.initial_h = h
        cfg.use_near_quadrature_matvec = near
        t0 = time.time()
        res = bem_solve(_spec(conds, charges), cfg, JsonlLogger(tempfile.mkdtemp()))
        dt = time.time() - t0
        st = res["gmres_stats"]
        out[f"{name}__sigma"] = np.asarray(res["surface_charge_density"], dtype=np.float64)
        out[f"{name}__meta"] = np.array([h, float(near), st["iters"], st["code"], st["resid"], st["tol_abs"],
                                         res["mesh_stats"]["n_panels"], res["mesh_stats"]["bc_residual_linf"], dt])
        print(f"solve {name}: N={res['mesh_stats']['n_panels']} iters={st['iters']} code={st['code']} {dt:.1f}s")
    np.savez_compressed(os.path.join(HERE, "solve_cases.npz"), **out)


def save_refine_cases():
    """electrodrive/core/bem.py:1550 bem_solve with more than one pass
    (h-refinement and best-pass selection, :1667-2495) and with a GMRES that
    cannot meet its tolerance (retry without the preconditioner, then the
    damped-Jacobi fallback, :2172-2302), FP64, CPU."""
    import tempfile

    from electrodrive.core.bem import bem_solve
    from electrodrive.utils.config import BEMConfig
    from electrodrive.utils.logging import JsonlLogger

    sphere = ([dict(type="sphere", radius=1.0, center=[0.0, 0.0, 0.0], potential=0.0)],
              [dict(type="point", q=1.0, pos=[0.0, 0.0, 2.0])])
    sphere1 = ([dict(type="sphere", radius=1.0, center=[0.0, 0.0, 0.0], potential=1.0)],
               [dict(type="point", q=1.0, pos=[0.0, 0.0, 2.0])])
    torus = ([dict(type="torus", major_radius=1.0, minor_radius=0.35, potential=1.0)],
             [dict(type="point", q=1.0, pos=[1.6, 0.3, 0.2])])
    # name: (spec, cfg overrides)
    cases = {
        # the first pass meets the target: the loop stops before max_refine_passes
        "sphere_stop_on_bc": (sphere, dict(initial_h=0.8, max_refine_passes=3, target_bc_inf_norm=1e-2)),
        # short cycles and a loose tolerance: each pass stops at a boundary
        # residual far above rounding, so the best-pass choice is reproducible
        # (full 256-step cycles end every pass at rounding level, where the
        # choice between passes is decided by rounding)
        "sphere_refine3_v1": (sphere1, dict(initial_h=0.8, max_refine_passes=3, target_bc_inf_norm=1e-12,
                                            gmres_restart=10, gmres_tol=1e-4)),
        "torus_refine2_near": (torus, dict(initial_h=0.25, max_refine_passes=2, target_bc_inf_norm=1e-12,
                                           use_near_quadrature_matvec=True, gmres_restart=10, gmres_tol=1e-4)),
        "sphere_fallback": (sphere, dict(initial_h=0.8, max_refine_passes=1, gmres_tol=1e-30, gmres_restart=20,
                                         gmres_maxiter=20)),
    }
    out = {}
    for name, ((conds, charges), over) in cases.items():
        cfg = BEMConfig()
        cfg.fp64 = True
        cfg.use_gpu = False
        for k, v in over.items():
            setattr(cfg, k, v)
        t0 = time.time()
        res = bem_solve(_spec(conds, charges), cfg, JsonlLogger(tempfile.mkdtemp()))
        dt = time.time() - t0
        if "error" in res:
            out[f"{name}__error"] = np.array(str(res["error"]))
            print(f"refine {name}: error {res['error']}")
            continue
        st = res["gmres_stats"]
        ms = res["mesh_stats"]
        hist = res["refinement_history"]
        out[f"{name}__sigma"] = np.asarray(res["surface_charge_density"], dtype=np.float64)
        out[f"{name}__passes"] = np.array([[p["pass"], p["h"], p["dof"], p["bc_resid_linf"], p["energy_A"],
                                            p["gmres_info"].get("iters", -1), p["gmres_info"].get("code", -1)]
                                           for p in hist], dtype=np.float64)
        out[f"{name}__best"] = np.array([ms["n_panels"], ms["h_final"], ms["bc_residual_linf"],
                                         res["solution"].meta.get("energy_A", np.nan), st.get("iters", -1),
                                         float(bool(st.get("success", True))), float(st.get("resid", np.nan)), dt])
        out[f"{name}__solver"] = np.array(str(st.get("solver", "gmres")))
        out[f"{name}__boundary_samples"] = np.asarray(res["boundary_samples"], dtype=np.float64)
        out[f"{name}__sample_points"] = np.asarray(res["sample_points"], dtype=np.float64)
        print(f"refine {name}: passes {[(p['dof'], p['bc_resid_linf']) for p in hist]} -> {ms['n_panels']} "
              f"solver {st.get('solver', 'gmres')} {dt:.1f}s")
    np.savez_compressed(os.path.join(HERE, "refine_cases.npz"), **out)


def save_icosphere_solve():
    """The sphere workload (5,120 icosphere panels, unit charge at (0,0,2),
    grounded, FP64, dense operator, GMRES(50) tol 1e-8) run through the
    reference's own building blocks on the icosphere arrays."""
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from electrodrive.core.bem_kernel import bem_matvec_gpu
    from electrodrive.core.bem_solver import gmres_restart
    from electrodrive.utils.config import K_E
    from electrodrive_gb300.core.bem_mesh import icosphere

    mesh = icosphere(4)
    C = torch.as_tensor(mesh.centroids)
    A = torch.as_tensor(mesh.areas)
    PV = mesh.vertices[mesh.triangles]
    t0 = time.time()
    si = torch.as_tensor(_ref_self_integrals(mesh.centroids, PV, 3))
    self_corr = si / A
    q, rq = 1.0, torch.tensor([0.0, 0.0, 2.0], dtype=torch.float64)
    V_free = K_E * q / torch.linalg.norm(C - rq[None, :], dim=1).clamp_min(1e-12)
    b = torch.zeros_like(A) - V_free
    x0 = b / si.clamp_min(1e-18)
    t1 = time.time()
    mv = lambda s: bem_matvec_gpu(sigma=s, src_centroids=C, areas=A, tile_size=1024, self_integrals=self_corr,
                                  backend="torch_tiled")
    sigma, info = gmres_restart(mv, b, restart=50, tol=1e-8, maxiter=2000, precond="jacobi", areas=A, A_diag=si,
                                x0=x0)
    t2 = time.time()
    np.savez_compressed(os.path.join(HERE, "icosphere5120_solve.npz"), self_integrals=si.numpy(),
                        sigma=sigma.numpy(), meta=np.array([info["iters"], info["code"], info["resid"],
                                                            info["tol_abs"], t1 - t0, t2 - t1]))
    print(f"icosphere solve: iters={info['iters']} code={info['code']} setup {t1 - t0:.1f}s solve {t2 - t1:.1f}s")


def save_targets_cases():
    """electrodrive/fmm3d/interaction_lists.py:531 build_interaction_lists
    between a source tree and a separate target tree."""
    out = {}
    # (source kind, n, seed, target kind, n, seed, dtype, source leaf, theta, shift, target leaf)
    cases = {
        "shifted_f32": ("uniform", 2000, 21, "uniform", 900, 22, torch.float32, 32, 0.5, 0.6, 32),
        "sphere_in_cube_f64": ("sphere", 1500, 23, "uniform", 700, 24, torch.float64, 24, 0.5, -0.5, 24),
        "leaf32_vs_leaf10_f32": ("clusters", 2500, 25, "uniform", 1200, 26, torch.float32, 32, 0.45, 0.1, 10),
    }
    for name, (ks, ns, ss, kt, nt, st, dtype, leaf, theta, shift, tleaf) in cases.items():
        src = gen_points(ks, ns, ss, dtype)
        tgt = gen_points(kt, nt, st, dtype) * 2.0 + shift
        tgt = tgt.to(dtype)
        stree = build_fmm_tree(src, leaf_size=leaf)
        ttree = build_fmm_tree(tgt, leaf_size=tleaf)
        lists = build_interaction_lists(stree, ttree, mac_theta=theta)
        out[f"{name}__sources"] = src.numpy()
        out[f"{name}__targets"] = tgt.numpy()
        out[f"{name}__meta"] = np.array([leaf, theta])
        out[f"{name}__target_leaf"] = np.array([tleaf])
        out[f"{name}__p2p_pairs"] = np.asarray(lists.p2p_pairs, dtype=np.int32).reshape(-1, 2)
        out[f"{name}__m2l_pairs"] = np.asarray(lists.m2l_pairs, dtype=np.int32).reshape(-1, 2)
        out[f"{name}__target_index_map"] = ttree.index_map.numpy().astype(np.int32)
        print(f"targets {name}: p2p={len(lists.p2p_pairs)} m2l={len(lists.m2l_pairs)}")
    np.savez_compressed(os.path.join(HERE, "targets_cases.npz"), **out)


def save_nearpot_cases():
    """electrodrive/core/bem.py:940 _apply_near_quadrature_potentials: the
    target-side near correction on a sphere and a torus mesh, at targets
    close to the surface, on centroids (the r < 1e-12 branch) and far away."""
    from electrodrive.core.bem import _apply_near_quadrature_potentials
    from electrodrive.core.bem_mesh import generate_mesh

    cases = {
        "sphere": (dict(type="sphere", radius=1.0, center=[0.0, 0.0, 0.0], potential=0.0), 0.4, 6.0, 3),
        "torus": (dict(type="torus", major_radius=1.0, minor_radius=0.35, potential=1.0), 0.45, 1.5, 4),
    }
    out = {}
    g = torch.Generator().manual_seed(91)
    for name, (cond, h, factor, depth) in cases.items():
        mesh = generate_mesh(_spec([cond], [dict(type="point", q=1.0, pos=[0.2, 0.1, 1.7])]), h)
        C = torch.as_tensor(mesh.centroids, dtype=torch.float64)
        A = torch.as_tensor(mesh.areas, dtype=torch.float64)
        PV = torch.as_tensor(np.asarray(mesh.vertices)[np.asarray(mesh.triangles)], dtype=torch.float64)
        n = C.shape[0]
        sig = torch.randn(n, generator=g, dtype=torch.float64)
        pick = torch.randperm(n, generator=g)[:40]
        near = C[pick] * (1.0 + 0.05 * torch.randn(40, 1, generator=g, dtype=torch.float64))
        far = torch.randn(10, 3, generator=g, dtype=torch.float64) * 3.0
        T = torch.cat([near, C[pick[:5]], far])
        v0 = torch.randn(T.shape[0], generator=g, dtype=torch.float64)
        # the reference edits the numpy view of its input in place: pass a copy
        v = _apply_near_quadrature_potentials(v0.clone(), T, C, A, sig, PV, distance_factor=factor, quad_order=2,
                                              max_depth=depth)
        for k, val in dict(centroids=C, areas=A, panel_vertices=PV, sigma=sig, targets=T, v_in=v0, v_out=v).items():
            out[f"{name}__{k}"] = val.numpy()
        out[f"{name}__meta"] = np.array([factor, 2, depth])
        print(f"nearpot {name}: N={n} M={T.shape[0]} |dv|={float((v - v0).norm()):.3g}")
    np.savez_compressed(os.path.join(HERE, "nearpot_cases.npz"), **out)


def save_efield_cases():
    """electrodrive/core/bem_kernel.py:914 bem_E_field_targets (dense induced
    field at targets) and electrodrive/core/bem.py:340
    _free_space_E_field_at_points, on seeded panels, densities and targets
    (inside, on and around the source cloud, and one target on a centroid)."""
    from electrodrive.core.bem import _free_space_E_field_at_points
    from electrodrive.core.bem_kernel import bem_E_field_targets

    out = {}
    for name, (n, m, seed, dtype) in {"cloud_f64": (1500, 400, 31, torch.float64),
                                      "cloud_f32": (1200, 300, 32, torch.float32)}.items():
        g = torch.Generator().manual_seed(seed)
        c = torch.rand(n, 3, generator=g, dtype=torch.float64).to(dtype)
        a = (torch.rand(n, generator=g, dtype=torch.float64) * 0.5 + 0.5).to(dtype) / n
        sig = (torch.rand(n, generator=g, dtype=torch.float64) * 2 - 1).to(dtype)
        t = (torch.rand(m, 3, generator=g, dtype=torch.float64) * 2.0 - 0.5).to(dtype)
        t[0] = c[7]  # a target on a source centroid: the 1e-24 clamp of r^2
        E = bem_E_field_targets(t, c, a, sig, tile_size=256, backend="torch_tiled")
        spec = SimpleNamespace(charges=[{"type": "point", "q": 1.5, "pos": [0.2, 0.3, 1.4]},
                                        {"type": "point", "q": -0.5, "pos": [0.9, -0.4, 0.1]}])
        Ef = _free_space_E_field_at_points(spec, t, dtype, torch.device("cpu"))
        for k, v in dict(centroids=c, areas=a, sigma=sig, targets=t, E=E, E_free=Ef).items():
            out[f"{name}__{k}"] = v.numpy()
        print(f"efield {name}: |E| {float(E.norm()):.4g}")
    np.savez_compressed(os.path.join(HERE, "efield_cases.npz"), **out)


def main():
    which = sys.argv[1:] or ["trees", "fmm", "gmres", "near", "solve", "refine", "ico", "targets", "efield",
                             "nearpot"]
    if "nearpot" in which:
        save_nearpot_cases()
    if "efield" in which:
        save_efield_cases()
    if "targets" in which:
        save_targets_cases()
    if "near" in which:
        save_near_cases()
    if "solve" in which:
        save_solve_cases()
    if "refine" in which:
        save_refine_cases()
    if "ico" in which:
        save_icosphere_solve()
    if "gmres" in which:
        save_gmres_cases()
    if "trees" in which:
        save_tree_case("uniform4096_f32", "uniform", 4096, 0, torch.float32, 64, 0.5)
        save_tree_case("clusters3000_f32", "clusters", 3000, 1, torch.float32, 32, 0.5)
        save_tree_case("lattice2000_f32", "lattice", 2000, 2, torch.float32, 16, 0.5)
        save_tree_case("coincident1200_f32", "coincident", 1200, 3, torch.float32, 8, 0.5)
        save_tree_case("sphere2500_f64", "sphere", 2500, 4, torch.float64, 24, 0.6)
        save_tree_case("uniform1500_theta03_f32", "uniform", 1500, 5, torch.float32, 20, 0.3)
        save_tree_case("deep_maxdepth3_f32", "clusters", 2000, 6, torch.float32, 4, 0.5, max_depth=3)
        save_tree_case("tiny5_f32", "uniform", 5, 7, torch.float32, 64, 0.5)
    if "fmm" in which:
        save_fmm_case("uniform512_f32", 512, 10, torch.float32, 64, 0.5, 8)
        save_fmm_case("uniform1024_f32", 1024, 11, torch.float32, 64, 0.5, 8)
    if "fmm_shapes" in which:
        # BEM-like and clustered point sets: points on the unit sphere, and two
        # tight Gaussian clusters over a sparse background with smaller leaves
        save_fmm_case("sphere1024_f32", 1024, 12, torch.float32, 64, 0.5, 8, kind="sphere")
        save_fmm_case("clusters1200_leaf32_f32", 1200, 13, torch.float32, 32, 0.5, 8, kind="clusters")


if __name__ == "__main__":
    main()
