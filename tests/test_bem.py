"""Panel quadrature, near-field corrections and the BEM solve.

CPU: the mesher and the oracle's quadrature restatements against fixtures
written by the reference (tests/golden/make_golden.py: near, solve, ico).
GPU: self integrals, near pairs (bit-exact), weights and their application,
the reference CUDA module's on-the-fly correction, bem_solve against the
reference's own bem_solve, and the 5,120-panel icosphere (unit charge at
(0,0,2), grounded) against the reference pipeline and the Kelvin image.
Tolerances: FP64 geometry 1e-12 relative; solutions 1e-6 relative L2 (both
are FP64 GMRES solves to the same tolerance); Kelvin: the discretisation
error of centroid collocation (3e-2 on sigma, 1e-2 on exterior potential).
"""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

NEAR = np.load(os.path.join(GOLDEN, "near_cases.npz"))
SOLVE = np.load(os.path.join(GOLDEN, "solve_cases.npz"))
ICO = np.load(os.path.join(GOLDEN, "icosphere5120_solve.npz"))
K_E = 1.0 / (4.0 * np.pi * 8.854187817e-12)
NEAR_CASES = ["sphere", "torus", "plane"]
MESH_SPECS = {
    "sphere": (dict(type="sphere", radius=1.0, center=[0.0, 0.0, 0.0], potential=0.0), 0.5),
    "torus": (dict(type="torus", major_radius=1.0, minor_radius=0.35, potential=1.0), 0.45),
    "plane": (dict(type="plane", z=0.0, potential=0.0), 1.2),
}


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _spec(cond, q=1.0, pos=(0.2, 0.1, 1.7)):
    return dict(conductors=[cond], charges=[dict(type="point", q=q, pos=list(pos))])


@pytest.mark.parametrize("name", NEAR_CASES)
def test_mesher_reproduces_reference_mesh(name):
    from electrodrive_gb300.core.bem_mesh import generate_mesh

    cond, h = MESH_SPECS[name]
    m = generate_mesh(_spec(cond), h)
    assert np.array_equal(m.centroids, NEAR[f"{name}__centroids"])
    assert np.array_equal(m.areas, NEAR[f"{name}__areas"])
    assert np.array_equal(m.vertices[m.triangles], NEAR[f"{name}__panel_vertices"])


@pytest.mark.parametrize("name", NEAR_CASES)
def test_oracle_quadrature_matches_reference(oracle, name):
    C, A, PV = (NEAR[f"{name}__{k}"] for k in ("centroids", "areas", "panel_vertices"))
    h, depth, depth_mv = NEAR[f"{name}__meta"]
    si = oracle.self_integrals(PV, C, 2, int(depth))
    assert rel(si, NEAR[f"{name}__self_integrals"]) < 1e-12
    pairs = oracle.near_pairs(C, A, 1.5)
    assert np.array_equal(pairs, NEAR[f"{name}__near_pairs"])
    w = oracle.near_weights(C, A, PV, pairs, 2, int(depth_mv))
    assert rel(w, NEAR[f"{name}__near_weights"]) < 1e-12


def test_icosphere_has_5120_panels_on_the_unit_sphere():
    from electrodrive_gb300.core.bem_mesh import icosphere

    m = icosphere(4)
    assert m.n_panels == 5120
    assert np.allclose(np.linalg.norm(m.vertices, axis=1), 1.0)
    assert abs(m.areas.sum() - 4 * np.pi) < 2e-3 * 4 * np.pi


def test_panel_vertices_gather_equals_host_gather():
    """bem_solve's panel vertex triples, gathered from the vertex and triangle
    arrays on the solve's device (here the CPU), equal vertices[triangles]."""
    from electrodrive_gb300.core.bem import panel_vertices_on
    from electrodrive_gb300.core.bem_mesh import icosphere, torus_mesh

    for m in (icosphere(2), torus_mesh(1.0, 0.35, 20, 8)):
        pv = panel_vertices_on(m, torch.device("cpu"))
        assert pv.dtype == torch.float64 and pv.shape == (m.n_panels, 3, 3) and pv.is_contiguous()
        assert np.array_equal(pv.numpy(), m.vertices[m.triangles])


@pytest.mark.gpu
@pytest.mark.parametrize("name", NEAR_CASES)
def test_gpu_near_field_matches_reference(cuda_lib, name):
    from electrodrive_gb300.core.bem_near import NearCorrection, self_integrals

    C, A, PV = (NEAR[f"{name}__{k}"] for k in ("centroids", "areas", "panel_vertices"))
    h, depth, depth_mv = NEAR[f"{name}__meta"]
    si = self_integrals(PV, C, order=2, depth=int(depth)).cpu().numpy()
    assert rel(si, NEAR[f"{name}__self_integrals"]) < 1e-12
    nc = NearCorrection(C, A, PV, distance_factor=1.5, order=2, depth=int(depth_mv), dtype=torch.float64)
    pairs, w = nc.export()
    assert np.array_equal(pairs.cpu().numpy(), NEAR[f"{name}__near_pairs"])
    assert rel(w.cpu().numpy(), NEAR[f"{name}__near_weights"]) < 1e-12
    sig = torch.as_tensor(NEAR[f"{name}__sigma"], device="cuda")
    out = torch.zeros_like(sig)
    nc.apply(sig, None, out)
    assert rel(out.cpu().numpy(), NEAR[f"{name}__v_corr"]) < 1e-12
    nc32 = NearCorrection(C, A, PV, distance_factor=1.5, order=2, depth=int(depth_mv), dtype=torch.float32)
    o32 = torch.zeros(sig.shape[0], device="cuda")
    nc32.apply(sig.float(), None, o32)
    assert rel(o32.cpu().numpy(), NEAR[f"{name}__v_corr"]) < 1e-5
    # the FP32 set cast from the FP64 one (no second pair search) is the same set
    cv = nc.astype(torch.float32)
    assert cv.n_pairs == nc32.n_pairs
    pc, wc = cv.export()
    assert torch.equal(pc, pairs) and torch.equal(wc, w)
    oc = torch.zeros_like(o32)
    cv.apply(sig.float(), None, oc)
    assert torch.equal(oc, o32)
    assert nc.astype(torch.float64) is nc


@pytest.mark.gpu
@pytest.mark.parametrize("order", [1, 2])
def test_on_the_fly_module_matches_oracle(cuda_lib, oracle, order):
    from electrodrive_gb300.core.bem_near import apply_near_quadrature_matvec_cuda

    C, A, PV = (NEAR[f"torus__{k}"] for k in ("centroids", "areas", "panel_vertices"))
    pairs = NEAR["torus__near_pairs"]
    w = oracle.near_weights(C, A, PV, pairs, order, 0)
    sig = NEAR["torus__sigma"]
    ref = np.zeros(C.shape[0])
    np.add.at(ref, pairs[:, 0], w * sig[pairs[:, 1]])
    T = lambda x: torch.as_tensor(x, device="cuda")
    rng = np.random.default_rng(1)
    pp = pairs[rng.permutation(pairs.shape[0])]  # the module accepts unsorted pairs
    out = apply_near_quadrature_matvec_cuda(torch.zeros(C.shape[0], dtype=torch.float64, device="cuda"), T(sig),
                                            centroids=T(C), areas=T(A), panel_vertices=T(PV), near_pairs=pp,
                                            quad_order=order)
    # delta_ij is a difference of two ~K_E A_j / r terms (identically zero for the
    # order-1 centroid rule), so compare against the size of those terms
    i, j = pairs[:, 0], pairs[:, 1]
    r = np.linalg.norm(C[i] - C[j], axis=1)
    scale = np.zeros(C.shape[0])
    np.add.at(scale, i, K_E * A[j] * np.abs(sig[j]) / r)
    assert np.all(np.abs(out.cpu().numpy() - ref) <= 1e-12 * scale + 1e-300)


@pytest.mark.gpu
def test_on_the_fly_module_long_and_empty_rows(cuda_lib, oracle):
    """Rows longer than one block's pair tile (999 pairs), empty rows, a block
    boundary inside the pair list, the pair rows reused for the same tensor
    and rebuilt after the tensor changes in place."""
    from electrodrive_gb300.core.bem_near import apply_near_quadrature_matvec_cuda

    rng = np.random.default_rng(11)
    n = 1000
    PV = rng.normal(size=(n, 3, 3)) * 0.05 + rng.uniform(-1, 1, size=(n, 1, 3))
    C = PV.mean(axis=1)
    A = 0.5 * np.linalg.norm(np.cross(PV[:, 1] - PV[:, 0], PV[:, 2] - PV[:, 0]), axis=1)
    sig = rng.uniform(-1, 1, n)
    rows = [np.stack([np.full(n - 1, 5), np.delete(np.arange(n), 5)], 1)]
    for i in range(40, n, 3):  # every third row from 40 on: a few random sources
        js = rng.choice(np.delete(np.arange(n), i), size=int(rng.integers(1, 12)), replace=False)
        rows.append(np.stack([np.full(js.size, i), np.sort(js)], 1))
    pairs = np.concatenate(rows).astype(np.int64)
    w = oracle.near_weights(C, A, PV, pairs, 2, 0)
    ref = np.zeros(n)
    np.add.at(ref, pairs[:, 0], w * sig[pairs[:, 1]])
    T = lambda x: torch.as_tensor(x, device="cuda")
    vfar = T(rng.uniform(-1, 1, n))
    pt = T(pairs[rng.permutation(pairs.shape[0])])
    call = lambda p: apply_near_quadrature_matvec_cuda(vfar, T(sig), centroids=T(C), areas=T(A), panel_vertices=T(PV),
                                                      near_pairs=p, quad_order=2).cpu().numpy()
    i, j = pairs[:, 0], pairs[:, 1]
    scale = np.zeros(n)
    np.add.at(scale, i, K_E * A[j] * np.abs(sig[j]) / np.linalg.norm(C[i] - C[j], axis=1))
    want = vfar.cpu().numpy() + ref
    for _ in range(2):  # the second call reuses the rows of the same tensor
        assert np.all(np.abs(call(pt) - want) <= 1e-12 * (scale + np.abs(want)) + 1e-300)
    pt[:, 1] = pt[:, 0]  # in place: every pair becomes (i, i); the rows must be rebuilt
    assert np.array_equal(call(pt), call(pt.clone()))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sphere_h05", "torus_h045_near"])
def test_bem_solve_matches_reference_bem_solve(cuda_lib, name):
    from electrodrive_gb300.core.bem import bem_solve
    from electrodrive_gb300.utils.config import BEMConfig

    h, near, iters, code, resid, tol_abs, npan, bc_res, _ = SOLVE[f"{name}__meta"]
    if name.startswith("sphere"):
        spec = dict(conductors=[dict(type="sphere", radius=1.0, center=[0, 0, 0], potential=0.0)],
                    charges=[dict(type="point", q=1.0, pos=[0.0, 0.0, 2.0])])
    else:
        spec = dict(conductors=[dict(type="torus", major_radius=1.0, minor_radius=0.35, potential=1.0)],
                    charges=[dict(type="point", q=1.0, pos=[1.6, 0.3, 0.2])])
    cfg = BEMConfig(fp64=True, initial_h=float(h), use_near_quadrature_matvec=bool(near), max_refine_passes=1)
    res = bem_solve(spec, cfg, operator="dense")
    st = res["gmres_stats"]
    err = rel(np.asarray(res["surface_charge_density"]), SOLVE[f"{name}__sigma"])
    msg = f"iters {st['iters']} vs {int(iters)}, resid {st['resid']:.3e} vs {resid:.3e}, sigma rel {err:.2e}"
    assert res["mesh_stats"]["n_panels"] == int(npan)
    assert st["code"] == int(code) and st["resid"] <= st["tol_abs"], msg
    assert abs(st["tol_abs"] - tol_abs) <= 1e-9 * tol_abs, msg
    # Cycles always run to the full restart length, long after the Krylov space
    # of these well-conditioned systems is exhausted, so the last update is
    # shaped by rounding: the reference's own gmres_restart, given identical
    # inputs in one process, ended the torus case after 256 iterations on its
    # first call and after 1,024 on later ones, with sigma differing by 5e-6
    # relative between its runs.  What is reproducible: the code, a whole
    # number of cycles, a true residual below tol_abs, and sigma to 2e-5.
    assert st["iters"] % cfg.gmres_restart == 0 and st["iters"] <= cfg.gmres_maxiter, msg
    if name.startswith("sphere"):
        assert st["iters"] == int(iters), msg
    assert err < (1e-6 if name.startswith("sphere") else 2e-5), msg


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sphere_h05", "torus_h045_near"])
@pytest.mark.parametrize("operator,mixed", [("fmm", False), ("fmm", True), ("dense", True)])
def test_fmm_and_mixed_solves_match_reference_bem_solve(cuda_lib, name, operator, mixed):
    """The FMM operator (p = 8, leaf 64, theta 0.5, plus the near correction)
    and the mixed FP32/FP64 refinement solver converge to the reference's own
    bem_solve density within 1e-5 relative L2 (the reference's run-to-run
    spread on the torus case is about 5e-6)."""
    from electrodrive_gb300.core.bem import bem_solve
    from electrodrive_gb300.utils.config import BEMConfig

    h, near = SOLVE[f"{name}__meta"][:2]
    if name.startswith("sphere"):
        spec = dict(conductors=[dict(type="sphere", radius=1.0, center=[0, 0, 0], potential=0.0)],
                    charges=[dict(type="point", q=1.0, pos=[0.0, 0.0, 2.0])])
    else:
        spec = dict(conductors=[dict(type="torus", major_radius=1.0, minor_radius=0.35, potential=1.0)],
                    charges=[dict(type="point", q=1.0, pos=[1.6, 0.3, 0.2])])
    cfg = BEMConfig(fp64=True, initial_h=float(h), use_near_quadrature_matvec=bool(near), max_refine_passes=1)
    res = bem_solve(spec, cfg, operator=operator, mixed=mixed, mixed_rtol=1e-7)
    st = res["gmres_stats"]
    assert res["mesh_stats"]["operator"] == operator
    assert st["code"] == 0 and st["success"]
    err = rel(np.asarray(res["surface_charge_density"]), SOLVE[f"{name}__sigma"])
    assert err < 1e-5, err


@pytest.mark.gpu
def test_icosphere_solve_matches_reference_and_kelvin(cuda_lib):
    from electrodrive_gb300.core.bem import bem_solve
    from electrodrive_gb300.core.bem_mesh import icosphere
    from electrodrive_gb300.utils.config import BEMConfig

    spec = dict(conductors=[dict(type="sphere", radius=1.0, center=[0, 0, 0], potential=0.0)],
                charges=[dict(type="point", q=1.0, pos=[0.0, 0.0, 2.0])])
    cfg = BEMConfig(fp64=True, gmres_restart=50, gmres_tol=1e-8, gmres_maxiter=2000)
    mesh = icosphere(4)
    res = bem_solve(spec, cfg, mesh=mesh, operator="dense", self_integral="quadrature")
    sigma = np.asarray(res["surface_charge_density"])
    iters, code = ICO["meta"][:2]
    assert res["gmres_stats"]["code"] == int(code) and res["gmres_stats"]["iters"] == int(iters)
    assert rel(sigma, ICO["sigma"]) < 1e-6
    # Kelvin image: q' = -q a / d at a^2 / d
    x = mesh.centroids
    d = np.linalg.norm(x - np.array([0, 0, 2.0]), axis=1)
    sig_k = -(4.0 - 1.0) / (4 * np.pi * d ** 3)
    assert rel(sigma, sig_k) < 3e-2
    g = torch.Generator().manual_seed(2)
    u = torch.randn(1000, 3, generator=g, dtype=torch.float64)
    u = u / u.norm(dim=1, keepdim=True)
    r = 1.2 + 1.8 * torch.rand(1000, 1, generator=g, dtype=torch.float64)
    pts = (u * r).numpy()
    v = res["solution"].eval(torch.as_tensor(pts, device="cuda")).cpu().numpy()
    vk = K_E * (1.0 / np.linalg.norm(pts - [0, 0, 2.0], axis=1) - 0.5 / np.linalg.norm(pts - [0, 0, 0.5], axis=1))
    assert rel(v, vk) < 1e-2
