"""Batched plans: K independent point sets packed into one plan.

Each instance's tree and lists are the ones a single plan builds for it, and
the batched matvec equals the per-instance matvecs bit for bit (the stage
kernels do the same work per node and row, only more of it per launch).
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _instances(seed, sizes):
    rng = np.random.default_rng(seed)
    pts = []
    for k, n in enumerate(sizes):
        kind = k % 3
        if kind == 0:
            p = rng.random((n, 3))
        elif kind == 1:
            u = rng.normal(size=(n, 3))
            p = u / np.linalg.norm(u, axis=1, keepdims=True) * rng.uniform(0.5, 2.0)
        else:
            p = rng.normal(size=(n, 3)) * 0.3 + rng.normal(size=3)
        pts.append(p)
    return pts


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_batched_matvec_equals_per_instance_matvecs(cuda_lib, dtype):
    from electrodrive_gb300._lib import Plan

    sizes = [700, 3000, 1, 128, 5000, 64]
    pts = _instances(3, sizes)
    off = np.concatenate([[0], np.cumsum(sizes)])
    allp = torch.as_tensor(np.concatenate(pts), dtype=dtype, device="cuda")
    rng = np.random.default_rng(4)
    sigma = torch.as_tensor(rng.uniform(-1, 1, off[-1]), dtype=dtype, device="cuda")
    areas = torch.as_tensor(rng.uniform(0.5, 1.5, off[-1]) / 1000, dtype=dtype, device="cuda")
    si = torch.as_tensor(rng.uniform(0, 10, off[-1]), dtype=dtype, device="cuda")
    batch = Plan(allp, leaf_size=32, expansion_order=8, instance_offsets=off)
    vb = batch.matvec(sigma, areas, si, k_e=1.0)
    tot_m2l = tot_p2p = tot_nodes = 0
    for k in range(len(sizes)):
        a, b = int(off[k]), int(off[k + 1])
        single = Plan(allp[a:b].contiguous(), leaf_size=32, expansion_order=8)
        tot_m2l += single.info.n_m2l_pairs
        tot_p2p += single.info.n_p2p_pairs
        tot_nodes += single.info.n_nodes
        vs = single.matvec(sigma[a:b].contiguous(), areas[a:b].contiguous(), si[a:b].contiguous(), k_e=1.0)
        assert torch.equal(vb[a:b], vs), k
    assert (batch.info.n_m2l_pairs, batch.info.n_p2p_pairs, batch.info.n_nodes) == (tot_m2l, tot_p2p, tot_nodes)


def test_batched_tree_export_is_the_offset_per_instance_trees(cuda_lib):
    from electrodrive_gb300._lib import Plan

    sizes = [900, 2000, 300]
    pts = _instances(7, sizes)
    off = np.concatenate([[0], np.cumsum(sizes)])
    allp = torch.as_tensor(np.concatenate(pts), dtype=torch.float32, device="cuda")
    tb = Plan(allp, leaf_size=64, instance_offsets=off).export_tree()
    node0 = 0
    for k in range(len(sizes)):
        a, b = int(off[k]), int(off[k + 1])
        ts = Plan(allp[a:b].contiguous(), leaf_size=64).export_tree()
        m = ts["node_radii"].shape[0]
        assert torch.equal(tb["index_map"][a:b].cpu(), ts["index_map"].cpu() + a)
        assert torch.equal(tb["node_radii"][node0:node0 + m].cpu(), ts["node_radii"].cpu())
        assert torch.equal(tb["node_ranges"][node0:node0 + m].cpu(), ts["node_ranges"].cpu() + a)
        par = ts["node_parents"].cpu()
        assert torch.equal(tb["node_parents"][node0:node0 + m].cpu(), torch.where(par >= 0, par + node0, par))
        node0 += m


def test_batched_dimer_solve_meets_the_tolerance_per_instance(cuda_lib):
    """Five dimers solved together (mixed precision, per-instance Krylov
    spaces and stopping): every instance meets 1e-6 in the FMM operator, its
    residual in the dense FP64 operator is 1e-6 plus the FMM's operator error,
    and its density agrees with its own dense FP64 solve to within what the
    residual allows (the conditioning of the close pair)."""
    from electrodrive_gb300.core.batch import BatchSystem, autotune_inner, dimer_case
    from electrodrive_gb300.core.bem import assemble_system
    from electrodrive_gb300.core.bem_solver import gmres_restart

    cases = [dimer_case(100 + i, n) for i, n in enumerate([1500, 2600, 1800, 3000, 2200])]
    system = BatchSystem(cases, leaf_size=32)
    tune = autotune_inner(system, leaf_sizes=(32, 64), orders=(6, 8))
    assert all(t["rel_error"] > 0 for t in tune["trials"])
    x, info = system.solve()
    assert info["code"] == 0
    res = system.residuals(x).cpu().numpy()
    assert res.max() <= 1e-6 * (1 + 1e-9), res
    for k, (mesh, spec) in enumerate(cases):
        sysd = assemble_system(mesh, spec, kind="dense")
        op = sysd["ops"][torch.float64]
        ref, rinfo = gmres_restart(op, sysd["b"], restart=100, tol=1e-10, maxiter=2000, precond="jacobi",
                                   A_diag=sysd["diag"], x0=sysd["x0"], early_exit=10)
        a, b = system.offsets[k], system.offsets[k + 1]
        xk = x[a:b].to(torch.float64)
        rd = float(torch.linalg.norm(sysd["b"] - op(xk)) / torch.linalg.norm(sysd["b"]))
        assert rd < 5e-6, (k, rd)
        err = float(torch.linalg.norm(xk - ref) / torch.linalg.norm(ref))
        assert err < 5e-4, (k, err)


def test_batched_learned_start_equals_per_instance_warm_start(cuda_lib):
    """BatchSystem.learned_start gives every instance the warm start that
    core.warm_start.warm_start gives it alone (same network, same FP32
    operator rows), and it starts much closer than the cold start."""
    import os

    from electrodrive_gb300.core.batch import BatchSystem, dimer_case
    from electrodrive_gb300.core.bem import assemble_system, segment_norms
    from electrodrive_gb300.core.warm_start import PointCloudNet, warm_start

    weights = os.path.join(os.path.dirname(__file__), "..", "electrodrive_gb300", "data", "pcn_weights.npz")
    net = PointCloudNet.load(weights, device="cuda")
    cases = [dimer_case(200 + i, n) for i, n in enumerate([1200, 2000, 1600])]
    system = BatchSystem(cases, leaf_size=64)
    x0 = system.learned_start(net)
    for k, (mesh, spec) in enumerate(cases):
        sysd = assemble_system(mesh, spec, kind="fmm", dtypes=(torch.float32,))
        xs = warm_start(net, mesh, sysd["b"], sysd["ops"][torch.float32])
        a, b = system.offsets[k], system.offsets[k + 1]
        assert float(torch.linalg.norm(x0[a:b] - xs) / torch.linalg.norm(xs)) < 1e-6, k
    bn = segment_norms(system.b, system.offsets)
    r_learned = segment_norms(system.b - system.op64(x0), system.offsets) / bn
    r_cold = segment_norms(system.b - system.op64(system.x0_cold), system.offsets) / bn
    assert bool((r_learned < r_cold).all()), (r_learned, r_cold)


def test_instance_mask_skips_inactive_instances_only(cuda_lib):
    """With an instance mask, the rows of active instances are bit-identical
    to the unmasked matvec; the mask is read when the kernels run."""
    from electrodrive_gb300._lib import Plan

    sizes = [900, 2500, 400, 3000]
    pts = _instances(8, sizes)
    off = np.concatenate([[0], np.cumsum(sizes)])
    allp = torch.as_tensor(np.concatenate(pts), dtype=torch.float32, device="cuda")
    rng = np.random.default_rng(9)
    sigma = torch.as_tensor(rng.uniform(-1, 1, off[-1]), dtype=torch.float32, device="cuda")
    areas = torch.full((int(off[-1]),), 1e-3, dtype=torch.float32, device="cuda")
    plan = Plan(allp, leaf_size=32, expansion_order=8, instance_offsets=off)
    full = plan.matvec(sigma, areas, None, k_e=1.0).clone()
    state = torch.zeros(4, 3, dtype=torch.float64, device="cuda")  # flags in column 1, stride 3
    state[[0, 2], 1] = 1.0
    plan.set_instance_mask(state[:, 1], 3)
    try:
        masked = plan.matvec(sigma, areas, None, k_e=1.0).clone()
        for k in (0, 2):
            a, b = int(off[k]), int(off[k + 1])
            assert torch.equal(masked[a:b], full[a:b]), k
        state[1, 1] = 1.0  # flags change on the device: the next matvec follows them
        again = plan.matvec(sigma, areas, None, k_e=1.0).clone()
        a, b = int(off[1]), int(off[2])
        assert torch.equal(again[a:b], full[a:b])
    finally:
        plan.set_instance_mask(None)
    assert torch.equal(plan.matvec(sigma, areas, None, k_e=1.0), full)
    single = Plan(allp[:900].contiguous(), leaf_size=32)
    with pytest.raises(Exception):
        single.set_instance_mask(state[:, 1], 3)  # needs a batched plan


@pytest.mark.parametrize("batched", [False, True])
def test_converted_plan_shares_the_partition(cuda_lib, batched):
    """edfmm_plan_convert: same dtype and order gives a bit-identical matvec;
    an FP32 plan converted from an FP64 one has the FP64 plan's tree and
    lists (geometry cast) and its matvec is within FP32 rounding of the FP64
    one; a batched plan keeps its instances (the mask works on the copy)."""
    from electrodrive_gb300._lib import Plan

    sizes = [1500, 4000, 700] if batched else [6000]
    pts = _instances(11, sizes)
    off = np.concatenate([[0], np.cumsum(sizes)])
    allp = torch.as_tensor(np.concatenate(pts), dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(12)
    sigma = torch.as_tensor(rng.uniform(-1, 1, off[-1]), dtype=torch.float64, device="cuda")
    areas = torch.full((int(off[-1]),), 1e-3, dtype=torch.float64, device="cuda")
    src = Plan(allp, leaf_size=32, expansion_order=8, instance_offsets=off if batched else None)
    v64 = src.matvec(sigma, areas, None, k_e=1.0).clone()
    same = src.convert(torch.float64)
    assert torch.equal(same.matvec(sigma, areas, None, k_e=1.0), v64)
    p32 = src.convert(torch.float32, 8)
    assert p32.dtype == torch.float32 and p32.info.expansion_order == 8
    for f in ("n_points", "n_nodes", "n_leaves", "n_m2l_pairs", "n_p2p_pairs", "p2p_interactions"):
        assert getattr(p32.info, f) == getattr(src.info, f), f
    t64, t32 = src.export_tree(), p32.export_tree()
    assert torch.equal(t64["index_map"], t32["index_map"])
    assert torch.equal(t64["node_children"], t32["node_children"])
    assert torch.equal(t64["node_centers"].float(), t32["node_centers"])
    l64, l32 = src.export_lists(), p32.export_lists()
    assert all(torch.equal(a, b) for a, b in zip(l64, l32))
    v32 = p32.matvec(sigma.float(), areas.float(), None, k_e=1.0).double()
    err = float(torch.linalg.norm(v32 - v64) / torch.linalg.norm(v64))
    fresh = Plan(allp.float(), leaf_size=32, expansion_order=8, instance_offsets=off if batched else None)
    vf = fresh.matvec(sigma.float(), areas.float(), None, k_e=1.0).double()
    err_fresh = float(torch.linalg.norm(vf - v64) / torch.linalg.norm(v64))
    # as close to the FP64 operator as an FP32 plan built from the FP32 points
    assert err < 1e-5 and err < 2 * err_fresh + 1e-7, (err, err_fresh)
    p6 = src.convert(torch.float32, 6)
    assert p6.info.expansion_order == 6 and p6.info.n_m2l_pairs == src.info.n_m2l_pairs
    v6 = p6.matvec(sigma.float(), areas.float(), None, k_e=1.0).double()
    assert float(torch.linalg.norm(v6 - v64) / torch.linalg.norm(v64)) < 1e-4
    del src  # the copies own their buffers
    assert torch.equal(p32.matvec(sigma.float(), areas.float(), None, k_e=1.0).double(), v32)
    if batched:
        assert p32.n_instances == len(sizes)
        state = torch.zeros(len(sizes), dtype=torch.float64, device="cuda")
        state[1] = 1.0
        p32.set_instance_mask(state, 1)
        try:
            m = p32.matvec(sigma.float(), areas.float(), None, k_e=1.0).double()
        finally:
            p32.set_instance_mask(None)
        a, b = int(off[1]), int(off[2])
        assert torch.equal(m[a:b], v32[a:b])
