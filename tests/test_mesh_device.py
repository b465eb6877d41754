"""Conductor meshes generated on the GPU (core.mesh_device, libedfmm
edfmm_mesh_grid / edfmm_mesh_finish) against the host generators, which
reproduce the reference's bem_mesh.py:27-212: vertices, triangles,
centroids, normals, areas and conductor ids equal bit for bit, degenerate
polar panels removed in the same order."""
import numpy as np
import pytest
import torch


@pytest.mark.parametrize("n_a,n_b", [(10, 20), (41, 80), (500, 200), (1001, 37)])
def test_one_dimensional_trig_tables_equal_the_meshgrid_trig(n_a, n_b):
    # the device path takes sin / cos of the 1-D coordinate arrays; the host
    # generators take them of the meshgrid: element by element they agree
    a = np.linspace(0.0, np.pi, n_a)
    b = np.linspace(0.0, 2.0 * np.pi, n_b, endpoint=False)
    A, B = np.meshgrid(a, b, indexing="ij")
    for f in (np.sin, np.cos):
        assert np.array_equal(f(A), np.broadcast_to(f(a)[:, None], A.shape))
        assert np.array_equal(f(B), np.broadcast_to(f(b)[None, :], B.shape))


def _same(dm, hm):
    h = dm.to_host()
    for k in ("vertices", "triangles", "centroids", "normals", "areas", "conductor_ids"):
        a, b = getattr(h, k), getattr(hm, k)
        assert a.shape == b.shape, k
        assert np.array_equal(a, b), (k, np.max(np.abs(a.astype(float) - b.astype(float))))


SPECS = [
    (dict(conductors=[dict(type="sphere", radius=1.0, center=[0.0, 0.0, 0.0])]), 0.2),
    (dict(conductors=[dict(type="sphere", radius=0.7, center=[0.3, -0.2, 1.1], id=4)]), 0.05),
    (dict(conductors=[dict(type="torus", major_radius=1.0, minor_radius=0.35, potential=1.0)]), 0.1),
    (dict(conductors=[dict(type="plane", z=-0.5)], charges=[dict(type="point", q=1.0, pos=[0.0, 0.0, 1.0])]), 0.6),
    (dict(conductors=[dict(type="sphere", radius=1.0, center=[0.0, 0.0, 0.0]),
                      dict(type="torus", major_radius=1.5, minor_radius=0.2, center=[4.0, 0.0, 0.0]),
                      dict(type="plane", z=-3.0)], charges=[dict(type="point", q=1.0, pos=[0.0, 0.0, 2.0])]), 0.3),
]


@pytest.mark.gpu
@pytest.mark.parametrize("k", range(len(SPECS)))
def test_device_mesh_equals_host_mesh(cuda_lib, k):
    from electrodrive_gb300.core.bem_mesh import generate_mesh
    from electrodrive_gb300.core.mesh_device import generate_mesh_device

    spec, h = SPECS[k]
    _same(generate_mesh_device(spec, h), generate_mesh(spec, h))


@pytest.mark.gpu
def test_device_torus_and_dimers_equal_host(cuda_lib):
    from electrodrive_gb300.core.batch import dimer_case, dimer_case_device
    from electrodrive_gb300.core.bem_mesh import torus_mesh
    from electrodrive_gb300.core.mesh_device import torus_mesh_device

    _same(torus_mesh_device(1.0, 0.35, 500, 200), torus_mesh(1.0, 0.35, 500, 200))
    for seed in (10, 11, 12, 13, 265):
        dm, dspec = dimer_case_device(seed)
        hm, hspec = dimer_case(seed)
        assert dspec == hspec
        _same(dm, hm)


@pytest.mark.gpu
def test_batch_system_from_device_meshes_equals_host_built(cuda_lib):
    """A batched system set up from dimers meshed on the GPU (no geometry
    from the host) equals the one set up from the host meshes: the same
    right-hand side, diagonal and operator, bit for bit."""
    from electrodrive_gb300.core.batch import BatchSystem, dimer_case, dimer_case_device

    seeds = (10, 11, 12)
    host = BatchSystem([dimer_case(s, 3000) for s in seeds])
    dev = BatchSystem([dimer_case_device(s, 3000) for s in seeds])
    assert dev.h2d_bytes == 0 and dev.offsets == host.offsets
    for k in ("b", "diag", "C64", "areas", "normals"):
        assert torch.equal(getattr(dev, k), getattr(host, k)), k
    x = torch.rand(host.n, generator=torch.Generator().manual_seed(0), dtype=torch.float64).to("cuda")
    assert torch.equal(dev.op64(x).clone(), host.op64(x).clone())
