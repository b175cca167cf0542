"""Batched realisations and random fields on the GPU against per-realisation FP64 solves
and the oracle's restatement of the field generator."""
import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch


def test_random_field_matches_oracle(cuda):
    from oracle import random_fields as orf
    from scatter_gb300 import device as dv
    from scatter_gb300.random_fields import lognormal_fields

    rng = np.random.default_rng(3)
    pts = rng.uniform(0, 10, size=(300, 3))
    f_gpu = dv.host(lognormal_fields(pts, seed=1234, R=3, lengths=(5.0, 1.0, 5.0), mean=50e6, sd=12.5e6,
                                     n_modes=64))
    f_ref = orf.lognormal_field(pts, 1234, 3, 64, (5.0, 1.0, 5.0), 50e6, 12.5e6)
    assert np.abs(np.log(f_gpu) - np.log(f_ref)).max() <= 2e-4


@pytest.mark.parametrize("model,angles", [("Exponential", 0.0), ("Matern", 0.0), ("Gaussian", [0.5, -0.3, 1.1]),
                                          ("Matern", [0.2, 0.0, 0.7])])
def test_random_field_models_match_oracle(cuda, model, angles):
    """The other covariance models and the rotation by angles (random_fields.py:79-88) on the
    GPU against the oracle's restatement of the same draws."""
    from oracle import random_fields as orf
    from scatter_gb300 import device as dv
    from scatter_gb300.random_fields import lognormal_fields, rotation

    rng = np.random.default_rng(5)
    pts = rng.uniform(0, 10, size=(300, 3))
    np.testing.assert_allclose(rotation(3, angles), orf.rotation(3, angles), rtol=0, atol=1e-15)
    f_gpu = dv.host(lognormal_fields(pts, seed=77, R=3, lengths=(4.0, 1.5, 6.0), mean=50e6, sd=12.5e6, n_modes=64,
                                     model=model, angles=angles))
    f_ref = orf.lognormal_field(pts, 77, 3, 64, (4.0, 1.5, 6.0), 50e6, 12.5e6, model=model,
                                rot=orf.rotation(3, angles))
    assert np.abs(np.log(f_gpu) - np.log(f_ref)).max() <= 2e-4


def test_random_field_statistics(cuda):
    from scatter_gb300 import device as dv
    from scatter_gb300.random_fields import lognormal_fields, lognormal_params

    pts = np.zeros((1, 3))
    R = 1024
    f = dv.host(lognormal_fields(pts, seed=7, R=R, lengths=(5.0, 5.0, 1.0), mean=50e6, sd=12.5e6)).ravel()
    mu, sig = lognormal_params(50e6, 12.5e6)
    g = np.log(f)
    assert abs(g.mean() - mu) <= 4 * sig / np.sqrt(R)
    assert abs(g.std() / sig - 1) <= 0.1
    # correlation at one correlation length along x: exp(-pi/4) for the Gaussian model
    pts2 = np.array([[0.0, 0.0, 0.0], [5.0, 0.0, 0.0]])
    h = np.log(dv.host(lognormal_fields(pts2, seed=7, R=R, lengths=(5.0, 5.0, 1.0), mean=50e6, sd=12.5e6)))
    rho = np.corrcoef(h[0], h[1])[0, 1]
    assert abs(rho - np.exp(-np.pi / 4)) <= 0.08


def test_batched_matches_per_realisation_fp64(cuda):
    """R realisations in one launch (FP32 products, FP64 state) vs R separate FP64 explicit
    solves with the same per-element E: relative L2 <= 1e-5."""
    from scatter_gb300 import device as dv
    from scatter_gb300 import meshgen
    from scatter_gb300.batched import BatchedExplicit
    from scatter_gb300.explicit import ExplicitLumped
    from scatter_gb300.force_external import ricker_table
    from scatter_gb300.random_fields import element_centroids, lognormal_fields
    from scatter_gb300.system_matrix import GenerateMatrix

    m = meshgen.box_model(8, 4, 4, 0.5, bottom="020", x_faces="200", z_faces="002")
    R = 4
    young = lognormal_fields(element_centroids(m), seed=11, R=R, lengths=(5.0, 1.0, 5.0), mean=50e6, sd=12.5e6)
    nu, rho = 0.3, 1900.0
    damping, absorbing, kdiv = [1, 0.02, 50, 0.02], [1, 1], 1e3
    dt, n_t = 5e-5, 400
    time = np.linspace(0, dt * (n_t - 1), n_t)
    top = m.top_nodes()
    node = int(top[len(top) // 2])
    table = ricker_table(m, node, -1e4, 20.0, 0.01, time)
    rec = [int(m.eq_nb_dof[m.node_index()[n], 1]) for n in top[::7]]
    b = BatchedExplicit(m, young, nu, rho, damping, absorbing, kdiv, dt)
    b.set_force(table)
    b.set_output(1, rec, n_t)
    b.run(0, n_t - 1)
    vb = b.velocities()
    ub, _ = b.state()
    yh = dv.host(young).astype(float)
    for r in range(R):
        g = GenerateMatrix(m.number_eq, 2)
        n_el = len(m.elem)
        g.generate_stiffness_and_mass(m, None, element_props=(yh[:, r], np.full(n_el, nu), np.full(n_el, rho)))
        g.absorbing_boundaries(m, None, absorbing, kdiv)
        g.damping_Rayleigh(damping)
        s = ExplicitLumped()
        s.initialise(m.number_eq, time)
        s.force_table = table
        s.calculate(g, g, g, None, 0, n_t - 1)
        assert rel_l2(vb[:, :, r], s.v[:, rec]) <= 1e-5
        assert rel_l2(ub[r], s.u[-1]) <= 1e-5


def test_batched_shapes_agree_bitwise(cuda):
    """Every kernel and shape the tuner may pick (the incidence-list kernel with 1 to 8
    realisations per thread, the tiled uniform hexa8 grid kernel with 1 or 2, the node-centric
    one with 2 to 8) gives bitwise the same histories: the per-realisation arithmetic and
    summation order are the same."""
    from scatter_gb300 import meshgen
    from scatter_gb300.batched import BatchedExplicit
    from scatter_gb300.force_external import ricker_table
    from scatter_gb300.random_fields import element_centroids, lognormal_fields

    m = meshgen.box_model(6, 4, 3, 0.5, bottom="020", x_faces="200", z_faces="002")
    R = 8
    young = lognormal_fields(element_centroids(m), seed=5, R=R, lengths=(5.0, 1.0, 5.0), mean=50e6, sd=12.5e6)
    dt, n_t = 5e-5, 120
    time = np.linspace(0, dt * (n_t - 1), n_t)
    top = m.top_nodes()
    table = ricker_table(m, int(top[len(top) // 2]), -1e4, 20.0, 0.002, time)
    rec = [int(m.eq_nb_dof[m.node_index()[n], 1]) for n in top[::5]]
    results = []
    shapes = ((1, 128, False), (1, 256, False), (2, 128, False), (4, 256, False), (8, 128, False), (1, 128, True),
              (1, 256, True), (2, 128, True), (2, 256, True), (2, 128, "node"), (4, 256, "node"), (8, 128, "node"),
              (2, 256, "node-wide"), (4, 128, "node-wide"))
    for rpt, tpb, grid in shapes:
        b = BatchedExplicit(m, young, 0.3, 1900.0, [1, 0.02, 50, 0.02], [1, 1], 1e3, dt)
        assert b.grid_tables is not None
        b.set_shape(rpt, tpb, grid)
        b.set_force(table)
        b.set_output(1, rec, n_t)
        b.run(0, n_t - 1)
        results.append((b.velocities(), b.state()[0]))
        b.close()
    assert np.abs(results[0][0]).max() > 0
    for vb, ub in results[1:]:
        np.testing.assert_array_equal(vb, results[0][0])
        np.testing.assert_array_equal(ub, results[0][1])


def test_batched_grid_kernel_on_a_notched_mesh(cuda):
    """The uniform-grid kernels (tiled and node-centric) on a box with a block of elements cut
    out of a top corner (halo points without nodes, nodes with fewer than 8 elements) give
    bitwise the incidence-list kernel's histories."""
    from scatter_gb300 import meshgen
    from scatter_gb300.batched import BatchedExplicit
    from scatter_gb300.force_external import ricker_table
    from scatter_gb300.mesher import ReadMesh
    from scatter_gb300.random_fields import element_centroids, lognormal_fields

    nx, ny, nz, h = 8, 5, 6, 0.5
    nodes, elem, _ = meshgen.box_hexa8(nx, ny, nz, h)
    X = nodes[:, 1:]
    idx = {int(n): k for k, n in enumerate(nodes[:, 0])}
    cen = np.stack([X[[idx[int(n)] for n in e]].mean(axis=0) for e in elem])
    lo = X.min(axis=0)
    keep = ~((cen[:, 0] > lo[0] + 2.0) & (cen[:, 1] > lo[1] + 1.5) & (cen[:, 2] > lo[2] + 1.0))
    elem = elem[keep]
    used = np.isin(nodes[:, 0], np.unique(elem))
    m = ReadMesh.from_arrays(nodes[used], elem, "hexa8", [[3, 1, "solid"]], np.ones(len(elem), dtype=np.int64))
    m.read_bc(meshgen.box_boundaries(nx * h, ny * h, nz * h, "111", "100", "001"))  # no Lysmer faces
    m.mapping()
    m.connectivities()
    R = 8
    young = lognormal_fields(element_centroids(m), seed=9, R=R, lengths=(2.0, 1.0, 2.0), mean=50e6, sd=12.5e6)
    dt, n_t = 5e-5, 100
    time = np.linspace(0, dt * (n_t - 1), n_t)
    top = m.top_nodes()
    table = ricker_table(m, int(top[0]), -1e4, 40.0, 0.002, time)
    rec = [int(m.eq_nb_dof[m.node_index()[n], 1]) for n in top[::2]]
    results = []
    for rpt, tpb, grid in ((4, 256, False), (1, 256, True), (2, 256, True), (4, 128, "node"), (8, 256, "node"),
                           (2, 256, "node-wide")):
        b = BatchedExplicit(m, young, 0.3, 1900.0, [1, 0.02, 50, 0.02], [1, 1], 1e3, dt)
        assert b.grid_tables is not None
        b.set_shape(rpt, tpb, grid)
        b.set_force(table)
        b.set_output(1, rec, n_t)
        b.run(0, n_t - 1)
        results.append((b.velocities(), b.state()[0]))
        b.close()
    assert np.abs(results[0][0]).max() > 0
    for vb, ub in results[1:]:
        np.testing.assert_array_equal(vb, results[0][0])
        np.testing.assert_array_equal(ub, results[0][1])


def _tc_case(notched):
    from scatter_gb300 import meshgen
    from scatter_gb300.mesher import ReadMesh

    nx, ny, nz, h = 9, 5, 6, 0.5
    if not notched:
        return meshgen.box_model(nx, ny, nz, h, bottom="020", x_faces="200", z_faces="002")
    nodes, elem, _ = meshgen.box_hexa8(nx, ny, nz, h)
    X = nodes[:, 1:]
    idx = {int(n): k for k, n in enumerate(nodes[:, 0])}
    cen = np.stack([X[[idx[int(n)] for n in e]].mean(axis=0) for e in elem])
    lo = X.min(axis=0)
    keep = ~((cen[:, 0] > lo[0] + 2.0) & (cen[:, 1] > lo[1] + 1.5) & (cen[:, 2] > lo[2] + 1.0))
    elem = elem[keep]
    used = np.isin(nodes[:, 0], np.unique(elem))
    m = ReadMesh.from_arrays(nodes[used], elem, "hexa8", [[3, 1, "solid"]], np.ones(len(elem), dtype=np.int64))
    m.read_bc(meshgen.box_boundaries(nx * h, ny * h, nz * h, "111", "100", "001"))
    m.mapping()
    m.connectivities()
    return m


@pytest.mark.parametrize("notched", [False, True])
def test_tensor_core_step(cuda, notched):
    """The tensor-core step (tcgen05, TF32 in three hi/lo products) on 128 realisations: against
    the CUDA-core kernel (FP32 products) for several column segment lengths, and against
    per-realisation FP64-class explicit solves, on a box with Lysmer faces and on a notched box
    (lattice points without nodes, nodes with fewer than 8 elements)."""
    from scatter_gb300 import device as dv
    from scatter_gb300.batched import BatchedExplicit
    from scatter_gb300.explicit import ExplicitLumped
    from scatter_gb300.force_external import ricker_table
    from scatter_gb300.random_fields import element_centroids, lognormal_fields
    from scatter_gb300.system_matrix import GenerateMatrix

    m = _tc_case(notched)
    R = 128
    young = lognormal_fields(element_centroids(m), seed=21, R=R, lengths=(2.0, 1.0, 2.0), mean=50e6, sd=12.5e6)
    nu, rho = 0.3, 1900.0
    damping, absorbing, kdiv = [1, 0.02, 50, 0.02], [1, 1], 1e3
    dt, n_t = 5e-5, 200
    time = np.linspace(0, dt * (n_t - 1), n_t)
    top = m.top_nodes()
    table = ricker_table(m, int(top[len(top) // 3]), -1e4, 40.0, 0.002, time)
    rec = [int(m.eq_nb_dof[m.node_index()[n], 1]) for n in top[::3]]

    def run(shape):
        b = BatchedExplicit(m, young, nu, rho, damping, absorbing, kdiv, dt)
        assert b.column_tables is not None
        if shape is None:
            b.set_shape(4, 256, False)
        else:
            b.set_tensor_core_shape(shape)
        b.set_force(table)
        b.set_output(1, rec, n_t)
        b.run(0, n_t - 1)
        b.status()
        out = (b.velocities(), b.state()[0])
        b.close()
        return out

    v0, u0 = run(None)
    assert np.abs(v0).max() > 0
    for seg in (100, 3, 1):  # the whole column, segments of 3 points, single planes
        vt, ut = run(seg)
        assert rel_l2(vt, v0) <= 2e-6, seg
        assert rel_l2(ut, u0) <= 2e-6, seg
    yh = dv.host(young).astype(float)
    n_el = len(m.elem)
    for r in (0, 77):
        g = GenerateMatrix(m.number_eq, 2)
        g.generate_stiffness_and_mass(m, None, element_props=(yh[:, r], np.full(n_el, nu), np.full(n_el, rho)))
        g.absorbing_boundaries(m, None, absorbing, kdiv)
        g.damping_Rayleigh(damping)
        s = ExplicitLumped()
        s.initialise(m.number_eq, time)
        s.force_table = table
        s.calculate(g, g, g, None, 0, n_t - 1)
        assert rel_l2(vt[:, :, r], s.v[:, rec]) <= 1e-5
