"""Ragged batching: meshes of different sizes and element types (hexa8, tetra10) concatenated
into one system and advanced by one explicit kernel per step, against each mesh advanced on
its own and against the oracle's explicit scheme."""
import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu

SPECS = [{"element": "hexa8", "dims": (3, 4, 2), "h": 0.5, "E": 80e6, "nu": 0.25, "rho": 1900.0},
         {"element": "tetra10", "dims": (2, 3, 2), "h": 0.5, "E": 150e6, "nu": 0.3, "rho": 2000.0},
         {"element": "hexa8", "dims": (4, 3, 3), "h": 0.5, "E": 40e6, "nu": 0.33, "rho": 1750.0}]
DAMPING = [1, 0.02, 50, 0.02]
DT, N_T = 5e-5, 240


@pytest.fixture(scope="module")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch


def _run(specs):
    from scatter_gb300.ragged import RaggedExplicit

    tg = np.arange(N_T) * DT
    r = RaggedExplicit(specs, DAMPING, DT, tg, f0=400.0, t0=2.5e-3)
    r.set_output(1, N_T)
    r.run(0, N_T - 1)
    v = r.velocities()
    r.close()
    return v


def test_union_equals_each_mesh_alone(cuda):
    v = _run(SPECS)
    assert np.abs(v).max() > 0
    for k, sp in enumerate(SPECS):
        alone = _run([sp])
        assert rel_l2(v[:, k], alone[:, 0]) <= 1e-12


def test_tetra10_mesh_vs_oracle(cuda):
    """The tetra10 mesh of the union (HRZ-lumped) against oracle/explicit.py with the same
    lumped mass, on the oracle's own element matrices and assembly."""
    from oracle import assembly as asm
    from oracle import elements as el
    from oracle import explicit
    from scatter_gb300 import meshgen
    from scatter_gb300.force_external import ricker_table
    from scatter_gb300.ragged import _top_centre

    v = _run(SPECS)
    sp = SPECS[1]
    m = meshgen.box_model(*sp["dims"], sp["h"], element="tetra10")
    n = len(m.elem)
    X = m.nodes[:, 1:][m.node_index()[m.elem]]
    Ke, Me = el.element_matrices("tetra10", X, np.full(n, sp["E"]), np.full(n, sp["nu"]), np.full(n, sp["rho"]))
    pairs = asm.element_pairs(m.eq_nb_elem)
    K = asm.assemble(m.eq_nb_elem, Ke, m.number_eq, pairs)
    M = asm.assemble(m.eq_nb_elem, Me, m.number_eq, pairs)
    Mx = Me[0][::3, ::3]
    ml = explicit.hrz(M, Mx.sum() / np.trace(Mx))
    assert ml.min() > 0
    alpha, beta = asm.rayleigh_coefficients(DAMPING)
    tg = np.arange(N_T) * DT
    table = ricker_table(m, _top_centre(m), -10e3, 400.0, 2.5e-3, tg)
    F = np.stack([table.dense(t) for t in range(N_T)])
    rec = int(m.eq_nb_dof[m.node_index()[_top_centre(m)], 1])
    _, V = explicit.solve(M, M * 0, K, alpha, beta, F, N_T, DT, rec=[rec], ml=ml)
    assert rel_l2(v[:, 1], V[:, 0]) <= 1e-10


def _run_mf(specs):
    from scatter_gb300.ragged import RaggedBatch

    tg = np.arange(N_T) * DT
    r = RaggedBatch(specs, DAMPING, DT, tg, f0=400.0, t0=2.5e-3)
    r.set_output(1, N_T)
    r.run(0, N_T - 1)
    v = r.velocities()
    r.close()
    return v


def test_matrix_free_union_equals_each_mesh_alone_and_the_assembled_union(cuda):
    """The matrix-free ragged kernel (FP32 products, pair accumulators): bitwise equal to each
    mesh advanced alone (the same per-node arithmetic), and within the batched path's bound
    of the assembled FP64-class union."""
    v = _run_mf(SPECS)
    ref = _run(SPECS)
    assert np.abs(v).max() > 0
    for k, sp in enumerate(SPECS):
        np.testing.assert_array_equal(v[:, k], _run_mf([sp])[:, 0])
        assert rel_l2(v[:, k], ref[:, k]) <= 1e-5
