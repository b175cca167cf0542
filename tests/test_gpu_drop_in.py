"""The time integrator as the reference drives it (scatter/scatter.py:119-159), on the GPU:
the plain method's small column configuration against the oracle and the 1D analytical
solution, the reference's own call form ``calculate(matrix.M, matrix.C, matrix.K, ...)``,
runs split over several calls, per-call force streaming, and a start from a non-zero
state (the writable u[0, :], v[0, :] of the duck type)."""
import numpy as np
import pytest

import column_case as cc
from helpers import rel_l2

pytestmark = pytest.mark.gpu

LAYOUTS = ["node-block", "csr"]


@pytest.fixture(scope="module")
def torch_cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    from scatter_gb300 import _native

    _native.load()
    return torch


def _column_system():
    from scatter_gb300.system_matrix import GenerateMatrix

    m, time, F, top_eq = cc.build()
    g = GenerateMatrix(m.number_eq, 2)
    g.generate_stiffness_and_mass(m, cc.MATS)
    g.absorbing_boundaries(m, cc.MATS, [1, 1], 1e3)  # no absorbing faces on this column: adds nothing
    g.damping_Rayleigh(cc.DAMPING)
    return g, m, time, F, top_eq


def _solver(layout, time, table, n_eq, receivers=None):
    from scatter_gb300.solvers import NewmarkExplicit

    s = NewmarkExplicit(layout=layout)
    s.output_interval = 1
    s.initialise(n_eq, time)
    s.force_table = table
    s.receivers = receivers
    s.update(0)
    return s


@pytest.mark.parametrize("layout", LAYOUTS)
def test_column_vs_oracle_and_analytical(torch_cuda, layout):
    """Config 1 in full (300 equations, 2000 steps): the GPU history against the oracle's
    direct-solve Newmark on the oracle's own matrices (<= 1e-10, u and v), and the top face's
    mean displacement against the 1D analytical solution (bound and its reasons in
    column_case.py)."""
    from oracle import newmark

    g, m, time, F, top_eq = _column_system()
    s = _solver(layout, time, F.table, m.number_eq)
    s.calculate(g.M, g.C, g.K, F.force_vector, 0, len(time) - 1)
    M, C, K = cc.oracle_matrices(m)
    Fd = np.stack([F.table.dense(t) for t in range(len(time))])
    U, V, _, _ = newmark.solve(M, C, K, Fd, time, 1)
    assert rel_l2(s.u, U) <= 1e-10
    assert rel_l2(s.v, V) <= 1e-10
    ua, _ = cc.analytical_top(time)
    assert rel_l2(s.u[:, top_eq].mean(axis=1), ua) <= cc.U_ANALYTICAL_RTOL
    s.close()


def test_reference_call_form_reaches_the_node_block_solver(torch_cuda):
    """calculate(matrix.M, matrix.C, matrix.K, ...) -- scipy matrices, as scatter.py:159 passes
    them -- runs the node-block FSAI solver from the generator's device arrays and gives the
    same bits as passing the generator; scipy matrices from elsewhere take the CSR loop."""
    import scipy.sparse as sp

    g, m, time, F, top_eq = _column_system()
    a = _solver("node-block", time, F.table, m.number_eq)
    a.calculate(g.M, g.C, g.K, F.force_vector, 0, len(time) - 1)
    assert a.preconditioner == "fsai"
    b = _solver("node-block", time, F.table, m.number_eq)
    b.calculate(g, g, g, F.force_vector, 0, len(time) - 1)
    np.testing.assert_array_equal(a.u, b.u)
    np.testing.assert_array_equal(a.v, b.v)
    c = _solver("node-block", time, F.table, m.number_eq)
    c.calculate(sp.csr_matrix(g.M), sp.csr_matrix(g.C), sp.csr_matrix(g.K), F.force_vector, 0, len(time) - 1)
    assert c.preconditioner == "csr"
    assert rel_l2(c.u, a.u) <= 1e-10
    for s in (a, b, c):
        s.close()


@pytest.mark.parametrize("layout", LAYOUTS)
def test_calls_in_chunks_and_streamed_force(torch_cuda, layout):
    """calculate over 0..n split into several calls continues the device run: the same bits as
    one call.  Streaming each call's force values host -> device gives the same bits again."""
    g, m, time, F, top_eq = _column_system()
    n = 300
    one = _solver(layout, time, F.table, m.number_eq, receivers=top_eq)
    one.calculate(g.M, g.C, g.K, None, 0, n)
    parts = _solver(layout, time, F.table, m.number_eq, receivers=top_eq)
    parts.stream_force = True
    for a, b in ((0, 7), (7, 8), (8, 150), (150, n)):
        parts.calculate(g.M, g.C, g.K, None, a, b)
    np.testing.assert_array_equal(one.u_rec[:n + 1], parts.u_rec[:n + 1])
    np.testing.assert_array_equal(one.v_rec[:n + 1], parts.v_rec[:n + 1])
    np.testing.assert_array_equal(one.a_rec[:n + 1], parts.a_rec[:n + 1])
    assert parts.device_solver.force.h2d_bytes == 8 * int(F.table.f_ptr[n + 1])
    one.close()
    parts.close()


@pytest.mark.parametrize("layout", LAYOUTS)
def test_nonzero_initial_state(torch_cuda, layout):
    """u[0, :] and v[0, :] written after initialise() (rose_utils.py:53-58) start the device run:
    a0 = M^-1 (f0 - C v0 - K u0), then the steps, against the oracle from the same state."""
    from oracle import newmark

    g, m, time, F, top_eq = _column_system()
    n_t = 400
    time = time[:n_t]
    from scatter_gb300.solvers import ForceTable

    table = ForceTable(F.table.f_ptr[:n_t + 1], F.table.f_eq[:F.table.f_ptr[n_t]], F.table.f_val[:F.table.f_ptr[n_t]],
                       m.number_eq)
    rng = np.random.default_rng(3)
    y = m.nodes[:, 2]  # rows of eq_nb_dof follow the node rows
    u0 = np.zeros(m.number_eq)
    v0 = np.zeros(m.number_eq)
    eq = m.eq_nb_dof
    for d, (amp_u, amp_v) in enumerate(((2e-6, 1e-4), (-5e-6, 3e-4), (1e-6, -2e-4))):
        free = ~np.isnan(eq[:, d])
        shape = np.sin(np.pi * y[free] / 20.0)  # smooth: a displaced, moving column
        u0[eq[free, d].astype(int)] = amp_u * shape * (1 + 0.1 * rng.standard_normal(free.sum()))
        v0[eq[free, d].astype(int)] = amp_v * shape
    s = _solver(layout, time, table, m.number_eq)
    s.u[0, :] = u0
    s.v[0, :] = v0
    s.calculate(g.M, g.C, g.K, None, 0, n_t - 1)
    M, C, K = cc.oracle_matrices(m)
    Fd = np.stack([table.dense(t) for t in range(n_t)])
    U, V, A, _ = newmark.solve(M, C, K, Fd, time, 1, u0=u0, v0=v0)
    np.testing.assert_array_equal(s.u[0], u0)
    assert rel_l2(s.a[0], A[0]) <= 1e-10
    assert rel_l2(s.u, U) <= 1e-10
    assert rel_l2(s.v, V) <= 1e-10
    s.close()


def test_continuing_call_reports_a_failure_when_settled(torch_cuda):
    """A continuing call queues its results and returns: a step that fails (here: the PCG
    iteration limit) raises ScatterGpuError when the outputs are read, and the solver is closed."""
    from scatter_gb300 import _native as nat
    from scatter_gb300.solvers import ForceTable, NewmarkExplicit

    g, m, time, F, top_eq = _column_system()
    n_t = 40
    t = F.table
    # no load before step 10: those steps converge at once from rest; the load then needs
    # more than the 2 iterations allowed
    first = int(t.f_ptr[10])
    ptr = np.concatenate([np.zeros(10, dtype=np.int64), t.f_ptr[10:n_t + 1] - first])
    table = ForceTable(ptr, t.f_eq[first:t.f_ptr[n_t]], t.f_val[first:t.f_ptr[n_t]], m.number_eq)
    s = NewmarkExplicit(max_iter=2)
    s.output_interval = 1
    s.initialise(m.number_eq, time[:n_t])
    s.force_table = table
    s.receivers = top_eq
    s.update(0)
    s.calculate(g, g, g, None, 0, 5)
    assert np.abs(s.u_rec[:6]).max() == 0.0
    s.calculate(g, g, g, None, 5, 15)  # queued: no error yet
    with pytest.raises(nat.ScatterGpuError):
        s.v_rec
    assert s.device_solver is None
