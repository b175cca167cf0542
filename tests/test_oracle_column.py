"""The small plain-method column (tests/column_case.py) on the CPU: the oracle's Newmark
against the 1D analytical solution, and the series restatement against its own limits."""
import numpy as np

import column_case as cc
from helpers import rel_l2


def test_series_limits():
    """u(x, 0) = 0 along the column, the time mean of u(L, t) over whole periods is the static
    p0 L / K, and v is the time derivative of u."""
    from oracle import analytical

    K, L, rho, p0 = 2e8, 10.0, 2000.0, 1e3
    c = np.sqrt(K / rho)
    x = np.linspace(0.5, L, 20)
    u0 = np.array([analytical.column_response(xi, [0.0], p0, K, rho, L, n_terms=4000)[0][0] for xi in x])
    assert np.abs(u0).max() <= 2e-3 * p0 * L / K
    period = 4 * L / c
    t = np.linspace(0, 3 * period, 30001)[:-1]
    u, v = analytical.column_response(L, t, p0, K, rho, L, n_terms=400)
    assert abs(u.mean() - p0 * L / K) <= 1e-3 * p0 * L / K
    du = np.gradient(u, t)
    inner = slice(100, -100)
    assert rel_l2(du[inner], v[inner]) <= 0.05  # central differences across the kinks


def test_column_oracle_vs_analytical():
    from oracle import newmark

    m, time, F, top_eq = cc.build()
    assert m.number_eq == 300 and len(m.nodes) == 189 and len(m.elem) == 80
    M, C, K = cc.oracle_matrices(m)
    Fd = np.stack([F.table.dense(t) for t in range(len(time))])
    U, V, _, _ = newmark.solve(M, C, K, Fd, time, 1)
    ua, _ = cc.analytical_top(time)
    assert rel_l2(U[:, top_eq].mean(axis=1), ua) <= cc.U_ANALYTICAL_RTOL
