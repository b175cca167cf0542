"""Known answers for the explicit scheme's restatement (oracle/explicit.py), which has no
reference counterpart.  For an undamped oscillator (w^2 = k/m) under a step force f0 from rest,
the scheme's recursion u_{n+1} - 2u_n + u_{n-1} = dt^2 (f0/m - w^2 u_n), u_0 = 0,
u_1 = dt^2 f0/m has the closed-form solution

    u_n = f0/k (1 - cos(W t_n) + w^2 dt^2 / (2 sin(W dt)) sin(W t_n)),   sin(W dt/2) = w dt/2,

and the reported velocity is (u_{n+1} - u_n)/dt.  A diagonal system of oscillators checks
every DOF against its own closed form."""
import numpy as np
import scipy.sparse as sp

from oracle import explicit


def _closed_form(w, f0, k, dt, n_t):
    W = 2 * np.arcsin(w * dt / 2) / dt
    t = np.arange(n_t) * dt
    return f0 / k * (1 - np.cos(W * t) + (w * dt) ** 2 / (2 * np.sin(W * dt)) * np.sin(W * t))


def test_oscillators_match_the_closed_form():
    m = np.array([2.0, 1.0, 0.5, 3.0])
    k = np.array([800.0, 50.0, 2000.0, 30.0])
    f0 = np.array([1.0, -2.0, 0.5, 4.0])
    w = np.sqrt(k / m)
    dt = 0.2 * 2 / w.max()  # a fifth of the stability limit of the stiffest oscillator
    n_t = 400
    M, K, Z = sp.diags(m), sp.diags(k), sp.csr_matrix((4, 4))
    U, V = explicit.solve(M, Z, K, 0.0, 0.0, np.tile(f0, (n_t, 1)), n_t, dt)
    for j in range(4):
        ref = _closed_form(w[j], f0[j], k[j], dt, n_t)
        np.testing.assert_allclose(U[:, j], ref, rtol=0, atol=1e-12 * abs(f0[j] / k[j]))
    # the reported velocity at step n+1 is the half-step velocity (u_{n+1} - u_n) / dt
    np.testing.assert_allclose(V[1:], np.diff(U, axis=0) / dt, rtol=1e-12, atol=1e-15)


def test_lumped_mass_of_a_consistent_matrix():
    # a 1D two-node bar element's consistent mass rho A l / 6 [[2, 1], [1, 2]]: row sums are half
    # the element mass on each node; the diagonal-scaled form keeps the total mass too
    Me = np.array([[2.0, 1.0], [1.0, 2.0]]) / 6.0
    np.testing.assert_allclose(explicit.lumped(Me), [0.5, 0.5])
    np.testing.assert_allclose(explicit.hrz(Me, Me.sum() / np.trace(Me)), [0.5, 0.5])


def test_rayleigh_damping_decays_the_free_response():
    # stiffness-proportional damping only: each mode decays, the static offset stays
    m, k = np.array([1.0, 1.0]), np.array([100.0, 400.0])
    f0 = np.array([1.0, 1.0])
    dt, n_t = 0.01, 6000
    U, _ = explicit.solve(sp.diags(m), sp.csr_matrix((2, 2)), sp.diags(k), 0.0, 0.01, np.tile(f0, (n_t, 1)), n_t,
                          dt)
    np.testing.assert_allclose(U[-1], f0 / k, rtol=1e-6)
    assert np.abs(U[1:] - f0 / k).max() > 0.5 * (f0 / k).min()
