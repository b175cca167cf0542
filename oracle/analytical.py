"""1D analytical wave propagation in a column (oracle; test infrastructure only).

Restates the reference's analytical check, integration_tests/analytical_solutions/
analytical_wave_prop.py:49-85 (OneDimWavePropagation.solution), which follows the
published series solution of Churchill, Operational Mathematics, 3rd ed., pp. 253-257:
a column of length L, fixed at x = 0, with a pressure step p0 applied at x = L at t = 0,
wave speed c = sqrt(K / rho) for the (constrained) modulus K:

    lambda_k = (2k - 1) pi / (2L)
    u(x, t) = p0/K (x + 8L/pi^2 sum_k (-1)^k / (2k-1)^2 sin(lambda_k x) cos(lambda_k c t))
    v(x, t) = p0/K 8L/pi^2 sum_k -(-1)^k lambda_k c / (2k-1)^2 sin(lambda_k x) sin(lambda_k c t)

summed over k = 1 .. n_terms - 1 as the reference does.  The reference passes the
constrained modulus E (1 - nu) / ((1 + nu)(1 - 2 nu)) when nu != 0
(integration_tests/test_benchmark_set_2.py:97-106 passes E with nu = 0).  Positive p0
stretches the column; a compressive top load gives the negated response.
"""
import numpy as np


def constrained_modulus(E, nu):
    return E * (1 - nu) / ((1 + nu) * (1 - 2 * nu))


def column_response(x, time, p0, K, rho, L, n_terms=1000):
    """(u, v) at height x above the fixed base for every t in ``time``."""
    t = np.asarray(time, dtype=float)
    c = np.sqrt(K / rho)
    k = np.arange(1, n_terms, dtype=float)
    lam = (2 * k - 1) * np.pi / (2 * L)
    sgn = np.where(k % 2 == 1, -1.0, 1.0) / (2 * k - 1) ** 2
    ph = np.outer(t, lam * c)
    su = (sgn * np.sin(lam * x) * np.cos(ph)).sum(axis=1)
    sv = (-sgn * lam * c * np.sin(lam * x) * np.sin(ph)).sum(axis=1)
    scale = 8 * L / np.pi ** 2
    return p0 / K * (x + scale * su), p0 / K * (scale * sv)
