"""Average-acceleration Newmark restated (oracle; test infrastructure only).

The reference calls PuggleSolvers 1.0.1 ``NewmarkExplicit`` (scatter/scatter.py:13,
120-121,155-159), a third-party package that is not vendored.  Its published
scheme, as wired by the reference, is Newmark with beta = 1/4, gamma = 1/2, the
consistent mass matrix and a constant effective matrix factorised once:

    a0 = M^-1 (F0 - C v0 - K u0)
    K^ = K + a4 C + a1 M
    u+ = K^-1 [F+ + M (a1 u + a2 v + a3 a) + C (a4 u + a5 v + a6 a)]
    a+ = a1 (u+ - u) - a2 v - a3 a
    v+ = v + dt ((1 - gamma) a + gamma a+)

with a1 = 1/(beta dt^2), a2 = 1/(beta dt), a3 = 1/(2 beta) - 1,
a4 = gamma/(beta dt), a5 = gamma/beta - 1, a6 = dt (gamma/(2 beta) - 1).
dt = time[1] - time[0] of the reference's time grid (scatter.py:117), constant.  Results are
stored every ``output_interval`` steps including step 0 (results read at
scatter/export_results.py:52-55).  This restatement reproduces every shipped
golden history (tests/test_oracle_golden.py).
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

BETA = 0.25
GAMMA = 0.5


def coefficients(dt, beta=BETA, gamma=GAMMA):
    return (1 / (beta * dt ** 2), 1 / (beta * dt), 1 / (2 * beta) - 1,
            gamma / (beta * dt), gamma / beta - 1, dt * (gamma / (2 * beta) - 1))


def solve(M, C, K, force, time, output_interval=1, u0=None, v0=None):
    """force: callable t -> F[n_eq] or dense array [n_t, n_eq].  Returns (u, v, a, out_time)."""
    M = sp.csc_matrix(M)
    C = sp.csc_matrix(C)
    K = sp.csc_matrix(K)
    n = M.shape[0]
    n_t = len(time)
    get = force if callable(force) else (lambda t: force[t])
    u = np.zeros(n) if u0 is None else np.array(u0, dtype=float)
    v = np.zeros(n) if v0 is None else np.array(v0, dtype=float)
    f0 = np.asarray(get(0), dtype=float)
    r0 = f0 - C @ v - K @ u
    a = spla.spsolve(M, r0) if np.any(r0) else np.zeros(n)
    out_idx = list(range(0, n_t, output_interval))
    U = np.zeros((len(out_idx), n))
    V = np.zeros_like(U)
    A = np.zeros_like(U)
    U[0], V[0], A[0] = u, v, a
    k = 1
    dt = time[1] - time[0]
    a1, a2, a3, a4, a5, a6 = coefficients(dt)
    lu = spla.splu(sp.csc_matrix(K + a4 * C + a1 * M))
    for t in range(1, n_t):
        rhs = np.asarray(get(t), dtype=float) + M @ (a1 * u + a2 * v + a3 * a) + C @ (a4 * u + a5 * v + a6 * a)
        un = lu.solve(rhs)
        an = a1 * (un - u) - a2 * v - a3 * a
        vn = v + dt * ((1 - GAMMA) * a + GAMMA * an)
        u, v, a = un, vn, an
        if t % output_interval == 0:
            U[k], V[k], A[k] = u, v, a
            k += 1
    return U, V, A, np.asarray(time)[out_idx]
