"""Explicit central-difference scheme with row-sum lumped mass (oracle; test infrastructure).

The reference has no lumped mass and no fixture for an explicit scheme (its mass is always
consistent, scatter/discretisation.py:203-222).  This is the CPU restatement of the explicit
path the GPU build adds, defined as:

    M_L = diag(row sums of M)                      (lumped mass, same total mass)
    C   = Cabs + alpha M_L + beta K                (Rayleigh with the lumped mass; Lysmer as assembled)
    a_n       = M_L^-1 (f_n - K (u_n + beta v_{n-1/2}) - alpha M_L v_{n-1/2} - Cabs v_{n-1/2})
    v_{n+1/2} = v_{n-1/2} + dt a_n
    u_{n+1}   = u_n + dt v_{n+1/2}

from rest (u_0 = 0, v_{-1/2} = 0); the velocity reported at step n+1 is v_{n+1/2}.  It is
conditionally stable (dt below the lumped-mass CFL limit) and converges to the same
continuum solution as the reference's Newmark scheme as dt, h -> 0.
"""
import numpy as np
import scipy.sparse as sp


def lumped(M):
    return np.asarray(sp.csr_matrix(M).sum(axis=1)).ravel()


def hrz(M, factor):
    """Diagonal-scaled lumped mass: factor * diag(M), factor = sum(M_e) / trace(M_e) of the
    element (the lumping the ragged path uses for quadratic tetrahedra)."""
    return factor * sp.csr_matrix(M).diagonal()


def solve(M, Cabs, K, alpha, beta, force, n_t, dt, output_interval=1, rec=None, ml=None):
    """force: dense [n_t, n] or callable t -> f; ml: lumped mass (default: row sums of M).
    Returns (U, V) at output steps (rows for steps 0, k, 2k, ...), restricted to ``rec``."""
    K = sp.csr_matrix(K)
    Cabs = sp.csr_matrix(Cabs)
    ml = lumped(M) if ml is None else np.asarray(ml, dtype=float)
    n = K.shape[0]
    get = force if callable(force) else (lambda t: force[t])
    u = np.zeros(n)
    v = np.zeros(n)
    sel = slice(None) if rec is None else np.asarray(rec)
    outs_u, outs_v = [u[sel].copy()], [v[sel].copy()]
    for t in range(n_t - 1):
        f = np.asarray(get(t), dtype=float)
        a = (f - K @ (u + beta * v) - alpha * ml * v - Cabs @ v) / ml
        v = v + dt * a
        u = u + dt * v
        if (t + 1) % output_interval == 0:
            outs_u.append(u[sel].copy())
            outs_v.append(v[sel].copy())
    return np.array(outs_u), np.array(outs_v)
