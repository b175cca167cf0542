"""The argument behind the Newmark PCG on the FP32 matrix, checked on the CPU (numpy, the small
column's effective matrix A = M + dt/2 C + dt^2/4 K): with Ah = A rounded to FP32 and
Al = A - Ah, L = sqrt(||Al||_1 ||Al||_inf) bounds ||Al||_2, so a CG on Ah that stops at
|r| + L |x - x0| <= tol |b| leaves the true residual |b - A x| within tol |b|.  The device
solver forms L and applies that stopping test (sc_nb_set_options bits 3 and 4)."""
import numpy as np
import scipy.sparse as sp

import column_case as cc


def _effective():
    m, _, _, _ = cc.build()
    M, C, K = cc.oracle_matrices(m)
    dt = cc.DT
    A = sp.csr_matrix(M + (dt / 2) * C + (dt * dt / 4) * K)
    Ah = A.copy()
    Ah.data = Ah.data.astype(np.float32).astype(np.float64)
    Al = A - Ah
    return A, Ah, Al


def _lo_norm(Al):
    a = abs(Al)
    return float(np.sqrt(a.sum(axis=0).max() * a.sum(axis=1).max()))


def test_lo_norm_bounds_the_lo_part():
    A, Ah, Al = _effective()
    L = _lo_norm(Al)
    assert 0 < L <= 2.0 ** -24 * abs(A).sum(axis=1).max()
    rng = np.random.default_rng(1)
    for _ in range(20):
        x = rng.standard_normal(A.shape[0])
        assert np.linalg.norm(Al @ x) <= L * np.linalg.norm(x)
    # against the spectral norm itself
    dense = Al.toarray()
    assert np.linalg.norm(dense, 2) <= L * (1 + 1e-12)


def _cg_fp32_matrix(A, Ah, L, b, x0, tol, max_it=500):
    """Jacobi-PCG on Ah from x0 with the FP32-matrix stopping test; returns x and whether the
    bound alone passed half the tolerance (the device solver restarts in pairs then).  The
    initial residual is the full one, b - A x0 (the device solver's pair residual); only the
    correction x - x0 goes through Ah, so b - A x = r - Al (x - x0)."""
    d = 1.0 / Ah.diagonal()
    x = x0.copy()
    r = b - A @ x0
    z = d * r
    p = z.copy()
    rz = r @ z
    nb = np.linalg.norm(b)
    for _ in range(max_it):
        w = Ah @ p
        alpha = rz / (p @ w)
        x += alpha * p
        r -= alpha * w
        e = L * np.linalg.norm(x - x0)
        if e > 0.5 * tol * nb:
            return x, True
        if np.linalg.norm(r) + e <= tol * nb:
            return x, False
        z = d * r
        rz, rz_old = r @ z, rz
        p = z + (rz / rz_old) * p
    raise AssertionError("no convergence")


def test_stopping_test_bounds_the_true_residual():
    """From a warm start with a small initial residual the bound holds and the true residual
    meets the tolerance; from rest (large residual) the bound passes half the tolerance, which
    is where the device solver restarts in pairs."""
    A, Ah, Al = _effective()
    L = _lo_norm(Al)
    rng = np.random.default_rng(7)
    x_true = rng.standard_normal(A.shape[0])
    b = A @ x_true
    tol = 1e-12
    for scale in (1e-10, 1e-9, 1e-8):
        x0 = x_true + scale * rng.standard_normal(A.shape[0]) * np.abs(x_true).max()
        x, gave_up = _cg_fp32_matrix(A, Ah, L, b, x0, tol)
        assert not gave_up
        assert np.linalg.norm(b - A @ x) <= tol * np.linalg.norm(b)
    _, gave_up = _cg_fp32_matrix(A, Ah, L, b, np.zeros_like(b), tol)
    assert gave_up
