"""The Newmark PCG's dot product r.z with the split FSAI preconditioner z = G^T G r, checked on
the CPU (numpy, the small column's effective matrix A = M + dt/2 C + dt^2/4 K).  The device
loop forms r.z as |G r|^2 in the lower preconditioner half (beside t = G r), so beta is known
before the upper half, which writes p = z + beta p itself.  The two forms are the same number
in exact arithmetic; with the device's FP16 factor and FP32 products they differ at FP32
rounding, and the PCG reaches the tolerance in the same number of iterations either way."""
import numpy as np
import scipy.sparse as sp

import column_case as cc


def _effective():
    m, _, _, _ = cc.build()
    M, C, K = cc.oracle_matrices(m)
    dt = cc.DT
    return sp.csr_matrix(M + (dt / 2) * C + (dt * dt / 4) * K)


def _fsai(A):
    """Lower-triangular FSAI factor on A's lower pattern: row i solves A[S, S] y = e_last on
    S = {j <= i : A_ij != 0} and takes g = y / sqrt(y_last), so G A G^T has a unit diagonal."""
    A = A.tocsr()
    n = A.shape[0]
    rows, cols, vals = [], [], []
    for i in range(n):
        S = A.indices[A.indptr[i]:A.indptr[i + 1]]
        S = np.sort(S[S <= i])
        e = np.zeros(len(S))
        e[-1] = 1.0
        y = np.linalg.solve(A[S][:, S].toarray(), e)
        g = y / np.sqrt(y[-1])
        rows += [i] * len(S)
        cols += list(S)
        vals += list(g)
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, n))


def _pcg(A, G, b, tol, dot_from_t, fp32, max_it=300):
    """PCG from rest with z = G^T (G r); rz either r.z or |t|^2 with t = G r.  fp32: r and t
    rounded to FP32 before the products, as the device's lower and upper halves read them."""
    GT = G.T.tocsr()
    x = np.zeros_like(b)
    r = b.copy()
    nb = np.linalg.norm(b)
    p = None
    rz_old = None
    for it in range(max_it + 1):
        rr = r.astype(np.float32).astype(np.float64) if fp32 else r
        t = G @ rr
        if fp32:
            t = t.astype(np.float32).astype(np.float64)
        z = GT @ t
        if fp32:
            z = z.astype(np.float32).astype(np.float64)
        rz = t @ t if dot_from_t else r @ z
        p = z if p is None else z + (rz / rz_old) * p
        rz_old = rz
        w = A @ p
        alpha = rz / (p @ w)
        x += alpha * p
        r -= alpha * w
        if np.linalg.norm(r) <= tol * nb:
            return x, it + 1
    raise AssertionError("no convergence")


def test_split_dot_equals_the_norm_of_g_r():
    A = _effective()
    G = _fsai(A)
    # G A G^T has a unit diagonal (the FSAI normalisation)
    assert np.allclose((G @ A @ G.T).diagonal(), 1.0, rtol=1e-10)
    rng = np.random.default_rng(3)
    for _ in range(10):
        r = rng.standard_normal(A.shape[0])
        t = G @ r
        assert abs(r @ (G.T @ t) - t @ t) <= 1e-13 * (t @ t)


def test_pcg_with_the_dot_from_the_lower_half():
    A = _effective()
    G16 = _fsai(A)
    G16.data = G16.data.astype(np.float16).astype(np.float64)  # the device's FP16 factor planes
    rng = np.random.default_rng(5)
    b = A @ rng.standard_normal(A.shape[0])
    tol = 1e-10
    for fp32 in (False, True):
        xa, ia = _pcg(A, G16, b, tol, dot_from_t=False, fp32=fp32)
        xb, ib = _pcg(A, G16, b, tol, dot_from_t=True, fp32=fp32)
        assert abs(ia - ib) <= 1, (fp32, ia, ib)
        for x in (xa, xb):
            assert np.linalg.norm(b - A @ x) <= 1.01 * tol * np.linalg.norm(b)
        if not fp32:  # exact-arithmetic forms: the same iterates to rounding
            assert ia == ib
            assert np.linalg.norm(xa - xb) <= 1e-12 * np.linalg.norm(xa)
