"""Global assembly restated in numpy (oracle; test infrastructure only).

Restates GenerateMatrix.generate_stiffness_and_mass (scatter/system_matrix.py:35-121):
for every element in order, the element's free equation numbers are sorted
(:90-95) and every (row, col) pair accumulates Ke/Me into a dict keyed by the
pair (:98-103), i.e. each global entry is the element-order sum of its
contributions; the result is a COO -> lil matrix over the element graph
(:108-121) that keeps explicit zeros.  Rayleigh damping restates
GenerateMatrix.damping_Rayleigh (system_matrix.py:166-198).
"""
import numpy as np
import scipy.sparse as sp


def element_pairs(eq_nb_elem):
    """(row, col, elem, local_i, local_j) for every free DOF pair of every element,
    ordered by element then by (sorted row eq, sorted col eq) as in system_matrix.py:90-103."""
    eq = np.asarray(eq_nb_elem, dtype=float)
    E, nd = eq.shape
    rows, cols, els, li, lj = [], [], [], [], []
    for e in range(E):
        free = np.where(~np.isnan(eq[e]))[0]
        i1 = eq[e, free].astype(np.int64)
        o = np.argsort(i1, kind="stable")
        i1, i2 = i1[o], free[o]
        R, C = np.meshgrid(i1, i1, indexing="ij")
        LI, LJ = np.meshgrid(i2, i2, indexing="ij")
        rows.append(R.ravel())
        cols.append(C.ravel())
        li.append(LI.ravel())
        lj.append(LJ.ravel())
        els.append(np.full(R.size, e))
    return (np.concatenate(rows), np.concatenate(cols), np.concatenate(els),
            np.concatenate(li), np.concatenate(lj))


def assemble(eq_nb_elem, Ke, n_eq, pairs=None):
    """Element-order summed CSR over the element graph (explicit zeros kept)."""
    r, c, e, li, lj = element_pairs(eq_nb_elem) if pairs is None else pairs
    v = np.asarray(Ke)[e, li, lj]
    key = r * n_eq + c
    order = np.argsort(key, kind="stable")  # stable: keeps element order inside a key
    key, v = key[order], v[order]
    starts = np.concatenate([[0], np.nonzero(np.diff(key))[0] + 1])
    vals = np.add.reduceat(v, starts)
    uk = key[starts]
    A = sp.csr_matrix((vals, (uk // n_eq, uk % n_eq)), shape=(n_eq, n_eq))
    # csr_matrix from COO with unique keys keeps explicit zeros
    A.sort_indices()
    return A


def drop_zeros(A):
    """scipy's sparse + sparse drops exact zeros (system_matrix.py:198,375-376)."""
    A = sp.csr_matrix(A, copy=True)
    A.eliminate_zeros()
    return A


def rayleigh_coefficients(damp):
    """(alpha, beta) from [f1, xi1, f2, xi2]: system_matrix.py:166-198."""
    f1, d1, f2, d2 = damp
    if f1 == f2:
        raise SystemExit("Frequencies for the Rayleigh damping are the same.")
    A = 0.5 * np.array([[1 / (2 * np.pi * f1), 2 * np.pi * f1], [1 / (2 * np.pi * f2), 2 * np.pi * f2]])
    return np.linalg.solve(A, np.array([d1, d2]))


def rayleigh(M, K, C0, damp):
    """C = C0 + (alpha M + beta K) with the reference's zero-dropping additions."""
    a, b = rayleigh_coefficients(damp)
    return drop_zeros(sp.csr_matrix(C0) + drop_zeros(sp.csr_matrix(M) * a + sp.csr_matrix(K) * b))
