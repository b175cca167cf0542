"""ctypes wrapper of the oracle's C Newmark/PCG loop (test infrastructure only)."""
import ctypes

import numpy as np
import scipy.sparse as sp

from . import cbuild

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(cbuild.build())
        P, I, L, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double
        _lib.oc_newmark_run.restype = I
        _lib.oc_newmark_run.argtypes = [L, P, P, P, P, P, D, D, I, I, I, I, P, P, P, P, P, P, I, P, P,
                                        ctypes.POINTER(L)]
        _lib.oc_threads.restype = I
    return _lib


def threads():
    return lib().oc_threads()


def _p(a):
    return None if a is None else a.ctypes.data


class NewmarkCPU:
    """State + CSR (shared pattern) for the C loop."""

    def __init__(self, M, C, K, dt, rtol=1e-12, max_iter=1000):
        pat = (sp.csr_matrix(M) + sp.csr_matrix(C) + sp.csr_matrix(K)).tocsr()
        pat.sort_indices()
        self.n = pat.shape[0]
        self.rowptr = pat.indptr.astype(np.int64)
        self.cols = pat.indices.astype(np.int32)

        def on(X):
            X = sp.csr_matrix(X)
            Z = sp.csr_matrix((np.zeros(pat.nnz), pat.indices, pat.indptr), shape=pat.shape) + X
            Z = sp.csr_matrix(Z)
            Z.sort_indices()
            if Z.nnz != pat.nnz:
                out = np.zeros(pat.nnz)
                r = np.repeat(np.arange(self.n), np.diff(Z.indptr)).astype(np.int64) * self.n + Z.indices
                s = np.repeat(np.arange(self.n), np.diff(pat.indptr)).astype(np.int64) * self.n + pat.indices
                out[np.searchsorted(s, r)] = Z.data
                return out
            return np.ascontiguousarray(Z.data)

        self.M, self.C, self.K = on(M), on(C), on(K)
        self.dt, self.rtol, self.max_iter = float(dt), float(rtol), int(max_iter)
        self.u = np.zeros(self.n)
        self.v = np.zeros(self.n)
        self.a = np.zeros(self.n)

    @classmethod
    def from_csr(cls, n, rowptr, cols, M, C, K, dt, rtol=1e-12, max_iter=1000):
        self = cls.__new__(cls)
        self.n = int(n)
        self.rowptr = np.ascontiguousarray(rowptr, dtype=np.int64)
        self.cols = np.ascontiguousarray(cols, dtype=np.int32)
        self.M, self.C, self.K = (np.ascontiguousarray(x, dtype=np.float64) for x in (M, C, K))
        self.dt, self.rtol, self.max_iter = float(dt), float(rtol), int(max_iter)
        self.u = np.zeros(self.n)
        self.v = np.zeros(self.n)
        self.a = np.zeros(self.n)
        return self

    def run(self, t_begin, n_steps, f_ptr, f_eq, f_val, rec=None):
        f_ptr = np.ascontiguousarray(f_ptr, dtype=np.int64)
        f_eq = np.ascontiguousarray(f_eq, dtype=np.int32)
        f_val = np.ascontiguousarray(f_val, dtype=np.float64)
        rec = None if rec is None else np.ascontiguousarray(rec, dtype=np.int32)
        out = None if rec is None else np.zeros((n_steps, len(rec)))
        it = ctypes.c_int64()
        rc = lib().oc_newmark_run(self.n, _p(self.rowptr), _p(self.cols), _p(self.M), _p(self.C), _p(self.K), self.dt,
                                  self.rtol, self.max_iter, int(t_begin), int(n_steps), len(f_ptr) - 1, _p(f_ptr),
                                  _p(f_eq), _p(f_val), _p(self.u), _p(self.v), _p(self.a),
                                  0 if rec is None else len(rec), _p(rec), _p(out), ctypes.byref(it))
        if rc:
            raise RuntimeError(f"oracle C Newmark failed with status {rc}")
        return out, it.value
