"""GPU time integrators with the duck type the reference drives (scatter/scatter.py:119-159).

``NewmarkExplicit`` has the interface of PuggleSolvers 1.0.1's class of that name as
the reference uses it:

    numerical = NewmarkExplicit()
    numerical.output_interval = k                       # scatter.py:137
    numerical.initialise(n_eq, time)                    # scatter.py:138
    numerical.update_rhs_at_time_step_func = F.update_load_at_t   # scatter.py:151
    numerical.update(0)                                 # scatter.py:158
    numerical.calculate(M, C, K, F0, 0, len(time) - 1)  # scatter.py:159
    numerical.u, numerical.v, numerical.a, numerical.output_time   # export_results.py:52-55

The scheme is the average-acceleration Newmark (beta = 1/4, gamma = 1/2) with consistent
mass that PuggleSolvers' NewmarkExplicit implements; the linear solve of each step is a
device-side Jacobi-PCG (``sc_newmark_*`` in include/scatter_gb300.h).
"""
import ctypes

import numpy as np
import scipy.sparse as sp
import torch

from . import _native as nat
from . import device as dv
from .system_matrix import DeviceCSR, GenerateMatrix


class ForceTable:
    """Force history as CSR over time steps: at step t, f = sum f_val[k] e_{f_eq[k]}."""

    def __init__(self, f_ptr, f_eq, f_val, n_eq):
        self.f_ptr = np.asarray(f_ptr, dtype=np.int64)
        self.f_eq = np.asarray(f_eq, dtype=np.int32)
        self.f_val = np.asarray(f_val, dtype=np.float64)
        self.n_eq = int(n_eq)

    @property
    def n_t(self):
        return len(self.f_ptr) - 1

    @classmethod
    def from_callback(cls, func, n_t, n_eq):
        """Sample a per-step force callback (dense vectors) into a table."""
        ptr, eqs, vals = [0], [], []
        for t in range(n_t):
            f = np.asarray(func(t), dtype=float)
            nz = np.nonzero(f)[0]
            eqs.append(nz)
            vals.append(f[nz])
            ptr.append(ptr[-1] + len(nz))
        return cls(ptr, np.concatenate(eqs) if eqs else [], np.concatenate(vals) if vals else [], n_eq)

    @classmethod
    def from_dense(cls, F):
        F = np.asarray(F, dtype=float)
        return cls.from_callback(lambda t: F[t], F.shape[0], F.shape[1])

    def dense(self, t):
        f = np.zeros(self.n_eq)
        s = slice(self.f_ptr[t], self.f_ptr[t + 1])
        f[self.f_eq[s]] = self.f_val[s]
        return f


def _device_matrices(M, C, K):
    """Upload scipy M, C, K onto their union pattern (structural entries, explicit zeros kept)."""
    mats = [sp.csr_matrix(x, dtype=float, copy=True) for x in (M, C, K)]
    n = mats[0].shape[0]
    keys = []
    for X in mats:
        X.sum_duplicates()
        r = np.repeat(np.arange(n, dtype=np.int64), np.diff(X.indptr))
        keys.append(r * n + X.indices)
    allk = np.unique(np.concatenate(keys))
    rows, cols = allk // n, allk % n
    indptr = np.zeros(n + 1, dtype=np.int64)
    indptr[1:] = np.cumsum(np.bincount(rows, minlength=n))
    vals = []
    for X, k in zip(mats, keys):
        v = np.zeros(len(allk))
        v[np.searchsorted(allk, k)] = X.data
        vals.append(dv.to_dev(v, torch.float64))
    pat = DeviceCSR(n, dv.to_dev(indptr, torch.int64), dv.to_dev(cols.astype(np.int32), torch.int32))
    return (pat, *vals)


class NewmarkGPU:
    """Device state + step loop on a shared CSR pattern (thin owner of the C-ABI handle)."""

    def __init__(self, pattern, M, C, K, dt, rtol=1e-12, max_iter=1000):
        self.pattern = pattern
        n = pattern.n
        self.n = n
        self.M, self.C, self.K = M, C, K
        self.A = dv.empty(max(pattern.nnz, 1), torch.float64)[:pattern.nnz]
        self.u = dv.zeros(n, torch.float64)
        self.v = dv.zeros(n, torch.float64)
        self.a = dv.zeros(n, torch.float64)
        wsn = nat.value("sc_newmark_workspace_doubles", n, 0)
        self.ws = dv.empty(wsn, torch.float64)
        h = ctypes.c_void_p()
        nat.call("sc_newmark_create", ctypes.byref(h), n, pattern.rowptr.data_ptr(), pattern.cols.data_ptr(),
                 M.data_ptr(), C.data_ptr(), K.data_ptr(), self.A.data_ptr(), float(dt), float(rtol), int(max_iter),
                 self.u.data_ptr(), self.v.data_ptr(), self.a.data_ptr(), self.ws.data_ptr(), wsn, dv.stream_ptr())
        self.h = h
        self._keep = []

    def set_force(self, table: ForceTable):
        self._keep_force = [dv.to_dev(table.f_ptr, torch.int64), dv.to_dev(table.f_eq, torch.int32),
                            dv.to_dev(table.f_val, torch.float64)]
        p, e, v = self._keep_force
        nat.call("sc_newmark_set_force", self.h, table.n_t, p.data_ptr(), e.data_ptr(), v.data_ptr())

    def set_output(self, interval, rec_eq, n_out, what=("u", "v", "a")):
        self.rec = dv.to_dev(np.asarray(rec_eq, dtype=np.int32), torch.int32)
        nr = self.rec.numel()
        self.out = {k: (dv.zeros(n_out * nr, torch.float64) if k in what else None) for k in ("u", "v", "a")}
        nat.call("sc_newmark_set_output", self.h, int(interval), nr, self.rec.data_ptr(),
                 *(dv.ptr(self.out[k]) for k in ("u", "v", "a")), int(n_out))
        self.n_out, self.n_rec = int(n_out), nr

    def initial_acceleration(self):
        nat.call("sc_newmark_initial_acceleration", self.h)

    def run(self, t_begin, t_end):
        nat.call("sc_newmark_run", self.h, int(t_begin), int(t_end))

    def status(self):
        tot = ctypes.c_int64()
        mx = ctypes.c_int()
        rc = nat.value("sc_newmark_status", self.h, ctypes.byref(tot), ctypes.byref(mx))
        return rc, tot.value, mx.value

    def outputs(self):
        return {k: (None if t is None else dv.host(t).reshape(self.n_out, self.n_rec)) for k, t in self.out.items()}

    def close(self):
        if getattr(self, "h", None):
            nat.value("sc_newmark_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class NewmarkExplicit:
    """GPU drop-in for PuggleSolvers' NewmarkExplicit as called by scatter/scatter.py:120-159."""

    def __init__(self, rtol=1e-12, max_iter=1000):
        self.output_interval = 1
        self.update_rhs_at_time_step_func = None
        self.rtol = rtol
        self.max_iter = max_iter
        self.receivers = None  # optional equation subset for the outputs (default: all)
        self.force_table = None  # optional ForceTable (skips sampling the callback)
        self.iterations = None

    def initialise(self, number_equations, time):
        self.number_equations = int(number_equations)
        self.time = np.asarray(time, dtype=float)
        n_out = len(range(0, len(self.time), self.output_interval))
        self.output_time = self.time[::self.output_interval][:n_out]
        self.u = np.zeros((n_out, self.number_equations))
        self.v = np.zeros_like(self.u)
        self.a = np.zeros_like(self.u)

    def update(self, t_idx):
        self.t_idx = t_idx

    def calculate(self, M, C, K, F, t_start_idx, t_end_idx):
        """Run steps t_start_idx .. t_end_idx on the GPU.  M, C, K: scipy matrices, or the
        GenerateMatrix that produced them (its device arrays are used without a copy)."""
        if isinstance(M, GenerateMatrix):
            g = M
            pat, Md, Cd, Kd = g.pattern, g.M_d, g.C_d, g.K_d
        else:
            pat, Md, Cd, Kd = _device_matrices(M, C, K)
        n = pat.n
        dt = self.time[1] - self.time[0]
        n_t = len(self.time)
        table = self.force_table
        if table is None:
            if self.update_rhs_at_time_step_func is not None:
                table = ForceTable.from_callback(self.update_rhs_at_time_step_func, n_t, n)
            else:
                F0 = np.asarray(F, dtype=float)
                table = ForceTable.from_callback(lambda t: F0, n_t, n)
        solver = NewmarkGPU(pat, Md, Cd, Kd, dt, self.rtol, self.max_iter)
        solver.set_force(table)
        rec = np.arange(n) if self.receivers is None else np.asarray(self.receivers)
        n_out = len(range(0, n_t, self.output_interval))
        solver.set_output(self.output_interval, rec, n_out)
        solver.initial_acceleration()
        solver.run(t_start_idx, t_end_idx)
        rc, tot, mx = solver.status()
        if rc != 0:
            raise nat.ScatterGpuError("sc_newmark_run", rc, nat.load().sc_status_string(rc).decode(), "")
        out = solver.outputs()
        self.iterations = (tot, mx)
        if self.receivers is None:
            self.u, self.v, self.a = out["u"], out["v"], out["a"]
        else:
            self.u_rec, self.v_rec, self.a_rec = out["u"], out["v"], out["a"]
        solver.close()
