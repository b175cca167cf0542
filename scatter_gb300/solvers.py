"""GPU time integrators with the duck type the reference drives (scatter/scatter.py:119-159).

``NewmarkExplicit`` has the interface of PuggleSolvers 1.0.1's class of that name as
the reference uses it:

    numerical = NewmarkExplicit()
    numerical.output_interval = k                       # scatter.py:137
    numerical.initialise(n_eq, time)                    # scatter.py:138
    numerical.u[0, :], numerical.v[0, :] = u0, v0       # optional initial state (rose_utils.py:53-58)
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
from .system_matrix import DeviceCSR, GenerateMatrix, generator_of


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


class _DeviceForce:
    """A force table on the device, as the step kernels read it: step pointers, target
    indices (equations or slots) and values.

    Resident (default): the whole history is copied once.  Streamed: the pointers and the
    indices go up once, and each run copies the values of the steps it reads -- steps
    t_begin .. t_end, since step t -> t + 1 clears the entries of step t and adds those of
    step t + 1 -- from pinned host memory on the solver's stream, as a caller feeding
    loads step by step would."""

    def __init__(self, table, index, stream=False):
        n = max(len(table.f_val), 1)
        self.ptr_h = np.asarray(table.f_ptr, dtype=np.int64)
        self.ptr = dv.to_dev(self.ptr_h, torch.int64)
        self.idx = dv.zeros(n, torch.int32)
        if len(table.f_val):
            self.idx[:len(table.f_val)] = index
        self.stream = bool(stream)
        if self.stream:
            self.val = dv.zeros(n, torch.float64)
            self.val_h = torch.from_numpy(np.ascontiguousarray(table.f_val, dtype=np.float64)).pin_memory()
            self.pushed = -1  # last step whose values are on the device
        else:
            self.val = dv.zeros(n, torch.float64)
            if len(table.f_val):
                self.val[:len(table.f_val)] = dv.to_dev(table.f_val, torch.float64)
        self.h2d_bytes = 0

    def push(self, t_begin, t_end):
        """Before a run over steps t_begin .. t_end: copy the values it reads (streamed)."""
        if not self.stream:
            return
        n_t = len(self.ptr_h) - 1
        first = max(t_begin, self.pushed + 1)
        last = min(t_end, n_t - 1)
        if last < first:
            return
        a, b = int(self.ptr_h[first]), int(self.ptr_h[last + 1])
        if b > a:
            self.val[a:b].copy_(self.val_h[a:b], non_blocking=True)
            self.h2d_bytes += (b - a) * 8
        self.pushed = last


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

    def __init__(self, pattern, M, C, K, dt, rtol=1e-12, max_iter=1000, spmv="pair", order_cap=True):
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
        # bit 0: the PCG SpMV in FP64 instead of FP32 pairs; bit 1: no cap on the warm-start
        # order at kinks of the force history
        nat.call("sc_newmark_set_options", self.h, {"pair": 0, "fp64": 1}[spmv] | (0 if order_cap else 2))
        self._keep = []

    def warm_start_status(self):
        """(the controller's current warm-start order, steps whose order the force history capped)."""
        o = ctypes.c_int()
        c = ctypes.c_int64()
        nat.call("sc_newmark_warm_start_status", self.h, ctypes.byref(o), ctypes.byref(c))
        return o.value, c.value

    def set_force(self, table: ForceTable, stream=False):
        """Force history (equation indices).  stream=True: values copied per run (push_force)."""
        eq = dv.to_dev(table.f_eq, torch.int32) if len(table.f_eq) else None
        self.force = _DeviceForce(table, eq, stream)
        f = self.force
        nat.call("sc_newmark_set_force", self.h, table.n_t, f.ptr.data_ptr(), f.idx.data_ptr(), f.val.data_ptr())

    def push_force(self, t_begin, t_end):
        self.force.push(t_begin, t_end)

    def set_output(self, interval, rec_eq, n_out, what=("u", "v", "a")):
        self.rec = dv.to_dev(np.asarray(rec_eq, dtype=np.int32), torch.int32)
        nr = self.rec.numel()
        self.out = {k: (dv.zeros(n_out * nr, torch.float64) if k in what else None) for k in ("u", "v", "a")}
        nat.call("sc_newmark_set_output", self.h, int(interval), nr, self.rec.data_ptr(),
                 *(dv.ptr(self.out[k]) for k in ("u", "v", "a")), int(n_out))
        self.n_out, self.n_rec = int(n_out), nr

    def set_state(self, u0, v0):
        """Initial displacement and velocity (equation order) in place of rest; before
        initial_acceleration(), which then solves M a0 = f(0) - C v0 - K u0."""
        self.u.copy_(dv.to_dev(np.asarray(u0, dtype=float), torch.float64))
        self.v.copy_(dv.to_dev(np.asarray(v0, dtype=float), torch.float64))

    def initial_acceleration(self):
        nat.call("sc_newmark_initial_acceleration", self.h)

    def run(self, t_begin, t_end):
        nat.call("sc_newmark_run", self.h, int(t_begin), int(t_end))

    def set_predictor(self, order):
        """Order (1..8) of the extrapolated accelerations each step's PCG starts from; 0 (the
        default) adapts the order to the iteration counts."""
        nat.call("sc_newmark_set_predictor", self.h, int(order))

    def status(self):
        tot = ctypes.c_int64()
        mx = ctypes.c_int()
        rc = nat.value("sc_newmark_status", self.h, ctypes.byref(tot), ctypes.byref(mx))
        return rc, tot.value, mx.value

    def status_to(self, dev3):
        """Queue (status, total iterations, largest per-step count) into dev3 (device int64[3])."""
        nat.call("sc_newmark_status_to", self.h, dev3.data_ptr())

    def outputs(self):
        return {k: (None if t is None else dv.host(t).reshape(self.n_out, self.n_rec)) for k, t in self.out.items()}

    def output_rows(self, r0, r1):
        """Output rows r0 .. r1 (host arrays [r1 - r0 + 1, n_rec]); None for what is not kept."""
        nr = self.n_rec
        return {k: (None if t is None else dv.host(t[r0 * nr:(r1 + 1) * nr]).reshape(-1, nr))
                for k, t in self.out.items()}

    def close(self):
        if getattr(self, "h", None):
            nat.value("sc_newmark_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class NodeBlockNewmark:
    """Node-block time loop for matrices assembled by GenerateMatrix (sc_nb_* C-ABI).

    State in slot space (slot = node * dim + dof); the eq <-> slot maps translate force
    entries, receivers and outputs from/to the reference's equation numbering."""

    def __init__(self, g, dt, rtol=1e-12, max_iter=1000, precond="fsai", spmv="pair", explicit="pair",
                 residual="pair", fp32_matrix="auto", order_cap=True):
        if g.adj_ptr is None:
            raise ValueError("GenerateMatrix has no node structure")
        self.g = g
        D, N = g.dim, g.n_nodes
        self.D, self.N = D, N
        self.n_s = D * N
        eqmap = g.eqmap_d.view(-1).long()
        free = eqmap >= 0
        slots = torch.arange(self.n_s, device=eqmap.device)
        self.eq2slot = torch.full((g.n_eq,), -1, dtype=torch.int64, device=eqmap.device)
        self.eq2slot[eqmap[free]] = slots[free]
        # Lysmer dashpots as a slot-space CSR
        if g.Cabs_d is not None:
            nz = torch.nonzero(g.Cabs_d).view(-1)
            rp = g.pattern.rowptr
            rows_eq = torch.searchsorted(rp, nz, right=True) - 1
            cols_eq = g.pattern.cols[nz].long()
            rs, cs, vs = self.eq2slot[rows_eq], self.eq2slot[cols_eq], g.Cabs_d[nz]
            key = rs * self.n_s + cs
            o = torch.argsort(key)
            rs, cs, vs = rs[o], cs[o], vs[o]
            cnt = torch.bincount(rs, minlength=self.n_s)
        else:
            cs = torch.zeros(0, dtype=torch.int64, device=eqmap.device)
            vs = torch.zeros(0, dtype=torch.float64, device=eqmap.device)
            cnt = torch.zeros(self.n_s, dtype=torch.int64, device=eqmap.device)
        self.cab_ptr = torch.zeros(self.n_s + 1, dtype=torch.int64, device=eqmap.device)
        self.cab_ptr[1:] = torch.cumsum(cnt, 0)
        self.cab_col = cs.to(torch.int32).contiguous()
        self.cab_val = vs.to(torch.float64).contiguous()
        if self.cab_col.numel() == 0:
            self.cab_col = torch.zeros(1, dtype=torch.int32, device=eqmap.device)
            self.cab_val = torch.zeros(1, dtype=torch.float64, device=eqmap.device)
        self.u = dv.zeros(self.n_s, torch.float64)
        self.v = dv.zeros(self.n_s, torch.float64)
        self.a = dv.zeros(self.n_s, torch.float64)
        self.u0_eq = self.v0_eq = None  # initial conditions other than rest (set_state)
        nnzb = int(g.adj.numel())
        wsb = nat.value("sc_nb_workspace_bytes", N, D, nnzb)
        self.ws = dv.empty(wsb, torch.uint8)
        h = ctypes.c_void_p()
        nat.call("sc_nb_create", ctypes.byref(h), N, D, g.eqmap_d.data_ptr(), g.adj_ptr.data_ptr(), g.adj.data_ptr(),
                 nnzb, g.pattern.rowptr.data_ptr(), g.pattern.cols.data_ptr(), g.K_d.data_ptr(), g.M_d.data_ptr(),
                 g.C_d.data_ptr(), int(cnt.sum().item()), self.cab_ptr.data_ptr(), self.cab_col.data_ptr(),
                 self.cab_val.data_ptr(), float(g.alpha), float(g.beta), float(dt), float(rtol), int(max_iter),
                 {"fsai": 0, "jacobi": 1}[precond], self.u.data_ptr(), self.v.data_ptr(), self.a.data_ptr(), self.ws.data_ptr(), wsb, dv.stream_ptr())
        self.h = h
        self.dt = dt
        # bit 0: PCG SpMV in FP64 instead of FP32 pairs; bit 1: explicit K w in FP64; bit 2: the
        # step's residual always in FP64 (by default it runs in pairs and hands over to FP64 by
        # itself when the load is nearly balanced by the elastic and inertial forces); bits 3, 4:
        # the PCG on the FP32 matrix (A's hi parts) never / at every step, instead of when the
        # bound on its error allows (the answer meets rtol either way); bit 5: no cap on the
        # warm-start order at kinks of the force history
        nat.call("sc_nb_set_options", self.h, {"pair": 0, "fp64": 1}[spmv] | {"pair": 0, "fp64": 2}[explicit] |
                 {"pair": 0, "fp64": 4}[residual] | {"auto": 0, "never": 8, "always": 16}[fp32_matrix] |
                 (0 if order_cap else 32))

    def warm_start_status(self):
        """(the controller's current warm-start order, steps whose order the force history capped)."""
        o = ctypes.c_int()
        c = ctypes.c_int64()
        nat.call("sc_nb_warm_start_status", self.h, ctypes.byref(o), ctypes.byref(c))
        return o.value, c.value

    def fp32_matrix_status(self):
        """(steps whose PCG started on the FP32 matrix, steps that switched to it during the
        solve, restarts in pairs, the bound L on ||A - Ah||_2)."""
        a = ctypes.c_int64()
        w = ctypes.c_int64()
        r = ctypes.c_int64()
        lo = ctypes.c_double()
        nat.call("sc_nb_a32_status", self.h, ctypes.byref(a), ctypes.byref(w), ctypes.byref(r), ctypes.byref(lo))
        return a.value, w.value, r.value, lo.value

    def residual_fp64(self):
        """True when the step's residual runs in FP64 (synchronises)."""
        f = ctypes.c_int()
        nat.call("sc_nb_residual_fp64", self.h, ctypes.byref(f))
        return bool(f.value)

    def set_predictor(self, order):
        """Order (1..8) of the extrapolated accelerations each step's PCG starts from; 0 (the
        default) adapts the order to the iteration counts."""
        nat.call("sc_nb_set_predictor", self.h, int(order))

    def set_force(self, table: ForceTable, stream=False):
        """Force history (equation indices, mapped to slots here).  stream=True: the values
        are copied from pinned host memory by push_force before each run."""
        eq = dv.to_dev(table.f_eq, torch.int64)
        slot = self.eq2slot[eq].to(torch.int32) if eq.numel() else None
        if slot is not None and bool((slot < 0).any()):
            raise ValueError("force on a fixed DOF")
        self.force = _DeviceForce(table, slot, stream)
        self.table = table
        f = self.force
        nat.call("sc_nb_set_force", self.h, table.n_t, f.ptr.data_ptr(), f.idx.data_ptr(), f.val.data_ptr())

    def push_force(self, t_begin, t_end):
        self.force.push(t_begin, t_end)

    def set_output(self, interval, rec_eq, n_out, what=("u", "v", "a")):
        rec = self.eq2slot[dv.to_dev(np.asarray(rec_eq, dtype=np.int64), torch.int64)].to(torch.int32).contiguous()
        self.rec = rec
        nr = rec.numel()
        self.out = {k: (dv.zeros(n_out * nr, torch.float64) if k in what else None) for k in ("u", "v", "a")}
        nat.call("sc_nb_set_output", self.h, int(interval), nr, rec.data_ptr(),
                 *(dv.ptr(self.out[k]) for k in ("u", "v", "a")), int(n_out))
        self.n_out, self.n_rec = int(n_out), nr

    def set_state(self, u0, v0):
        """Initial displacement and velocity in equation order (the reference solver's
        u[0, :] and v[0, :]) in place of rest; before initial_acceleration()."""
        self.u0_eq, self.v0_eq = np.asarray(u0, dtype=float), np.asarray(v0, dtype=float)
        free = self.eq2slot >= 0
        self.u[self.eq2slot[free]] = dv.to_dev(self.u0_eq, torch.float64)[free]
        self.v[self.eq2slot[free]] = dv.to_dev(self.v0_eq, torch.float64)[free]

    def initial_acceleration(self):
        """a0 = M^-1 (f(0) - C v0 - K u0); zero for a start from rest without load at t = 0
        (pulse, heaviside, moving loads all start at 0), else solved with the CSR path."""
        t = self.table
        loaded = t.f_ptr[1] > t.f_ptr[0] and np.any(t.f_val[t.f_ptr[0]:t.f_ptr[1]] != 0)
        if loaded or self.u0_eq is not None:
            g = self.g
            csr = NewmarkGPU(g.pattern, g.M_d, g.C_d, g.K_d, self.dt)
            csr.set_force(t)
            if self.u0_eq is not None:
                csr.set_state(self.u0_eq, self.v0_eq)
            csr.initial_acceleration()
            a_eq = csr.a
            free = self.eq2slot >= 0
            self.a[self.eq2slot[free]] = a_eq[free]
            csr.close()
        # step-0 output row
        for k, buf in self.out.items():
            if buf is not None:
                src = {"u": self.u, "v": self.v, "a": self.a}[k]
                buf[:self.n_rec] = src[self.rec.long()]

    def run(self, t_begin, t_end):
        nat.call("sc_nb_run", self.h, int(t_begin), int(t_end))

    def status(self):
        tot = ctypes.c_int64()
        mx = ctypes.c_int()
        fb = ctypes.c_int()
        rc = nat.value("sc_nb_status", self.h, ctypes.byref(tot), ctypes.byref(mx), ctypes.byref(fb))
        self.fsai_fallback_rows = fb.value
        return rc, tot.value, mx.value

    def status_to(self, dev3):
        """Queue (status, total iterations, largest per-step count) into dev3 (device int64[3])."""
        nat.call("sc_nb_status_to", self.h, dev3.data_ptr())

    def time_spmv(self, reps=20, a32=False):
        """ms per launch and algorithmic bytes per launch of the PCG SpMV; a32: the form that
        applies the FP32 matrix (A's hi planes) alone."""
        ms = ctypes.c_float()
        by = ctypes.c_int64()
        nat.call("sc_nb_time_spmv_a32", self.h, int(bool(a32)), int(reps), ctypes.byref(ms), ctypes.byref(by))
        return ms.value, by.value

    def apply(self, which, x_eq):
        """Op x for testing: x in the reference's equation numbering (host) -> Op x (host)."""
        ops = {"A": 0, "K": 1, "M": 2, "P": 3, "Cabs": 4}
        x = torch.zeros(self.n_s, dtype=torch.float64, device=self.u.device)
        x[self.eq2slot] = dv.to_dev(np.asarray(x_eq, dtype=float), torch.float64)
        y = torch.zeros_like(x)
        nat.call("sc_nb_apply", self.h, ops[which], x.data_ptr(), y.data_ptr())
        return dv.host(y[self.eq2slot])

    def run_explicit(self, t_begin, t_end):
        nat.call("sc_nb_explicit_run", self.h, int(t_begin), int(t_end))

    def tune_explicit(self, reps=5):
        """Pick the explicit step's threads per node row by timing; returns (choice, ms/step)."""
        tpr, ms = ctypes.c_int(), ctypes.c_float()
        nat.call("sc_nb_tune_explicit", self.h, int(reps), ctypes.byref(tpr), ctypes.byref(ms))
        return tpr.value, ms.value

    def time_explicit(self, reps=20):
        ms = ctypes.c_float()
        nat.call("sc_nb_time_explicit", self.h, int(reps), ctypes.byref(ms))
        return ms.value

    def outputs(self):
        return {k: (None if t is None else dv.host(t).reshape(self.n_out, self.n_rec)) for k, t in self.out.items()}

    def output_rows(self, r0, r1):
        """Output rows r0 .. r1 (host arrays [r1 - r0 + 1, n_rec]); None for what is not kept."""
        nr = self.n_rec
        return {k: (None if t is None else dv.host(t[r0 * nr:(r1 + 1) * nr]).reshape(-1, nr))
                for k, t in self.out.items()}

    def state_eq(self):
        """u, v, a in the reference's equation numbering (host arrays)."""
        free = self.eq2slot
        return tuple(dv.host(x[free]) for x in (self.u, self.v, self.a))

    def close(self):
        if getattr(self, "h", None):
            nat.value("sc_nb_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class NewmarkExplicit:
    """GPU drop-in for PuggleSolvers' NewmarkExplicit as called by scatter/scatter.py:120-159.

    ``calculate(M, C, K, F, t_start, t_end)`` takes the matrices as scipy CSR or as the
    GenerateMatrix that assembled them.  Scipy matrices that this package's GenerateMatrix
    handed out (``m.M, m.C, m.K``, the reference's call form) are recognised and run from
    the generator's device arrays on the node-block solver; any other scipy matrices are
    uploaded and run on the CSR loop.

    The device solver outlives the call: a later call with the same matrices, time grid and
    force that starts where the previous one ended (t_start == previous t_end) continues
    the run on the device, and fills rows t_start .. t_end of the outputs.  With
    ``stream_force = True`` each call copies the force values of its own steps host ->
    device (pinned memory) instead of the whole history at set-up.  ``close()`` frees the
    device solver.

    A continuing call returns once its steps, the device -> host copies of their outputs and
    of the run's status are queued: the outputs (u, v, a, or u_rec, v_rec, a_rec with
    receivers) and ``iterations`` are settled when they are read or at the next call, which
    queues its own steps first, so the GPU runs one call's steps while the host handles the
    previous call's results.  A failed step raises at that point."""

    def __init__(self, rtol=1e-12, max_iter=1000, layout="node-block", spmv="pair", residual="pair",
                 fp32_matrix="auto"):
        self.output_interval = 1
        self.layout = layout  # "node-block" (matrices from GenerateMatrix) or "csr"
        self.spmv = spmv  # PCG SpMV arithmetic (both layouts): "pair" (FP32 pairs) or "fp64"
        self.residual = residual  # node-block step residual: "pair" (hands over to FP64 by itself) or "fp64"
        # node-block PCG on the FP32 matrix when its error bound allows ("auto"), "never" or "always"
        self.fp32_matrix = fp32_matrix
        self.update_rhs_at_time_step_func = None
        self.rtol = rtol
        self.max_iter = max_iter
        self.receivers = None  # optional equation subset for the outputs (default: all)
        self.force_table = None  # optional ForceTable (skips sampling the callback)
        self.stream_force = False
        self._iterations = None
        self.preconditioner = None
        self._live = None  # (key, device solver, last step reached)
        self._pending = None  # queued outputs and status of the last continuing call
        self._rec = {}

    def initialise(self, number_equations, time):
        self.close()
        self.number_equations = int(number_equations)
        self.time = np.asarray(time, dtype=float)
        n_out = len(range(0, len(self.time), self.output_interval))
        self.output_time = self.time[::self.output_interval][:n_out]
        # u, v, a [n_out, n_eq] are made on first use: a run that records receivers only never
        # touches them (at 1.79 M equations and 10,001 outputs each would be 134 GiB)
        self._hist = {}
        self._hist_shape = (n_out, self.number_equations)

    def _history(self, key):
        self._settle()
        if key not in self._hist:
            self._hist[key] = np.zeros(self._hist_shape)  # zero pages, committed as written
        return self._hist[key]

    u = property(lambda self: self._history("u"), lambda self, x: self._hist.__setitem__("u", x))
    v = property(lambda self: self._history("v"), lambda self, x: self._hist.__setitem__("v", x))
    a = property(lambda self: self._history("a"), lambda self, x: self._hist.__setitem__("a", x))

    def _receiver(self, key):
        self._settle()
        return self._rec.get(key)

    u_rec = property(lambda self: self._receiver("u"))
    v_rec = property(lambda self: self._receiver("v"))
    a_rec = property(lambda self: self._receiver("a"))

    @property
    def iterations(self):
        """(total PCG iterations of the run, largest per step)."""
        self._settle()
        return self._iterations

    def update(self, t_idx):
        self.t_idx = t_idx

    def _force(self, n, n_t, F):
        table = self.force_table
        if table is None:
            if self.update_rhs_at_time_step_func is not None:
                table = ForceTable.from_callback(self.update_rhs_at_time_step_func, n_t, n)
            else:
                F0 = np.asarray(F, dtype=float)
                table = ForceTable.from_callback(lambda t: F0, n_t, n)
            self.force_table = table
        return table

    def _start(self, g, mats, F, t_start_idx, t_end_idx):
        """New device solver, initial state, initial acceleration and the run's first steps."""
        pat, Md, Cd, Kd = mats
        n = pat.n
        dt = self.time[1] - self.time[0]
        n_t = len(self.time)
        table = self._force(n, n_t, F)
        rec = np.arange(n) if self.receivers is None else np.asarray(self.receivers)
        n_out = len(range(0, n_t, self.output_interval))
        # the reference solver's u[0, :] and v[0, :] are writable initial conditions
        ic = None
        hist = getattr(self, "_hist", {})
        if any(k in hist and np.any(hist[k][0]) for k in ("u", "v")):
            ic = (np.array(self.u[0], dtype=float), np.array(self.v[0], dtype=float))
        attempts = ["fsai", "csr"] if (g is not None and self.layout == "node-block" and g.adj_ptr is not None) \
            else ["csr"]
        for kind in attempts:
            if kind == "csr":
                solver = NewmarkGPU(pat, Md, Cd, Kd, dt, self.rtol, self.max_iter, spmv=self.spmv)
            else:
                solver = NodeBlockNewmark(g, dt, self.rtol, self.max_iter, precond=kind, spmv=self.spmv,
                                          residual=self.residual, fp32_matrix=self.fp32_matrix)
            solver.set_force(table, stream=self.stream_force)
            solver.set_output(self.output_interval, rec, n_out)
            if ic is not None:
                solver.set_state(*ic)
            solver.push_force(0, 0)  # the initial acceleration reads the force at t = 0
            solver.initial_acceleration()
            solver.push_force(t_start_idx, t_end_idx)
            solver.run(t_start_idx, t_end_idx)
            rc, tot, mx = solver.status()
            self.preconditioner = kind
            # the node-block PCG stops with a breakdown status when A is not positive definite:
            # the reference's tetra10 operators can make it so (its 4-point rule leaves the
            # consistent mass singular, and its tri6 Lysmer dashpot matrix is indefinite).
            # Redo the solve with the CSR FP64 loop, which runs the reference's iteration as is
            if rc == 3 and kind == "fsai":
                solver.close()
                continue
            break
        return solver, rc, tot, mx, (0, t_end_idx)

    def calculate(self, M, C, K, F, t_start_idx, t_end_idx):
        """Run steps t_start_idx .. t_end_idx on the GPU.  M, C, K: scipy matrices, or the
        GenerateMatrix that produced them (its device arrays are used without a copy)."""
        if isinstance(M, GenerateMatrix):
            g = M
        else:
            g = generator_of(M, C, K)
        key = (id(g) if g is not None else (id(M), id(C), id(K)), id(self.time), id(self.force_table),
               self.layout, self.spmv, self.residual, self.fp32_matrix, self.output_interval)
        live = self._live
        if live is not None and live[0] == key and t_start_idx == live[2] and t_end_idx >= t_start_idx:
            solver = live[1]
            solver.push_force(t_start_idx, t_end_idx)
            solver.run(t_start_idx, t_end_idx)
            # the matrices stay referenced while the run is live, so their ids stay theirs
            self._live = (key, solver, t_end_idx, (M, C, K))
            # the previous call's results, while this call's steps run behind them
            self._settle()
            self._queue(solver, (t_start_idx, t_end_idx))
            return
        self.close()
        mats = (g.pattern, g.M_d, g.C_d, g.K_d) if g is not None else _device_matrices(M, C, K)
        solver, rc, tot, mx, rows = self._start(g, mats, F, t_start_idx, t_end_idx)
        key = key[:2] + (id(self.force_table),) + key[3:]
        if rc != 0:
            solver.close()
            raise nat.ScatterGpuError("time loop", rc, nat.load().sc_status_string(rc).decode(), "")
        self._live = (key, solver, t_end_idx, (M, C, K))
        self._iterations = (tot, mx)
        self._copy_outputs(solver, rows)

    def _out_rows(self, solver, rows):
        k = self.output_interval
        return -(-rows[0] // k), min(rows[1] // k, solver.n_out - 1)

    def _dst(self, solver):
        """The host arrays the outputs go to."""
        if self.receivers is None:
            return {"u": self._history("u"), "v": self._history("v"), "a": self._history("a")}
        nr = solver.n_rec
        if self._rec.get("u") is None or self._rec["u"].shape != (solver.n_out, nr):
            self._rec = {name: np.zeros((solver.n_out, nr)) for name in ("u", "v", "a")}
        return self._rec

    def _copy_outputs(self, solver, rows):
        """Output rows of steps rows[0] .. rows[1] from the device into the host arrays."""
        r0, r1 = self._out_rows(solver, rows)
        if r1 < r0:
            return
        dst = self._dst(solver)
        for name, rows_h in solver.output_rows(r0, r1).items():
            if rows_h is not None:
                dst[name][r0:r1 + 1] = rows_h

    def _queue(self, solver, rows):
        """Queue the device -> host copies of the outputs of steps rows[0] .. rows[1] and of the
        run's status into pinned buffers, and an event after them (no synchronisation)."""
        r0, r1 = self._out_rows(solver, rows)
        if getattr(self, "_st_dev", None) is None or self._st_dev.device != solver.u.device:
            self._st_dev = torch.zeros(3, dtype=torch.int64, device=solver.u.device)
            self._st_host = torch.zeros(3, dtype=torch.int64).pin_memory()
            self._stage = {}
        solver.status_to(self._st_dev)
        self._st_host.copy_(self._st_dev, non_blocking=True)
        staged = {}
        if r1 >= r0:
            nr = solver.n_rec
            n = (r1 - r0 + 1) * nr
            for name, t in solver.out.items():
                if t is None:
                    continue
                buf = self._stage.get(name)
                if buf is None or buf.numel() < n:
                    buf = self._stage[name] = torch.empty(n, dtype=torch.float64).pin_memory()
                buf[:n].copy_(t[r0 * nr:(r1 + 1) * nr], non_blocking=True)
                staged[name] = buf[:n]
        ev = torch.cuda.Event()
        ev.record()
        self._pending = (solver, r0, r1, staged, ev)

    def _settle(self, raise_errors=True):
        """Wait for the queued copies of the last continuing call and deliver them."""
        p = getattr(self, "_pending", None)
        if p is None:
            return
        self._pending = None
        solver, r0, r1, staged, ev = p
        ev.synchronize()
        rc, tot, mx = (int(x) for x in self._st_host.tolist())
        if staged:
            dst = self._dst(solver)
            nr = solver.n_rec
            for name, buf in staged.items():
                dst[name][r0:r1 + 1] = buf.numpy().reshape(-1, nr)
        self._iterations = (tot, mx)
        if rc != 0 and raise_errors:
            self.close()
            raise nat.ScatterGpuError("time loop", rc, nat.load().sc_status_string(rc).decode(), "")

    @property
    def device_solver(self):
        """The live device solver (NodeBlockNewmark or NewmarkGPU), or None."""
        return None if self._live is None else self._live[1]

    def close(self):
        self._settle(raise_errors=False)
        if getattr(self, "_live", None) is not None:
            self._live[1].close()
            self._live = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
