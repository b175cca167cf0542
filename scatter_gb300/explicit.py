"""Explicit central-difference scheme with lumped mass on the GPU (no reference counterpart).

The reference's time integrators (PuggleSolvers, scatter/scatter.py:120-131) use the
consistent mass (scatter/discretisation.py:203-222).  This scheme is the added fast path:

    M_L = row sums of M;  C = Cabs + alpha M_L + beta K
    a_n = M_L^-1 (f_n - K (u_n + beta v_{n-1/2}) - alpha M_L v_{n-1/2} - Cabs v_{n-1/2})
    v_{n+1/2} = v_{n-1/2} + dt a_n,   u_{n+1} = u_n + dt v_{n+1/2}

one fused kernel per step (``sc_nb_explicit_run``).  ``ExplicitLumped`` has the solver duck
type of ``NewmarkExplicit``; the velocity reported at step n+1 is v_{n+1/2}.
"""
import numpy as np
import torch

from . import _native as nat
from . import device as dv
from .solvers import ForceTable, NodeBlockNewmark
from .system_matrix import GenerateMatrix, generator_of


def critical_time_step(g: GenerateMatrix):
    """2 / omega_max with omega_max^2 bounded by Gershgorin on M_L^-1 K (a lower bound on the
    true CFL limit of the lumped scheme)."""
    rp = g.pattern.rowptr
    ml = torch.empty(g.n_eq, dtype=torch.float64, device=rp.device)
    ka = torch.empty(g.n_eq, dtype=torch.float64, device=rp.device)
    nat.call("sc_csr_row_sums", g.n_eq, rp.data_ptr(), g.M_d.data_ptr(), 0, ml.data_ptr(), dv.stream_ptr())
    nat.call("sc_csr_row_sums", g.n_eq, rp.data_ptr(), g.K_d.data_ptr(), 1, ka.data_ptr(), dv.stream_ptr())
    bound = float((ka / ml).max().item())
    if float(ml.min().item()) <= 0:
        raise ValueError("lumped mass has non-positive entries (row-sum lumping of this element type)")
    return 2.0 / np.sqrt(bound)


class ExplicitLumped:
    def __init__(self, check_cfl=True, arithmetic="pair"):
        self.arithmetic = arithmetic  # K w products: "pair" (FP32 pairs) or "fp64"
        self.output_interval = 1
        self.update_rhs_at_time_step_func = None
        self.force_table = None
        self.receivers = None
        self.check_cfl = check_cfl

    def initialise(self, number_equations, time):
        self.number_equations = int(number_equations)
        self.time = np.asarray(time, dtype=float)
        n_out = len(range(0, len(self.time), self.output_interval))
        self.output_time = self.time[::self.output_interval][:n_out]
        self.u = np.zeros((n_out, self.number_equations))
        self.v = np.zeros(self.u.shape)  # zero pages: a receivers-only run never writes them
        self.a = np.zeros(self.u.shape)

    def update(self, t_idx):
        self.t_idx = t_idx

    def calculate(self, M, C, K, F, t_start_idx, t_end_idx):
        g = M if isinstance(M, GenerateMatrix) else generator_of(M, C, K)
        if g is None:
            raise TypeError("the explicit GPU scheme takes the GenerateMatrix that assembled M, C, K, or the "
                            "scipy matrices it handed out")
        if np.any(self.u[0]) or np.any(self.v[0]):
            # the central-difference state is (u_n, v_{n-1/2}): it starts from rest only
            raise NotImplementedError("the explicit GPU scheme starts from rest (u[0] = v[0] = 0)")
        dt = self.time[1] - self.time[0]
        if self.check_cfl:
            dtc = critical_time_step(g)
            if dt > dtc:
                raise ValueError(f"explicit scheme unstable: dt {dt:.3e} > critical {dtc:.3e}")
        n_t = len(self.time)
        table = self.force_table
        if table is None:
            func = self.update_rhs_at_time_step_func or (lambda t: F)
            table = ForceTable.from_callback(func, n_t, g.n_eq)
        s = NodeBlockNewmark(g, dt, explicit=self.arithmetic)
        s.set_force(table)
        rec = np.arange(g.n_eq) if self.receivers is None else np.asarray(self.receivers)
        n_out = len(range(0, n_t, self.output_interval))
        s.set_output(self.output_interval, rec, n_out, what=("u", "v"))
        for k in ("u", "v"):
            s.out[k][:s.n_rec] = {"u": s.u, "v": s.v}[k][s.rec.long()]
        s.run_explicit(t_start_idx, t_end_idx)
        torch.cuda.synchronize()
        out = s.outputs()
        if self.receivers is None:
            self.u, self.v = out["u"], out["v"]
        else:
            self.u_rec, self.v_rec = out["u"], out["v"]
        self.solver_handle = s
        s.close()
