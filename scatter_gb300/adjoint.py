"""Gradient of a receiver-velocity misfit w.r.t. per-element E and rho (explicit scheme).

No reference counterpart: the reference has no differentiation.  ``ExplicitAdjoint``
evaluates J = 1/2 sum_n |P v_n - d_n|^2 for the explicit lumped-mass scheme and its
gradient with the hand-written discrete adjoint of ``sc_nb_adjoint`` (checkpoint every
``checkpoint`` steps, recompute, backward).  ``ReceiverMisfit`` wraps it as a
torch.autograd.Function of (E, rho).
"""
import ctypes

import numpy as np
import torch

from . import _native as nat
from . import device as dv
from .batched import element_types
from .lysmer import boundary_faces
from .solvers import NodeBlockNewmark
from .system_matrix import ELEM_NODES, FACE_NODES, FACE_TYPES, GenerateMatrix, model_arrays


class _AdjDesc(ctypes.Structure):
    _fields_ = [("n_steps", ctypes.c_int), ("checkpoint", ctypes.c_int), ("n_rec", ctypes.c_int),
                ("rec_slot", ctypes.c_void_p), ("target", ctypes.c_void_p), ("n_elem", ctypes.c_int),
                ("n_en", ctypes.c_int), ("elem", ctypes.c_void_p), ("ke_type", ctypes.c_void_p),
                ("ke1", ctypes.c_void_p), ("young", ctypes.c_void_p), ("rho", ctypes.c_void_p),
                ("ml1", ctypes.c_void_p), ("l_eptr", ctypes.c_void_p), ("l_row", ctypes.c_void_p),
                ("l_col", ctypes.c_void_p), ("l_c", ctypes.c_void_p), ("l_s", ctypes.c_void_p)]


class ExplicitAdjoint:
    def __init__(self, model, nu, damping, absorbing, k_div, dt, n_steps, rec_eq, table, checkpoint=200, order=2):
        if int(model.dimension) != 3:
            raise NotImplementedError("the adjoint is 3D")
        self.model, self.damping, self.absorbing, self.k_div = model, damping, absorbing, k_div
        self.dt, self.n_steps, self.table, self.checkpoint, self.order = dt, int(n_steps), table, int(checkpoint), order
        self.rec_eq = np.asarray(rec_eq, dtype=np.int64)
        etype = str(model.element_type)
        self.n_en = ELEM_NODES[etype]
        nodes, _, elem_idx, eqmap = model_arrays(model)
        self.elem_idx, self.eqmap = elem_idx, eqmap
        n_elem = len(elem_idx)
        self.nu = np.broadcast_to(np.asarray(nu, dtype=float), (n_elem,)).copy()
        # unit element stiffness and mass per element shape
        first, ktype = element_types(model, self.nu)
        nd = 3 * self.n_en
        coords = dv.to_dev(nodes[:, 1:][elem_idx[first]], torch.float64)
        one = dv.to_dev(np.ones(len(first)), torch.float64)
        nu_t = dv.to_dev(self.nu[first], torch.float64)
        ke = dv.empty(len(first) * nd * nd, torch.float64)
        me = dv.empty(len(first) * nd * nd, torch.float64)
        nat.call("sc_element_matrices", nat.ELEMENT_CODES[etype], order, len(first), coords.data_ptr(), one.data_ptr(),
                 nu_t.data_ptr(), one.data_ptr(), ke.data_ptr(), me.data_ptr(), dv.stream_ptr())
        torch.cuda.current_stream().synchronize()
        self.ke1 = ke.to(torch.float32)
        self.ke_type = dv.to_dev(ktype, torch.int32)
        Me1 = dv.host(me).reshape(len(first), self.n_en, 3, self.n_en, 3)
        Mc = np.einsum("tacbc->tabc", Me1)  # [types, a, b, c]: component-c mass coupling
        free = (eqmap[elem_idx] >= 0).astype(float)  # [E, n_en, 3]
        self.ml1 = dv.to_dev(np.einsum("eabc,ebc->eac", Mc[ktype], free), torch.float32)
        self.elem = dv.to_dev(elem_idx, torch.int32)

    def _lysmer_entries(self, E, rho, eq2slot):
        faces = boundary_faces(self.model, (E, self.nu, rho), self.absorbing)
        n_face = len(faces["eqs"])
        nf = FACE_NODES[FACE_TYPES[str(self.model.element_type)]]
        n_elem = len(E)
        if n_face == 0:
            z = np.zeros(1)
            return np.zeros(n_elem + 1, np.int64), z.astype(np.int32), z.astype(np.int32), z, z
        xy = dv.to_dev(faces["xy"], torch.float64)
        Fm = dv.empty(n_face * nf * nf, torch.float64)
        nat.call("sc_face_matrices", nat.ELEMENT_CODES[FACE_TYPES[str(self.model.element_type)]], self.order, n_face,
                 xy.data_ptr(), Fm.data_ptr(), dv.stream_ptr())
        F = dv.host(Fm).reshape(n_face, nf, nf)
        eqs = faces["eqs"]
        rows = eq2slot[np.repeat(eqs, nf, axis=1).ravel()]
        cols = eq2slot[np.tile(eqs, (1, nf)).ravel()]
        lc = (F * faces["fct"][:, None, :]).ravel()
        ls = (np.abs(F) * faces["fct2"][:, None, :]).ravel() / self.k_div
        el = np.repeat(faces["elem"], nf * nf)
        o = np.argsort(el, kind="stable")
        eptr = np.zeros(n_elem + 1, np.int64)
        eptr[1:] = np.cumsum(np.bincount(el, minlength=n_elem))
        return eptr, rows[o].astype(np.int32), cols[o].astype(np.int32), lc[o], ls[o]

    def prepare(self, E, rho):
        """Operators, device handle and descriptor at (E, rho); reusable for several targets."""
        return _Prepared(self, np.asarray(E, dtype=float), np.asarray(rho, dtype=float))

    def evaluate(self, E, rho, target):
        """J, dJ/dE, dJ/drho (numpy) for per-element E, rho and target [n_steps+1, n_rec]."""
        p = self.prepare(E, rho)
        try:
            return p.gradient(target)
        finally:
            p.close()


class _Prepared:
    def __init__(self, adj, E, rho):
        self.adj = adj
        g = GenerateMatrix(adj.model.number_eq, adj.order)
        g.generate_stiffness_and_mass(adj.model, None, element_props=(E, adj.nu, rho))
        g.absorbing_boundaries(adj.model, None, adj.absorbing, adj.k_div)
        g.damping_Rayleigh(adj.damping)
        s = NodeBlockNewmark(g, adj.dt, precond="jacobi")
        s.set_force(adj.table)
        self.solver = s
        e2s = dv.host(s.eq2slot)
        eptr, lr, lcol, lc, ls = adj._lysmer_entries(E, rho, e2s)
        self.rec = dv.to_dev(e2s[adj.rec_eq].astype(np.int32), torch.int32)
        self._keep = [dv.to_dev(x, t) for x, t in ((E, torch.float64), (rho, torch.float64), (eptr, torch.int64),
                                                    (lr, torch.int32), (lcol, torch.int32), (lc, torch.float32),
                                                    (ls, torch.float32))]
        self.n_elem = len(E)

    def forward(self):
        """Receiver velocities [n_steps+1, n_rec] of the explicit scheme from rest (host)."""
        a = self.adj
        s = self.solver
        s.u.zero_()
        s.v.zero_()
        s.set_output(1, a.rec_eq, a.n_steps + 1, what=("v",))
        s.run_explicit(0, a.n_steps)
        return dv.host(s.out["v"]).reshape(a.n_steps + 1, len(a.rec_eq))

    def gradient(self, target):
        a = self.adj
        tgt = dv.to_dev(np.asarray(target, dtype=float), torch.float64)
        if tgt.numel() != (a.n_steps + 1) * len(a.rec_eq):
            raise ValueError("target must be [n_steps + 1, n_receivers]")
        E_d, rho_d, ep_d, lr_d, lc_d, lcv_d, lsv_d = self._keep
        d = _AdjDesc(a.n_steps, a.checkpoint, len(a.rec_eq), self.rec.data_ptr(), tgt.data_ptr(), self.n_elem,
                     a.n_en, a.elem.data_ptr(), a.ke_type.data_ptr(), a.ke1.data_ptr(), E_d.data_ptr(),
                     rho_d.data_ptr(), a.ml1.data_ptr(), ep_d.data_ptr(), lr_d.data_ptr(), lc_d.data_ptr(),
                     lcv_d.data_ptr(), lsv_d.data_ptr())
        gE = dv.zeros(self.n_elem, torch.float64)
        gR = dv.zeros(self.n_elem, torch.float64)
        J = ctypes.c_double()
        nat.call("sc_nb_adjoint", self.solver.h, ctypes.byref(d), ctypes.byref(J), gE.data_ptr(), gR.data_ptr())
        return J.value, dv.host(gE), dv.host(gR)

    def timings(self):
        """Device ms of the last gradient's phases: forward with checkpoints, recompute of the
        last segment, the rest of the reverse sweep (backward steps fused with the previous
        segment's recompute, element gradients), and the whole reverse sweep."""
        ms = (ctypes.c_float * 4)()
        nat.call("sc_nb_adjoint_timings", self.solver.h, ms)
        return tuple(float(x) for x in ms)

    def close(self):
        self.solver.close()


class ReceiverMisfit(torch.autograd.Function):
    """J(E, rho) with the adjoint gradient as its backward."""

    @staticmethod
    def forward(ctx, E, rho, adj, target):
        J, gE, gR = adj.evaluate(E.detach().cpu().numpy(), rho.detach().cpu().numpy(), target)
        ctx.save_for_backward(torch.as_tensor(gE, dtype=E.dtype, device=E.device),
                              torch.as_tensor(gR, dtype=rho.dtype, device=rho.device))
        return torch.tensor(J, dtype=E.dtype, device=E.device)

    @staticmethod
    def backward(ctx, grad_out):
        gE, gR = ctx.saved_tensors
        return grad_out * gE, grad_out * gR, None, None
