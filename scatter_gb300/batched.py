"""Batched realisations on the GPU: R per-element Young's modulus fields advanced together.

Each realisation is the explicit lumped-mass scheme of ``scatter_gb300.explicit`` applied to
the model with that realisation's per-element E (the reference's random-field materials,
scatter/random_fields.py:109-118), density and Poisson ratio shared.  One kernel per step
advances all realisations (``sc_batch_*``); see include/scatter_gb300.h.
"""
import ctypes

import numpy as np
import torch

from . import _native as nat
from . import device as dv
from .lysmer import boundary_faces
from .solvers import ForceTable
from .system_matrix import ELEM_NODES, FACE_NODES, FACE_TYPES, GenerateMatrix, model_arrays


class _Desc(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_int), ("n_elem", ctypes.c_int), ("n_en", ctypes.c_int), ("R", ctypes.c_int),
                ("n_types", ctypes.c_int), ("elem", ctypes.c_void_p), ("inc_ptr", ctypes.c_void_p),
                ("inc", ctypes.c_void_p), ("ke_type", ctypes.c_void_p), ("ke1", ctypes.c_void_p),
                ("young", ctypes.c_void_p), ("ml", ctypes.c_void_p), ("fixed", ctypes.c_void_p),
                ("alpha", ctypes.c_double), ("beta", ctypes.c_double), ("dt", ctypes.c_double),
                ("l_ptr", ctypes.c_void_p), ("l_col", ctypes.c_void_p), ("l_elem", ctypes.c_void_p),
                ("l_c", ctypes.c_void_p), ("l_s", ctypes.c_void_p), ("node_nen", ctypes.c_void_p)]


def element_types(model, nu, tol=1e-9):
    """Group elements with identical shape (node offsets) and Poisson ratio: one unit-E
    stiffness per group."""
    nodes, _, elem_idx, _ = model_arrays(model)
    X = nodes[:, 1:][elem_idx]
    off = X - X[:, :1, :]
    scale = max(np.abs(off).max(), 1e-300)
    sig = np.c_[np.round(off.reshape(len(X), -1) / (scale * tol)), np.round(np.asarray(nu) / tol)]
    _, first, inv = np.unique(sig, axis=0, return_index=True, return_inverse=True)
    return first, inv.ravel().astype(np.int32)


class BatchedExplicit:
    def __init__(self, model, young, nu, rho, damping, absorbing, k_div, dt, order=2):
        """young: per-element, per-realisation E [n_elem, R] (numpy or CUDA float32)."""
        dv.require_cuda()
        etype = str(model.element_type)
        if int(model.dimension) != 3:
            raise NotImplementedError("batched realisations are 3D")
        n_en = ELEM_NODES[etype]
        nodes, _, elem_idx, eqmap = model_arrays(model)
        n_elem, N = len(elem_idx), len(nodes)
        nu = np.broadcast_to(np.asarray(nu, dtype=float), (n_elem,)).copy()
        rho = np.broadcast_to(np.asarray(rho, dtype=float), (n_elem,)).copy()
        ones = np.ones(n_elem)
        # mass (independent of E) and pattern from a unit-E assembly
        g = GenerateMatrix(model.number_eq, order)
        g.generate_stiffness_and_mass(model, None, element_props=(ones, nu, rho))
        self.g = g
        alpha, beta = GenerateMatrix.rayleigh_coefficients(damping)
        s = dv.stream_ptr()
        # lumped mass in slot space
        rp = g.pattern.rowptr
        ml_eq = torch.empty(g.n_eq, dtype=torch.float64, device=rp.device)
        nat.call("sc_csr_row_sums", g.n_eq, rp.data_ptr(), g.M_d.data_ptr(), 0, ml_eq.data_ptr(), s)
        em = torch.as_tensor(eqmap.reshape(-1), device=rp.device).long()
        free = em >= 0
        self.ml = torch.ones(3 * N, dtype=torch.float64, device=rp.device)
        self.ml[free] = ml_eq[em[free]]
        self.fixed = (~free).to(torch.int32)
        self.eq2slot = torch.full((g.n_eq,), -1, dtype=torch.int64, device=rp.device)
        self.eq2slot[em[free]] = torch.arange(3 * N, device=rp.device)[free]
        # unit-E element stiffness per element type
        first, ktype = element_types(model, nu)
        coords = dv.to_dev(nodes[:, 1:][elem_idx[first]], torch.float64)
        nd = 3 * n_en
        ke = dv.empty(len(first) * nd * nd, torch.float64)
        # keep every argument tensor alive until the asynchronous launch has consumed it
        e_one = dv.to_dev(np.ones(len(first)), torch.float64)
        nu_t = dv.to_dev(nu[first], torch.float64)
        nat.call("sc_element_matrices", nat.ELEMENT_CODES[etype], order, len(first), coords.data_ptr(),
                 e_one.data_ptr(), nu_t.data_ptr(), None, ke.data_ptr(), None, s)
        torch.cuda.current_stream().synchronize()
        del e_one, nu_t
        self.ke1 = ke.to(torch.float32)
        self.ke_type = dv.to_dev(ktype, torch.int32)
        self.n_types = len(first)
        # node -> element incidence
        self.elem = dv.to_dev(elem_idx, torch.int32)
        self.inc_ptr = dv.empty(N + 1, torch.int32)
        self.inc = dv.empty(n_elem * n_en, torch.int32)
        work = dv.empty(N, torch.int32)
        nat.call("sc_node_incidence", n_elem, n_en, N, self.elem.data_ptr(), self.inc_ptr.data_ptr(),
                 self.inc.data_ptr(), work.data_ptr(), s)
        # Lysmer entries scaled per realisation (unit E here)
        self._lysmer(model, (ones, nu, rho), absorbing, k_div, order, N)
        self.young = (young if torch.is_tensor(young) else dv.to_dev(np.asarray(young, dtype=np.float32),
                                                                         torch.float32)).contiguous()
        R = int(self.young.shape[1])
        self.R, self.N, self.n_en = R, N, n_en
        self.u = dv.zeros(3 * N * R, torch.float64)
        self.v = dv.zeros(3 * N * R, torch.float64)
        d = _Desc(N, n_elem, n_en, R, self.n_types, self.elem.data_ptr(), self.inc_ptr.data_ptr(), self.inc.data_ptr(),
                  self.ke_type.data_ptr(), self.ke1.data_ptr(), self.young.data_ptr(), self.ml.data_ptr(),
                  self.fixed.data_ptr(), float(alpha), float(beta), float(dt), self.l_ptr.data_ptr(),
                  self.l_col.data_ptr(), self.l_elem.data_ptr(), self.l_c.data_ptr(), self.l_s.data_ptr(), None)
        self._desc = d
        h = ctypes.c_void_p()
        nat.call("sc_batch_create", ctypes.byref(h), ctypes.byref(d), self.u.data_ptr(), self.v.data_ptr(), s)
        self.h = h
        self.dt = dt

    def _lysmer(self, model, props, absorbing, k_div, order, N):
        etype = str(model.element_type)
        faces = boundary_faces(model, props, absorbing)
        nf = FACE_NODES[FACE_TYPES[etype]]
        n_face = len(faces["eqs"])
        dev = self.ml.device
        if n_face == 0:
            self.l_ptr = torch.zeros(3 * N + 1, dtype=torch.int64, device=dev)
            self.l_col = torch.zeros(1, dtype=torch.int32, device=dev)
            self.l_elem = torch.zeros(1, dtype=torch.int32, device=dev)
            self.l_c = torch.zeros(1, dtype=torch.float32, device=dev)
            self.l_s = torch.zeros(1, dtype=torch.float32, device=dev)
            return
        xy = dv.to_dev(faces["xy"], torch.float64)
        Fm = dv.empty(n_face * nf * nf, torch.float64)
        nat.call("sc_face_matrices", nat.ELEMENT_CODES[FACE_TYPES[etype]], order, n_face, xy.data_ptr(), Fm.data_ptr(),
                 dv.stream_ptr())
        F = dv.host(Fm).reshape(n_face, nf, nf)
        eqs = faces["eqs"]
        rows = np.repeat(eqs, nf, axis=1).ravel()
        cols = np.tile(eqs, (1, nf)).ravel()
        c = (F * faces["fct"][:, None, :]).ravel()
        sv = (np.abs(F) * faces["fct2"][:, None, :]).ravel() / k_div
        el = np.repeat(faces["elem"], nf * nf)
        e2s = dv.host(self.eq2slot)
        rs, cs = e2s[rows], e2s[cols]
        o = np.argsort(rs, kind="stable")
        rs, cs, c, sv, el = rs[o], cs[o], c[o], sv[o], el[o]
        ptr = np.zeros(3 * N + 1, dtype=np.int64)
        ptr[1:] = np.cumsum(np.bincount(rs, minlength=3 * N))
        self.l_ptr = dv.to_dev(ptr, torch.int64)
        self.l_col = dv.to_dev(cs.astype(np.int32), torch.int32)
        self.l_elem = dv.to_dev(el.astype(np.int32), torch.int32)
        self.l_c = dv.to_dev(c.astype(np.float32), torch.float32)
        self.l_s = dv.to_dev(sv.astype(np.float32), torch.float32)

    def config(self):
        """(realisations per thread, threads per block, tuned ms per step) of the step kernel."""
        rpt, tpb, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        nat.call("sc_batch_config", self.h, ctypes.byref(rpt), ctypes.byref(tpb), ctypes.byref(ms))
        return rpt.value, tpb.value, ms.value

    def set_shape(self, realisations_per_thread, threads_per_block):
        """Override the tuned kernel shape (testing aid)."""
        nat.call("sc_batch_set_shape", self.h, int(realisations_per_thread), int(threads_per_block))

    def set_force(self, table: ForceTable):
        eq = dv.to_dev(table.f_eq, torch.int64)
        slot = self.eq2slot[eq].to(torch.int32) if eq.numel() else torch.zeros(1, dtype=torch.int32,
                                                                                device=self.ml.device)
        val = dv.to_dev(table.f_val, torch.float64) if eq.numel() else torch.zeros(1, dtype=torch.float64,
                                                                                    device=self.ml.device)
        self._force = [dv.to_dev(table.f_ptr, torch.int64), slot.contiguous(), val]
        p, e, v = self._force
        nat.call("sc_batch_set_force", self.h, table.n_t, p.data_ptr(), e.data_ptr(), v.data_ptr())

    def set_output(self, interval, rec_eq, n_out):
        rec = self.eq2slot[dv.to_dev(np.asarray(rec_eq, dtype=np.int64), torch.int64)].to(torch.int32).contiguous()
        self.rec = rec
        self.n_rec, self.n_out = rec.numel(), int(n_out)
        self.out_v = dv.zeros(self.n_out * self.n_rec * self.R, torch.float64)
        nat.call("sc_batch_set_output", self.h, int(interval), self.n_rec, rec.data_ptr(), self.out_v.data_ptr(),
                 self.n_out)

    def run(self, t_begin, t_end):
        nat.call("sc_batch_run", self.h, int(t_begin), int(t_end))

    def velocities(self):
        """[n_out, n_rec, R] receiver velocities (host)."""
        return dv.host(self.out_v).reshape(self.n_out, self.n_rec, self.R)

    def state(self):
        """u, v [R, n_eq] in the reference's equation numbering (host)."""
        e2s = self.eq2slot
        u = self.u.view(3 * self.N, self.R)[e2s].T
        v = self.v.view(3 * self.N, self.R)[e2s].T
        return dv.host(u), dv.host(v)

    def close(self):
        if getattr(self, "h", None):
            nat.value("sc_batch_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
