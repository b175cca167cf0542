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


def incidence_by_local_index(elem_idx, n_nodes):
    """Node -> element incidence (CSR), each node's elements ordered by the node's local index
    in the element, then by element."""
    E, n_en = elem_idx.shape
    node = elem_idx.ravel()
    la = np.tile(np.arange(n_en), E)
    el = np.repeat(np.arange(E), n_en)
    o = np.lexsort((el, la, node))
    ptr = np.zeros(n_nodes + 1, dtype=np.int64)
    ptr[1:] = np.cumsum(np.bincount(node, minlength=n_nodes))
    if ptr[-1] >= 2**31:
        raise ValueError("incidence list too long for int32 offsets")
    return ptr.astype(np.int32), el[o].astype(np.int32)


# natural coordinates (0 / 1 for -1 / +1) of the hexa8 nodes in the reference's order
# (scatter/element_types.py:52-104)
HEX8_NAT = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])


HEX8_TILE = (4, 4, 2)  # lattice points per tile along xi, eta, zeta (the kernel's kTX, kTY, kTZ)


def hex8_lattice(xyz, elem_idx):
    """Integer lattice coordinates [n_nodes, 3] (from 0) of a uniform hexa8 grid along the
    natural axes of its first element, or None when the mesh is not one (the conditions are
    those of hex8_grid_tables)."""
    n_nodes = len(xyz)
    e0 = elem_idx[0]
    A = np.stack([xyz[e0[1]] - xyz[e0[0]], xyz[e0[3]] - xyz[e0[0]], xyz[e0[4]] - xyz[e0[0]]], axis=1)
    if abs(np.linalg.det(A)) <= 1e-12 * np.abs(A).max() ** 3:
        return None
    L = np.linalg.solve(A, (xyz - xyz[e0[0]]).T).T
    Li = np.rint(L)
    if np.abs(L - Li).max() > 1e-6:
        return None
    Li = Li.astype(np.int64)
    Li -= Li.min(axis=0)
    if np.any(Li[elem_idx] != Li[elem_idx[:, :1]] + HEX8_NAT[None]):
        return None
    ext = Li.max(axis=0) + 1
    key = Li[:, 0] + ext[0] * (Li[:, 1] + ext[1] * Li[:, 2])
    if len(np.unique(key)) != n_nodes:
        return None
    return Li


HEX8_COLUMN = (4, 4)  # lattice points per column across the first two axes (the kernel's kCX, kCY)


def hex8_column_tables(xyz, elem_idx, cross=HEX8_COLUMN):
    """(nodes [n_col, nzp, 36], elems [n_col, nzp - 1, 25], nzp) for the tensor-core step on a
    uniform hexa8 grid, None for other meshes.  Columns of cross[0] x cross[1] lattice points
    across the first two lattice axes, numbered first axis fastest; per column and plane z
    (third axis) the nodes of the column's ring -- its points grown by one on each side,
    point (hx, hy) at hx + (cross[0] + 2) hy -- and the elements whose local node 0 is at ring
    point (ex, ey) < (cross[0] + 1, cross[1] + 1), at ex + (cross[0] + 1) ey; -1 where none."""
    Li = hex8_lattice(xyz, elem_idx)
    if Li is None:
        return None
    ext = Li.max(axis=0) + 1
    cx, cy = cross
    nc = -(-ext[:2] // np.array(cross))
    box = np.array([nc[0] * cx + 2, nc[1] * cy + 2, ext[2]])  # one point of margin across
    def key(x, y, z):
        return (x + 1) + box[0] * ((y + 1) + box[1] * z)
    dense_n = np.full(int(np.prod(box)), -1, dtype=np.int64)
    dense_n[key(Li[:, 0], Li[:, 1], Li[:, 2])] = np.arange(len(Li))
    dense_e = np.full(int(np.prod(box)), -1, dtype=np.int64)
    L0 = Li[elem_idx[:, 0]]
    dense_e[key(L0[:, 0], L0[:, 1], L0[:, 2])] = np.arange(len(elem_idx))
    C = np.arange(int(np.prod(nc)))
    x0, y0 = (C % nc[0]) * cx, (C // nc[0]) * cy
    nzp = int(ext[2])
    hx, hy = np.meshgrid(np.arange(cx + 2), np.arange(cy + 2), indexing="xy")
    hx, hy = hx.ravel(), hy.ravel()  # point hx + (cx + 2) hy
    z = np.arange(nzp)
    px = x0[:, None, None] - 1 + hx[None, None, :]
    py = y0[:, None, None] - 1 + hy[None, None, :]
    nodes = dense_n[key(px, py, z[None, :, None])]
    ex, ey = np.meshgrid(np.arange(cx + 1), np.arange(cy + 1), indexing="xy")
    ex, ey = ex.ravel(), ey.ravel()
    qx = x0[:, None, None] - 1 + ex[None, None, :]
    qy = y0[:, None, None] - 1 + ey[None, None, :]
    elems = dense_e[key(qx, qy, z[None, :-1, None])]
    return nodes.astype(np.int32), elems.astype(np.int32), nzp


def hex8_grid_tables(xyz, elem_idx, tile=HEX8_TILE):
    """(halo [n_tiles, (tx+2)(ty+2)(tz+2)], elem8 [n_nodes, 8]) of a uniform hexa8 grid, None
    for other meshes.  The nodes must sit on an integer lattice along the natural axes of the
    first element (every element the same shape and orientation), each element's local node l
    at its first node's lattice point plus the natural offset of l, at most one node per
    lattice point.  halo lists per tile the nodes of the tile grown by one point on every side
    (-1 where there is none), point (hx, hy, hz) at hx + (tx+2) (hy + (ty+2) hz); tiles are
    numbered x fastest.  elem8 [a, la] is the element in which node a is local node la."""
    n_nodes, E = len(xyz), len(elem_idx)
    Li = hex8_lattice(xyz, elem_idx)
    if Li is None:
        return None
    tile = np.asarray(tile)
    ext = Li.max(axis=0) + 1
    nt = -(-ext // tile)
    box = nt * tile + 2  # padded lattice: one point of margin on every side
    key = (Li[:, 0] + 1) + box[0] * ((Li[:, 1] + 1) + box[1] * (Li[:, 2] + 1))
    dense = np.full(int(np.prod(box)), -1, dtype=np.int64)
    dense[key] = np.arange(n_nodes)
    elem8 = np.full((n_nodes, 8), -1, dtype=np.int64)
    for la in range(8):
        elem8[elem_idx[:, la], la] = np.arange(E)
    hb = tile + 2
    T = np.arange(int(np.prod(nt)))
    tx, ty, tz = T % nt[0], (T // nt[0]) % nt[1], T // (nt[0] * nt[1])
    H = np.arange(int(np.prod(hb)))
    hx, hy, hz = H % hb[0], (H // hb[0]) % hb[1], H // (hb[0] * hb[1])
    px = tx[:, None] * tile[0] + hx[None]
    py = ty[:, None] * tile[1] + hy[None]
    pz = tz[:, None] * tile[2] + hz[None]
    halo = dense[px + box[0] * (py + box[1] * pz)]
    return halo.astype(np.int32), elem8.astype(np.int32)


class BatchedExplicit:
    def __init__(self, model, young, nu, rho, damping, absorbing, k_div, dt, order=2, tensor_cores=True):
        """young: per-element, per-realisation E [n_elem, R] (numpy or CUDA float32).
        tensor_cores: offer the tensor-core step kernel to the tuner (uniform hexa8 grids, R a
        multiple of 128)."""
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
        # node -> element incidence, each node's list sorted by the node's local index in the
        # element (then element): the summation order of both step kernels
        self.elem = dv.to_dev(elem_idx, torch.int32)
        ptr, inc = incidence_by_local_index(elem_idx, N)
        self.inc_ptr = dv.to_dev(ptr, torch.int32)
        self.inc = dv.to_dev(inc, torch.int32)
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
        # uniform hexa8 grids: the neighbour-register kernel joins the tuner's candidates
        self.grid_tables = None
        if etype == "hexa8" and self.n_types == 1:
            self.grid_tables = hex8_grid_tables(nodes[:, 1:].astype(float), elem_idx)
        if self.grid_tables is not None:
            self._halo = dv.to_dev(self.grid_tables[0], torch.int32)
            self._elem8 = dv.to_dev(self.grid_tables[1], torch.int32)
            nat.call("sc_batch_set_hex8_grid", self.h, len(self.grid_tables[0]), self._halo.data_ptr(),
                     self._elem8.data_ptr())
        # ... and, for whole groups of 128 realisations, the tensor-core kernel
        self.column_tables = None
        if self.grid_tables is not None and R % 128 == 0 and tensor_cores:
            self.column_tables = hex8_column_tables(nodes[:, 1:].astype(float), elem_idx)
        if self.column_tables is not None:
            cn, ce, nzp = self.column_tables
            self._col_nodes = dv.to_dev(cn, torch.int32)
            self._col_elems = dv.to_dev(ce, torch.int32)
            nat.call("sc_batch_set_hex8_columns", self.h, len(cn), nzp, self._col_nodes.data_ptr(),
                     self._col_elems.data_ptr())

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

    KERNELS = {0: "incidence lists (k_batch_step)", 1: "uniform hexa8 grid, tiled (k_batch_step_hex8g)",
               2: "tensor cores (k_batch_step_tc)", 3: "uniform hexa8 grid, node-centric (k_batch_step_hex8c)",
               4: "uniform hexa8 grid, node-centric, wide register budget (k_batch_step_hex8c_wide)"}

    def config(self):
        """(realisations per thread, threads per block, tuned ms per step, kernel) of the step
        kernel; kernel 0 incidence lists, 1 the tiled uniform hexa8 grid kernel, 2 the
        tensor-core kernel (whose first value is then its column segment length), 3 the
        node-centric uniform hexa8 kernel."""
        rpt, tpb, ms, grid = ctypes.c_int(), ctypes.c_int(), ctypes.c_float(), ctypes.c_int()
        nat.call("sc_batch_config", self.h, ctypes.byref(rpt), ctypes.byref(tpb), ctypes.byref(ms), ctypes.byref(grid))
        return rpt.value, tpb.value, ms.value, grid.value

    def set_shape(self, realisations_per_thread, threads_per_block, grid=False):
        """Override the tuned kernel and shape (testing aid): grid False the incidence-list
        kernel, True the tiled uniform hexa8 kernel, "node" the node-centric one, "node-wide" the
        node-centric one at the wide register budget."""
        if grid == "node-wide":
            nat.call("sc_batch_set_node_shape_budget", self.h, int(realisations_per_thread), int(threads_per_block), 1)
            return
        fn = {False: "sc_batch_set_shape", True: "sc_batch_set_grid_shape", "node": "sc_batch_set_node_shape"}[grid]
        nat.call(fn, self.h, int(realisations_per_thread), int(threads_per_block))

    def set_tensor_core_shape(self, segment):
        """Select the tensor-core kernel with column segments of `segment` points (testing aid)."""
        nat.call("sc_batch_set_tc_shape", self.h, int(segment))

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

    def status(self):
        """Synchronise; raises if a tensor-core step gave up waiting for its tensor-core work."""
        nat.call("sc_batch_status", self.h)

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
