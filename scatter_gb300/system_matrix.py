"""GPU global matrices: drop-in for scatter/system_matrix.py ``GenerateMatrix``.

Same constructor and methods as the reference (scatter/system_matrix.py:16-198,256-376):

    m = GenerateMatrix(n_eq, int_order)
    m.generate_stiffness_and_mass(model, materials)
    m.absorbing_boundaries(model, materials, [a_p, a_s], k_div)
    m.damping_Rayleigh([f1, xi1, f2, xi2])
    m.K, m.M, m.C            # scipy CSR (downloaded on first access)

The matrices live on the GPU in CSR over the reference's equation numbering, all three on
the element-graph pattern (the reference's M pattern).  The scipy matrices handed out
follow the reference's sparsity semantics: ``.M`` keeps the element graph with its stored
zeros (system_matrix.py:98-121), while ``.K`` and ``.C`` drop the entries whose assembled
value is exactly 0.0, as the reference's scipy additions do (system_matrix.py:198,375-376).

The scipy matrices are read-only views of what is on the device and remember the
generator that made them, so a time integrator given ``(m.M, m.C, m.K)`` -- the
reference's own call form, scatter/scatter.py:159 -- can run on the device arrays
directly (``generator_of``).
"""
import weakref

import numpy as np
import scipy.sparse as sp
import torch

from . import _native as nat
from . import device as dv

FACE_TYPES = {"hexa8": "quad4", "hexa20": "quad8", "tetra4": "tri3", "tetra10": "tri6"}
FACE_NODES = {"quad4": 4, "quad8": 8, "tri3": 3, "tri6": 6}
ELEM_NODES = {"hexa8": 8, "hexa20": 20, "tetra4": 4, "tetra10": 10, "quad4": 4, "quad8": 8, "tri3": 3, "tri6": 6}


def model_arrays(model):
    """Pull the mesh arrays the path needs from a ReadMesh-like object (ours or the reference's)."""
    nodes = np.asarray(model.nodes, dtype=float)
    ids = nodes[:, 0].astype(np.int64)
    id2idx = np.full(int(ids.max()) + 1, -1, dtype=np.int64)
    id2idx[ids] = np.arange(len(ids))
    elem_ids = np.asarray(model.elem, dtype=np.int64)
    elem_idx = id2idx[elem_ids]
    if (elem_idx < 0).any():
        raise ValueError("element references an unknown node id")
    eq = np.asarray(model.eq_nb_dof, dtype=float)
    eqmap = np.where(np.isnan(eq), -1, np.nan_to_num(eq, nan=-1)).astype(np.int32)
    return nodes, id2idx, elem_idx.astype(np.int32), eqmap


def element_properties(model, materials):
    """Per-element E, nu, rho through the physical-group names (system_matrix.py:51-71)."""
    names = {}
    for row in model.materials:
        names[int(row[1])] = str(row[2])
    mi = np.asarray(model.materials_index, dtype=np.int64)
    uniq, inv = np.unique(mi, return_inverse=True)
    table = np.array([[materials[names[int(u)]][k] for k in ("Young", "poisson", "density")] for u in uniq],
                     dtype=float).reshape(-1, 3)
    vals = table[inv.ravel()]
    return vals[:, 0].copy(), vals[:, 1].copy(), vals[:, 2].copy()


class DeviceCSR:
    """Shared-pattern CSR on the GPU: rowptr int64 [n+1], cols int32 [nnz]."""

    def __init__(self, n, rowptr, cols):
        self.n = int(n)
        self.rowptr = rowptr
        self.cols = cols
        self.nnz = int(cols.numel())

    def to_scipy(self, values):
        return sp.csr_matrix((dv.host(values), dv.host(self.cols), dv.host(self.rowptr)), shape=(self.n, self.n))


def _csr_from_elements(n_nodes, n_en, dim, elem_idx_d, eqmap_d, n_eq):
    """Steps 1-3 of the assembly: incidence, adjacency, CSR pattern (all on the GPU)."""
    s = dv.stream_ptr()
    n_elem = elem_idx_d.numel() // n_en
    inc_ptr = dv.empty(n_nodes + 1, torch.int32)
    inc = dv.empty(max(n_elem * n_en, 1), torch.int32)
    work = dv.empty(max(n_nodes, 1), torch.int32)
    nat.call("sc_node_incidence", n_elem, n_en, n_nodes, elem_idx_d.data_ptr(), inc_ptr.data_ptr(), inc.data_ptr(),
             work.data_ptr(), s)
    deg = dv.empty(n_nodes, torch.int32)
    nat.call("sc_node_adjacency", n_nodes, n_en, elem_idx_d.data_ptr(), inc_ptr.data_ptr(), inc.data_ptr(), None,
             deg.data_ptr(), None, s)
    adj_ptr = dv.empty(n_nodes + 1, torch.int64)
    adj_ptr[:n_nodes] = deg.to(torch.int64)
    scan_work = dv.empty(nat.value("sc_scan_work_size", n_nodes), torch.int64)
    nat.call("sc_exclusive_scan_i64", n_nodes, adj_ptr.data_ptr(), adj_ptr.data_ptr(), scan_work.data_ptr(), s)
    n_adj = int(adj_ptr[n_nodes].item())
    adj = dv.empty(max(n_adj, 1), torch.int32)
    nat.call("sc_node_adjacency", n_nodes, n_en, elem_idx_d.data_ptr(), inc_ptr.data_ptr(), inc.data_ptr(),
             adj_ptr.data_ptr(), None, adj.data_ptr(), s)
    rowptr = dv.zeros(n_eq + 1, torch.int64)
    nat.call("sc_csr_pattern", n_nodes, dim, eqmap_d.data_ptr(), adj_ptr.data_ptr(), adj.data_ptr(), None,
             rowptr.data_ptr(), None, s)
    scan_work = dv.empty(nat.value("sc_scan_work_size", n_eq), torch.int64)
    nat.call("sc_exclusive_scan_i64", n_eq, rowptr.data_ptr(), rowptr.data_ptr(), scan_work.data_ptr(), s)
    nnz = int(rowptr[n_eq].item())
    cols = dv.empty(max(nnz, 1), torch.int32)[:nnz]
    nat.call("sc_csr_pattern", n_nodes, dim, eqmap_d.data_ptr(), adj_ptr.data_ptr(), adj.data_ptr(),
             rowptr.data_ptr(), None, cols.data_ptr(), s)
    return inc_ptr, inc, adj_ptr, adj, DeviceCSR(n_eq, rowptr, cols)


class GenerateMatrix:
    r"""GPU global stiffness, mass and damping (drop-in for the reference's GenerateMatrix)."""

    def __init__(self, nb_equations: int, order: int) -> None:
        self.n_eq = int(nb_equations)
        self.order = int(order)
        self.pattern = None
        self.K_d = self.M_d = self.C_d = None
        self.K0_d = None
        self.Cabs_d = None
        self.Kabs_d = None
        self.alpha = self.beta = 0.0
        self.props = None
        self._cache = {}
        self.n_nodes = self.dim = None
        self.adj_ptr = self.adj = self.eqmap_d = None

    # -------------------------------------------------------------- element integration + assembly
    def generate_stiffness_and_mass(self, data, material: dict, element_props=None) -> None:
        """Element Ke/Me on the GPU, then deterministic CSR assembly (system_matrix.py:35-121).
        element_props: optional per-element (E, nu, rho) arrays used instead of ``material``
        (the per-element materials the reference's random-field path creates)."""
        dv.require_cuda()
        etype = str(data.element_type)
        dim = int(data.dimension)
        n_en = ELEM_NODES[etype]
        nodes, id2idx, elem_idx, eqmap = model_arrays(data)
        E, nu, rho = element_properties(data, material) if element_props is None else \
            tuple(np.asarray(x, dtype=float) for x in element_props)
        self.props = (E, nu, rho)
        n_elem, n_nodes = len(elem_idx), len(nodes)
        s = dv.stream_ptr()
        xyz_d = dv.to_dev(nodes[:, 1:1 + dim], torch.float64)
        elem_d = dv.to_dev(elem_idx, torch.int32)
        coords = xyz_d[elem_d.long()].contiguous()  # [E, n_en, dim]
        nd = n_en * dim
        Ke = dv.empty(n_elem * nd * nd, torch.float64)
        Me = dv.empty(n_elem * nd * nd, torch.float64)
        E_d, nu_d, rho_d = (dv.to_dev(x, torch.float64) for x in (E, nu, rho))
        nat.call("sc_element_matrices", nat.ELEMENT_CODES[etype], self.order, n_elem, coords.data_ptr(),
                 E_d.data_ptr(), nu_d.data_ptr(), rho_d.data_ptr(), Ke.data_ptr(), Me.data_ptr(), s)
        eqmap_d = dv.to_dev(eqmap, torch.int32)
        inc_ptr, inc, adj_ptr, adj, pat = _csr_from_elements(n_nodes, n_en, dim, elem_d, eqmap_d, self.n_eq)
        K = dv.zeros(max(pat.nnz, 1), torch.float64)[:pat.nnz]
        M = dv.zeros(max(pat.nnz, 1), torch.float64)[:pat.nnz]
        nat.call("sc_assemble_values", n_nodes, n_en, dim, elem_d.data_ptr(), eqmap_d.data_ptr(), inc_ptr.data_ptr(),
                 inc.data_ptr(), adj_ptr.data_ptr(), adj.data_ptr(), pat.rowptr.data_ptr(), pat.cols.data_ptr(),
                 Ke.data_ptr(), Me.data_ptr(), K.data_ptr(), M.data_ptr(), s)
        del Ke, Me
        self.pattern = pat
        self.n_nodes, self.dim = n_nodes, dim
        self.adj_ptr, self.adj, self.eqmap_d = adj_ptr, adj[:int(adj_ptr[n_nodes].item())], eqmap_d
        self.K0_d = K
        self.K_d = K
        self.M_d = M
        self.C_d = dv.zeros(max(pat.nnz, 1), torch.float64)[:pat.nnz]
        self._cache.clear()

    # -------------------------------------------------------------- Lysmer
    def absorbing_boundaries(self, data, material: dict, parameters_viscous: list, parameters_stiff: float) -> None:
        """Lysmer dashpots into C and springs into K (system_matrix.py:256-376), face detection
        and node ordering on the host (O(boundary)), face integrals and scatter on the GPU."""
        from .lysmer import boundary_faces

        if self.pattern is None:
            raise RuntimeError("generate_stiffness_and_mass must run first")
        etype = str(data.element_type)
        if int(data.dimension) != 3:
            # the reference exits for 2D absorbing faces (system_matrix.py:324-326) and only
            # re-adds zero matrices otherwise; nothing to add here
            if np.any(np.asarray(data.BC) == 2):
                raise SystemExit("Absorbing boundaries not implemented for 2D yet")
            return
        faces = boundary_faces(data, self.props, parameters_viscous)
        nf = FACE_NODES[FACE_TYPES[etype]]
        nnz = self.pattern.nnz
        self.Cabs_d = dv.zeros(max(nnz, 1), torch.float64)[:nnz]
        self.Kabs_d = dv.zeros(max(nnz, 1), torch.float64)[:nnz]
        n_face = len(faces["eqs"])
        if n_face:
            s = dv.stream_ptr()
            xy = dv.to_dev(faces["xy"], torch.float64)
            Fm = dv.empty(n_face * nf * nf, torch.float64)
            nat.call("sc_face_matrices", nat.ELEMENT_CODES[FACE_TYPES[etype]], self.order, n_face, xy.data_ptr(),
                     Fm.data_ptr(), s)
            eqs = dv.to_dev(faces["eqs"], torch.int32)
            fct = dv.to_dev(faces["fct"], torch.float64)
            fct2 = dv.to_dev(faces["fct2"], torch.float64)
            row_ptr = dv.empty(self.n_eq + 1, torch.int32)
            order = dv.empty(n_face * nf * nf, torch.int32)
            work = dv.empty(self.n_eq, torch.int32)
            nat.call("sc_group_rows", n_face, nf, eqs.data_ptr(), self.n_eq, row_ptr.data_ptr(), order.data_ptr(),
                     work.data_ptr(), s)
            nat.call("sc_lysmer_values", n_face, nf, eqs.data_ptr(), Fm.data_ptr(), fct.data_ptr(), fct2.data_ptr(),
                     self.n_eq, row_ptr.data_ptr(), order.data_ptr(), self.pattern.rowptr.data_ptr(),
                     self.pattern.cols.data_ptr(), self.Cabs_d.data_ptr(), self.Kabs_d.data_ptr(), s)
        # C = C + C_abs ; K = K + K_abs / k_div (system_matrix.py:375-376)
        K = dv.empty(max(nnz, 1), torch.float64)[:nnz]
        nat.call("sc_combine", nnz, 1.0, self.K0_d.data_ptr(), 1.0 / parameters_stiff, self.Kabs_d.data_ptr(), 0.0,
                 None, K.data_ptr(), dv.stream_ptr())
        C = dv.empty(max(nnz, 1), torch.float64)[:nnz]
        nat.call("sc_combine", nnz, 1.0, self.C_d.data_ptr(), 1.0, self.Cabs_d.data_ptr(), 0.0, None, C.data_ptr(),
                 dv.stream_ptr())
        self.K_d = K
        self.C_d = C
        self._cache.clear()

    # -------------------------------------------------------------- Rayleigh
    @staticmethod
    def rayleigh_coefficients(damp):
        """(alpha, beta) from [f1, xi1, f2, xi2] (system_matrix.py:177-187)."""
        f1, d1, f2, d2 = damp
        if f1 == f2:
            raise SystemExit("Frequencies for the Rayleigh damping are the same.")
        A = 1 / 2 * np.array([[1 / (2 * np.pi * f1), 2 * np.pi * f1], [1 / (2 * np.pi * f2), 2 * np.pi * f2]])
        return np.linalg.solve(A, np.array([d1, d2]))

    def damping_Rayleigh(self, damp) -> None:
        """C = C + (alpha M + beta K) on the GPU (system_matrix.py:166-198)."""
        a, b = self.rayleigh_coefficients(damp)
        # C = C_abs + (alpha M + beta K): kept as coefficients for the node-block solver
        self.alpha, self.beta = self.alpha + float(a), self.beta + float(b)
        a, b = float(a), float(b)
        nnz = self.pattern.nnz
        C = dv.empty(max(nnz, 1), torch.float64)[:nnz]
        nat.call("sc_combine", nnz, 1.0, self.C_d.data_ptr(), a, self.M_d.data_ptr(), b,
                 self.K_d.data_ptr(), C.data_ptr(), dv.stream_ptr())
        self.C_d = C
        self._cache.clear()

    # -------------------------------------------------------------- scipy views
    def _scipy(self, key, values):
        if key not in self._cache:
            A = self.pattern.to_scipy(values)
            if key in ("K", "C"):
                A.eliminate_zeros()  # scipy's sparse + sparse drops exact zeros
            for arr in (A.data, A.indices, A.indptr):
                arr.flags.writeable = False  # a view of the device matrix: edits would not reach it
            A._scatter_gb300_source = (weakref.ref(self), key)
            self._cache[key] = A
        return self._cache[key]

    def device_values(self, A):
        """The device value array behind a scipy matrix this generator handed out, or None."""
        src = getattr(A, "_scatter_gb300_source", None)
        if src is None or src[0]() is not self or self._cache.get(src[1]) is not A:
            return None
        return {"K": self.K_d, "M": self.M_d, "C": self.C_d}[src[1]]

    @property
    def K(self):
        return self._scipy("K", self.K_d)

    @property
    def M(self):
        return self._scipy("M", self.M_d)

    @property
    def C(self):
        return self._scipy("C", self.C_d)


def generator_of(M, C, K):
    """The GenerateMatrix whose current .M, .C, .K are exactly these scipy objects, or None.

    Each matrix handed out carries a weak link to its generator; the link only counts while
    the object is still the generator's current one (any later assembly step replaces it)."""
    src = getattr(M, "_scatter_gb300_source", None)
    g = src[0]() if src is not None else None
    if g is None:
        return None
    ok = (g.device_values(M) is g.M_d and g.device_values(C) is g.C_d and g.device_values(K) is g.K_d)
    return g if ok else None
