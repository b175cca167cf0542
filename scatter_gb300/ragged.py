"""Ragged batching: independent meshes of uneven size and element type advanced together.

No reference counterpart (the reference solves one mesh per call).  Each mesh is assembled on
its own (scatter/system_matrix.py semantics, its own homogeneous material), then the meshes'
node-block systems are concatenated block-diagonally -- node, equation and pattern offsets --
into one system that the explicit scheme of sc_nb_explicit_run advances with one kernel (one
graph launch) per step for all meshes.  Every node row belongs to one mesh, so a row's
products are the ones the mesh alone would compute; the sliced-ELL width adapts per slice to
the mesh's row lengths (hexa8 and tetra10 rows differ).  The step kernel's threads per node
row are picked by timing (sc_nb_tune_explicit).

Lumped mass per mesh: row sums of the consistent mass (hexa8), or, for the quadratic
tetrahedron, whose consistent-mass row sums are negative at the corners (the reference's
4-point rule gives -1/20 of the element mass there), the diagonal scaled to the element mass
(HRZ: m_ii = M_ii * sum(M_e) / trace(M_e), one factor per element shape for straight-sided
elements).
"""
import ctypes
from types import SimpleNamespace

import numpy as np
import torch

from . import _native as nat
from . import device as dv
from .force_external import ricker_table
from .solvers import ForceTable, NodeBlockNewmark
from .system_matrix import ELEM_NODES, GenerateMatrix, model_arrays


def mesh_specs(n_meshes, seed, hexa_edges=(10, 80), tetra_edges=(5, 40), h=0.5):
    """Seeded mesh descriptions: element type (hexa8 or tetra10 made of hexes split into 6
    tets), edge counts per axis drawn uniformly, homogeneous E in [20, 200] MPa, nu in
    [0.2, 0.35], rho in [1700, 2100]."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_meshes):
        etype = "hexa8" if rng.random() < 0.5 else "tetra10"
        lo, hi = hexa_edges if etype == "hexa8" else tetra_edges
        nx, ny, nz = (int(x) for x in rng.integers(lo, hi + 1, size=3))
        out.append({"element": etype, "dims": (nx, ny, nz), "h": h, "E": float(rng.uniform(20e6, 200e6)),
                    "nu": float(rng.uniform(0.2, 0.35)), "rho": float(rng.uniform(1700.0, 2100.0))})
    return out


def _top_centre(model):
    top = model.top_nodes()
    X = model.nodes[model.node_index()[top], 1:]
    c = 0.5 * (X.min(axis=0) + X.max(axis=0))
    return int(top[np.argmin(((X[:, [0, 2]] - c[[0, 2]]) ** 2).sum(axis=1))])


def hrz_factor(model, nu, rho, order=2):
    """sum(M_e) / trace(M_e) of the model's first element (one x-component block)."""
    etype = str(model.element_type)
    nodes, _, elem_idx, _ = model_arrays(model)
    n_en = ELEM_NODES[etype]
    X = dv.to_dev(nodes[:, 1:][elem_idx[:1]], torch.float64)
    one = dv.to_dev(np.ones(1), torch.float64)
    nu_t = dv.to_dev(np.array([nu]), torch.float64)
    rho_t = dv.to_dev(np.array([rho]), torch.float64)
    nd = 3 * n_en
    ke = dv.empty(nd * nd, torch.float64)
    me = dv.empty(nd * nd, torch.float64)
    nat.call("sc_element_matrices", nat.ELEMENT_CODES[etype], order, 1, X.data_ptr(), one.data_ptr(), nu_t.data_ptr(),
             rho_t.data_ptr(), ke.data_ptr(), me.data_ptr(), dv.stream_ptr())
    Me = dv.host(me).reshape(n_en, 3, n_en, 3)[:, 0, :, 0]
    return float(Me.sum() / np.trace(Me))


def lumped_mass(Me, ktype, elem_idx, free, rho, hrz=False):
    """Lumped mass per node and component [n_nodes, 3] from per-type unit-rho element mass
    blocks Me [types, n_en, n_en] (one component; the consistent mass is m_ab I): row sums over
    free columns (the row sums of the assembled mass), or the diagonal scaled to the element
    mass (hrz).  Fixed components get 1."""
    N = len(free)
    ml = np.zeros((N, 3))
    if hrz:
        f = Me.sum(axis=(1, 2)) / np.einsum("taa->t", Me)
        contrib = np.einsum("taa,t->ta", Me, f)[ktype][:, :, None] * np.ones(3)
    else:
        contrib = np.einsum("eab,ebc->eac", Me[ktype], free[elem_idx].astype(float))
    np.add.at(ml, elem_idx, contrib * rho)
    return np.where(free, ml, 1.0)


class RaggedExplicit:
    def __init__(self, specs, damping, dt, time_grid, load_amplitude=-10e3, f0=20.0, t0=0.05, order=2,
                 bottom="111", x_faces="100", z_faces="001", tune=True):
        from . import meshgen

        dv.require_cuda()
        self.specs = specs
        parts = []
        node_off = eq_off = nnz_off = adj_off = 0
        rowptrs, colss, Ks, Ms, Cs, adj_ptrs, adjs, eqmaps, mls = [], [], [], [], [], [], [], [], []
        f_tables, rec_eq = [], []
        s = dv.stream_ptr()
        alpha = beta = None
        for sp in specs:
            nx, ny, nz = sp["dims"]
            m = meshgen.box_model(nx, ny, nz, sp["h"], element=sp["element"], bottom=bottom, x_faces=x_faces,
                                  z_faces=z_faces)
            mats = {"solid": {"density": sp["rho"], "Young": sp["E"], "poisson": sp["nu"]}}
            g = GenerateMatrix(m.number_eq, order)
            g.generate_stiffness_and_mass(m, mats)
            g.damping_Rayleigh(damping)
            alpha, beta = g.alpha, g.beta
            n_eq, N = g.n_eq, g.n_nodes
            rp = g.pattern.rowptr
            # lumped mass in the mesh's equation numbering
            ml = torch.empty(n_eq, dtype=torch.float64, device=rp.device)
            if sp["element"] == "tetra10":
                rows = torch.repeat_interleave(torch.arange(n_eq, device=rp.device), (rp[1:] - rp[:-1]).long())
                diag = g.M_d[g.pattern.cols.long() == rows]
                ml = diag * hrz_factor(m, sp["nu"], sp["rho"], order)
            else:
                nat.call("sc_csr_row_sums", n_eq, rp.data_ptr(), g.M_d.data_ptr(), 0, ml.data_ptr(), s)
            rowptrs.append(rp[:-1] + nnz_off)
            colss.append(g.pattern.cols + eq_off)
            Ks.append(g.K_d)
            Ms.append(g.M_d)
            Cs.append(g.C_d)
            adj_ptrs.append(g.adj_ptr[:-1] + adj_off)
            adjs.append(g.adj + node_off)
            em = g.eqmap_d.clone()
            em[em >= 0] += eq_off
            eqmaps.append(em)
            mls.append(ml)
            tg = np.asarray(time_grid, dtype=float)
            ft = ricker_table(m, _top_centre(m), load_amplitude, f0, t0, tg)
            f_tables.append((ft, eq_off))
            rec_eq.append(int(m.eq_nb_dof[m.node_index()[_top_centre(m)], 1]) + eq_off)
            parts.append({"n_eq": n_eq, "n_nodes": N, "eq_off": eq_off, "node_off": node_off, "element": sp["element"]})
            node_off += N
            eq_off += n_eq
            nnz_off += g.pattern.nnz
            adj_off += int(g.adj_ptr[N].item())
            del g
        dev = rowptrs[0].device
        pattern = SimpleNamespace(rowptr=torch.cat(rowptrs + [torch.tensor([nnz_off], dtype=torch.int64, device=dev)]),
                                  cols=torch.cat(colss).to(torch.int32).contiguous(), n=eq_off, nnz=nnz_off)
        self.union = SimpleNamespace(
            pattern=pattern, K_d=torch.cat(Ks), M_d=torch.cat(Ms), C_d=torch.cat(Cs), Cabs_d=None,
            adj_ptr=torch.cat(adj_ptrs + [torch.tensor([adj_off], dtype=torch.int64, device=dev)]),
            adj=torch.cat(adjs).to(torch.int32).contiguous(), eqmap_d=torch.cat(eqmaps).contiguous(),
            n_nodes=node_off, dim=3, n_eq=eq_off, alpha=alpha, beta=beta)
        self.parts = parts
        self.n_eq, self.n_nodes = eq_off, node_off
        del Ks, Ms, Cs
        # force: every mesh's table, entries of a step concatenated mesh by mesh
        n_t = len(time_grid)
        counts = np.zeros(n_t, dtype=np.int64)
        for ft, _ in f_tables:
            counts += np.diff(ft.f_ptr)
        ptr = np.r_[0, np.cumsum(counts)]
        f_eq = np.empty(ptr[-1], dtype=np.int64)
        f_val = np.empty(ptr[-1])
        fill = ptr[:-1].copy()
        for ft, off in f_tables:
            c = np.diff(ft.f_ptr)
            step = np.repeat(np.arange(n_t), c)
            pos = fill[step] + (np.arange(len(step)) - np.repeat(ft.f_ptr[:-1], c))
            f_eq[pos] = ft.f_eq + off
            f_val[pos] = ft.f_val
            fill += c
        self.table = ForceTable(ptr, f_eq, f_val, eq_off)
        self.rec_eq = np.asarray(rec_eq, dtype=np.int64)
        self.dt = dt
        self.solver = NodeBlockNewmark(self.union, dt, precond="jacobi")
        ml_slot = torch.ones(self.solver.n_s, dtype=torch.float64, device=dev)
        ml_eq = torch.cat(mls)
        ml_slot[self.solver.eq2slot] = ml_eq
        self._ml_slot = ml_slot
        nat.call("sc_nb_set_lumped_mass", self.solver.h, ml_slot.data_ptr())
        self.solver.set_force(self.table)
        self.tuned = self.solver.tune_explicit() if tune else None

    def set_output(self, interval, n_out):
        self.solver.set_output(interval, self.rec_eq, n_out, what=("v",))

    def run(self, t_begin, t_end):
        self.solver.run_explicit(t_begin, t_end)

    def velocities(self):
        """[n_out, n_meshes]: vertical velocity at each mesh's top-centre node."""
        return self.solver.outputs()["v"]

    def close(self):
        self.solver.close()


class RaggedBatch:
    """The same meshes advanced matrix-free: one thread per node gathers its incident elements'
    unit-E stiffness (one FP32 table per element shape and nu) scaled by the mesh's E, FP32
    products with (hi, lo) pair accumulators for u and v (the batched path's arithmetic,
    csrc/sc_batch.cu with one realisation and per-node element types).  No global matrix is
    stored, so the memory is a few tens of bytes per DOF and the kernel is compute-bound."""

    def __init__(self, specs, damping, dt, time_grid, load_amplitude=-10e3, f0=20.0, t0=0.05, order=2,
                 bottom="111", x_faces="100", z_faces="001"):
        from . import meshgen
        from .batched import _Desc, element_types
        from .system_matrix import GenerateMatrix

        dv.require_cuda()
        s = dv.stream_ptr()
        alpha, beta = GenerateMatrix.rayleigh_coefficients(damping)
        nen_max = max(ELEM_NODES[sp["element"]] for sp in specs)
        nd_max = 3 * nen_max
        elems, types, young, k1s, fixed, mls, nens, inc_ptrs, incs = [], [], [], [], [], [], [], [], []
        node_off = elem_off = type_off = inc_off = 0
        f_parts, rec_slot = [], []
        self.parts = []
        for sp in specs:
            nx, ny, nz = sp["dims"]
            m = meshgen.box_model(nx, ny, nz, sp["h"], element=sp["element"], bottom=bottom, x_faces=x_faces,
                                  z_faces=z_faces)
            etype = str(m.element_type)
            n_en = ELEM_NODES[etype]
            nodes, _, elem_idx, eqmap = model_arrays(m)
            N, n_el = len(nodes), len(elem_idx)
            nu = np.full(n_el, sp["nu"])
            first, ktype = element_types(m, nu)
            # unit-E stiffness and unit-rho mass per element shape
            X = dv.to_dev(nodes[:, 1:][elem_idx[first]], torch.float64)
            one = dv.to_dev(np.ones(len(first)), torch.float64)
            nu_t = dv.to_dev(nu[first], torch.float64)
            nd = 3 * n_en
            ke = dv.empty(len(first) * nd * nd, torch.float64)
            me = dv.empty(len(first) * nd * nd, torch.float64)
            nat.call("sc_element_matrices", nat.ELEMENT_CODES[etype], order, len(first), X.data_ptr(), one.data_ptr(),
                     nu_t.data_ptr(), one.data_ptr(), ke.data_ptr(), me.data_ptr(), s)
            torch.cuda.current_stream().synchronize()
            Ke = dv.host(ke).reshape(len(first), nd, nd)
            Me = dv.host(me).reshape(len(first), n_en, 3, n_en, 3)[:, :, 0, :, 0]  # per-component block
            kp = np.zeros((len(first), nd_max, nd_max), dtype=np.float32)
            kp[:, :nd, :nd] = Ke
            k1s.append(kp)
            # lumped mass per slot: row sums over free columns, or the diagonal scaled to the
            # element mass for the quadratic tetrahedron
            free = (eqmap >= 0)
            mls.append(lumped_mass(Me, ktype, elem_idx, free, sp["rho"], hrz=etype == "tetra10").ravel())
            fixed.append((~free).astype(np.int32).ravel())
            # connectivity, padded to the largest element type
            ep = np.zeros((n_el, nen_max), dtype=np.int64)
            ep[:, :n_en] = elem_idx + node_off
            ep[:, n_en:] = ep[:, :1]
            elems.append(ep)
            types.append(ktype.astype(np.int64) + type_off)
            young.append(np.full(n_el, sp["E"], dtype=np.float32))
            nens.append(np.full(N, n_en, dtype=np.uint8))
            # node -> element incidence of the mesh, offset into the union
            el_d = dv.to_dev(elem_idx.astype(np.int32), torch.int32)
            ip = dv.empty(N + 1, torch.int32)
            inc = dv.empty(n_el * n_en, torch.int32)
            work = dv.empty(N, torch.int32)
            nat.call("sc_node_incidence", n_el, n_en, N, el_d.data_ptr(), ip.data_ptr(), inc.data_ptr(),
                     work.data_ptr(), s)
            inc_ptrs.append(dv.host(ip)[:-1].astype(np.int64) + inc_off)
            incs.append(dv.host(inc).astype(np.int64) + elem_off)
            # force and receiver in slot space
            tg = np.asarray(time_grid, dtype=float)
            c = _top_centre(m)
            ft = ricker_table(m, c, load_amplitude, f0, t0, tg)
            inv = np.full(int(m.number_eq), -1, dtype=np.int64)
            nn, cc = np.nonzero(free)
            inv[eqmap[nn, cc]] = (nn + node_off) * 3 + cc
            f_parts.append((ft, inv))
            rec_slot.append((int(m.node_index()[c]) + node_off) * 3 + 1)
            self.parts.append({"element": etype, "n_eq": int(m.number_eq), "n_nodes": N})
            node_off += N
            elem_off += n_el
            type_off += len(first)
            inc_off += n_el * n_en
        self.n_nodes, self.n_elem = node_off, elem_off
        self.n_eq = sum(p["n_eq"] for p in self.parts)
        n_t = len(time_grid)
        counts = np.zeros(n_t, dtype=np.int64)
        for ft, _ in f_parts:
            counts += np.diff(ft.f_ptr)
        ptr = np.r_[0, np.cumsum(counts)]
        f_slot = np.empty(ptr[-1], dtype=np.int64)
        f_val = np.empty(ptr[-1])
        fill = ptr[:-1].copy()
        for ft, inv in f_parts:
            cnt = np.diff(ft.f_ptr)
            step = np.repeat(np.arange(n_t), cnt)
            pos = fill[step] + (np.arange(len(step)) - np.repeat(ft.f_ptr[:-1], cnt))
            f_slot[pos] = inv[ft.f_eq]
            f_val[pos] = ft.f_val
            fill += cnt
        self._t = {
            "elem": dv.to_dev(np.concatenate(elems).astype(np.int32), torch.int32),
            "ke_type": dv.to_dev(np.concatenate(types).astype(np.int32), torch.int32),
            "ke1": dv.to_dev(np.concatenate(k1s), torch.float32),
            "young": dv.to_dev(np.concatenate(young), torch.float32),
            "ml": dv.to_dev(np.concatenate(mls), torch.float64),
            "fixed": dv.to_dev(np.concatenate(fixed), torch.int32),
            "inc_ptr": dv.to_dev(np.r_[np.concatenate(inc_ptrs), inc_off].astype(np.int32), torch.int32),
            "inc": dv.to_dev(np.concatenate(incs).astype(np.int32), torch.int32),
            "node_nen": dv.to_dev(np.concatenate(nens), torch.uint8),
            "l_ptr": torch.zeros(3 * node_off + 1, dtype=torch.int64, device="cuda"),
            "l_i": torch.zeros(1, dtype=torch.int32, device="cuda"),
            "l_f": torch.zeros(1, dtype=torch.float32, device="cuda"),
            "f_ptr": dv.to_dev(ptr, torch.int64), "f_slot": dv.to_dev(f_slot.astype(np.int32), torch.int32),
            "f_val": dv.to_dev(f_val, torch.float64),
            "rec": dv.to_dev(np.asarray(rec_slot, dtype=np.int32), torch.int32)}
        t = self._t
        self.u = dv.zeros(3 * node_off, torch.float64)
        self.v = dv.zeros(3 * node_off, torch.float64)
        d = _Desc(node_off, elem_off, nen_max, 1, int(t["ke1"].shape[0]), t["elem"].data_ptr(), t["inc_ptr"].data_ptr(),
                  t["inc"].data_ptr(), t["ke_type"].data_ptr(), t["ke1"].data_ptr(), t["young"].data_ptr(),
                  t["ml"].data_ptr(), t["fixed"].data_ptr(), float(alpha), float(beta), float(dt), t["l_ptr"].data_ptr(),
                  t["l_i"].data_ptr(), t["l_i"].data_ptr(), t["l_f"].data_ptr(), t["l_f"].data_ptr(),
                  t["node_nen"].data_ptr())
        self._desc = d
        h = ctypes.c_void_p()
        nat.call("sc_batch_create", ctypes.byref(h), ctypes.byref(d), self.u.data_ptr(), self.v.data_ptr(), s)
        self.h = h
        nat.call("sc_batch_set_force", self.h, n_t, t["f_ptr"].data_ptr(), t["f_slot"].data_ptr(),
                 t["f_val"].data_ptr())
        rpt, tpb, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        nat.call("sc_batch_config", self.h, ctypes.byref(rpt), ctypes.byref(tpb), ctypes.byref(ms), None)
        self.tuned = (tpb.value, ms.value)

    def set_output(self, interval, n_out):
        self.n_out = int(n_out)
        self.out_v = dv.zeros(self.n_out * len(self.parts), torch.float64)
        nat.call("sc_batch_set_output", self.h, int(interval), len(self.parts), self._t["rec"].data_ptr(),
                 self.out_v.data_ptr(), self.n_out)

    def run(self, t_begin, t_end):
        nat.call("sc_batch_run", self.h, int(t_begin), int(t_end))

    def velocities(self):
        """[n_out, n_meshes]: vertical velocity at each mesh's top-centre node."""
        return dv.host(self.out_v).reshape(self.n_out, len(self.parts))

    def close(self):
        if getattr(self, "h", None):
            nat.value("sc_batch_destroy", self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
