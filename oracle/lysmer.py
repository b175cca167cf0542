"""Lysmer absorbing boundaries restated (oracle; test infrastructure only).

Restates GenerateMatrix.absorbing_boundaries (scatter/system_matrix.py:256-376)
with utils.clockwise_sort_2D_elements / are_collinear (scatter/utils.py:141-196),
including the reference's behaviour that matters for parity:

* a face is detected per direction i when exactly ``nb_nodes_lower_elem`` of the
  element's nodes are absorbing in direction i (:314);
* the face's in-plane coordinates are put in the clockwise order of
  clockwise_sort_2D_elements (corners by angle, then the remaining mid-side
  nodes in Python set order) and integrated as a SurfaceElement (:322-336);
* the resulting node matrix is scattered into rows/cols of the *sorted*
  equation numbers of the face nodes (:355-357), not the sorted-coordinate
  order, and the dashpot factor multiplies columns (:362-370);
* ``|F| * (Ec or G) / absorbing_BC_stiff`` is added to K (:373,376).
"""
import numpy as np
import scipy.sparse as sp

from . import elements as el


def _are_collinear(coords):
    """utils.py:178-196."""
    x1, y1 = coords[0]
    x2, y2 = coords[1]
    slope = (y2 - y1) / (x2 - x1) if x2 != x1 else float("inf")
    for i in range(2, len(coords)):
        x1, y1 = coords[i - 1]
        x2, y2 = coords[i]
        ns = (y2 - y1) / (x2 - x1) if x2 != x1 else float("inf")
        if ns != slope:
            return False
    return True


def clockwise_sort(points):
    """utils.py:141-175: angle sort about the lowest-y point, corners first, then the
    remaining points in the order Python's set symmetric difference yields them."""
    pts = [np.asarray(p, dtype=float) for p in points]
    ref = min(pts, key=lambda p: p[1])
    srt = sorted(pts, key=lambda p: np.arctan2(p[1] - ref[1], p[0] - ref[0]))
    corner = [srt[0]]
    base = 0
    for i in range(len(srt) - 1):
        if not _are_collinear(srt[base:i + 2]):
            corner.append(srt[i])
            base = i
    s1 = set(map(tuple, srt))
    s2 = set(map(tuple, corner))
    middle = list(map(list, s1.symmetric_difference(s2)))
    corner.extend(middle)
    return np.array(corner)


def absorbing(model, props, parameters_viscous, parameters_stiff, order=2):
    """Return (C_abs, K_abs) as CSR; ``model`` is a dict with nodes, elem, BC, BC_dir,
    eq_nb_dof, element_type, materials_index; ``props`` maps element -> (E, nu, rho)."""
    nodes = np.asarray(model["nodes"], dtype=float)
    elem = np.asarray(model["elem"], dtype=np.int64)
    BC = np.asarray(model["BC"])
    BC_dir = np.asarray(model["BC_dir"])
    eq_nb_dof = np.asarray(model["eq_nb_dof"], dtype=float)
    etype = str(model["element_type"])
    dim = el.DIM[etype]
    n_eq = int(model["number_eq"])
    # entries collected per face in face order and summed by the sparse constructor (the
    # reference adds face by face into lil matrices, system_matrix.py:362-376); the
    # equation -> (node, dof) inverse of eq_nb_dof replaces the reference's np.where search
    c_r, c_c, c_v, k_v = [], [], [], []
    free = ~np.isnan(eq_nb_dof)
    eq_node = np.full(n_eq, -1, dtype=np.int64)
    eq_dof = np.full(n_eq, -1, dtype=np.int64)
    nn, dd = np.nonzero(free)
    eq_node[eq_nb_dof[nn, dd].astype(np.int64)] = nn
    eq_dof[eq_nb_dof[nn, dd].astype(np.int64)] = dd
    if dim != 3:
        return sp.csr_matrix((n_eq, n_eq)), sp.csr_matrix((n_eq, n_eq))
    ftype = el.LOWER[etype]
    nf = el.NODES[ftype]
    id2idx = {int(n): i for i, n in enumerate(nodes[:, 0])}
    absorb = BC == 2
    E_, nu_, rho_ = props
    # elements with no absorbing node contribute nothing: visit only the others
    ids = nodes[:, 0].astype(np.int64)
    idmap = np.full(int(ids.max()) + 1, -1, dtype=np.int64)
    idmap[ids] = np.arange(len(ids))
    touching = np.nonzero(absorb.any(axis=1)[idmap[elem]].any(axis=1))[0]
    for e in touching:
        idx = [id2idx[int(n)] for n in elem[e]]
        sel = [i for i in idx if absorb[i].any()]
        if not sel:
            continue
        E, nu, rho = float(E_[e]), float(nu_[e]), float(rho_[e])
        Ec = E * (1 - nu) / ((1 + nu) * (1 - 2 * nu))
        G = E / (2 * (1 + nu))
        vp = np.sqrt(Ec / rho)
        vs = np.sqrt(G / rho)
        bt = absorb[sel]
        for d in range(dim):
            if bt[:, d].sum() != nf:
                continue
            col = np.where(bt[:, d])[0]
            fidx = [sel[k] for k in col]
            xy = np.delete(nodes[fidx, 1:], d, axis=1)
            xy = clockwise_sort(xy)
            F = el.face_matrix(ftype, xy[None], order)[0]
            i1 = np.sort(eq_nb_dof[fidx, d]).astype(np.int64)
            fct = np.full(nf, parameters_viscous[1] * rho * vs)
            fct2 = np.full(nf, G)
            for k, val in enumerate(i1):
                if BC_dir[eq_node[val], eq_dof[val]] == 1:
                    fct[k] = parameters_viscous[0] * rho * vp
                    fct2[k] = Ec
            c_r.append(np.repeat(i1, nf))
            c_c.append(np.tile(i1, nf))
            c_v.append((F * fct).ravel())
            k_v.append((np.abs(F) * fct2).ravel())
    if not c_r:
        return sp.csr_matrix((n_eq, n_eq)), sp.csr_matrix((n_eq, n_eq))
    r, c = np.concatenate(c_r), np.concatenate(c_c)
    C = sp.csr_matrix((np.concatenate(c_v), (r, c)), shape=(n_eq, n_eq))
    Kst = sp.csr_matrix((np.concatenate(k_v), (r, c)), shape=(n_eq, n_eq))
    C.sum_duplicates()
    Kst.sum_duplicates()
    return C, Kst / parameters_stiff
