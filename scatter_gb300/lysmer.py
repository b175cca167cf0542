"""Host-side face detection and node ordering for the Lysmer absorbing boundaries.

O(boundary) integer/permutation work that feeds the GPU face integrals
(``sc_face_matrices``) and scatter (``sc_lysmer_values``).  It keeps the reference's
behaviour of GenerateMatrix.absorbing_boundaries (scatter/system_matrix.py:256-376),
which parity with the reference requires:

* a face of element e in direction d exists when exactly ``nb_nodes_lower_elem`` of the
  element's nodes are absorbing (BC == 2) in direction d (:314); faces are taken in element
  order, then direction order;
* the face's in-plane coordinates (coordinate d removed) are ordered as
  utils.clockwise_sort_2D_elements (scatter/utils.py:141-175) does: angle about the first
  lowest-y point, corner detection by exact slope comparison, then the remaining (mid-side)
  points in Python set order -- the face integral is evaluated in that order (:328-336);
* its rows/columns go to the face nodes' equation numbers sorted ascending (:355-357), with
  the dashpot / spring factor of column k taken from the node holding the k-th smallest
  equation: a_p rho v_p and E_c if BC_dir == 1 there, else a_s rho v_s and G (:362-370).
"""
import numpy as np

from .system_matrix import ELEM_NODES, FACE_NODES, FACE_TYPES, model_arrays


def _collinear(pts):
    (x1, y1), (x2, y2) = pts[0], pts[1]
    slope = (y2 - y1) / (x2 - x1) if x2 != x1 else float("inf")
    for i in range(2, len(pts)):
        (x1, y1), (x2, y2) = pts[i - 1], pts[i]
        s = (y2 - y1) / (x2 - x1) if x2 != x1 else float("inf")
        if s != slope:
            return False
    return True


def clockwise_order(xy):
    """Node order of utils.clockwise_sort_2D_elements for one face (returns a permutation)."""
    pts = [tuple(map(float, p)) for p in xy]
    ref = min(range(len(pts)), key=lambda i: pts[i][1])
    rx, ry = pts[ref]
    ang = [float(np.arctan2(p[1] - ry, p[0] - rx)) for p in pts]
    srt = sorted(range(len(pts)), key=lambda i: ang[i])
    corner = [srt[0]]
    base = 0
    for i in range(len(srt) - 1):
        if not _collinear([pts[k] for k in srt[base:i + 2]]):
            corner.append(srt[i])
            base = i
    s_all = set(pts[k] for k in srt)
    s_cor = set(pts[k] for k in corner)
    middle = list(s_all.symmetric_difference(s_cor))
    lookup = {pts[k]: k for k in srt}
    return corner + [lookup[m] for m in middle]


def _linear_order(xy):
    """Vectorised clockwise order for faces without mid-side nodes ([F, nf, 2] -> [F, nf]).
    With no collinear triple of corners the reference's result is the plain angle order."""
    F = xy.shape[0]
    ref = np.argmin(xy[:, :, 1], axis=1)  # first lowest-y point, as min() returns
    r = xy[np.arange(F), ref]
    ang = np.arctan2(xy[:, :, 1] - r[:, None, 1], xy[:, :, 0] - r[:, None, 0])
    return np.argsort(ang, axis=1, kind="stable")


def boundary_faces(model, props, parameters_viscous):
    """Faces with their ordered in-plane coordinates, sorted equation numbers and factors."""
    etype = str(model.element_type)
    ftype = FACE_TYPES[etype]
    nf = FACE_NODES[ftype]
    n_en = ELEM_NODES[etype]
    nodes, id2idx, elem_idx, eqmap = model_arrays(model)
    BC = np.asarray(model.BC)
    BC_dir = np.asarray(model.BC_dir)
    absorb = BC == 2
    E, nu, rho = props
    A = absorb[elem_idx]  # [E, n_en, 3]
    cnt = A.sum(axis=1)  # [E, 3]
    fe, fd = np.nonzero(cnt == nf)  # element-major, direction-minor = the reference's order
    n_face = len(fe)
    out = {"eqs": np.zeros((n_face, nf), np.int32), "xy": np.zeros((n_face, nf, 2)),
           "fct": np.zeros((n_face, nf)), "fct2": np.zeros((n_face, nf)), "elem": fe.astype(np.int64)}
    if n_face == 0:
        return out
    # face nodes in element order
    sel = A[fe, :, fd]  # [F, n_en]
    pos = np.argsort(~sel, axis=1, kind="stable")[:, :nf]  # element-order positions of the nf nodes
    fnodes = elem_idx[fe[:, None], pos]  # [F, nf] node indices
    xyz = nodes[fnodes, 1:]  # [F, nf, 3]
    keep = np.array([[k for k in range(3) if k != d] for d in range(3)])[fd]  # [F, 2]
    xy = np.take_along_axis(xyz, keep[:, None, :], axis=2)
    if nf in (3, 4):
        order = _linear_order(xy)
    else:
        order = np.array([clockwise_order(f) for f in xy])
    out["xy"] = np.take_along_axis(xy, order[:, :, None], axis=1)
    feq = eqmap[fnodes, fd[:, None]]  # [F, nf]
    srt = np.argsort(feq, axis=1, kind="stable")
    out["eqs"] = np.take_along_axis(feq, srt, axis=1).astype(np.int32)
    node_sorted = np.take_along_axis(fnodes, srt, axis=1)
    normal = BC_dir[node_sorted, fd[:, None]] == 1
    Ee, nue, rhoe = E[fe], nu[fe], rho[fe]
    Ec = Ee * (1 - nue) / ((1 + nue) * (1 - 2 * nue))
    G = Ee / (2 * (1 + nue))
    vp = np.sqrt(Ec / rhoe)
    vs = np.sqrt(G / rhoe)
    out["fct"] = np.where(normal, (parameters_viscous[0] * rhoe * vp)[:, None], (parameters_viscous[1] * rhoe * vs)[:, None])
    out["fct2"] = np.where(normal, Ec[:, None], G[:, None])
    if np.any(out["eqs"] < 0):
        raise ValueError("absorbing face node without an equation number")
    return out
