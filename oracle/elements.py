"""Element library restated in numpy (oracle; test infrastructure only).

Restates scatter/element_types.py (shape functions, gmsh node order),
scatter/discretisation.py:436-497 (Gauss rules), :107-238 (volume Jacobian, B,
N, Ke, Me), :241-433 (2D solids and faces) and scatter/material_models.py:5-43.
Vectorised over elements: ``xyz`` is ``[E, n_en, dim]``.
"""
import math

import numpy as np

NODES = {"hexa8": 8, "hexa20": 20, "tetra4": 4, "tetra10": 10,
         "quad4": 4, "quad8": 8, "tri3": 3, "tri6": 6}
DIM = {"hexa8": 3, "hexa20": 3, "tetra4": 3, "tetra10": 3, "quad4": 2, "quad8": 2, "tri3": 2, "tri6": 2}
FAMILY = {"hexa8": "quad", "hexa20": "quad", "quad4": "quad", "quad8": "quad",
          "tetra4": "tetra", "tetra10": "tetra", "tri3": "tri", "tri6": "tri"}
LOWER = {"hexa8": "quad4", "hexa20": "quad8", "tetra4": "tri3", "tetra10": "tri6"}


def gauss(family, n):
    """Points [ng, d] and weights [ng]; discretisation.py:436-497 (hex loops :33-55)."""
    if family == "quad":
        if n == 1:
            x, w = [0.0], [2.0]
        elif n == 2:
            x, w = [-math.sqrt(1 / 3), math.sqrt(1 / 3)], [1.0, 1.0]
        elif n == 3:
            x, w = [-math.sqrt(3 / 5), 0.0, math.sqrt(3 / 5)], [5 / 9, 8 / 9, 5 / 9]
        else:
            raise ValueError("integration order not supported")
        return np.array(x), np.array(w)
    if family == "tri":
        if n == 1:
            p, w = [[1 / 3, 1 / 3]], [1 / 2]
        elif n == 2:
            p, w = [[1 / 6, 1 / 6], [2 / 3, 1 / 6], [1 / 6, 2 / 3]], [1 / 6] * 3
        elif n == 3:
            p, w = [[1 / 3, 1 / 3], [1 / 5, 1 / 5], [3 / 5, 1 / 5], [1 / 5, 3 / 5]], [-27 / 96, 25 / 96, 25 / 96, 25 / 96]
        else:
            raise ValueError("integration order not supported")
        return np.array(p), np.array(w)
    if family == "tetra":
        if n == 1:
            p, w = [[1 / 4, 1 / 4, 1 / 4]], [1 / 6]
        elif n == 2:
            a = 1 / 4 - 1 / 20 * math.sqrt(5)
            b = 1 / 4 + 3 / 20 * math.sqrt(5)
            p, w = [[a, a, a], [a, a, b], [a, b, a], [b, a, a]], [1 / 24] * 4
        else:
            raise ValueError("integration order not supported")
        return np.array(p), np.array(w)
    raise ValueError(family)


def points(etype, order):
    """Natural points [ng, d] and weights [ng] in the reference's loop order."""
    fam = FAMILY[etype]
    if fam == "quad":
        x, w = gauss("quad", order)
        if DIM[etype] == 3:
            P = np.array([[x[i], x[j], x[k]] for i in range(order) for j in range(order) for k in range(order)])
            W = np.array([w[i] * w[j] * w[k] for i in range(order) for j in range(order) for k in range(order)])
        else:
            P = np.array([[x[i], x[j]] for i in range(order) for j in range(order)])
            W = np.array([w[i] * w[j] for i in range(order) for j in range(order)])
        return P, W
    return gauss(fam, order)


def shape(etype, p):
    """N [n], dN [n, d] at natural point p; element_types.py (see per-type comments)."""
    if etype == "hexa8":  # element_types.py:52-104
        u, v, w = p
        sg = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                       [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=float)
        a, b, c = 1 + sg[:, 0] * u, 1 + sg[:, 1] * v, 1 + sg[:, 2] * w
        N = a * b * c / 8
        dN = np.stack([sg[:, 0] * b * c, sg[:, 1] * a * c, sg[:, 2] * a * b], axis=1) / 8
        return N, dN
    if etype == "hexa20":  # element_types.py:155-254
        u, v, w = p
        sg = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                       [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=float)
        N = np.zeros(20)
        dN = np.zeros((20, 3))
        for i in range(8):
            su, sv, sw = sg[i]
            a, b, c = 1 + su * u, 1 + sv * v, 1 + sw * w
            s = su * u + sv * v + sw * w - 2
            N[i] = a * b * c * s / 8
            dN[i] = [su * b * c * s / 8 + a * b * c * su / 8,
                     sv * a * c * s / 8 + a * b * c * sv / 8,
                     sw * a * b * s / 8 + a * b * c * sw / 8]
        # mid-side nodes: (axis along which the node is mid-edge, signs of the other two)
        mids = {8: (0, None, -1, -1), 9: (1, -1, None, -1), 10: (2, -1, -1, None), 11: (1, 1, None, -1),
                12: (2, 1, -1, None), 13: (0, None, 1, -1), 14: (2, 1, 1, None), 15: (2, -1, 1, None),
                16: (0, None, -1, 1), 17: (1, -1, None, 1), 18: (1, 1, None, 1), 19: (0, None, 1, 1)}
        x = np.array([u, v, w])
        for i, (ax, s0, s1, s2) in mids.items():
            sgn = [s0, s1, s2]
            f = [1 - x[k] ** 2 if k == ax else 1 + sgn[k] * x[k] for k in range(3)]
            df = [-2 * x[k] if k == ax else sgn[k] for k in range(3)]
            N[i] = f[0] * f[1] * f[2] / 4
            dN[i] = [df[0] * f[1] * f[2] / 4, f[0] * df[1] * f[2] / 4, f[0] * f[1] * df[2] / 4]
        return N, dN
    if etype == "quad4":  # element_types.py:303-333
        u, v = p
        sg = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], dtype=float)
        a, b = 1 + sg[:, 0] * u, 1 + sg[:, 1] * v
        return a * b / 4, np.stack([sg[:, 0] * b, sg[:, 1] * a], axis=1) / 4
    if etype == "quad8":  # element_types.py:382-424 (serendipity corners are bilinear there)
        u, v = p
        sg = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], dtype=float)
        a, b = 1 + sg[:, 0] * u, 1 + sg[:, 1] * v
        N = np.zeros(8)
        dN = np.zeros((8, 2))
        N[:4] = a * b / 4
        dN[:4] = np.stack([sg[:, 0] * b, sg[:, 1] * a], axis=1) / 4
        N[4], dN[4] = (1 - u * u) * (1 - v) / 2, [-u * (1 - v), -(1 - u * u) / 2]
        N[5], dN[5] = (1 + u) * (1 - v * v) / 2, [(1 - v * v) / 2, -v * (1 + u)]
        N[6], dN[6] = (1 - u * u) * (1 + v) / 2, [-u * (1 + v), (1 - u * u) / 2]
        N[7], dN[7] = (1 - u) * (1 - v * v) / 2, [-(1 - v * v) / 2, -v * (1 - u)]
        return N, dN
    if etype == "tri3":  # element_types.py:475-501
        u, v = p
        return np.array([1 - u - v, u, v]), np.array([[-1.0, -1.0], [1.0, 0.0], [0.0, 1.0]])
    if etype == "tri6":  # element_types.py:552-587 (dN[0,0] and dN[0,1] as written there)
        u, v = p
        L = 1 - u - v
        N = np.array([(2 * L - 1) * L, (2 * u - 1) * u, (2 * v - 1) * v, 4 * L * u, 4 * u * v, 4 * L * v])
        dN = np.array([[1 - 4 * L, 1 - 4 * L], [4 * u - 1, 0], [0, 4 * v - 1],
                       [4 * L - 4 * u, -4 * u], [4 * v, 4 * u], [-4 * v, 4 * L - 4 * v]], dtype=float)
        return N, dN
    if etype == "tetra4":  # element_types.py:646-683
        u, v, w = p
        return (np.array([1 - u - v - w, u, v, w]),
                np.array([[-1.0, -1, -1], [1, 0, 0], [0, 1, 0], [0, 0, 1]]))
    if etype == "tetra10":  # element_types.py:742-802
        u, v, w = p
        L = 1 - u - v - w
        N = np.array([(2 * L - 1) * L, (2 * u - 1) * u, (2 * v - 1) * v, (2 * w - 1) * w,
                      4 * u * L, 4 * u * v, 4 * v * L, 4 * w * L, 4 * v * w, 4 * u * w])
        d0 = 4 * u + 4 * v + 4 * w - 3
        dN = np.array([[d0, d0, d0], [4 * u - 1, 0, 0], [0, 4 * v - 1, 0], [0, 0, 4 * w - 1],
                       [4 * L - 4 * u, -4 * u, -4 * u], [4 * v, 4 * u, 0], [-4 * v, 4 * L - 4 * v, -4 * v],
                       [-4 * w, -4 * w, 4 * L - 4 * w], [0, 4 * w, 4 * v], [4 * w, 0, 4 * u]], dtype=float)
        return N, dN
    raise ValueError(etype)


def tables(etype, order):
    """N [ng, n], dN [ng, n, d], W [ng] at the Gauss points."""
    P, W = points(etype, order)
    Ns, dNs = zip(*[shape(etype, p) for p in P])
    return np.array(Ns), np.array(dNs), W


def d_matrix(E, nu, dim):
    """Isotropic elastic D, per element: material_models.py:5-43.  Returns [E, 6|3, 6|3]."""
    E = np.atleast_1d(np.asarray(E, dtype=float))
    nu = np.atleast_1d(np.asarray(nu, dtype=float)) * np.ones_like(E)
    f = E / ((1 + nu) * (1 - 2 * nu))
    if dim == 3:
        D = np.zeros((len(E), 6, 6))
        for i in range(3):
            for j in range(3):
                D[:, i, j] = np.where(i == j, 1 - nu, nu)
            D[:, 3 + i, 3 + i] = (1 - 2 * nu) / 2
    else:
        D = np.zeros((len(E), 3, 3))
        D[:, 0, 0] = D[:, 1, 1] = 1 - nu
        D[:, 0, 1] = D[:, 1, 0] = nu
        D[:, 2, 2] = (1 - 2 * nu) / 2
    return D * f[:, None, None]


def geometry(etype, xyz, order):
    """detJ [E, ng] and global derivatives [E, ng, n, d]; discretisation.py:107-137, :361-373."""
    N, dN, W = tables(etype, order)
    d = DIM[etype]
    X = np.asarray(xyz, dtype=float)[:, :, :d]
    J = np.einsum("gnd,enk->egkd", dN, X)  # J[e,g,k,d] = sum_n x_k dN/dxi_d  (= (dN^T X)^T)
    detJ = np.linalg.det(J)
    Jinv = np.linalg.inv(J)
    dNx = np.einsum("gnd,egdk->egnk", dN, Jinv)
    return N, dNx, detJ, W


def b_matrix(dNx):
    """Strain-displacement B [E, ng, 6|3, d*n]; discretisation.py:139-158 (3D), :375-392 (2D)."""
    E, G, n, d = dNx.shape
    if d == 3:
        B = np.zeros((E, G, 6, 3 * n))
        B[:, :, 0, 0::3] = dNx[..., 0]
        B[:, :, 1, 1::3] = dNx[..., 1]
        B[:, :, 2, 2::3] = dNx[..., 2]
        B[:, :, 3, 0::3] = dNx[..., 1]
        B[:, :, 3, 1::3] = dNx[..., 0]
        B[:, :, 4, 1::3] = dNx[..., 2]
        B[:, :, 4, 2::3] = dNx[..., 1]
        B[:, :, 5, 0::3] = dNx[..., 2]
        B[:, :, 5, 2::3] = dNx[..., 0]
    else:
        B = np.zeros((E, G, 3, 2 * n))
        B[:, :, 0, 0::2] = dNx[..., 0]
        B[:, :, 1, 1::2] = dNx[..., 1]
        B[:, :, 2, 0::2] = dNx[..., 1]
        B[:, :, 2, 1::2] = dNx[..., 0]
    return B


def element_matrices(etype, xyz, E, nu, rho, order=2):
    """Ke, Me [E, d*n, d*n]: Ke = sum_g B^T D B detJ w (discretisation.py:177-201, :394-408),
    Me = rho sum_g N^T N detJ w, consistent (discretisation.py:203-222, :410-418)."""
    N, dNx, detJ, W = geometry(etype, xyz, order)
    d = DIM[etype]
    n = N.shape[1]
    B = b_matrix(dNx)
    D = d_matrix(E, nu, d)
    dw = detJ * W[None, :]
    Ke = np.einsum("egsi,est,egtj,eg->eij", B, D, B, dw)
    m = np.einsum("ga,gb,eg->eab", N, N, dw) * np.asarray(rho, dtype=float).reshape(-1, 1, 1)
    Me = np.zeros((len(m), d * n, d * n))
    for c in range(d):
        Me[:, c::d, c::d] = m
    return Ke, Me


def face_matrix(ftype, xy, order=2):
    """Scalar face mass F[a, b] = sum_g Na Nb detJ w for 2D faces (discretisation.py:420-433,
    evaluated on the face's in-plane coordinates exactly as given).  xy: [F, n, 2]."""
    N, dNx, detJ, W = geometry(ftype, xy, order)
    return np.einsum("ga,gb,eg->eab", N, N, detJ * W[None, :])
