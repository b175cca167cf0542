"""Mesh reading, boundary planes and equation numbering (host side, vectorised).

Drop-in for scatter/mesher.py ``ReadMesh`` on the path the solver needs: same attributes
and the same numbering, computed with array operations instead of the reference's
O(elements x nodes) loops (mesher.py:312-326, :328-391).

    m = ReadMesh("model.msh"); m.read_gmsh(); m.read_bc(boundaries)
    m.mapping(); m.connectivities(); m.get_mesh_edges()

``ReadMesh.from_arrays`` builds the same object from generated nodes/elements.
"""
import os

import numpy as np

GMSH_TYPES = {2: ("tri3", 2, None, None), 9: ("tri6", 2, None, None), 3: ("quad4", 2, None, None),
              5: ("hexa8", 3, "quad4", 4), 17: ("hexa20", 3, "quad8", 8), 4: ("tetra4", 3, "tri3", 3),
              11: ("tetra10", 3, "tri6", 6)}
HEX8_FACES = np.array([[0, 1, 2, 3], [0, 1, 4, 5], [4, 5, 6, 7], [2, 3, 6, 7], [0, 3, 4, 7], [1, 2, 5, 6]])


def _section(lines, start, end):
    i = next(k for k, s in enumerate(lines) if s.startswith(start))
    j = next(k for k, s in enumerate(lines) if s.startswith(end))
    return lines[i + 2:j]


def define_plane(p1, p2, p3):
    """Plane through three points and the unit normal's absolute components (utils.py:32-59)."""
    p1, p2, p3 = (np.asarray(p, dtype=float) for p in (p1, p2, p3))
    cp = np.cross(p3 - p1, p2 - p1)
    d = np.dot(cp, p3)
    return [cp[0], cp[1], cp[2], d], np.abs(cp / np.linalg.norm(cp))


class ReadMesh:
    def __init__(self, file_name=None):
        if file_name is not None:
            if not os.path.isfile(file_name):
                raise SystemExit("ERROR: Mesh file does not exit.")
            if os.path.splitext(file_name)[-1] != ".msh":
                raise SystemExit("ERROR: Mesh file is not a valid file")
        self.file_name = file_name
        self.nodes = []
        self.elem = []
        self.materials = []
        self.materials_index = []
        self.element_type = None
        self.lower_element_type = None
        self.nb_nodes_lower_elem = None
        self.nb_nodes_elem = None
        self.dimension = 3
        self.BC = self.BC_dir = None
        self.number_eq = 0
        self.type_BC = None
        self.eq_nb_dof = None
        self.eq_nb_elem = None
        self.type_BC_elem = None
        self.boundary_elem = np.zeros((0, 4), dtype=np.int64)

    # ------------------------------------------------------------------ input
    @classmethod
    def from_arrays(cls, nodes, elem, element_type, materials, materials_index):
        """nodes [N, 4] (id, x, y, z), elem [E, n_en] node ids, materials [[dim, id, name]]."""
        m = cls(None)
        m.nodes = np.asarray(nodes, dtype=float)
        m.elem = np.asarray(elem, dtype=np.int64)
        code = {v[0]: k for k, v in GMSH_TYPES.items()}[element_type]
        m._set_type(code)
        m.materials = [list(x) for x in materials]
        m.materials_index = np.asarray(materials_index, dtype=np.int64)
        m.nb_nodes_elem = m.elem.shape[1]
        return m

    def _set_type(self, code):
        et, dim, low, nlow = GMSH_TYPES[code]
        self.element_type, self.dimension = et, dim
        self.lower_element_type = low if low else []
        self.nb_nodes_lower_elem = nlow if nlow else []

    def read_gmsh(self):
        """gmsh 2.2 ASCII reader (mesher.py:55-228); one volume (or 2D) element type."""
        with open(self.file_name) as f:
            lines = f.read().splitlines()
        nodes = np.array([[float(x) for x in s.split()] for s in _section(lines, "$Nodes", "$EndNodes")])
        names = []
        for s in _section(lines, "$PhysicalNames", "$EndPhysicalNames"):
            a, b, c = s.split(maxsplit=2)
            names.append([int(a), int(b), c.replace('"', "")])
        if any(n[2] == "rose" for n in names):
            raise NotImplementedError("ROSE train-track coupling is outside this GPU path")
        elem = [list(map(int, s.split())) for s in _section(lines, "$Elements", "$EndElements")]
        types = {e[1] for e in elem}
        if not all(t in GMSH_TYPES for t in types):
            raise SystemExit("ERROR: Element type not supported")
        if len(types) != 1:
            raise SystemExit("ERROR: mesh mixes element types")
        self._set_type(types.pop())
        arr = np.array(elem, dtype=np.int64)
        self.nodes = nodes
        self.elem = arr[:, 5:]
        self.materials_index = arr[:, 3]
        self.materials = names
        self.nb_nodes_elem = self.elem.shape[1]

    # ------------------------------------------------------------------ boundary conditions
    def read_bc(self, bc):
        """Per-node BC type (0 free, 1 fixed, 2 absorbing) and normal flags (mesher.py:230-274)."""
        n = len(self.nodes)
        self.BC = np.zeros((n, self.dimension), dtype=int)
        self.BC_dir = np.zeros((n, self.dimension), dtype=int)
        X = self.nodes[:, 1:]
        for name in bc:
            typ, pts = bc[name][0], bc[name][1]
            if self.dimension == 3:
                plane, direction = define_plane(pts[0], pts[1], pts[2])
                res = X[:, 0] * plane[0] + X[:, 1] * plane[1] + X[:, 2] * plane[2] - plane[3]
            elif self.dimension == 2:
                p0, p1 = np.asarray(pts[0], dtype=float), np.asarray(pts[1], dtype=float)
                vec = p1 - p0
                direction = np.array([-vec[1], vec[0]])
                dist = lambda p: np.linalg.norm(np.asarray(p)[None, :] - X, axis=1)  # noqa: E731
                res = dist(p0) + dist(p1) - np.linalg.norm(p0 - p1)
            else:
                raise SystemExit(f"ERROR: dimension: {self.dimension}, is  not supported")
            idx = np.where(np.isclose(res, 0.0, atol=1e-5))[0]
            for j, val in enumerate(typ):
                self.BC[idx, j] = np.maximum(self.BC[idx, j], int(val))
                self.BC_dir[idx, j] = np.maximum(self.BC_dir[idx, j], abs(int(direction[j])))

    def mapping(self):
        """Equation numbers node-major, DOF-minor; fixed DOFs NaN (mesher.py:276-310)."""
        if np.any((self.BC < 0) | (self.BC > 2)):
            bad = self.BC[(self.BC < 0) | (self.BC > 2)][0]
            raise SystemExit(f"Error in the boundary condition definition. \n{bad} is not a valid boundary condition.")
        free = (self.BC != 1).ravel()
        eq = np.full(free.shape, np.nan)
        eq[free] = np.arange(int(free.sum()))
        self.eq_nb_dof = eq.reshape(self.BC.shape)
        self.number_eq = int(free.sum())
        tb = np.full(self.BC.shape, "Normal", dtype="<U6")
        tb[self.BC == 1] = "Fixed"
        tb[self.BC == 2] = "Absorb"
        self.type_BC = tb

    def node_index(self):
        ids = self.nodes[:, 0].astype(np.int64)
        id2idx = np.full(int(ids.max()) + 1, -1, dtype=np.int64)
        id2idx[ids] = np.arange(len(ids))
        return id2idx

    def connectivities(self):
        """Per-element equation numbers (mesher.py:312-326), by array gather."""
        idx = self.node_index()[self.elem]
        self.eq_nb_elem = self.eq_nb_dof[idx].reshape(len(self.elem), -1)
        self.type_BC_elem = self.type_BC[idx].reshape(len(self.elem), -1)

    # ------------------------------------------------------------------ surfaces
    def get_mesh_edges(self):
        """Boundary faces of hexa8 meshes as node-id rows (mesher.py:328-391), vectorised.

        As in the reference: boundary nodes are nodes attached to fewer than 8 elements;
        an element with more than 4 boundary nodes contributes each of its 6 surfaces whose
        nodes are all boundary nodes, an element with exactly 4 contributes those 4 nodes in
        element order; rows are then made unique (sorted)."""
        if self.element_type != "hexa8":
            return
        idx = self.node_index()[self.elem]
        count = np.bincount(idx.ravel(), minlength=len(self.nodes))
        bnode = count < 8
        isb = bnode[idx]  # [E, 8]
        nb = isb.sum(axis=1)
        rows = []
        many = np.nonzero(nb > 4)[0]
        if len(many):
            full = isb[many][:, HEX8_FACES].all(axis=2)  # [k, 6]
            e, s = np.nonzero(full)
            rows.append(self.elem[many[e][:, None], HEX8_FACES[s]])
        four = np.nonzero(nb == 4)[0]
        if len(four):
            pos = np.argsort(~isb[four], axis=1, kind="stable")[:, :4]
            rows.append(np.take_along_axis(self.elem[four], pos, axis=1))
        if np.any((nb > 0) & (nb < 4)):
            raise ValueError("hexa8 element touching the boundary with fewer than 4 nodes")
        self.boundary_elem = np.unique(np.concatenate(rows), axis=0) if rows else np.zeros((0, 4), np.int64)

    def get_top_surface(self):
        """Top faces: centroid strictly inside the x/z range and above the lowest (mesher.py:393-424)."""
        eps = 1e-10
        X = self.nodes[:, 1:]
        c = X[self.node_index()[self.boundary_elem]].mean(axis=1)
        keep = ((c[:, 0] > c[:, 0].min() + eps) & (c[:, 0] < c[:, 0].max() - eps) & (c[:, 1] > c[:, 1].min() + eps)
                & (c[:, 2] > c[:, 2].min() + eps) & (c[:, 2] < c[:, 2].max() - eps))
        return self.boundary_elem[keep]

    def top_nodes(self):
        """Node ids on the highest y plane."""
        y = self.nodes[:, 2]
        return self.nodes[np.isclose(y, y.max()), 0].astype(np.int64)
