"""Structured meshes for the benchmark configurations (hexa8 boxes, tetra10 from split hexes).

Axes follow the reference meshes: y vertical (0 at the base, up), x along the box, z into
-z (0 to -Lz).  Hexa8 node order gives detJ > 0 (u -> +x, v -> +y, w -> +z), as
scatter/element_types.py expects.  Node ids are 1-based with x fastest, then z, then y.
Meshes can be written as gmsh 2.2 ASCII so the reference's reader can load them too.
"""
import itertools

import numpy as np

from .mesher import ReadMesh


def box_nodes(nx, ny, nz, h):
    i, k, j = np.meshgrid(np.arange(nx + 1), np.arange(nz + 1), np.arange(ny + 1), indexing="ij")
    # order: x fastest, then z, then y
    I = np.transpose(i, (2, 1, 0)).ravel()
    K = np.transpose(k, (2, 1, 0)).ravel()
    J = np.transpose(j, (2, 1, 0)).ravel()
    xyz = np.stack([I * h, J * h, -K * h], axis=1).astype(float)
    ids = np.arange(1, len(xyz) + 1)
    return np.c_[ids, xyz], (nx + 1, nz + 1, ny + 1)


def _nid(i, j, k, nx, nz):
    return 1 + i + (nx + 1) * (k + (nz + 1) * j)


def box_hexa8(nx, ny, nz, h):
    nodes, _ = box_nodes(nx, ny, nz, h)
    i, j, k = (a.ravel() for a in np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"))
    # element order: x fastest, then z, then y (matches the node order's locality)
    o = np.lexsort((i, k, j))
    i, j, k = i[o], j[o], k[o]
    f = lambda a, b, c: _nid(a, b, c, nx, nz)  # noqa: E731
    elem = np.stack([f(i, j, k + 1), f(i + 1, j, k + 1), f(i + 1, j + 1, k + 1), f(i, j + 1, k + 1),
                     f(i, j, k), f(i + 1, j, k), f(i + 1, j + 1, k), f(i, j + 1, k)], axis=1)
    centroid_y = (j + 0.5) * h
    return nodes, elem, centroid_y


def box_tetra10(nx, ny, nz, h):
    """Each hexa8 split into 6 tetrahedra along its main diagonal (conforming), with mid-side
    nodes shared between neighbours; gmsh tetra10 node order with detJ > 0."""
    nodes, elem8, cy8 = box_hexa8(nx, ny, nz, h)
    X = nodes[:, 1:]
    # cube corner (a,b,c) in {0,1}^3 -> hexa8 local index with u->x, v->y, w->z
    corner = {(0, 0, 0): 0, (1, 0, 0): 1, (1, 1, 0): 2, (0, 1, 0): 3, (0, 0, 1): 4, (1, 0, 1): 5, (1, 1, 1): 6,
              (0, 1, 1): 7}
    paths = []
    for perm in itertools.permutations(range(3)):
        p = [0, 0, 0]
        seq = [corner[tuple(p)]]
        for ax in perm:
            p[ax] = 1
            seq.append(corner[tuple(p)])
        paths.append(seq)
    tets = elem8[:, paths].reshape(-1, 4)  # [E*6, 4] node ids
    cy = np.repeat(cy8, 6)
    P = X[tets - 1]
    det = np.einsum("ij,ij->i", np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0]), P[:, 3] - P[:, 0])
    flip = det < 0
    tets[flip, 1], tets[flip, 2] = tets[flip, 2].copy(), tets[flip, 1].copy()
    edges = [(0, 1), (1, 2), (0, 2), (0, 3), (2, 3), (1, 3)]  # tetra10 nodes 4..9 (element_types.py:719-741)
    pairs = np.stack([np.sort(tets[:, list(e)], axis=1) for e in edges], axis=1).reshape(-1, 2)
    uniq, inv = np.unique(pairs, axis=0, return_inverse=True)
    mid_ids = len(nodes) + 1 + np.arange(len(uniq))
    mid_xyz = 0.5 * (X[uniq[:, 0] - 1] + X[uniq[:, 1] - 1])
    nodes = np.r_[nodes, np.c_[mid_ids, mid_xyz]]
    elem = np.c_[tets, mid_ids[inv.ravel()].reshape(-1, 6)]
    return nodes, elem, cy


def box_planes(Lx, Ly, Lz):
    """Boundary plane points for the six faces of [0,Lx] x [0,Ly] x [-Lz,0]."""
    z = -Lz
    return {"bottom": [[0, 0, 0], [Lx, 0, 0], [0, 0, z], [Lx, 0, z]],
            "top": [[0, Ly, 0], [Lx, Ly, 0], [0, Ly, z], [Lx, Ly, z]],
            "left": [[0, 0, 0], [0, 0, z], [0, Ly, 0], [0, Ly, z]],
            "right": [[Lx, 0, 0], [Lx, 0, z], [Lx, Ly, 0], [Lx, Ly, z]],
            "front": [[0, 0, 0], [Lx, 0, 0], [0, Ly, 0], [Lx, Ly, 0]],
            "back": [[0, 0, z], [Lx, 0, z], [0, Ly, z], [Lx, Ly, z]]}


def box_boundaries(Lx, Ly, Lz, bottom="111", x_faces="100", z_faces="001"):
    P = box_planes(Lx, Ly, Lz)
    return {"bottom": [bottom, P["bottom"]], "left": [x_faces, P["left"]], "right": [x_faces, P["right"]],
            "front": [z_faces, P["front"]], "back": [z_faces, P["back"]]}


def box_model(nx, ny, nz, h, element="hexa8", layers=None, bottom="111", x_faces="100", z_faces="001"):
    """ReadMesh-equivalent model of a structured box with BCs applied and equations numbered.

    layers: list of (y_min, name) -- elements whose centroid y >= y_min get ``name``
    (checked in order, last match wins); default one material "solid"."""
    if element == "hexa8":
        nodes, elem, cy = box_hexa8(nx, ny, nz, h)
    elif element == "tetra10":
        nodes, elem, cy = box_tetra10(nx, ny, nz, h)
    else:
        raise ValueError(element)
    names = ["solid"] if not layers else [n for _, n in layers]
    mid = np.ones(len(elem), dtype=np.int64)
    if layers:
        for k, (ymin, _) in enumerate(layers):
            mid[cy >= ymin] = k + 1
    materials = [[3, k + 1, n] for k, n in enumerate(names)]
    m = ReadMesh.from_arrays(nodes, elem, element, materials, mid)
    Lx, Ly, Lz = nx * h, ny * h, nz * h
    m.read_bc(box_boundaries(Lx, Ly, Lz, bottom, x_faces, z_faces))
    m.mapping()
    m.connectivities()
    m.get_mesh_edges()
    m.dims = (nx, ny, nz, h)
    return m


def column_model(nx=2, ny=20, nz=2, h=0.5, bottom="111"):
    return box_model(nx, ny, nz, h, bottom=bottom)


def write_gmsh(path, model):
    """gmsh 2.2 ASCII (the layout scatter/mesher.py:55-228 reads)."""
    code = {"hexa8": 5, "hexa20": 17, "tetra4": 4, "tetra10": 11, "quad4": 3, "tri3": 2, "tri6": 9}[model.element_type]
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$PhysicalNames\n")
        f.write(f"{len(model.materials)}\n")
        for dim, i, n in model.materials:
            f.write(f'{dim} {i} "{n}"\n')
        f.write("$EndPhysicalNames\n$Nodes\n")
        f.write(f"{len(model.nodes)}\n")
        for r in model.nodes:
            f.write(f"{int(r[0])} {float(r[1])!r} {float(r[2])!r} {float(r[3])!r}\n")
        f.write("$EndNodes\n$Elements\n")
        f.write(f"{len(model.elem)}\n")
        for k, (e, mi) in enumerate(zip(model.elem, model.materials_index)):
            f.write(f"{k + 1} {code} 2 {int(mi)} 1 " + " ".join(str(int(x)) for x in e) + "\n")
        f.write("$EndElements\n")
