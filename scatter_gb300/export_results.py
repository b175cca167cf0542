"""Result export: drop-in for scatter/export_results.py ``Write`` (pickle dict + legacy VTK).

The pickle layout is the reference's (export_results.py:68-141):
``{time, nodes, position, displacement|velocity|acceleration: {node_id: {x, y[, z]: array}}}``
with zeros for fixed DOFs.  VTK files follow the layout of the reference's VTK writer as
seen in its golden files (integration_tests/results_mean/VTK): unstructured grid,
displacement / velocity / boundary_conditions point vectors, material index and material
properties as cell scalars; written by this module (the reference's vtk_tools dependency is
not needed).
"""
import os
import pickle
from collections import defaultdict

import numpy as np

VTK_CELL = {"hexa8": 12, "hexa20": 25, "quad4": 9, "tri3": 5, "tri6": 22, "tetra4": 10, "tetra10": 24}
VTK_ORDER = {"hexa8": list(range(8)), "hexa20": list(range(20)), "quad4": [0, 1, 2, 3], "tri3": [0, 1, 2],
             "tri6": list(range(6)), "tetra4": [0, 1, 2, 3], "tetra10": [0, 1, 2, 3, 4, 5, 6, 7, 9, 8]}


class Write:
    def __init__(self, output_folder, model, materials, numerical):
        os.makedirs(output_folder, exist_ok=True)
        self.output_folder = output_folder
        self.element_type = model.element_type
        self.nodes = np.asarray(model.nodes)[:, 0].astype(int)
        self.eq_nb_dof = np.asarray(model.eq_nb_dof, dtype=float)
        self.coordinates = np.asarray(model.nodes)[:, 1:]
        self.elements = np.asarray(model.elem)[:, VTK_ORDER[model.element_type]] - 1
        self.time = numerical.output_time
        self.dis = numerical.u
        self.vel = numerical.v
        self.acc = numerical.a
        self.mat = model.materials
        self.mat_idx = model.materials_index
        self.materials = materials
        self.bc = np.asarray(model.BC)
        self.n_dim = model.dimension
        self.data = {}
        self.parse_data()

    def parse_data(self):
        """export_results.py:68-103."""
        self.data.update({"time": self.time, "nodes": list(map(int, self.nodes)), "position": self.coordinates,
                          "displacement": defaultdict(dict), "velocity": defaultdict(dict),
                          "acceleration": defaultdict(dict)})
        labels = ["x", "y", "z"][:self.n_dim]
        zeros = np.zeros(len(self.time))
        for i, nid in enumerate(self.nodes):
            for k, lab in enumerate(labels):
                dof = self.eq_nb_dof[i][k]
                if np.isnan(dof):
                    u = v = a = zeros
                else:
                    u, v, a = self.dis[:, int(dof)], self.vel[:, int(dof)], self.acc[:, int(dof)]
                self.data["displacement"][str(int(nid))][lab] = u
                self.data["velocity"][str(int(nid))][lab] = v
                self.data["acceleration"][str(int(nid))][lab] = a

    def pickle(self, name="data", write=True, nodes="all"):
        """export_results.py:105-141."""
        if not write:
            return
        if nodes != "all":
            idx = [self.data["nodes"].index(int(i)) for i in nodes]
            data = {"time": self.data["time"], "nodes": nodes, "position": [self.data["position"][i] for i in idx],
                    "displacement": defaultdict(dict), "velocity": defaultdict(dict),
                    "acceleration": defaultdict(dict)}
            for n in nodes:
                for key in ("displacement", "velocity", "acceleration"):
                    data[key].update({str(n): self.data[key][str(n)]})
        else:
            data = self.data
        with open(os.path.join(self.output_folder, f"{name}.pickle"), "wb") as f:
            pickle.dump(data, f)

    def vtk(self, name="data", binary=True, write=True, output_interval=1):
        """One legacy VTK file per output time (export_results.py:143-213)."""
        if not write:
            return
        props = list(set(tuple(m.keys()) for m in self.materials.values()))[0]
        names = {int(r[1]): r[2] for r in self.mat}
        mat_index = np.asarray(self.mat_idx, dtype=float)
        mat_prop = np.array([[self.materials[names[int(i)]][p] for p in props] for i in self.mat_idx], dtype=float)
        bc = np.zeros((self.bc.shape[0], 3), dtype=self.bc.dtype)
        bc[:, :self.bc.shape[1]] = self.bc
        folder = os.path.join(self.output_folder, "VTK")
        os.makedirs(folder, exist_ok=True)
        n_nodes = len(self.nodes)
        for out_t in range(int(len(self.time) / output_interval)):
            t = int(out_t * output_interval)
            D = np.zeros((n_nodes, 3))
            V = np.zeros((n_nodes, 3))
            for k, lab in enumerate(["x", "y", "z"][:self.n_dim]):
                for i, nid in enumerate(self.nodes):
                    D[i, k] = self.data["displacement"][str(int(nid))][lab][t]
                    V[i, k] = self.data["velocity"][str(int(nid))][lab][t]
            path = os.path.join(folder, f"{name}_{out_t}.vtk")
            _write_vtk(path, f"{name}_{out_t}", binary, self.coordinates, self.elements, VTK_CELL[self.element_type],
                       [("displacement", D), ("velocity", V), ("boundary_conditions", bc)],
                       [("material_index", mat_index)] + [(f"material_prop_{p}", mat_prop[:, j])
                                                          for j, p in enumerate(props)])


def _write_vtk(path, title, binary, X, cells, cell_type, point_vectors, cell_scalars):
    """Legacy VTK unstructured grid; binary blocks are big-endian, as the format requires."""
    n, nc = len(X), len(cells)
    npe = cells.shape[1]
    with open(path, "wb") as f:
        def line(s):
            f.write((s + "\n").encode())

        line("# vtk DataFile Version 2.0")
        line(title)
        line("BINARY" if binary else "ASCII")
        line("DATASET UNSTRUCTURED_GRID")
        line(f"POINTS {n} float")
        if binary:
            f.write(np.asarray(X, dtype=">f4").tobytes())
            line("")
        else:
            for r in X:
                line(" ".join(repr(float(v)) for v in r))
        line(f"CELLS {nc} {nc * (npe + 1)}")
        conn = np.c_[np.full(nc, npe), cells]
        if binary:
            f.write(conn.astype(">i4").tobytes())
            line("")
        else:
            for r in conn:
                line(" ".join(str(int(v)) for v in r))
        line(f"CELL_TYPES {nc}")
        if binary:
            f.write(np.full(nc, cell_type, dtype=">i4").tobytes())
            line("")
        else:
            for _ in range(nc):
                line(str(cell_type))
        line(f"POINT_DATA {n}")
        for name, A in point_vectors:
            integer = np.issubdtype(A.dtype, np.integer)
            line(f"VECTORS {name} double")
            if binary:
                f.write(np.asarray(A, dtype=">f8").tobytes())
                line("")
            else:
                for r in A:
                    line(" ".join(str(int(v)) if integer else repr(float(v)) for v in r))
        line(f"CELL_DATA {nc}")
        for name, a in cell_scalars:
            line(f"SCALARS {name} double")
            line("LOOKUP_TABLE default")
            if binary:
                f.write(np.asarray(a, dtype=">f8").tobytes())
                line("")
            else:
                for v in a:
                    line(repr(float(v)))
