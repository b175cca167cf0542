"""Generate the golden fixtures in this folder from the reference implementation.

Run where the reference source tree is present, with ``SCATTER_REF`` naming its
root (the folder that holds ``scatter/`` and ``integration_tests/``)::

    SCATTER_REF=/path/to/scatter python tests/golden/make_golden.py

What it writes (``*.npz``, all small):

* ``mesh_<case>.npz`` -- the reference's own ``ReadMesh`` output for each test
  mesh and boundary set (nodes, elements, BC, BC_dir, equation map ...), so the
  tests can run on a machine without the reference or its ``.msh`` files.
* ``mat_<case>.npz`` -- the reference's assembled K, M, C (CSR) after
  ``generate_stiffness_and_mass``, ``absorbing_boundaries`` and
  ``damping_Rayleigh`` (scatter/system_matrix.py:35-121,166-198,256-376), plus
  the absorbing-boundary parts alone.  ``K_dropped`` / ``C_dropped`` list the
  entries (row * n_eq + col, ascending) of M's pattern -- the element graph --
  that K and C do not store: the reference's scipy additions drop the entries
  whose sums come out exactly 0.0 (system_matrix.py:198,375-376).
* ``elem_<etype>.npz`` -- element Ke, Me from ``VolumeElement`` /
  ``SurfaceElement`` (scatter/discretisation.py:8-433) for a few elements.
* ``load_<case>.npz`` -- the dense force vector per time step from
  ``Force.update_load_at_t`` (scatter/force_external.py:55-349), stored sparse.
* ``hist_<case>.npz`` -- the reference's shipped golden time histories
  (integration_tests/test_data/*.pickle, results_mean_2d/data.pickle and the
  hexa8 ``results_mean/VTK`` series), read with a restricted unpickler.

The reference imports packages that are absent here (rose, PuggleSolvers,
shapely); they are replaced by stub modules that are never exercised on the
paths used, except shapely's Polygon/Point for the ``moving_at_plane`` load,
which gets a small convex-polygon stand-in (hull by angle sort, area centroid,
strict-interior containment -- shapely's published semantics for convex
polygons).  NumPy >= 2.5 rejects the 2D shape functions' (n, 1) ``N`` arrays in
``SurfaceElement.matrix_N`` (scatter/discretisation.py:382); ``N`` is flattened
after ``shape_functions`` for QuadFour/QuadEight/TriThree/TriSix.
"""
import hashlib
import io
import os
import pickle
import sys
import types

import numpy as np
import scipy.sparse as sp

REF = os.environ.get("SCATTER_REF", "")
HERE = os.path.dirname(os.path.abspath(__file__))


# ----------------------------------------------------------------------------- shims
def _install_shims():
    def stub(name, **attrs):
        m = types.ModuleType(name)
        m.__dict__.update(attrs)
        sys.modules[name] = m
        return m

    class _Unused:
        def __init__(self, *a, **k):
            raise RuntimeError("stubbed dependency used")

    class Point:
        def __init__(self, c):
            self.c = np.asarray(c, dtype=float)

    class Polygon:
        """Convex polygon stand-in for shapely (hull, centroid, strict contains)."""

        def __init__(self, pts):
            pts = np.asarray(pts, dtype=float)
            c = pts.mean(axis=0)
            order = np.argsort(np.arctan2(pts[:, 1] - c[1], pts[:, 0] - c[0]))
            self.p = pts[order]

        @property
        def convex_hull(self):
            return self

        @property
        def centroid(self):
            p, q = self.p, np.roll(self.p, -1, axis=0)
            cr = p[:, 0] * q[:, 1] - q[:, 0] * p[:, 1]
            a = cr.sum() / 2
            cx = ((p[:, 0] + q[:, 0]) * cr).sum() / (6 * a)
            cy = ((p[:, 1] + q[:, 1]) * cr).sum() / (6 * a)
            ns = types.SimpleNamespace()
            ns.xy = (np.array([cx]), np.array([cy]))
            return ns

        def contains(self, pt):
            p, q = self.p, np.roll(self.p, -1, axis=0)
            cr = (q[:, 0] - p[:, 0]) * (pt.c[1] - p[:, 1]) - (q[:, 1] - p[:, 1]) * (pt.c[0] - p[:, 0])
            return bool(np.all(cr > 0) or np.all(cr < 0))

    stub("rose")
    stub("rose.model")
    stub("rose.model.model_part", Material=_Unused, Section=_Unused)
    stub("rose.model.train_track_interaction", CoupledTrainTrack=_Unused, List=list)
    stub("rose.pre_process")
    stub("rose.pre_process.default_trains", set_train=_Unused)
    stub("solvers")
    stub("solvers.newmark_solver", NewmarkSolver=_Unused)
    stub("shapely")
    stub("shapely.geometry", Point=Point)
    stub("shapely.geometry.polygon", Polygon=Polygon)
    if REF not in sys.path:
        sys.path.insert(0, REF)

    from scatter import element_types as et

    for cls in (et.QuadFour, et.QuadEight, et.TriThree, et.TriSix):
        orig = cls.shape_functions

        def patched(self, xy, _orig=orig):
            _orig(self, xy)
            self.N = np.asarray(self.N, dtype=float).reshape(-1)

        cls.shape_functions = patched


_install_shims()
from scatter import discretisation, force_external, material_models, mesher, system_matrix, validator  # noqa: E402


class _RestrictedUnpickler(pickle.Unpickler):
    """Only the globals the reference's fixtures use (checked with pickletools)."""

    ALLOWED = {
        ("numpy.core.multiarray", "_reconstruct"): ("numpy._core.multiarray", "_reconstruct"),
        ("numpy._core.multiarray", "_reconstruct"): ("numpy._core.multiarray", "_reconstruct"),
        ("numpy", "ndarray"): ("numpy", "ndarray"),
        ("numpy", "dtype"): ("numpy", "dtype"),
        ("collections", "defaultdict"): ("collections", "defaultdict"),
        ("builtins", "dict"): ("builtins", "dict"),
        ("builtins", "list"): ("builtins", "list"),
    }

    def find_class(self, module, name):
        if (module, name) not in self.ALLOWED:
            raise pickle.UnpicklingError(f"global {module}.{name} not allowed")
        m, n = self.ALLOWED[(module, name)]
        __import__(m)
        return getattr(sys.modules[m], n)


def load_pickle(path):
    with open(path, "rb") as f:
        return _RestrictedUnpickler(io.BytesIO(f.read())).load()


# ----------------------------------------------------------------------------- cases
def bc_column3d(x, y, z, bottom="010"):
    return {"bottom": [bottom, [[0, 0, 0], [x, 0, 0], [0, 0, z], [x, 0, z]]],
            "left": ["100", [[0, 0, 0], [0, 0, z], [0, y, 0], [0, y, z]]],
            "right": ["100", [[x, 0, 0], [x, 0, z], [x, y, 0], [x, y, z]]],
            "front": ["001", [[0, 0, 0], [z, 0, 0], [0, y, 0], [x, y, 0]]],
            "back": ["001", [[0, 0, z], [x, 0, z], [0, y, z], [x, y, z]]]}


def bc_column2d(x, y):
    return {"bottom": ["01", [[0, 0, 0], [x, 0, 0]]],
            "left": ["10", [[0, 0, 0], [0, y, 0]]],
            "right": ["10", [[x, 0, 0], [x, y, 0]]]}


MAT_COLUMN = {"solid": {"density": 1500, "Young": 30e6, "poisson": 0.2},
              "bottom": {"density": 1200, "Young": 300e6, "poisson": 0.25}}
MAT_BENCH2 = {"solid": {"density": 1500, "Young": 30e6, "poisson": 0.0}}
MAT_CUBE = {"solid": {"density": 1500, "Young": 10e6, "poisson": 0.2},
            "bottom": {"density": 1200, "Young": 300e6, "poisson": 0.25}}

BENCH2_NODES = {"tri3": [3, 4, 25], "tri6": [3, 4, 47, 48, 49],
                "tetra4": [3, 4, 7, 8, 29, 69, 91, 92, 132],
                "tetra10": [3, 4, 7, 8, 51, 52, 53, 135, 136, 137, 183, 184, 185, 186, 187, 188,
                            432, 433, 434, 435, 436, 437, 438, 439, 440]}

# name -> (mesh file, boundaries, materials, damping, absorbing, k_div, load, time_step)
CASES = {
    "column_hexa8_pulse": ("column.msh", bc_column3d(0.1, 20, -0.1), MAT_COLUMN, [1, 0.001, 30, 0.001],
                           [1, 1], 1e3, {"force": [0, -1000, 0], "node": [3, 4, 7, 8], "time": 0.5,
                                         "type": "pulse"}, 0.5e-3),
    "column_hexa8_abs": ("column.msh", bc_column3d(0.1, 20, -0.1, "020"), MAT_COLUMN, [1, 0.001, 30, 0.001],
                         [1, 1], 1e3, {"force": [0, -1000, 0], "node": [3, 4, 7, 8], "time": 0.5,
                                       "type": "heaviside"}, 0.5e-3),
    "column_hexa20_pulse": ("column_high_order.msh", bc_column3d(0.1, 20, -0.1), MAT_COLUMN,
                            [1, 0.001, 30, 0.001], [1, 1], 1e3,
                            {"force": [0, -1000, 0], "node": [3, 4, 7, 8], "time": 0.5, "type": "pulse"}, 0.5e-3),
    "column_hexa20_abs": ("column_high_order.msh", bc_column3d(0.1, 20, -0.1, "020"), MAT_COLUMN,
                          [1, 0.001, 30, 0.001], [1, 1], 1e3,
                          {"force": [0, -1000, 0], "node": [3, 4, 7, 8], "time": 0.5, "type": "heaviside"}, 0.5e-3),
    "quad4_2d": ("column_2D.msh", bc_column2d(1, 10), MAT_COLUMN, [1, 0.005, 20, 0.005], [1, 1], 1e3,
                 {"force": [0, -1e6, 0], "node": [3, 4, 25], "time": 1.0, "type": "heaviside"}, 5e-3),
    "cube_moving": ("cube.msh", bc_column3d(10, 10, -10), MAT_CUBE, [1, 0.0, 30, 0.0], [1, 1], 1e3,
                    {"force": [0, -1000, 0], "node": [8], "time": 1, "type": "moving", "speed": 10,
                     "ini_steps": 50}, 0.5e-2),
    "cube_plane": ("cube.msh", bc_column3d(10, 10, -10), MAT_CUBE, [1, 0.0, 30, 0.0], [1, 1], 1e3,
                   {"force": [0, -1000, 0], "start_coord": [0.5, -0.5], "time": 1, "type": "moving_at_plane",
                    "direction": [0.5, -1], "speed": 10, "ini_steps": 50}, 0.5e-2),
}
for _et, _nodes in BENCH2_NODES.items():
    _nd = 2 if _et.startswith("tri") else 3
    _bc = bc_column2d(1, 10) if _nd == 2 else bc_column3d(1, 10, -1)
    CASES[f"{_et}_bench2"] = (f"column_{_nd}D_{_et}.msh", _bc, MAT_BENCH2, [1, 0.001, 30, 0.001], [1, 1], 1e3,
                              {"force": [0, 1000 / len(_nodes), 0], "node": list(_nodes), "time": 1,
                               "type": "heaviside"}, 5e-4)
# absorbing boundaries on the quadratic / simplex 3D elements (matrix level only)
for _et in ("tetra4", "tetra10"):
    CASES[f"{_et}_abs"] = (f"column_3D_{_et}.msh", bc_column3d(1, 10, -1, "020"), MAT_BENCH2,
                           [1, 0.001, 30, 0.001], [1, 1], 1e3,
                           {"force": [0, 1000, 0], "node": [3], "time": 0.01, "type": "heaviside"}, 5e-4)
# absorbing on five faces of the 10x10x10 cube (matrix level)
CASES["cube_abs5"] = ("cube.msh", {"bottom": ["020", [[0, 0, 0], [10, 0, 0], [0, 0, -10], [10, 0, -10]]],
                                   "left": ["200", [[0, 0, 0], [0, 0, -10], [0, 10, 0], [0, 10, -10]]],
                                   "right": ["200", [[10, 0, 0], [10, 0, -10], [10, 10, 0], [10, 10, -10]]],
                                   "front": ["002", [[0, 0, 0], [10, 0, 0], [0, 10, 0], [10, 10, 0]]],
                                   "back": ["002", [[0, 0, -10], [10, 0, -10], [0, 10, -10], [10, 10, -10]]]},
                      MAT_CUBE, [1, 0.02, 50, 0.02], [1, 1], 1e3,
                      {"force": [0, -1000, 0], "node": [8], "time": 0.05, "type": "heaviside"}, 0.5e-2)

# cases whose full K/M/C go into the fixture (the rest store pattern hashes + checksums)
FULL_MATRICES = {"column_hexa8_pulse", "column_hexa8_abs", "column_hexa20_pulse", "column_hexa20_abs",
                 "quad4_2d", "tri3_bench2", "tri6_bench2", "tetra4_bench2", "tetra4_abs"}


def read_model(mesh_file, boundaries):
    m = mesher.ReadMesh(os.path.join(REF, "integration_tests", "mesh", mesh_file))
    m.read_gmsh()
    m.read_bc(boundaries)
    m.mapping()
    m.connectivities()
    m.get_mesh_edges()
    return m


def pattern_hash(a):
    a = a.tocsr()
    a.sort_indices()
    h = hashlib.sha256()
    h.update(np.asarray(a.indptr, dtype=np.int64).tobytes())
    h.update(np.asarray(a.indices, dtype=np.int64).tobytes())
    return h.hexdigest()


def pattern_keys(a):
    """Stored entries of a sparse matrix as sorted keys row * n + col (int64)."""
    a = sp.csr_matrix(a)
    a.sum_duplicates()
    rows = np.repeat(np.arange(a.shape[0], dtype=np.int64), np.diff(a.indptr))
    return np.sort(rows * a.shape[1] + a.indices.astype(np.int64))


def csr_parts(prefix, a, out, full):
    a = sp.csr_matrix(a)
    a.sort_indices()
    out[prefix + "_shape"] = np.array(a.shape)
    out[prefix + "_nnz"] = np.array(a.nnz)
    out[prefix + "_hash"] = np.array(pattern_hash(a))
    out[prefix + "_absum"] = np.array(np.abs(a.data).sum())
    out[prefix + "_diag"] = a.diagonal()
    if full:
        out[prefix + "_indptr"] = a.indptr.astype(np.int64)
        out[prefix + "_indices"] = a.indices.astype(np.int32)
        out[prefix + "_data"] = a.data


def mesh_arrays(m):
    d = {"nodes": np.asarray(m.nodes, dtype=float), "elem": np.asarray(m.elem, dtype=np.int64),
         "materials_index": np.asarray(m.materials_index, dtype=np.int64),
         "material_names": np.array([str(x[2]) for x in m.materials]),
         "material_ids": np.array([int(x[1]) for x in m.materials]),
         "BC": np.asarray(m.BC), "BC_dir": np.asarray(m.BC_dir),
         "eq_nb_dof": np.asarray(m.eq_nb_dof), "eq_nb_elem": np.asarray(m.eq_nb_elem),
         "number_eq": np.array(m.number_eq), "element_type": np.array(m.element_type),
         "dimension": np.array(m.dimension)}
    if len(m.boundary_elem):
        d["boundary_elem"] = np.asarray(m.boundary_elem, dtype=np.int64)
    return d


def gen_case(name, spec):
    mesh_file, bcs, mats, damping, absorbing, kdiv, load, dt = spec
    m = read_model(mesh_file, bcs)
    out = {"case_" + k: np.array(repr(v)) for k, v in
           dict(mesh=mesh_file, boundaries=bcs, materials=mats, damping=damping, absorbing=absorbing,
                k_div=kdiv, load=load, dt=dt).items()}
    np.savez_compressed(os.path.join(HERE, f"mesh_{name}.npz"), **mesh_arrays(m), **out)

    g = system_matrix.GenerateMatrix(m.number_eq, 2)
    g.generate_stiffness_and_mass(m, mats)
    mats_out = {}
    full = name in FULL_MATRICES
    csr_parts("K0", g.K, mats_out, full)
    csr_parts("M", g.M, mats_out, full)
    if m.dimension == 3:
        # absorbing parts alone: start from empty K and C
        g2 = system_matrix.GenerateMatrix(m.number_eq, 2)
        g2.K = sp.lil_matrix(g.K.shape)
        g2.C = sp.lil_matrix(g.K.shape)
        g2.absorbing_boundaries(m, mats, absorbing, kdiv)
        csr_parts("Cabs", g2.C, mats_out, True)
        csr_parts("Kabs", g2.K, mats_out, True)
        g.absorbing_boundaries(m, mats, absorbing, kdiv)
    g.damping_Rayleigh(damping)
    csr_parts("K", g.K, mats_out, full)
    csr_parts("C", g.C, mats_out, full)
    mkeys = pattern_keys(g.M)
    for key, X in (("K", g.K), ("C", g.C)):
        kept = pattern_keys(X)
        if not np.isin(kept, mkeys).all():
            raise RuntimeError(f"{name}: {key} stores an entry outside M's pattern")
        mats_out[key + "_dropped"] = np.setdiff1d(mkeys, kept)
    np.savez_compressed(os.path.join(HERE, f"mat_{name}.npz"), **mats_out)

    # loads: dense vector per step, stored as COO over (step, eq)
    load = dict(load)
    validator.ValidateLoad.validate(load)
    time = np.linspace(0, load["time"], int(np.ceil(load["time"] / dt) + 1))
    F = force_external.Force()
    top = m.get_top_surface() if load["type"] == "moving_at_plane" else []
    F.initialise_load(load, time, m, None, top_surface_elements=top)
    steps, eqs, vals = [], [], []
    for t in range(len(time)):
        f = np.array(F.update_load_at_t(t), dtype=float)
        nz = np.nonzero(f)[0]
        steps.append(np.full(len(nz), t))
        eqs.append(nz)
        vals.append(f[nz])
    np.savez_compressed(os.path.join(HERE, f"load_{name}.npz"), time=time, step=np.concatenate(steps),
                        eq=np.concatenate(eqs), val=np.concatenate(vals),
                        n_eq=np.array(m.number_eq))
    print(f"{name}: n_eq={m.number_eq} nnzM={g.M.nnz} nnzK={g.K.nnz} steps={len(time)}")


def gen_elements():
    """Element Ke/Me from the reference's VolumeElement/SurfaceElement for a few elements."""
    picks = {"hexa8": ("column.msh", MAT_COLUMN["solid"]), "hexa20": ("column_high_order.msh", MAT_COLUMN["solid"]),
             "tetra4": ("column_3D_tetra4.msh", MAT_COLUMN["solid"]),
             "tetra10": ("column_3D_tetra10.msh", MAT_COLUMN["solid"]),
             "quad4": ("column_2D.msh", MAT_COLUMN["solid"]), "tri3": ("column_2D_tri3.msh", MAT_COLUMN["solid"]),
             "tri6": ("column_2D_tri6.msh", MAT_COLUMN["solid"])}
    for et, (mf, mat) in picks.items():
        m = mesher.ReadMesh(os.path.join(REF, "integration_tests", "mesh", mf))
        m.read_gmsh()
        xyz_all, Ke_all, Me_all = [], [], []
        nodes = {int(n[0]): n[1:] for n in m.nodes}
        for e in m.elem[:4]:
            xyz = np.array([nodes[int(n)] for n in e])
            if m.dimension == 3:
                s = discretisation.VolumeElement(et, 2)
            else:
                s = discretisation.SurfaceElement(et, 2)
            s.generate(xyz)
            D = material_models.stiffness_elasticity(mat["Young"], mat["poisson"], m.dimension)
            Ke_all.append(s.compute_stiffness(D))
            Me_all.append(s.compute_mass(mat["density"]))
            xyz_all.append(xyz)
        np.savez_compressed(os.path.join(HERE, f"elem_{et}.npz"), xyz=np.array(xyz_all), Ke=np.array(Ke_all),
                            Me=np.array(Me_all), E=np.array(mat["Young"]), nu=np.array(mat["poisson"]),
                            rho=np.array(mat["density"]))
    # quad8 has no mesh in the reference: a distorted 8-node quad and the 3-point rule too
    from scatter.element_types import QuadEight  # noqa: F401
    xy = np.array([[0, 0], [1.1, 0.1], [1.2, 1.0], [-0.1, 0.9], [0.55, 0.05], [1.15, 0.55], [0.55, 0.95],
                   [-0.05, 0.45]], dtype=float)
    Ke_all, Me_all, A_all = [], [], []
    for order in (2, 3):
        s = discretisation.SurfaceElement("quad8", order)
        s.generate(np.c_[xy, np.zeros(8)])
        D = material_models.stiffness_elasticity(30e6, 0.2, 2)
        Ke_all.append(s.compute_stiffness(D))
        Me_all.append(s.compute_mass(1500.0))
        A_all.append(s.compute_abs_bound())
    np.savez_compressed(os.path.join(HERE, "elem_quad8.npz"), xyz=xy, Ke=np.array(Ke_all), Me=np.array(Me_all),
                        Fabs=np.array(A_all), orders=np.array([2, 3]), E=np.array(30e6), nu=np.array(0.2),
                        rho=np.array(1500.0))


def gen_histories():
    root = os.path.join(REF, "integration_tests")
    for et in BENCH2_NODES:
        nd = 2 if et.startswith("tri") else 3
        d = load_pickle(os.path.join(root, "test_data", f"column_{nd}D_{et}.pickle"))
        np.savez_compressed(os.path.join(HERE, f"hist_{et}_bench2.npz"), time=np.asarray(d["time"]),
                            node=np.array(3), dis_y=np.asarray(d["displacement"]["3"]["y"]),
                            vel_y=np.asarray(d["velocity"]["3"]["y"]))
    d = load_pickle(os.path.join(root, "results_mean_2d", "data.pickle"))
    nodes = [int(n) for n in d["nodes"]]
    out = {"time": np.asarray(d["time"]), "nodes": np.array(nodes)}
    for key, short in (("displacement", "dis"), ("velocity", "vel"), ("acceleration", "acc")):
        out[short] = np.stack([np.stack([np.asarray(d[key][str(n)][c]) for c in ("x", "y")], axis=-1)
                               for n in nodes], axis=1)  # [n_t, n_nodes, 2]
    np.savez_compressed(os.path.join(HERE, "hist_quad4_2d.npz"), **out)

    # hexa8 column, pulse load: VTK series data_0..data_1000 (ASCII doubles)
    vtk_dir = os.path.join(root, "results_mean", "VTK")
    n_files = len([f for f in os.listdir(vtk_dir) if f.endswith(".vtk")])
    keep = np.array([3, 4, 7, 8] + list(range(20, 804, 49)))  # node ids (1-based)
    dis = np.zeros((n_files, len(keep), 3))
    vel = np.zeros((n_files, len(keep), 3))
    snaps = {}
    for i in range(n_files):
        with open(os.path.join(vtk_dir, f"data_{i}.vtk")) as f:
            lines = f.read().splitlines()
        i_d = lines.index("VECTORS displacement double")
        i_v = lines.index("VECTORS velocity double")
        n_pts = int(lines[4].split()[1])
        D = np.array([[float(x) for x in lines[i_d + 1 + k].split()] for k in range(n_pts)])
        V = np.array([[float(x) for x in lines[i_v + 1 + k].split()] for k in range(n_pts)])
        dis[i] = D[keep - 1]
        vel[i] = V[keep - 1]
        if i in (250, 1000):
            snaps[f"dis_all_{i}"] = D
            snaps[f"vel_all_{i}"] = V
    np.savez_compressed(os.path.join(HERE, "hist_column_hexa8_pulse.npz"), nodes=keep, dis=dis, vel=vel,
                        dt=np.array(0.5e-3), n_steps=np.array(n_files), **snaps)


if __name__ == "__main__":
    if not REF or not os.path.isdir(os.path.join(REF, "scatter")):
        raise SystemExit("set SCATTER_REF to the reference source tree (the folder holding scatter/)")
    gen_elements()
    for name, spec in CASES.items():
        gen_case(name, spec)
    gen_histories()
