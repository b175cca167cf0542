"""Result export (scatter_gb300/export_results.py) against the reference's formats: the pickle
dict of export_results.py:68-141, and the legacy VTK files of its shipped
integration_tests/results_mean/VTK series (hexa8 column).  Every node's displacement and
velocity at output 1000 of that series are committed golden values: written back out here, they
must come out at the same place in the same layout."""
import pickle
from types import SimpleNamespace

import numpy as np

from helpers import model_ns, npz

N_PTS, N_CELLS = 804, 200
# the section lines of the reference's files (data lines left out); the title is the file name
REF_SECTIONS = ["# vtk DataFile Version 2.0", "{title}", "ASCII", "DATASET UNSTRUCTURED_GRID",
                f"POINTS {N_PTS} float", f"CELLS {N_CELLS} {N_CELLS * 9}", f"CELL_TYPES {N_CELLS}",
                f"POINT_DATA {N_PTS}", "VECTORS displacement double", "VECTORS velocity double",
                "VECTORS boundary_conditions double", f"CELL_DATA {N_CELLS}", "SCALARS material_index double",
                "LOOKUP_TABLE default", "SCALARS material_prop_density double", "LOOKUP_TABLE default",
                "SCALARS material_prop_Young double", "LOOKUP_TABLE default", "SCALARS material_prop_poisson double",
                "LOOKUP_TABLE default"]


def _writer(tmp_path):
    """Write() over the column mesh with two outputs: zeros, then the golden output-1000 state
    (accelerations: a ramp over the equations)."""
    from scatter_gb300.export_results import Write

    ns, model, spec = model_ns("column_hexa8_pulse")
    h = npz("hist_column_hexa8_pulse.npz")
    eq = model["eq_nb_dof"]
    free = ~np.isnan(eq)
    n_eq = model["number_eq"]
    U, V, A = np.zeros((2, n_eq)), np.zeros((2, n_eq)), np.zeros((2, n_eq))
    U[1, eq[free].astype(int)] = h["dis_all_1000"][free]
    V[1, eq[free].astype(int)] = h["vel_all_1000"][free]
    A[1] = np.arange(n_eq) * 1e-3
    num = SimpleNamespace(output_time=np.array([0.0, 1000 * float(h["dt"])]), u=U, v=V, a=A)
    return Write(str(tmp_path), ns, spec["materials"], num), model, h


def _is_number(tok):
    try:
        float(tok)
        return True
    except ValueError:
        return False


def test_vtk_ascii_layout_and_values(tmp_path):
    w, model, h = _writer(tmp_path)
    assert np.all(h["dis_all_1000"][np.isnan(model["eq_nb_dof"])] == 0)
    w.vtk(binary=False)
    lines = (tmp_path / "VTK" / "data_1.vtk").read_text().splitlines()
    sections = [s for s in lines if s and not _is_number(s.split()[0])]
    assert sections == [s.format(title="data_1") for s in REF_SECTIONS]

    def block(header, n):
        i = lines.index(header)
        return np.array([[float(x) for x in lines[i + 1 + k].split()] for k in range(n)])

    np.testing.assert_array_equal(block("VECTORS displacement double", N_PTS), h["dis_all_1000"])
    np.testing.assert_array_equal(block("VECTORS velocity double", N_PTS), h["vel_all_1000"])
    np.testing.assert_array_equal(block("VECTORS boundary_conditions double", N_PTS), model["BC"])
    np.testing.assert_array_equal(block(f"POINTS {N_PTS} float", N_PTS), model["nodes"][:, 1:])
    cells = block(f"CELLS {N_CELLS} {N_CELLS * 9}", N_CELLS)
    np.testing.assert_array_equal(cells[:, 0], 8)
    np.testing.assert_array_equal(cells[:, 1:], model["elem"] - 1)
    np.testing.assert_array_equal(block(f"CELL_TYPES {N_CELLS}", N_CELLS)[:, 0], 12)
    first = (tmp_path / "VTK" / "data_0.vtk").read_text().splitlines()
    i = first.index("VECTORS displacement double")
    assert all(float(x) == 0.0 for k in range(N_PTS) for x in first[i + 1 + k].split())


def test_vtk_binary_matches_ascii(tmp_path):
    w, model, h = _writer(tmp_path)
    w.vtk(binary=True)
    b = (tmp_path / "VTK" / "data_1.vtk").read_bytes()

    def block(header, n, dtype):
        i = b.index(header.encode() + b"\n") + len(header) + 1
        return np.frombuffer(b[i:i + n * np.dtype(dtype).itemsize], dtype=dtype)

    assert b.split(b"\n")[2] == b"BINARY"
    np.testing.assert_array_equal(block("VECTORS displacement double", 3 * N_PTS, ">f8").reshape(-1, 3),
                                  h["dis_all_1000"])
    np.testing.assert_array_equal(block("VECTORS velocity double", 3 * N_PTS, ">f8").reshape(-1, 3),
                                  h["vel_all_1000"])
    np.testing.assert_array_equal(block(f"POINTS {N_PTS} float", 3 * N_PTS, ">f4").reshape(-1, 3),
                                  model["nodes"][:, 1:].astype(np.float32))
    conn = block(f"CELLS {N_CELLS} {N_CELLS * 9}", 9 * N_CELLS, ">i4").reshape(-1, 9)
    np.testing.assert_array_equal(conn[:, 1:], model["elem"] - 1)


def test_pickle_dict(tmp_path):
    w, model, h = _writer(tmp_path)
    w.pickle()
    with open(tmp_path / "data.pickle", "rb") as f:
        d = pickle.load(f)
    assert set(d) == {"time", "nodes", "position", "displacement", "velocity", "acceleration"}
    ids = model["nodes"][:, 0].astype(int)
    assert d["nodes"] == ids.tolist()
    np.testing.assert_array_equal(d["position"], model["nodes"][:, 1:])
    eq = model["eq_nb_dof"]
    for i, nid in enumerate(ids):
        for k, lab in enumerate("xyz"):
            got = d["displacement"][str(nid)][lab]
            want = np.zeros(2) if np.isnan(eq[i, k]) else w.dis[:, int(eq[i, k])]
            np.testing.assert_array_equal(got, want)
            assert got[1] == h["dis_all_1000"][i, k]
            a = d["acceleration"][str(nid)][lab]
            assert a[1] == (0.0 if np.isnan(eq[i, k]) else int(eq[i, k]) * 1e-3)
    # a subset of nodes keeps the same layout
    w.pickle(name="sub", nodes=[3, 8])
    with open(tmp_path / "sub.pickle", "rb") as f:
        s = pickle.load(f)
    assert s["nodes"] == [3, 8] and set(s["velocity"]) == {"3", "8"}
    np.testing.assert_array_equal(np.asarray(s["position"]), model["nodes"][[2, 7], 1:])
    np.testing.assert_array_equal(s["velocity"]["8"]["y"], d["velocity"]["8"]["y"])
