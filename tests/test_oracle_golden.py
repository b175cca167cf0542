"""The oracle (CPU restatement) against the reference's own golden vectors.

Pins the oracle before it is trusted as the checker of the CUDA path: element
matrices, assembled K/M/C, absorbing-boundary matrices and force tables produced by
the reference's code (tests/golden/make_golden.py), and the reference's shipped time
histories.
"""
import numpy as np
import pytest

from helpers import case, full_field, golden_csr, golden_load_table, npz, oracle_system, pattern_hash, rel_l2
from oracle import elements as el
from oracle import loads, newmark
from oracle.assembly import rayleigh_coefficients

ETYPES = ["hexa8", "hexa20", "tetra4", "tetra10", "quad4", "tri3", "tri6"]
CASES = ["column_hexa8_pulse", "column_hexa8_abs", "column_hexa20_pulse", "column_hexa20_abs", "quad4_2d",
         "tri3_bench2", "tri6_bench2", "tetra4_bench2", "tetra10_bench2", "tetra4_abs", "tetra10_abs", "cube_abs5",
         "cube_moving"]


@pytest.mark.parametrize("etype", ETYPES)
def test_element_matrices(etype):
    d = npz(f"elem_{etype}.npz")
    n = len(d["Ke"])
    Ke, Me = el.element_matrices(etype, d["xyz"], np.full(n, float(d["E"])), np.full(n, float(d["nu"])),
                                 np.full(n, float(d["rho"])))
    assert np.abs(Ke - d["Ke"]).max() <= 1e-13 * np.abs(d["Ke"]).max()
    assert np.abs(Me - d["Me"]).max() <= 1e-13 * np.abs(d["Me"]).max()


def test_quad8_and_third_order_rules():
    d = npz("elem_quad8.npz")
    for i, o in enumerate(d["orders"]):
        Ke, Me = el.element_matrices("quad8", d["xyz"][None], [float(d["E"])], [float(d["nu"])], [float(d["rho"])],
                                     order=int(o))
        F = el.face_matrix("quad8", d["xyz"][None], int(o))
        assert np.abs(Ke[0] - d["Ke"][i]).max() <= 1e-13 * np.abs(d["Ke"][i]).max()
        assert np.abs(Me[0] - d["Me"][i]).max() <= 1e-13 * np.abs(d["Me"][i]).max()
        assert np.abs(np.kron(F[0], np.eye(2)) - d["Fabs"][i]).max() <= 1e-15


@pytest.mark.parametrize("name", CASES)
def test_assembly_lysmer_rayleigh(name):
    model, spec, M, C, K, Ca, Ka = oracle_system(name)
    g = npz(f"mat_{name}.npz")
    # M keeps the element-graph pattern: bit-exact
    assert pattern_hash(M) == str(g["M_hash"])
    # absorbing parts: pattern and values
    if "Cabs_hash" in g.files:
        assert pattern_hash(Ca) == str(g["Cabs_hash"])
        gC, gK = golden_csr(g, "Cabs"), golden_csr(g, "Kabs")
        if gC.nnz:
            assert abs(Ca - gC).max() <= 1e-14 * abs(gC).max()
            assert abs(Ka - gK).max() <= 1e-14 * abs(gK).max()
    for key, X in (("K", K), ("M", M), ("C", C)):
        ref = golden_csr(g, key)
        if ref is not None:
            assert abs(X - ref).max() <= 1e-13 * abs(ref).max()
        diag = g[key + "_diag"]
        scale = max(np.abs(diag).max(), 1e-300)
        assert np.abs(X.diagonal() - diag).max() <= 1e-13 * scale
        absum = float(g[key + "_absum"])
        if absum == 0.0:
            assert not np.any(X.data)
        else:
            assert abs(np.abs(X.data).sum() / absum - 1) <= 1e-12


@pytest.mark.parametrize("name", ["column_hexa8_pulse", "column_hexa8_abs", "quad4_2d", "tri3_bench2",
                                  "tetra10_bench2", "cube_moving", "cube_plane"])
def test_force_tables(name):
    model, spec = case(name)
    load = dict(spec["load"])
    time = loads.time_grid(load["time"], spec["dt"])
    top = model.get("boundary_elem")
    if load["type"] == "moving_at_plane":
        top = _top_surface(model)
    F = loads.table(load, time, model, top)
    Fg, tg = golden_load_table(name)
    np.testing.assert_array_equal(time, tg)
    assert np.abs(F - Fg).max() <= 1e-12 * max(np.abs(Fg).max(), 1)


def _top_surface(model):
    """mesher.get_top_surface (scatter/mesher.py:393-424) on the golden boundary elements."""
    be = model["boundary_elem"]
    c = model["nodes"][:, 1:][be - 1].mean(axis=1)
    eps = 1e-10
    keep = ((c[:, 0] > c[:, 0].min() + eps) & (c[:, 0] < c[:, 0].max() - eps) & (c[:, 1] > c[:, 1].min() + eps)
            & (c[:, 2] > c[:, 2].min() + eps) & (c[:, 2] < c[:, 2].max() - eps))
    return be[keep]


@pytest.mark.parametrize("name", ["tri3_bench2", "tri6_bench2", "tetra4_bench2", "tetra10_bench2"])
def test_newmark_benchmark_set_2(name):
    """integration_tests/test_benchmark_set_2.py fixtures (node 3, y)."""
    model, spec, M, C, K, _, _ = oracle_system(name)
    load = dict(spec["load"])
    time = loads.time_grid(load["time"], spec["dt"])
    F = loads.table(load, time, model)
    U, V, A, _ = newmark.solve(M, C, K, F, time, 1)
    h = npz(f"hist_{name}.npz")
    idx = np.where(model["nodes"][:, 0].astype(int) == 3)[0][0]
    e = int(model["eq_nb_dof"][idx, 1])
    assert rel_l2(U[:, e], h["dis_y"]) <= 1e-10
    assert rel_l2(V[:, e], h["vel_y"]) <= 1e-10


def test_newmark_quad4_all_nodes():
    """integration_tests/results_mean_2d/data.pickle: every node, u, v, a."""
    model, spec, M, C, K, _, _ = oracle_system("quad4_2d")
    load = dict(spec["load"])
    time = loads.time_grid(load["time"], spec["dt"])
    U, V, A, _ = newmark.solve(M, C, K, loads.table(load, time, model), time, 1)
    h = npz("hist_quad4_2d.npz")
    ids = model["nodes"][:, 0].astype(int)
    sel = [np.where(ids == n)[0][0] for n in h["nodes"]]
    for X, key in ((U, "dis"), (V, "vel"), (A, "acc")):
        assert rel_l2(full_field(X, model["eq_nb_dof"])[:, sel], h[key]) <= 1e-10


def test_newmark_hexa8_vtk_series():
    """integration_tests/results_mean/VTK (hexa8 column, pulse, 1001 steps)."""
    model, spec, M, C, K, _, _ = oracle_system("column_hexa8_pulse")
    load = dict(spec["load"])
    time = loads.time_grid(load["time"], spec["dt"])
    U, V, A, _ = newmark.solve(M, C, K, loads.table(load, time, model), time, 1)
    h = npz("hist_column_hexa8_pulse.npz")
    ids = model["nodes"][:, 0].astype(int)
    sel = [np.where(ids == n)[0][0] for n in h["nodes"]]
    Uf, Vf = full_field(U, model["eq_nb_dof"]), full_field(V, model["eq_nb_dof"])
    assert rel_l2(Uf[:, sel], h["dis"]) <= 1e-10
    assert rel_l2(Vf[:, sel], h["vel"]) <= 1e-10
    assert rel_l2(Uf[1000], h["dis_all_1000"]) <= 1e-10
    assert rel_l2(Vf[250], h["vel_all_250"]) <= 1e-10


def test_rayleigh_closed_form():
    """unit_test/test_gen_matrix.py:13-60."""
    f1, d1, f2, d2 = 1, 0.01, 30, 0.01
    a, b = rayleigh_coefficients([f1, d1, f2, d2])
    a_ref = (4 * d2 * f1 ** 2 * f2 - 4 * d1 * f1 * f2 ** 2) * np.pi / (f1 ** 2 - f2 ** 2)
    b_ref = (d1 * f1 - d2 * f2) / ((f1 ** 2 - f2 ** 2) * np.pi)
    assert abs(a - a_ref) <= 1e-12 * abs(a_ref)
    assert abs(b - b_ref) <= 1e-12 * abs(b_ref)
    with pytest.raises(SystemExit):
        rayleigh_coefficients([1, 0.01, 1, 0.01])


def test_tetra10_lysmer_indefinite():
    """The reference's tetra10 dashpot matrix (tri6 faces with its face-node ordering) is
    indefinite, unlike the tetra4 and hexa8 ones; with the singular tetra10 consistent mass of
    its 4-point rule, the Newmark matrix M + dt/2 C + dt^2/4 K is then indefinite and the time
    loop diverges in the reference as well as here.  Pinned on the reference's own matrices."""
    import scipy.linalg as la

    def min_eig(name):
        C = golden_csr(npz(f"mat_{name}.npz"), "Cabs").toarray()
        return la.eigvalsh(0.5 * (C + C.T))[0], np.abs(C).max()

    lo, scale = min_eig("tetra10_abs")
    assert lo < -0.1 * scale
    for name in ("tetra4_abs", "column_hexa8_abs"):
        lo, scale = min_eig(name)
        assert lo >= -1e-12 * scale
    # the oracle's own tetra10 dashpot matrix is the same one
    model, spec, M, C, K, Ca, Ka = oracle_system("tetra10_abs")
    assert abs(Ca - golden_csr(npz("mat_tetra10_abs.npz"), "Cabs")).max() <= 1e-14 * abs(Ca).max()
