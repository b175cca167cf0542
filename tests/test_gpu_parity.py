"""CUDA path against the oracle and the reference's golden vectors (GPU)."""
import numpy as np
import pytest

from helpers import (case, element_coords, element_props, full_field, golden_csr, model_ns, npz, oracle_system,
                     pattern_hash, rel_l2)

pytestmark = pytest.mark.gpu

ETYPES = ["hexa8", "hexa20", "tetra4", "tetra10", "quad4", "tri3", "tri6"]


@pytest.fixture(scope="module")
def torch_cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    from scatter_gb300 import _native

    _native.load()
    return torch


def _element_gpu(torch, etype, xyz, E, nu, rho, order=2):
    from scatter_gb300 import _native as nat
    from scatter_gb300 import device as dv

    n, n_en, dim = xyz.shape
    nd = n_en * dim
    x = dv.to_dev(xyz, torch.float64)
    Ke = dv.empty(n * nd * nd, torch.float64)
    Me = dv.empty(n * nd * nd, torch.float64)
    Ed, nud, rhod = (dv.to_dev(np.asarray(v, dtype=float), torch.float64) for v in (E, nu, rho))
    nat.call("sc_element_matrices", nat.ELEMENT_CODES[etype], order, n, x.data_ptr(), Ed.data_ptr(), nud.data_ptr(),
             rhod.data_ptr(), Ke.data_ptr(), Me.data_ptr(), dv.stream_ptr())
    torch.cuda.synchronize()
    return dv.host(Ke).reshape(n, nd, nd), dv.host(Me).reshape(n, nd, nd)


@pytest.mark.parametrize("etype", ETYPES)
def test_element_matrices_vs_reference(torch_cuda, etype):
    d = npz(f"elem_{etype}.npz")
    n = len(d["Ke"])
    Ke, Me = _element_gpu(torch_cuda, etype, d["xyz"][:, :, :(3 if etype in ("hexa8", "hexa20", "tetra4", "tetra10")
                                                                 else 2)],
                          np.full(n, float(d["E"])), np.full(n, float(d["nu"])), np.full(n, float(d["rho"])))
    assert np.abs(Ke - d["Ke"]).max() <= 1e-13 * np.abs(d["Ke"]).max()
    assert np.abs(Me - d["Me"]).max() <= 1e-13 * np.abs(d["Me"]).max()


@pytest.mark.parametrize("order", [1, 2, 3])
def test_quad8_and_orders_vs_oracle(torch_cuda, order):
    from oracle import elements as el

    d = npz("elem_quad8.npz")
    Ke, Me = _element_gpu(torch_cuda, "quad8", d["xyz"][None], [float(d["E"])], [float(d["nu"])], [float(d["rho"])],
                          order)
    Ko, Mo = el.element_matrices("quad8", d["xyz"][None], [float(d["E"])], [float(d["nu"])], [float(d["rho"])], order)
    assert np.abs(Ke - Ko).max() <= 1e-13 * np.abs(Ko).max()
    assert np.abs(Me - Mo).max() <= 1e-13 * np.abs(Mo).max()


@pytest.mark.parametrize("etype,order", [("hexa8", 1), ("hexa8", 3), ("hexa20", 3), ("tetra4", 1), ("tetra10", 1),
                                         ("tri6", 3), ("tri3", 1), ("quad4", 3)])
def test_other_gauss_orders_vs_oracle(torch_cuda, etype, order):
    from oracle import elements as el

    d = npz(f"elem_{etype}.npz")
    n = len(d["Ke"])
    dim = 3 if etype in ("hexa8", "hexa20", "tetra4", "tetra10") else 2
    xyz = d["xyz"][:, :, :dim]
    args = (np.full(n, float(d["E"])), np.full(n, float(d["nu"])), np.full(n, float(d["rho"])))
    Ke, Me = _element_gpu(torch_cuda, etype, xyz, *args, order=order)
    Ko, Mo = el.element_matrices(etype, xyz, *args, order=order)
    assert np.abs(Ke - Ko).max() <= 1e-13 * np.abs(Ko).max()
    assert np.abs(Me - Mo).max() <= 1e-13 * np.abs(Mo).max()


ASM_CASES = ["column_hexa8_pulse", "column_hexa8_abs", "column_hexa20_pulse", "column_hexa20_abs", "quad4_2d",
             "tri3_bench2", "tri6_bench2", "tetra4_bench2", "tetra10_bench2", "tetra4_abs", "tetra10_abs",
             "cube_abs5", "cube_moving"]


def _gpu_system(name):
    from scatter_gb300.system_matrix import GenerateMatrix

    ns, model, spec = model_ns(name)
    g = GenerateMatrix(ns.number_eq, 2)
    g.generate_stiffness_and_mass(ns, spec["materials"])
    g.absorbing_boundaries(ns, spec["materials"], spec["absorbing"], spec["k_div"])
    g.damping_Rayleigh(spec["damping"])
    return g, ns, model, spec


@pytest.mark.parametrize("name", ASM_CASES)
def test_assembly_vs_reference_and_oracle(torch_cuda, name):
    g, ns, model, spec = _gpu_system(name)
    mats = npz(f"mat_{name}.npz")
    _, _, Mo, Co, Ko, Cao, Kao = oracle_system(name)
    M, K, C = g.M, g.K, g.C
    # pattern: element graph, bit-exact with the reference's M
    assert pattern_hash(M) == str(mats["M_hash"])
    assert pattern_hash(K) == str(mats["M_hash"]) and pattern_hash(C) == str(mats["M_hash"])
    for X, Xo, key in ((M, Mo, "M"), (K, Ko, "K"), (C, Co, "C")):
        scale = max(abs(Xo).max(), 1e-300)
        assert abs(X - Xo).max() <= 1e-13 * scale, key
        ref = golden_csr(mats, key)
        if ref is not None:
            assert abs(X - ref).max() <= 1e-13 * scale, key
            # every stored reference entry is a stored entry here (structural subset)
            r1, o1 = ref.copy(), X.copy()
            r1.data[:] = 1.0
            o1.data[:] = 1.0
            assert (r1 - r1.multiply(o1)).count_nonzero() == 0, key
    if g.Cabs_d is not None and "Cabs_data" in mats.files:
        Cabs = g.pattern.to_scipy(g.Cabs_d)
        Kabs = g.pattern.to_scipy(g.Kabs_d)
        gC, gK = golden_csr(mats, "Cabs"), golden_csr(mats, "Kabs")
        if gC.nnz:
            assert abs(Cabs - gC).max() <= 1e-14 * abs(gC).max()
            assert abs(Kabs / spec["k_div"] - gK).max() <= 1e-14 * abs(gK).max()


def test_assembly_is_deterministic(torch_cuda):
    g1, *_ = _gpu_system("tetra10_bench2")
    g2, *_ = _gpu_system("tetra10_bench2")
    for a, b in ((g1.K_d, g2.K_d), (g1.M_d, g2.M_d), (g1.C_d, g2.C_d)):
        assert torch_cuda.equal(a, b)


def _gpu_history(name, rtol=1e-12, receivers=None):
    from oracle import loads
    from scatter_gb300.solvers import ForceTable, NewmarkExplicit

    g, ns, model, spec = _gpu_system(name)
    load = dict(spec["load"])
    time = loads.time_grid(load["time"], spec["dt"])
    F = loads.table(load, time, model)
    solver = NewmarkExplicit(rtol=rtol)
    solver.output_interval = 1
    solver.initialise(ns.number_eq, time)
    solver.force_table = ForceTable.from_dense(F)
    solver.receivers = receivers
    solver.update(0)
    solver.calculate(g, g, g, F[0], 0, len(time) - 1)
    return solver, model, spec, time, F


@pytest.mark.parametrize("name", ["tri3_bench2", "tri6_bench2", "tetra4_bench2", "tetra10_bench2"])
def test_newmark_vs_benchmark_set_2(torch_cuda, name):
    solver, model, spec, time, F = _gpu_history(name)
    h = npz(f"hist_{name}.npz")
    idx = np.where(model["nodes"][:, 0].astype(int) == 3)[0][0]
    e = int(model["eq_nb_dof"][idx, 1])
    assert rel_l2(solver.u[:, e], h["dis_y"]) <= 1e-10
    assert rel_l2(solver.v[:, e], h["vel_y"]) <= 1e-10


def test_newmark_vs_oracle_full_history(torch_cuda):
    from oracle import newmark

    solver, model, spec, time, F = _gpu_history("column_hexa8_abs")
    _, _, Mo, Co, Ko, _, _ = oracle_system("column_hexa8_abs")
    U, V, A, _ = newmark.solve(Mo, Co, Ko, F, time, 1)
    assert rel_l2(solver.u, U) <= 1e-10
    assert rel_l2(solver.v, V) <= 1e-10
    assert rel_l2(solver.a, A) <= 1e-9


def test_newmark_hexa8_vtk_series(torch_cuda):
    solver, model, spec, time, F = _gpu_history("column_hexa8_pulse")
    h = npz("hist_column_hexa8_pulse.npz")
    ids = model["nodes"][:, 0].astype(int)
    sel = [np.where(ids == n)[0][0] for n in h["nodes"]]
    Uf, Vf = full_field(solver.u, model["eq_nb_dof"]), full_field(solver.v, model["eq_nb_dof"])
    assert rel_l2(Uf[:, sel], h["dis"]) <= 1e-10
    assert rel_l2(Vf[:, sel], h["vel"]) <= 1e-10
    assert rel_l2(Uf[1000], h["dis_all_1000"]) <= 1e-10


def test_newmark_quad4_all_nodes(torch_cuda):
    solver, model, spec, time, F = _gpu_history("quad4_2d")
    h = npz("hist_quad4_2d.npz")
    ids = model["nodes"][:, 0].astype(int)
    sel = [np.where(ids == n)[0][0] for n in h["nodes"]]
    for X, key in ((solver.u, "dis"), (solver.v, "vel"), (solver.a, "acc")):
        assert rel_l2(full_field(X, model["eq_nb_dof"])[:, sel], h[key]) <= 1e-10


def test_newmark_receivers_and_interval(torch_cuda):
    """Receiver subset + output interval give the same rows as the full history."""
    full, *_ = _gpu_history("column_hexa8_pulse")
    rec = np.array([5, 17, 400, 799])
    from oracle import loads
    from scatter_gb300.solvers import ForceTable, NewmarkExplicit

    g, ns, model, spec = _gpu_system("column_hexa8_pulse")
    load = dict(spec["load"])
    time = loads.time_grid(load["time"], spec["dt"])
    F = loads.table(load, time, model)
    s = NewmarkExplicit()
    s.output_interval = 10
    s.initialise(ns.number_eq, time)
    s.force_table = ForceTable.from_dense(F)
    s.receivers = rec
    s.calculate(g, g, g, F[0], 0, len(time) - 1)
    np.testing.assert_array_equal(s.u_rec, full.u[::10][:, rec])
    np.testing.assert_array_equal(s.v_rec, full.v[::10][:, rec])


def test_newmark_not_converged_status(torch_cuda):
    """A CG iteration cap of 1 returns SC_NOT_CONVERGED (status read on the host, no fault)."""
    from scatter_gb300 import _native as nat

    with pytest.raises(nat.ScatterGpuError) as ei:
        from oracle import loads
        from scatter_gb300.solvers import ForceTable, NewmarkExplicit

        g, ns, model, spec = _gpu_system("tetra4_bench2")
        load = dict(spec["load"])
        time = loads.time_grid(load["time"], spec["dt"])[:50]
        F = loads.table(load, time, model)
        s = NewmarkExplicit(max_iter=1)
        s.initialise(ns.number_eq, time)
        s.force_table = ForceTable.from_dense(F)
        s.calculate(g, g, g, F[0], 0, len(time) - 1)
    assert ei.value.code == 2
