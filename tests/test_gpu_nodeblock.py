"""Node-block operators (sliced-ELL A, K, M, dashpots, FSAI preconditioner) against the
eq-space CSR matrices, and the eager execution mode against the graph mode."""
import os

import numpy as np
import pytest

from helpers import model_ns, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch


def _box(element):
    from scatter_gb300 import meshgen
    from scatter_gb300.system_matrix import GenerateMatrix

    mats = {"lower": {"density": 2000.0, "Young": 150e6, "poisson": 0.25},
            "upper": {"density": 1800.0, "Young": 30e6, "poisson": 0.3}}
    m = meshgen.box_model(6, 4, 4, 0.5, element=element, layers=[(0.0, "lower"), (1.5, "upper")],
                          bottom="020", x_faces="200", z_faces="002")
    g = GenerateMatrix(m.number_eq, 2)
    g.generate_stiffness_and_mass(m, mats)
    g.absorbing_boundaries(m, mats, [1, 1], 1e3)
    g.damping_Rayleigh([1, 0.02, 50, 0.02])
    return g


def _golden(name):
    from scatter_gb300.system_matrix import GenerateMatrix

    ns, model, spec = model_ns(name)
    g = GenerateMatrix(ns.number_eq, 2)
    g.generate_stiffness_and_mass(ns, spec["materials"])
    g.absorbing_boundaries(ns, spec["materials"], spec["absorbing"], spec["k_div"])
    g.damping_Rayleigh(spec["damping"])
    return g


CASES = [("box", "hexa8"), ("box", "tetra10"), ("golden", "column_hexa8_abs"), ("golden", "column_hexa20_abs"),
         ("golden", "tetra4_abs"), ("golden", "quad4_2d"), ("golden", "tri6_bench2")]


@pytest.mark.parametrize("kind,name", CASES)
def test_node_block_operators(cuda, kind, name):
    from scatter_gb300.solvers import NodeBlockNewmark

    g = _box(name) if kind == "box" else _golden(name)
    dt = 5e-5
    s = NodeBlockNewmark(g, dt)
    M, C, K = g.M, g.C, g.K
    A = M + (dt / 2) * C + (dt * dt / 4) * K
    rng = np.random.default_rng(0)
    x = rng.standard_normal(g.n_eq)
    for which, X in (("A", A), ("K", K), ("M", M)):
        y = s.apply(which, x)
        assert rel_l2(y, X @ x) <= 1e-13, which
    if g.Cabs_d is not None:
        Cabs = g.pattern.to_scipy(g.Cabs_d)
        assert rel_l2(s.apply("Cabs", x), Cabs @ x) <= 1e-13
        # Rayleigh structure used by the residual: C = Cabs + alpha M + beta K
        assert rel_l2(Cabs @ x + g.alpha * (M @ x) + g.beta * (K @ x), C @ x) <= 1e-12
    # preconditioner: symmetric positive definite (FP16 factor planes, FP32 products)
    z = rng.standard_normal(g.n_eq)
    Px, Pz = s.apply("P", x), s.apply("P", z)
    assert abs(z @ Px - x @ Pz) <= 1e-5 * abs(x @ Px)
    assert x @ Px > 0
    s.close()


def test_eager_mode_matches_graph_mode(cuda):
    """SCATTER_GB300_EAGER=1 launches the same kernels without a graph: identical bits."""
    from oracle import loads
    from scatter_gb300.solvers import ForceTable, NewmarkExplicit

    g = _golden("tetra4_bench2")
    ns, model, spec = model_ns("tetra4_bench2")
    load = dict(spec["load"])
    time = loads.time_grid(load["time"], spec["dt"])[:200]
    F = loads.table(load, time, model)
    outs = []
    for eager in ("0", "1"):
        os.environ["SCATTER_GB300_EAGER"] = eager
        try:
            s = NewmarkExplicit()
            s.initialise(ns.number_eq, time)
            s.force_table = ForceTable.from_dense(F)
            s.calculate(g, g, g, F[0], 0, len(time) - 1)
            outs.append((s.u.copy(), s.iterations))
        finally:
            os.environ.pop("SCATTER_GB300_EAGER", None)
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    assert outs[0][1] == outs[1][1]


def _ricker_box():
    """Box with Lysmer dashpots, Rayleigh damping and a Ricker point load on the top: a smooth
    load history over 400 steps."""
    from scatter_gb300 import meshgen
    from scatter_gb300.force_external import ricker_table
    from scatter_gb300.system_matrix import GenerateMatrix

    mats = {"lower": {"density": 2000.0, "Young": 150e6, "poisson": 0.25},
            "upper": {"density": 1800.0, "Young": 30e6, "poisson": 0.3}}
    m = meshgen.box_model(10, 6, 6, 0.5, layers=[(0.0, "lower"), (1.5, "upper")], bottom="020", x_faces="200",
                          z_faces="002")
    g = GenerateMatrix(m.number_eq, 2)
    g.generate_stiffness_and_mass(m, mats)
    g.absorbing_boundaries(m, mats, [1, 1], 1e3)
    g.damping_Rayleigh([1, 0.02, 50, 0.02])
    dt, n_t = 5e-5, 401
    time = np.arange(n_t) * dt
    top = m.top_nodes()
    table = ricker_table(m, int(top[len(top) // 2]), -1e4, 40.0, 0.004, time)
    rec = np.asarray([int(m.eq_nb_dof[m.node_index()[n], 1]) for n in top[::3]], dtype=np.int64)
    return g, table, rec, dt, n_t


def _warm_start_runs(make, orders, table, rec, n_t):
    runs = {}
    for order in orders:
        s = make()
        if order:
            s.set_predictor(order)
        s.set_force(table)
        s.set_output(1, rec, n_t, what=("u",))
        s.initial_acceleration()
        s.run(0, n_t - 1)
        rc, iters, _ = s.status()
        assert rc == 0
        runs[order] = (s.outputs()["u"].copy(), iters)
        s.close()
    return runs


def test_warm_start_order_changes_iterations_not_the_answer(cuda):
    """Fixed warm-start orders 1..8 and the adaptive default reach the same displacements
    (the PCG tolerance), and the adaptive order needs fewer PCG iterations than order 2 on a
    smooth load history."""
    from scatter_gb300.solvers import NodeBlockNewmark

    g, table, rec, dt, n_t = _ricker_box()
    runs = _warm_start_runs(lambda: NodeBlockNewmark(g, dt), (0, 1, 2, 4, 6, 8), table, rec, n_t)
    ref = runs[2][0]
    assert np.abs(ref).max() > 0
    for order, (u, _) in runs.items():
        assert rel_l2(u, ref) <= 1e-10, order
    assert runs[0][1] < runs[2][1]


def test_csr_warm_start_order_changes_iterations_not_the_answer(cuda):
    """The CSR loop (scipy matrices, Jacobi-PCG) with the same warm start: every order reaches
    the node-block loop's displacements to the PCG tolerance, and the adaptive order needs
    fewer iterations than the linear extrapolation (order 1)."""
    from scatter_gb300.solvers import NewmarkGPU, NodeBlockNewmark, _device_matrices

    g, table, rec, dt, n_t = _ricker_box()
    pat, Md, Cd, Kd = _device_matrices(g.M, g.C, g.K)
    runs = _warm_start_runs(lambda: NewmarkGPU(pat, Md, Cd, Kd, dt), (0, 1, 2, 4, 8), table, rec, n_t)
    ref = _warm_start_runs(lambda: NodeBlockNewmark(g, dt), (0,), table, rec, n_t)[0][0]
    assert np.abs(ref).max() > 0
    for order, (u, _) in runs.items():
        assert rel_l2(u, ref) <= 1e-10, order
    assert runs[0][1] < runs[1][1]


@pytest.mark.parametrize("residual", ["pair", "fp64"])
def test_residual_arithmetic_and_handover(cuda, residual):
    """The step's residual in pair arithmetic (default) and in FP64 (option), on the small
    column settling under a constant top load with heavy Rayleigh damping: once the elastic
    forces carry the load (slow motion), the pair residual hands over to the FP64 one, and both
    arithmetics reach the oracle's direct solve to 1e-10 (u, v).  A wave step (the first ones)
    stays in pairs."""
    import column_case as cc
    from oracle import assembly as asm
    from oracle import newmark
    from scatter_gb300.solvers import NodeBlockNewmark
    from scatter_gb300.system_matrix import GenerateMatrix

    damping = [1, 0.9, 50, 0.9]
    m, _, _, top_eq = cc.build()
    g = GenerateMatrix(m.number_eq, 2)
    g.generate_stiffness_and_mass(m, cc.MATS)
    g.absorbing_boundaries(m, cc.MATS, [1, 1], 1e3)
    g.damping_Rayleigh(damping)
    dt, n_t = 1e-3, 1500
    time = np.linspace(0, dt * (n_t - 1), n_t)
    from scatter_gb300.force_external import Force

    top = m.top_nodes()
    load = {"type": "heaviside", "force": [0, -cc.P0 / len(top), 0], "node": list(top), "time": time[-1],
            "ini_steps": 5}
    F = Force()
    F.initialise_load(load, time, m, None)
    s = NodeBlockNewmark(g, dt, residual=residual)
    s.set_force(F.table)
    s.set_output(1, np.arange(m.number_eq), n_t)
    s.initial_acceleration()
    s.run(0, 10)
    early = s.residual_fp64()
    s.run(10, n_t - 1)
    rc, _, _ = s.status()
    assert rc == 0
    late = s.residual_fp64()
    out = s.outputs()
    s.close()
    if residual == "pair":
        assert not early and late  # waves first, then the settled column hands over
    else:
        assert early and late
    M, C, K = cc.oracle_matrices(m)
    C = asm.rayleigh(M, K, M * 0, damping)
    Fd = np.stack([F.table.dense(t) for t in range(n_t)])
    U, V, _, _ = newmark.solve(M, C, K, Fd, time, 1)
    assert rel_l2(out["u"], U) <= 1e-10
    assert rel_l2(out["v"], V) <= 1e-10


def test_fp32_matrix_meets_the_tolerance(cuda):
    """The PCG on the FP32 matrix (A's hi parts) stops on |r| + L |x - x0| <= rtol |b|, with L
    a bound on ||A - Ah||_2: every mode reaches the pair-only displacements to the PCG
    tolerance.  'always' starts every step on Ah and restarts the early steps (large r0) in
    pairs; 'auto' starts a step on Ah, or switches to it during the solve, only where the bound
    allows, and needs no restart on this smooth load."""
    from scatter_gb300.solvers import NodeBlockNewmark

    g, table, rec, dt, n_t = _ricker_box()
    out = {}
    for mode in ("never", "auto", "always"):
        s = NodeBlockNewmark(g, dt, fp32_matrix=mode)
        s.set_force(table)
        s.set_output(1, rec, n_t, what=("u",))
        s.initial_acceleration()
        s.run(0, n_t - 1)
        rc, iters, _ = s.status()
        assert rc == 0, mode
        out[mode] = (s.outputs()["u"].copy(), iters, s.fp32_matrix_status())
        s.close()
    ref = out["never"][0]
    assert np.abs(ref).max() > 0
    a32, switched, restarts, lo = out["never"][2]
    assert a32 == 0 and switched == 0 and restarts == 0 and lo > 0
    for mode in ("auto", "always"):
        assert rel_l2(out[mode][0], ref) <= 1e-10, mode
    a32, switched, restarts, _ = out["always"][2]
    assert a32 > 0 and restarts > 0
    a32, switched, restarts, _ = out["auto"][2]
    assert a32 + switched > 0 and restarts == 0


@pytest.mark.parametrize("layout", ["node-block", "csr"])
def test_order_cap_at_a_load_kink(cuda, layout):
    """A heaviside load that ramps over 5 steps: the warm-start order is capped while its window
    straddles the ramp's end, which takes fewer PCG iterations over the first 30 steps, and the
    answer is the uncapped one to the PCG tolerance (both Newmark solvers)."""
    from scatter_gb300 import meshgen
    from scatter_gb300.force_external import Force
    from scatter_gb300.solvers import NewmarkGPU, NodeBlockNewmark, _device_matrices
    from scatter_gb300.system_matrix import GenerateMatrix

    mats = {"lower": {"density": 2000.0, "Young": 150e6, "poisson": 0.25},
            "upper": {"density": 1800.0, "Young": 30e6, "poisson": 0.3}}
    m = meshgen.box_model(10, 6, 6, 0.5, layers=[(0.0, "lower"), (1.5, "upper")], bottom="020", x_faces="200",
                          z_faces="002")
    g = GenerateMatrix(m.number_eq, 2)
    g.generate_stiffness_and_mass(m, mats)
    g.absorbing_boundaries(m, mats, [1, 1], 1e3)
    g.damping_Rayleigh([1, 0.02, 50, 0.02])
    dt, n_t = 5e-5, 31
    time = np.arange(n_t) * dt
    top = m.top_nodes()
    load = {"type": "heaviside", "force": [0, -1e4, 0], "node": [int(top[len(top) // 2])], "time": time[-1],
            "ini_steps": 5}
    F = Force()
    F.initialise_load(load, time, m, None)
    out = {}
    if layout == "csr":
        pat, Md, Cd, Kd = _device_matrices(g.M, g.C, g.K)
    for cap in (True, False):
        if layout == "csr":
            s = NewmarkGPU(pat, Md, Cd, Kd, dt, order_cap=cap)
        else:
            s = NodeBlockNewmark(g, dt, order_cap=cap)
        s.set_force(F.table)
        s.set_output(1, np.arange(m.number_eq), n_t, what=("u",))
        s.initial_acceleration()
        s.run(0, n_t - 1)
        rc, iters, _ = s.status()
        assert rc == 0
        out[cap] = (s.outputs()["u"].copy(), iters, s.warm_start_status()[1])
        s.close()
    assert out[True][2] > 0 and out[False][2] == 0
    assert out[True][1] < out[False][1]
    assert rel_l2(out[True][0], out[False][0]) <= 1e-10
