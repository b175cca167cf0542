"""The oracle's discrete adjoint (explicit lumped-mass scheme) against central finite
differences of its own forward, and its forward against the oracle's explicit scheme on the
assembled matrices."""
import numpy as np
import pytest

import adjoint_case as case
from oracle import adjoint as adj
from oracle import assembly as asm
from oracle import explicit, lysmer
from oracle.assembly import rayleigh_coefficients


@pytest.fixture(scope="module")
def setup():
    m, table, rec_eq, (E, nu, rho), (E0, rho0) = case.build()
    ops = case.OracleOps(m, nu).operators()
    alpha, beta = rayleigh_coefficients(case.DAMPING)
    F = np.stack([table.dense(t) for t in range(case.N_STEPS + 1)])
    Vr0, _ = adj.forward(ops, E0, rho0, alpha, beta, F, case.DT, case.N_STEPS, rec_eq)
    return m, ops, alpha, beta, F, rec_eq, E, nu, rho, Vr0


def test_unit_pieces_rebuild_the_assembled_system(setup):
    """sum_e E_e (K1 + S1), sqrt(rho E) C1 and rho ml1 equal the assembled K, Lysmer C and
    row-sum lumped M, and the adjoint's forward equals the explicit scheme."""
    from oracle import elements as el

    m, ops, alpha, beta, F, rec_eq, E, nu, rho, _ = setup
    K, Cab, ml = ops.build(E, rho)
    X = m.nodes[:, 1:][m.node_index()[m.elem]]
    Ke, Me = el.element_matrices("hexa8", X, E, nu, rho)
    pairs = asm.element_pairs(m.eq_nb_elem)
    mdl = {"nodes": m.nodes, "elem": m.elem, "BC": m.BC, "BC_dir": m.BC_dir, "eq_nb_dof": m.eq_nb_dof,
           "element_type": "hexa8", "number_eq": m.number_eq}
    Ca, Ka = lysmer.absorbing(mdl, (E, nu, rho), case.ABSORBING, case.K_DIV)
    Kf = asm.assemble(m.eq_nb_elem, Ke, m.number_eq, pairs) + Ka
    Mf = asm.assemble(m.eq_nb_elem, Me, m.number_eq, pairs)
    assert abs(K - Kf).max() <= 1e-12 * abs(Kf).max()
    assert abs(Cab - Ca).max() <= 1e-12 * abs(Ca).max()
    assert np.abs(ml - explicit.lumped(Mf)).max() <= 1e-12 * ml.max()
    Vr, _ = adj.forward(ops, E, rho, alpha, beta, F, case.DT, case.N_STEPS, rec_eq)
    _, V = explicit.solve(Mf, Ca, Kf, alpha, beta, F, case.N_STEPS + 1, case.DT, rec=rec_eq)
    assert np.abs(Vr - V).max() <= 1e-12 * np.abs(V).max()


def test_gradient_matches_central_differences(setup):
    m, ops, alpha, beta, F, rec_eq, E, nu, rho, Vr0 = setup
    J, gE, gR = adj.gradient(ops, E, rho, alpha, beta, F, case.DT, case.N_STEPS, rec_eq, Vr0)
    assert J > 0

    def J_at(Ep, rp):
        Vr, _ = adj.forward(ops, Ep, rp, alpha, beta, F, case.DT, case.N_STEPS, rec_eq)
        return adj.misfit(Vr, Vr0)

    rng = np.random.default_rng(3)
    for kind in ("E", "rho", "both"):
        dE = rng.standard_normal(len(E)) * E if kind != "rho" else np.zeros(len(E))
        dR = rng.standard_normal(len(E)) * rho if kind != "E" else np.zeros(len(E))
        h = 1e-6
        fd = (J_at(E + h * dE, rho + h * dR) - J_at(E - h * dE, rho - h * dR)) / (2 * h)
        an = gE @ dE + gR @ dR
        assert abs(fd - an) <= 1e-6 * abs(an), (kind, fd, an)
    # one element at a time for E (every entry of the gradient, not only projections)
    for e in range(len(E)):
        d = np.zeros(len(E))
        d[e] = 1e-6 * E[e]
        fd = (J_at(E + d, rho) - J_at(E - d, rho)) / (2 * d[e])
        assert abs(fd - gE[e]) <= 1e-5 * np.abs(gE).max(), (e, fd, gE[e])
