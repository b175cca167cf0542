"""Small seeded inversion case shared by the adjoint tests: a 3 x 2 x 2 hexa8 box at 0.5 m
with Lysmer dashpots on sides and base, Rayleigh damping, a Ricker point load on a top node,
receivers on the top face, per-element E and rho perturbed around two layers."""
import numpy as np
import scipy.sparse as sp

DT, N_STEPS, CHECKPOINT = 1e-4, 80, 24  # 80 = 3 x 24 + 8: a ragged last segment
DAMPING = [1, 0.02, 200, 0.02]
ABSORBING, K_DIV = [1, 1], 1e3
MATS = {"lower": {"density": 2000.0, "Young": 150e6, "poisson": 0.25},
        "upper": {"density": 1800.0, "Young": 30e6, "poisson": 0.3}}


def build():
    from scatter_gb300 import meshgen
    from scatter_gb300.force_external import ricker_table
    from scatter_gb300.system_matrix import element_properties

    m = meshgen.box_model(3, 2, 2, 0.5, element="hexa8", layers=[(0.0, "lower"), (0.5, "upper")], bottom="020",
                          x_faces="200", z_faces="002")
    E0, nu, rho0 = element_properties(m, MATS)
    rng = np.random.default_rng(7)
    E = E0 * (1 + 0.2 * rng.uniform(-1, 1, len(E0)))
    rho = rho0 * (1 + 0.1 * rng.uniform(-1, 1, len(rho0)))
    time = np.arange(N_STEPS + 1) * DT
    top = m.top_nodes()
    table = ricker_table(m, int(top[len(top) // 2]), 1e4, 250.0, 3e-3, time, direction=1)
    idx = m.node_index()[top]
    rec_eq = np.asarray(m.eq_nb_dof[idx, 1], dtype=np.int64)
    return m, table, rec_eq, (E, nu, rho), (E0, rho0)


class OracleOps:
    """Per-element unit pieces for oracle.adjoint.Operators, from the oracle's own element
    matrices and Lysmer code (one element at a time)."""

    def __init__(self, m, nu):
        from oracle import elements as el
        from oracle import lysmer

        n_eq, n_el = int(m.number_eq), len(m.elem)
        X = m.nodes[:, 1:][m.node_index()[m.elem]]
        Ke, Me = el.element_matrices("hexa8", X, np.ones(n_el), nu, np.ones(n_el))
        eqs = np.asarray(m.eq_nb_elem, dtype=float)
        self.K1, self.S1, self.C1 = [], [], []
        ml_rows, ml_cols, ml_vals = [], [], []
        mdl = {"nodes": m.nodes, "BC": m.BC, "BC_dir": m.BC_dir, "eq_nb_dof": m.eq_nb_dof, "element_type": "hexa8",
               "number_eq": n_eq}
        for e in range(n_el):
            ok = ~np.isnan(eqs[e])
            q = eqs[e][ok].astype(np.int64)
            k = Ke[e][np.ix_(ok, ok)]
            self.K1.append(sp.csr_matrix((k.ravel(), (np.repeat(q, len(q)), np.tile(q, len(q)))), shape=(n_eq, n_eq)))
            ml = Me[e][np.ix_(ok, ok)].sum(axis=1)
            ml_rows += [e] * len(q)
            ml_cols += list(q)
            ml_vals += list(ml)
            C1, S1 = lysmer.absorbing(dict(mdl, elem=m.elem[e:e + 1]), ([1.0], [nu[e]], [1.0]), ABSORBING, K_DIV)
            self.C1.append(C1)
            self.S1.append(S1)
        self.ml1 = sp.csr_matrix((ml_vals, (ml_rows, ml_cols)), shape=(n_el, n_eq))

    def operators(self):
        from oracle.adjoint import Operators

        return Operators(self.K1, self.S1, self.C1, self.ml1)
