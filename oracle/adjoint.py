"""Discrete adjoint of the explicit lumped-mass scheme (oracle; test infrastructure only).

The reference has no adjoint; this is the FP64 CPU restatement the GPU adjoint is checked
against (and which is itself checked against central finite differences).

Model, per element e with parameters (E_e, rho_e) and fixed Poisson ratio:
    K   = sum_e E_e K1_e + sum_faces E_e S1_f          (elastic + Lysmer springs)
    M_L = sum_e rho_e ml1_e                            (row-sum lumped unit mass)
    Cab = sum_faces sqrt(rho_e E_e) C1_f                (Lysmer dashpots: rho v_p = sqrt(rho E E_c1))
    D   = beta K + Cab + alpha M_L
Forward (explicit.py): v_{n+1} = v_n + dt M_L^-1 (f_n - K u_n - D v_n), u_{n+1} = u_n + dt v_{n+1}.
Misfit J = 1/2 sum_{n=1..N} |P v_n - d_n|^2 (P picks the receiver equations).
Backward, with g = mu_v + dt mu_u and y = M_L^-1 g (K, Cab symmetric):
    mu_u <- mu_u - dt K y
    mu_v <- g - dt D y + P^T (P v_n - d_n)
    dJ/dE_e   += -dt y^T [dK/dE_e (u_n + beta v_n) + dCab/dE_e v_n]
    dJ/drho_e += -dt y^T [ml1_e (a_n + alpha v_n) + dCab/drho_e v_n]
"""
import numpy as np
import scipy.sparse as sp


class Operators:
    """Parameter-dependent operators from per-element pieces (all eq-space)."""

    def __init__(self, K1, S1, C1, ml1, elem_of_face_entries=None):
        # K1: list of sparse matrices per element (unit E); S1, C1: per-element sparse (faces of
        # that element summed); ml1: [n_elem, n_eq] sparse rows -> lumped unit mass per element
        self.K1, self.S1, self.C1, self.ml1 = K1, S1, C1, ml1

    def build(self, E, rho):
        K = sum(E[e] * (self.K1[e] + self.S1[e]) for e in range(len(E)))
        Cab = sum(np.sqrt(rho[e] * E[e]) * self.C1[e] for e in range(len(E)))
        ml = np.asarray((self.ml1.T @ rho)).ravel()
        return sp.csr_matrix(K), sp.csr_matrix(Cab), ml


def forward(ops, E, rho, alpha, beta, F, dt, n_steps, rec, store=False):
    K, Cab, ml = ops.build(E, rho)
    n = K.shape[0]
    u = np.zeros(n)
    v = np.zeros(n)
    U, V, A = [u.copy()], [v.copy()], []
    Vr = [v[rec].copy()]
    for t in range(n_steps):
        a = (F[t] - K @ (u + beta * v) - Cab @ v - alpha * ml * v) / ml
        v = v + dt * a
        u = u + dt * v
        Vr.append(v[rec].copy())
        if store:
            U.append(u.copy())
            V.append(v.copy())
            A.append(a.copy())
    return np.array(Vr), (U, V, A, K, Cab, ml)


def misfit(Vr, d):
    return 0.5 * float(((Vr[1:] - d[1:]) ** 2).sum())


def gradient(ops, E, rho, alpha, beta, F, dt, n_steps, rec, d):
    Vr, (U, V, A, K, Cab, ml) = forward(ops, E, rho, alpha, beta, F, dt, n_steps, rec, store=True)
    J = misfit(Vr, d)
    n = K.shape[0]
    mu_u = np.zeros(n)
    mu_v = np.zeros(n)
    mu_v[rec] += Vr[n_steps] - d[n_steps]
    gE = np.zeros(len(E))
    gr = np.zeros(len(rho))
    for t in range(n_steps - 1, -1, -1):
        g = mu_v + dt * mu_u
        y = g / ml
        u, v, a = U[t], V[t], A[t]
        w = u + beta * v
        for e in range(len(E)):
            dK = ops.K1[e] + ops.S1[e]
            dC = ops.C1[e]
            s = np.sqrt(rho[e] * E[e])
            gE[e] += -dt * (y @ (dK @ w) + y @ (dC @ v) * 0.5 * s / E[e])
            mlr = np.asarray(ops.ml1[e].todense()).ravel()
            gr[e] += -dt * (y @ (mlr * (a + alpha * v)) + y @ (dC @ v) * 0.5 * s / rho[e])
        Ky = K @ y
        mu_u = mu_u - dt * Ky
        mu_v = g - dt * (beta * Ky + Cab @ y + alpha * ml * y)
        if t >= 1:
            mu_v[rec] += V[t][rec] - d[t]
    return J, gE, gr
