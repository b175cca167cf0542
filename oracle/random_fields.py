"""Random-field restatement (oracle; test infrastructure only).

The reference draws its fields with gstools' SRF (scatter/random_fields.py:59-120; gstools
1.7.0, not installed here), so the generator itself is parity-unpinned.  This restates the
GPU generator's published method in float64 numpy: the randomisation (spectral) method for
the covariance models the reference offers (random_fields.py:79-88) -- Gaussian
exp(-(pi/4) h^2), Exponential exp(-h), Matern(nu) -- with wave vectors drawn from each model's
spectral density (normal, multivariate Cauchy, multivariate t with 2 nu degrees of freedom,
the last through a Marsaglia-Tsang gamma draw), scaled by the axis lengths and rotated by the
`angles` rotation; counter-based splitmix64 uniforms; and the reference's log-normal transform
(random_fields.py:73-77).  The Linear model is refused beyond 1D: the triangular covariance is
not positive definite there, so no Gaussian field in 2D or 3D has it.
"""
import math

import numpy as np

M64 = (1 << 64) - 1


def mix64(z):
    z = (z + 0x9E3779B97F4A7C15) & M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def uniform01(seed, r, j, k):
    h = mix64((seed + 0x632BE59BD9B4E019 * (r + 1)) & M64)
    h = mix64((h + j * 0x9E3779B97F4A7C15 + k) & M64)
    return ((h >> 11) + 0.5) * (1.0 / 9007199254740992.0)


MODELS = {"Gaussian": 0, "Exponential": 1, "Matern": 2}


def normal01(seed, r, j, k):
    u1, u2 = uniform01(seed, r, j, k), uniform01(seed, r, j, k + 1)
    return math.sqrt(-2.0 * math.log(u1)) * math.cos(2 * math.pi * u2)


def gamma_draw(seed, r, j, a):
    """Gamma(a, 1), Marsaglia & Tsang (2000); a < 1 boosted by U^(1/a) (uniform 15); attempt t
    draws its normal from uniforms 16 + 3t, 17 + 3t and its acceptance uniform from 18 + 3t."""
    boost = uniform01(seed, r, j, 15) ** (1.0 / a) if a < 1.0 else 1.0
    aa = a + 1.0 if a < 1.0 else a
    d = aa - 1.0 / 3.0
    c = 1.0 / math.sqrt(9.0 * d)
    g = d
    for t in range(64):
        x = normal01(seed, r, j, 16 + 3 * t)
        v1 = 1.0 + c * x
        if v1 <= 0.0:
            continue
        v = v1 ** 3
        if math.log(uniform01(seed, r, j, 18 + 3 * t)) < 0.5 * x * x + d - d * v + d * math.log(v):
            g = d * v
            break
    return g * boost


def rotation(dim, angles):
    """R with k = R kappa: Givens rotations in the planes (x, y), (x, z), (y, z) in that order
    (the rotation planes of the anisotropy frame, one angle per plane; missing angles are 0),
    embedded in 3D."""
    ang = np.zeros(3)
    a = np.atleast_1d(np.asarray(angles, dtype=float))
    n = dim * (dim - 1) // 2
    ang[:min(n, len(a))] = a[:n]
    Rm = np.eye(3)
    for (i, j), th in zip([(0, 1), (0, 2), (1, 2)], ang):
        G = np.eye(3)
        G[i, i] = G[j, j] = np.cos(th)
        G[i, j], G[j, i] = -np.sin(th), np.sin(th)
        Rm = Rm @ G
    return Rm


def modes(seed, R, N, lengths, model="Gaussian", nu=1.0, rot=None):
    """[R, N, 5]: (k_x, k_y, k_z, Z1, Z2) per realisation and mode."""
    code = MODELS[model]
    il = 1.0 / np.asarray(lengths, dtype=float)
    Rm = np.eye(3) if rot is None else np.asarray(rot, dtype=float)
    out = np.zeros((R, N, 5))
    for r in range(R):
        for j in range(N):
            n = []
            for p in range(3):
                u1, u2 = uniform01(seed, r, j, 2 * p), uniform01(seed, r, j, 2 * p + 1)
                rad = np.sqrt(-2.0 * np.log(u1))
                n += [rad * np.cos(2 * np.pi * u2), rad * np.sin(2 * np.pi * u2)]
            if code == 0:
                scale = np.sqrt(np.pi / 2.0)
            elif code == 1:
                scale = 1.0 / abs(normal01(seed, r, j, 6))
            else:
                scale = np.sqrt(nu / (2.0 * gamma_draw(seed, r, j, nu)))
            out[r, j, :3] = Rm @ (np.array(n[:3]) * scale * il)
            out[r, j, 3:] = n[3:5]
    return out


def correlation(model, h, nu=1.0):
    """The models' correlation at scaled distance h (what the fields' statistics must show)."""
    from scipy.special import gamma, kv

    h = np.asarray(h, dtype=float)
    if model == "Gaussian":
        return np.exp(-np.pi / 4 * h ** 2)
    if model == "Exponential":
        return np.exp(-h)
    s = np.sqrt(nu) * np.maximum(h, 1e-300)
    return np.where(h > 0, 2 ** (1 - nu) / gamma(nu) * s ** nu * kv(nu, s), 1.0)


def lognormal_params(mean, sd):
    """random_fields.py:73-75."""
    var = np.log((sd / mean) ** 2 + 1)
    mu = np.log(mean ** 2 / np.sqrt(mean ** 2 + sd ** 2))
    return mu, np.sqrt(var)


def lognormal_field(points, seed, R, N, lengths, mean, sd, model="Gaussian", nu=1.0, rot=None):
    """[n_points, R] log-normal values."""
    md = modes(seed, R, N, lengths, model, nu, rot)
    mu, sig = lognormal_params(mean, sd)
    X = np.asarray(points, dtype=float)
    out = np.zeros((len(X), R))
    for r in range(R):
        ph = X @ md[r, :, :3].T
        g = (md[r, :, 3] * np.cos(ph) + md[r, :, 4] * np.sin(ph)).sum(axis=1) * np.sqrt(1.0 / N)
        out[:, r] = np.exp(mu + sig * g)
    return out
