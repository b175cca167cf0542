"""Random-field restatement (oracle; test infrastructure only).

The reference draws its fields with gstools' SRF (scatter/random_fields.py:59-120; gstools
1.7.0, not installed here), so the generator itself is parity-unpinned.  This restates the
GPU generator's published method -- randomisation (spectral) method for a Gaussian
covariance exp(-(pi/4)|r/l|^2), counter-based splitmix64 normals -- in float64 numpy, and the
reference's log-normal transform (random_fields.py:73-77).
"""
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


def modes(seed, R, N, lengths):
    lx, ly, lz = lengths
    sc = np.sqrt(np.pi / 2.0) / np.array([lx, ly, lz])
    out = np.zeros((R, N, 5))
    for r in range(R):
        for j in range(N):
            n = []
            for p in range(3):
                u1, u2 = uniform01(seed, r, j, 2 * p), uniform01(seed, r, j, 2 * p + 1)
                rad = np.sqrt(-2.0 * np.log(u1))
                n += [rad * np.cos(2 * np.pi * u2), rad * np.sin(2 * np.pi * u2)]
            out[r, j, :3] = np.array(n[:3]) * sc
            out[r, j, 3:] = n[3:5]
    return out


def lognormal_params(mean, sd):
    """random_fields.py:73-75."""
    var = np.log((sd / mean) ** 2 + 1)
    mu = np.log(mean ** 2 / np.sqrt(mean ** 2 + sd ** 2))
    return mu, np.sqrt(var)


def lognormal_field(points, seed, R, N, lengths, mean, sd):
    """[n_points, R] log-normal values."""
    md = modes(seed, R, N, lengths)
    mu, sig = lognormal_params(mean, sd)
    X = np.asarray(points, dtype=float)
    out = np.zeros((len(X), R))
    for r in range(R):
        ph = X @ md[r, :, :3].T
        g = (md[r, :, 3] * np.cos(ph) + md[r, :, 4] * np.sin(ph)).sum(axis=1) * np.sqrt(1.0 / N)
        out[:, r] = np.exp(mu + sig * g)
    return out
