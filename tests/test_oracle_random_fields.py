"""The random-field restatement (oracle/random_fields.py) against the covariance model the
reference asks gstools for (scatter/random_fields.py:59-120: Gaussian model, anisotropic
lengths, log-normal transform of :73-77).  gstools itself is absent, so this checks the model's
statistics, not gstools' bits: the log-field's mean and spread, and its correlation
exp(-(pi/4)(r/l)^2) along each axis with that axis's length."""
import numpy as np

from oracle import random_fields as orf

R, N = 512, 64
LENGTHS = (5.0, 2.0, 1.0)
MEAN, SD = 50e6, 12.5e6


def _log_fields():
    # origin, then one correlation length along x, y, z, then 1 m along x
    pts = np.array([[0, 0, 0], [5, 0, 0], [0, 2, 0], [0, 0, 1], [1, 0, 0]], dtype=float)
    return np.log(orf.lognormal_field(pts, 2024, R, N, LENGTHS, MEAN, SD))  # [5, R]


def test_lognormal_parameters():
    mu, sig = orf.lognormal_params(MEAN, SD)
    # the transform's own identities: E[exp(g)] = mean, sd[exp(g)] = sd
    assert np.isclose(np.exp(mu + sig ** 2 / 2), MEAN, rtol=1e-14)
    assert np.isclose(np.sqrt(np.exp(sig ** 2) - 1) * np.exp(mu + sig ** 2 / 2), SD, rtol=1e-12)


def test_field_statistics_and_anisotropic_correlation():
    g = _log_fields()
    mu, sig = orf.lognormal_params(MEAN, SD)
    # one point over the realisations: the mean and the spread of the log-field
    assert abs(g[0].mean() - mu) <= 4 * sig / np.sqrt(R)
    assert abs(g[0].std() / sig - 1) <= 0.1
    # correlation at one correlation length along each axis: exp(-pi/4); standard error of a
    # correlation near 0.46 over 512 samples is about 0.035
    for k in (1, 2, 3):
        rho = np.corrcoef(g[0], g[k])[0, 1]
        assert abs(rho - np.exp(-np.pi / 4)) <= 0.1, k
    # 1 m along x is a fifth of that axis's length
    rho = np.corrcoef(g[0], g[4])[0, 1]
    assert abs(rho - np.exp(-np.pi / 4 / 25)) <= 0.03


def test_fields_are_reproducible_and_independent_across_realisations():
    pts = np.array([[0.3, 1.1, -0.7]])
    a = orf.lognormal_field(pts, 99, 4, 16, LENGTHS, MEAN, SD)
    b = orf.lognormal_field(pts, 99, 4, 16, LENGTHS, MEAN, SD)
    np.testing.assert_array_equal(a, b)
    c = orf.lognormal_field(pts, 100, 4, 16, LENGTHS, MEAN, SD)
    assert not np.any(a == c)
    # realisation r depends only on (seed, r): the first 2 of 4 equal a 2-realisation draw
    d = orf.lognormal_field(pts, 99, 2, 16, LENGTHS, MEAN, SD)
    np.testing.assert_array_equal(a[:, :2], d)
