"""The random-field restatement (oracle/random_fields.py) against the covariance model the
reference asks gstools for (scatter/random_fields.py:59-120: Gaussian model, anisotropic
lengths, log-normal transform of :73-77).  gstools itself is absent, so this checks the model's
statistics, not gstools' bits: the log-field's mean and spread, and its correlation
exp(-(pi/4)(r/l)^2) along each axis with that axis's length."""
import numpy as np
import pytest

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


def _corr_along_axes(model, lengths, rot=None, seed=2024, R=512, N=64, pts=None):
    pts = np.array(pts if pts is not None else [[0, 0, 0], [lengths[0], 0, 0], [0, lengths[1], 0], [0, 0, lengths[2]],
                                                 [2 * lengths[0], 0, 0]], dtype=float)
    g = np.log(orf.lognormal_field(pts, seed, R, N, lengths, MEAN, SD, model=model, rot=rot))
    return [np.corrcoef(g[0], g[k])[0, 1] for k in range(1, len(pts))]


@pytest.mark.parametrize("model", ["Exponential", "Matern"])
def test_other_models_correlation(model):
    """Exponential exp(-h) and Matern (nu = 1) h K_1(h), the other models the reference offers
    (random_fields.py:81-84): correlation at one length along each axis and at two along x."""
    rho = _corr_along_axes(model, LENGTHS)
    want1, want2 = orf.correlation(model, [1.0, 2.0])
    for k in range(3):
        assert abs(rho[k] - want1) <= 0.1, (model, k, rho[k], want1)
    assert abs(rho[3] - want2) <= 0.1, (model, rho[3], want2)


def test_models_have_the_lognormal_marginal():
    mu, sig = orf.lognormal_params(MEAN, SD)
    for model in ("Exponential", "Matern"):
        g = np.log(orf.lognormal_field(np.zeros((1, 3)), 5, 1024, 64, LENGTHS, MEAN, SD, model=model))[0]
        assert abs(g.mean() - mu) <= 4 * sig / np.sqrt(1024), model
        assert abs(g.std() / sig - 1) <= 0.1, model


def test_angles_rotate_the_anisotropy_frame():
    """lengths (6, 1, 1) rotated by pi/2 in the (x, y) plane: the long axis points along y."""
    rot = orf.rotation(3, [np.pi / 2, 0.0, 0.0])
    np.testing.assert_allclose(rot @ [1.0, 0, 0], [0, 1.0, 0], atol=1e-15)
    rho = _corr_along_axes("Gaussian", (6.0, 1.0, 1.0), rot=rot, pts=[[0, 0, 0], [0, 6, 0], [6, 0, 0]])
    assert abs(rho[0] - np.exp(-np.pi / 4)) <= 0.1
    assert abs(rho[1]) <= 0.1
    # 2D: one angle, in the (x, y) plane
    np.testing.assert_allclose(orf.rotation(2, 0.4), orf.rotation(3, [0.4, 0, 0]))


def test_gamma_draws_have_the_gamma_moments():
    for a in (0.5, 1.0, 2.5):
        g = np.array([orf.gamma_draw(11, 0, j, a) for j in range(4000)])
        assert abs(g.mean() - a) <= 4 * np.sqrt(a / 4000), a
        assert abs(g.var() / a - 1) <= 0.15, a


def test_linear_model_is_refused_beyond_1d(tmp_path):
    from scatter_gb300.random_fields import RF

    props = {"theta": 5, "seed_number": 1, "material": "soil", "key_material": "Young", "std_value": 1e6,
             "aniso_x": 1, "aniso_z": 1, "model_name": "Linear"}
    rf = RF(props, {"soil": {"Young": 1e7, "poisson": 0.3, "density": 1900}}, str(tmp_path), "hexa8")
    with pytest.raises(ValueError, match="1D only"):
        rf.generate_gstools_rf(np.array([[1, 0, 0, 0.0]]), np.array([[1]]), 3)
