"""The oracle's marginal likelihood against the reference's own checks
(ctests/test_sparse_gp.cpp:102-118, 225-290): the plain form (column-pivoted
QR of Qff + Lambda) and the stable form agree, and the analytic hyperparameter
gradient matches central differences (perturbation 1e-6) of the likelihood
after set_hyperparameters."""
import numpy as np
import pytest

from tests import fixtures


@pytest.fixture(scope="module")
def lm():
    return fixtures.likelihood_model()


def test_plain_and_stable_likelihoods_agree(lm):
    gp = lm["gp"]
    l1 = gp.compute_likelihood()
    assert l1 == pytest.approx(gp.data_fit + gp.complexity_penalty + gp.constant_term,
                               rel=1e-15)
    l2 = gp.compute_likelihood_stable()
    l3 = gp.compute_likelihood_gradient_stable()
    assert abs(l1 - l2) < 1e-12 * abs(l1)
    assert abs(l2 - l3) < 1e-12 * abs(l2)
    assert np.linalg.eigvalsh(gp.Kuu_mat).min() > 1e-3   # well conditioned


def test_gradient_matches_finite_differences(lm):
    gp = lm["gp"]
    h = gp.hyperparameters.copy()
    gp.compute_likelihood_gradient_stable()
    g = gp.likelihood_gradient.copy()
    pert = 1e-6
    for i in range(4):
        vals = []
        for sgn in (1, -1):
            hh = h.copy()
            hh[i] += sgn * pert
            gp.set_hyperparameters(hh)
            vals.append(gp.compute_likelihood_gradient_stable())
        fd = (vals[0] - vals[1]) / (2 * pert)
        assert abs(fd - g[i]) < 1e-5 * abs(g[i]) + 1e-4, (i, fd, g[i])
    gp.set_hyperparameters(h)


def test_two_kernel_gradient_matches_finite_differences():
    """Two kernels (sparse_gp.cpp:775-829 masks each kernel's gradient to its
    own Kuu block and Kuf rows): all five components against central
    differences."""
    gp = fixtures.likelihood_model(second_kernel=(1.5, [3, 3]))["gp"]
    h = gp.hyperparameters.copy()
    assert len(h) == 5
    gp.compute_likelihood_gradient_stable()
    g = gp.likelihood_gradient.copy()
    pert = 1e-6
    for i in range(5):
        vals = []
        for sgn in (1, -1):
            hh = h.copy()
            hh[i] += sgn * pert
            gp.set_hyperparameters(hh)
            vals.append(gp.compute_likelihood_stable())
        fd = (vals[0] - vals[1]) / (2 * pert)
        assert abs(fd - g[i]) < 1e-5 * abs(g[i]) + 1e-4, (i, fd, g[i])
    gp.set_hyperparameters(h)
