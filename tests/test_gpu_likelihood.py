"""The marginal likelihood and its hyperparameter gradient on the GPU
(fpp_likelihood_gradient_stable through SparseGP) against the oracle on the
same training set, and against central differences of the GPU's own
likelihood after set_hyperparameters (the check of
ctests/test_sparse_gp.cpp:225-290)."""
import numpy as np
import pytest

import flare_pp_gb300 as fg
from tests import fixtures

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pair():
    lm = fixtures.likelihood_model()
    ogp = lm["gp"]
    b2 = fg.B2("chebyshev", "quadratic", [0.0, lm["rc"]], [], [2, 4, 2])
    gp = fg.SparseGP([fg.NormalizedDotProduct(2.0, 2)], 1.0, 2.0, 3.0)
    frames = []
    for k, of in enumerate(ogp.training_structures):
        s = fg.Structure(of.cell, of.species, of.positions, lm["rc"], [b2])
        s.energy, s.forces, s.stresses = of.energy, of.forces, of.stresses
        gp.add_training_structure(s, [0, 3, 5] if k == 1 else (-1,))
        frames.append(s)
    for k, atoms in enumerate(ogp.sparse_indices[0]):
        gp.add_specific_environments(frames[k], atoms)
    gp.update_matrices_QR()
    return gp, ogp


def test_likelihood_and_gradient_match_oracle(gpu_lib, pair):
    gp, ogp = pair
    np.testing.assert_array_equal(gp.label_kind, ogp.label_kind)
    ref = ogp.compute_likelihood_stable()
    got = gp.compute_likelihood_stable()
    assert abs(got - ref) < 1e-9 * abs(ref)
    ref = ogp.compute_likelihood_gradient_stable()
    got = gp.compute_likelihood_gradient_stable()
    assert abs(got - ref) < 1e-9 * abs(ref)
    for a, b, name in ((gp.data_fit, ogp.data_fit, "data fit"),
                       (gp.complexity_penalty, ogp.complexity_penalty, "complexity")):
        assert abs(a - b) < 1e-9 * max(abs(b), 1.0), name
    np.testing.assert_allclose(gp.likelihood_gradient, ogp.likelihood_gradient,
                               rtol=1e-7, atol=0)


def test_gradient_matches_finite_differences(gpu_lib, pair):
    gp, _ = pair
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


def test_KnK_and_errors(gpu_lib, pair):
    from flare_pp_gb300._lib import FlareGpuError
    gp, _ = pair
    KnK = gp.compute_KnK()
    for t in range(3):
        one = (gp.label_kind == t).astype(float)
        ref = gp.Kuf @ (one[:, None] * gp.Kuf.T)
        np.testing.assert_allclose(KnK[t], ref, rtol=0, atol=1e-12 * max(np.abs(ref).max(), 1))
    gp.precompute_KnK()
    np.testing.assert_allclose(gp.Kuf_e_noise_Kfu[0] * 2.0 ** 4, KnK[0], rtol=1e-15)
    saved = gp.energy_noise
    gp.energy_noise = 0.0
    with pytest.raises(FlareGpuError, match="non-zero"):
        gp.compute_likelihood_stable()
    gp.energy_noise = saved
