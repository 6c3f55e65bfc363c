"""SparseGP with two kernels over two descriptors (sparse_gp.h:48-49: a B2
and a B3 NormalizedDotProduct kernel, as ctests/test_sparse_gp.cpp fits):
per-kernel sparse sets, Kuu block diagonal over the kernels, Kuf rows
stacked, the QR solve, and every prediction summing the kernels' parts,
against the oracle's multi-kernel SparseGP."""
import numpy as np
import pytest

import flare_pp_gb300 as fg
from flare_pp_gb300 import synth
from oracle.b2 import B2 as OB2
from oracle.b3 import B3 as OB3
from oracle.geometry import Structure as OStructure
from oracle.kernel import NormalizedDotProduct as ONDP
from oracle.sparse_gp import SparseGP as OSGP

pytestmark = pytest.mark.gpu

RC = 5.0
HYPS = [(2.0, 2), (1.5, 2)]


def _descriptors():
    ob = [OB2("chebyshev", "quadratic", [0, RC], [], [2, 5, 3]),
          OB3("chebyshev", "quadratic", [0, RC], [], [2, 3, 2])]
    gb = [fg.B2("chebyshev", "quadratic", [0, RC], [], [2, 5, 3]),
          fg.B3("chebyshev", "quadratic", [0, RC], [], [2, 3, 2])]
    return ob, gb


@pytest.fixture(scope="module")
def trained():
    ob, gb = _descriptors()
    ogp = OSGP([ONDP(s, p) for s, p in HYPS], 0.001, 0.05, 0.006)
    ggp = fg.SparseGP([fg.NormalizedDotProduct(s, p) for s, p in HYPS], 0.001, 0.05, 0.006)
    cells = synth.fcc_batch(n_structures=4, seed=505, lo=24, hi=48)
    rng = np.random.default_rng(12)
    for k, (cell, sp, pos) in enumerate(cells):
        e, f, st, _ = synth.lennard_jones(cell, pos)
        os_ = OStructure(cell, sp, pos, RC, ob)
        gs = fg.Structure(cell, sp, pos, RC, gb)
        for s in (os_, gs):
            s.energy, s.forces, s.stresses = np.array([e]), f.reshape(-1), st
        ogp.add_training_structure(os_)
        ggp.add_training_structure(gs)
        atoms = sorted(rng.choice(len(sp), 5, replace=False).tolist())
        ogp.add_specific_environments(os_, atoms)
        ggp.add_specific_environments(gs, atoms)
    ogp.update_matrices_QR()
    ggp.update_matrices_QR()
    cell, sp, pos = synth.fcc_batch(n_structures=1, seed=606, lo=32, hi=40)[0]
    return dict(ogp=ogp, ggp=ggp, ob=ob, gb=gb, test=(cell, sp, pos))


def test_training_matches_oracle(gpu_lib, trained):
    ogp, ggp = trained["ogp"], trained["ggp"]
    assert [sd.n_clusters for sd in ggp.sparse_descriptors] == \
        [sd.n_clusters for sd in ogp.sparse_descriptors]
    np.testing.assert_allclose(ggp.Kuu, ogp.Kuu_mat, rtol=0,
                               atol=1e-10 * np.abs(ogp.Kuu_mat).max())
    np.testing.assert_allclose(ggp.Kuf, ogp.Kuf_mat, rtol=0,
                               atol=1e-9 * np.abs(ogp.Kuf_mat).max())
    np.testing.assert_allclose(ggp.alpha, ogp.alpha, rtol=0,
                               atol=1e-5 * np.abs(ogp.alpha).max())
    assert len(ggp.hyperparameters) == 5


def test_predictions_match_oracle(gpu_lib, trained):
    ogp, ggp = trained["ogp"], trained["ggp"]
    cell, sp, pos = trained["test"]
    os_ = OStructure(cell, sp, pos, RC, trained["ob"])
    gs = fg.Structure(cell, sp, pos, RC, trained["gb"])
    ogp.predict_SOR(os_)
    ggp.predict_mean(gs)
    scale = np.abs(os_.mean_efs).max()
    np.testing.assert_allclose(gs.mean_efs, os_.mean_efs, rtol=0, atol=1e-7 * scale)
    ggp.predict_SOR(gs)
    np.testing.assert_allclose(gs.mean_efs, os_.mean_efs, rtol=0, atol=1e-7 * scale)
    np.testing.assert_allclose(gs.variance_efs, os_.variance_efs, rtol=0,
                               atol=1e-6 * np.abs(os_.variance_efs).max())
    ogp.predict_DTC(os_)
    ggp.predict_DTC(gs)
    np.testing.assert_allclose(gs.variance_efs, os_.variance_efs, rtol=0,
                               atol=1e-6 * np.abs(os_.variance_efs).max())
    ref = ogp.compute_cluster_uncertainties(os_)
    got = ggp.compute_cluster_uncertainties(gs)
    assert len(got) == 2
    for r, g, (sig, _) in zip(ref, got, HYPS):
        np.testing.assert_allclose(g, r, rtol=0, atol=1e-7 * sig * sig)


def test_mapped_forms_sum_the_kernels(gpu_lib, trained):
    """The mapped (pair-style) form of each kernel, summed: equals the
    kernel-form mean for power 2 (FP64), and the mixed form is within the
    gates; each kernel writes its own potential file."""
    ogp, ggp = trained["ogp"], trained["ggp"]
    cell, sp, pos = trained["test"]
    os_ = OStructure(cell, sp, pos, RC, trained["ob"])
    ogp.predict_mean(os_)
    ref = os_.mean_efs
    n = len(sp)
    gs = fg.Structure(cell, sp, pos, RC, trained["gb"])
    e, f, s = ggp.predict_mapped(gs, "fp64")
    assert abs(e - ref[0]) < 1e-8 * max(1.0, abs(ref[0]))
    np.testing.assert_allclose(f.ravel(), ref[1:-6], rtol=0,
                               atol=1e-8 * np.abs(ref[1:-6]).max())
    e, f, s = ggp.predict_mapped(gs, "mixed")
    assert abs(e - ref[0]) / n < 1e-6
    assert np.abs(f.ravel() - ref[1:-6]).max() < 1e-4
    assert len(ggp.mapping_coefficients_kernels) == 2


def test_json_round_trip(gpu_lib, trained, tmp_path):
    ggp = trained["ggp"]
    fn = tmp_path / "gp.json"
    ggp.to_json(fn)
    back = fg.SparseGP.from_json(fn)
    assert len(back.kernels) == 2
    cell, sp, pos = trained["test"]
    g1 = fg.Structure(cell, sp, pos, RC, trained["gb"])
    g2 = fg.Structure(cell, sp, pos, RC, trained["gb"])
    ggp.predict_SOR(g1)
    back.predict_SOR(g2)
    np.testing.assert_allclose(g2.mean_efs, g1.mean_efs, rtol=0,
                               atol=1e-12 * np.abs(g1.mean_efs).max())
    np.testing.assert_allclose(g2.variance_efs, g1.variance_efs, rtol=0,
                               atol=1e-12 * np.abs(g1.variance_efs).max())


def test_likelihood_gradient_matches_oracle(gpu_lib, trained):
    """The gradient in (sigma_B2, sigma_B3, sigma_e, sigma_f, sigma_s) against
    the oracle's multi-kernel gradient (each kernel masked to its own Kuu block
    and Kuf rows), and against central differences of the GPU likelihood for
    the components where differences are stable.  With sigma_e = 1e-3 the
    energy-noise difference quotient is dominated by rounding (the oracle's
    own swings from 5.7e2 to 2.6e4 as the step shrinks from 1e-3 to 1e-5 of
    sigma_e), so that component is checked against the oracle only."""
    ogp, ggp = trained["ogp"], trained["ggp"]
    h0 = ggp.hyperparameters.copy()
    assert len(h0) == 5
    np.testing.assert_allclose(h0, ogp.hyperparameters, rtol=1e-15)
    ggp.set_hyperparameters(h0)
    got = ggp.compute_likelihood_gradient_stable()
    ref = ogp.compute_likelihood_gradient_stable()
    # the two QR solves (cuSOLVER, numpy) of this tight-noise fit differ at
    # ~1e-9 of the likelihood
    assert abs(got - ref) < 1e-8 * abs(ref)
    g = ggp.likelihood_gradient.copy()
    np.testing.assert_allclose(g, ogp.likelihood_gradient, rtol=1e-5, atol=0)
    try:
        for i in (0, 1, 3, 4):
            pert = 1e-3 * h0[i]
            vals = []
            for sgn in (1, -1):
                h = h0.copy()
                h[i] += sgn * pert
                ggp.set_hyperparameters(h)
                vals.append(ggp.compute_likelihood_stable())
            fd = (vals[0] - vals[1]) / (2 * pert)
            assert abs(fd - g[i]) < 1e-4 * abs(g[i]) + 1.0, (i, fd, g[i])
    finally:
        ggp.set_hyperparameters(h0)
