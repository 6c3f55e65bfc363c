"""The oracle's sparse GP against the reference's own bffs/sparse_gp.cpp
(with the kernels, descriptors and structure code it calls), compiled
unmodified against small Eigen and nlohmann_json stand-ins
(tests/golden/make_golden.py -> sgp_golden.npz): one B2 kernel and a B2 + B3
model on the tests.fixtures.sgp_scenario frames (one frame trained on a force
subset).  Checked: the label vector and noise vector (bit-exact), Kuu and Kuf,
the QR solve's alpha, R_inv and L_inv, the stable likelihood and its
hyperparameter gradient (before and after set_hyperparameters), predict_mean /
SOR / DTC and the cluster uncertainties of a held-out frame, and each
kernel's mapping coefficients (NormalizedDotProduct::
compute_mapping_coefficients, power 1 and 2) and variance map
(compute_varmap_coefficients, power 1) of the trained model.  The stand-in's
Cholesky and Householder QR round differently from numpy's LAPACK, so the
solve's outputs agree to ~1e-11 of their scale rather than bit for bit."""
import os

import numpy as np
import pytest

from oracle.b2 import B2 as OB2
from oracle.b3 import B3 as OB3
from oracle.geometry import Structure as OStructure
from oracle import predict as opred
from oracle.kernel import NormalizedDotProduct as ONDP
from oracle.sparse_gp import SparseGP as OSGP
from tests import fixtures

GOLD = os.path.join(os.path.dirname(__file__), "golden", "sgp_golden.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _close(mine, ref, rel):
    mine = np.asarray(mine, dtype=float).ravel()
    ref = np.asarray(ref, dtype=float).ravel()
    assert mine.shape == ref.shape, (mine.shape, ref.shape)
    scale = max(np.abs(ref).max(), 1e-300)
    np.testing.assert_allclose(mine, ref, rtol=0, atol=rel * scale)


def _model(two, power):
    sc = fixtures.sgp_scenario(two, power)
    rc = sc["rc"]
    descs = [OB2("chebyshev", "quadratic", [0, rc], [], list(s)) if kind == "B2" else
             OB3("chebyshev", "quadratic", [0, rc], [], list(s)) for kind, s in sc["descs"]]
    gp = OSGP([ONDP(s, p) for s, p in sc["hyps"]], *sc["noises"])
    strucs = []
    for (cell, sp, pos, e, f, st), atoms in zip(sc["frames"], sc["train_atoms"]):
        s = OStructure(cell, sp, pos, rc, descs)
        s.energy, s.forces, s.stresses = e, f, st
        gp.add_training_structure(s, atoms if atoms is not None else (-1,))
        strucs.append(s)
    for s, atoms in zip(strucs, sc["sparse_atoms"]):
        gp.add_specific_environments(s, atoms)
    gp.update_matrices_QR()
    test = OStructure(*sc["test"], rc, descs)
    return gp, test


@pytest.mark.parametrize("tag,two,power", [("one", False, 2.0), ("two", True, 2.0),
                                            ("pow1", False, 1.0)])
def test_sparse_gp_matches_reference(gold, tag, two, power):
    gp, test = _model(two, power)
    k = f"{tag}/"
    np.testing.assert_array_equal(gp.y, gold[k + "y"].ravel())
    np.testing.assert_array_equal(gp.noise_vector, gold[k + "noise_vector"].ravel())
    np.testing.assert_array_equal(gp.hyperparameters, gold[k + "hyperparameters"].ravel())
    _close(gp.Kuu_mat, gold[k + "Kuu"], 1e-13)
    _close(gp.Kuf_mat, gold[k + "Kuf"], 1e-13)
    _close(gp.L_inv, gold[k + "L_inv"], 1e-11)
    _close(gp.R_inv, gold[k + "R_inv"], 1e-11)
    _close(gp.alpha, gold[k + "alpha"], 1e-11)
    gp.compute_likelihood_stable()
    for f in ("log_marginal_likelihood", "data_fit", "complexity_penalty"):
        _close(getattr(gp, f), gold[k + "stable/" + f], 1e-12)
    v = gp.compute_likelihood_gradient_stable()
    _close(v, gold[k + "grad/value"], 1e-12)
    _close(gp.likelihood_gradient, gold[k + "grad/likelihood_gradient"], 1e-10)
    for what in ("mean", "SOR", "DTC"):
        getattr(gp, "predict_" + what)(test)
        _close(test.mean_efs, gold[k + f"predict/{what}/mean_efs"], 1e-10)
        if what != "mean":
            _close(test.variance_efs, gold[k + f"predict/{what}/variance_efs"], 1e-10)
    unc = gp.compute_cluster_uncertainties(test)
    for ki, u in enumerate(unc):
        _close(u, gold[k + f"cluster_uncertainties/{ki}"], 1e-10)
    o = 0
    for ki, (kern, sd) in enumerate(zip(gp.kernels, gp.sparse_descriptors)):
        a = gp.alpha[o:o + sd.n_clusters]
        m = (kern.compute_map_coeff_pow2(sd, a) if power == 2 else
             kern.compute_map_coeff_pow1(sd, a))
        _close(m, gold[k + f"mapping/{ki}"], 1e-10)
        if power == 1:
            vm = opred.varmap_coefficients(sd, gp.Kuu_inverse, kern.sigma, 1, alpha_ind=o)
            _close(vm, gold[k + f"varmap/{ki}"], 1e-10)
        o += sd.n_clusters
    gp.set_hyperparameters(gold[k + "set_hyps/hyps"])
    _close(gp.alpha, gold[k + "set_hyps/alpha"], 1e-10)
    v = gp.compute_likelihood_gradient_stable()
    _close(v, gold[k + "set_hyps/grad/value"], 1e-12)
    _close(gp.likelihood_gradient, gold[k + "set_hyps/grad/likelihood_gradient"], 1e-10)
