"""The model's JSON state in the layout of SparseGP::to_json / from_json
(src/flare_pp/bffs/sparse_gp.h:101-111, sparse_gp.cpp:1406-1417): a round trip
predicts the same energies, forces, stresses and variances, as the
reference's own round-trip test checks (tests/test_sparse_gp.py:84-136)."""
import json

import numpy as np
import pytest

import flare_pp_gb300 as fg
from flare_pp_gb300 import synth
from tests import fixtures

pytestmark = pytest.mark.gpu


def test_sparse_gp_json_round_trip(gpu_lib, tmp_path):
    m = fixtures.config1_model(n_frames=2, n_sparse=20)
    ogp = m["gp"]
    b2 = fg.B2("chebyshev", "quadratic", [0.0, 5.0], [], [1, 8, 3])
    gp = fg.SparseGP([fg.NormalizedDotProduct(2.0, 2)], 0.001, 0.05, 0.006)
    frames = []
    for of in ogp.training_structures:
        s = fg.Structure(of.cell, of.species, of.positions, 5.0, [b2])
        s.energy, s.forces, s.stresses = of.energy, of.forces, of.stresses
        gp.add_training_structure(s)
        frames.append(s)
    for k, atoms in enumerate(ogp.sparse_indices[0]):
        gp.add_specific_environments(frames[k], atoms)
    gp.update_matrices_QR()
    fn = tmp_path / "sgp.json"
    gp.to_json(str(fn))
    # the reference's field names (NLOHMANN_DEFINE_TYPE_INTRUSIVE list)
    j = json.load(open(fn))
    for key in ("kernels", "sparse_descriptors", "alpha", "R_inv", "L_inv", "Sigma",
                "Kuu_inverse", "training_structures", "noise_vector", "y"):
        assert key in j
    gp2 = fg.SparseGP.from_json(str(fn))
    cell, sp, pos = synth.fcc_al_108(101, 5)
    a = fg.Structure(cell, sp, pos, 5.0)
    b = fg.Structure(cell, sp, pos, 5.0)
    gp.predict_SOR(a)
    gp2.predict_SOR(b)
    np.testing.assert_allclose(b.mean_efs, a.mean_efs, rtol=0, atol=1e-12)
    np.testing.assert_allclose(b.variance_efs, a.variance_efs, rtol=1e-12, atol=1e-14)
    e1, f1, s1 = gp.predict_mapped(a, "mixed")
    e2, f2, s2 = gp2.predict_mapped(b, "mixed")
    assert e1 == e2
    np.testing.assert_array_equal(f1, f2)
    gp2.predict_local_uncertainties(b)
    gp.predict_local_uncertainties(a)
    np.testing.assert_allclose(b.local_uncertainties[0], a.local_uncertainties[0],
                               rtol=0, atol=1e-12)
