"""fpp_predict_energy_uncertainty: the energy, energy variance (predict_SOR,
sparse_gp.cpp:630-649) and per-atom variances (compute_cluster_uncertainties,
sparse_gp.cpp:93-133) at MD sizes, against the FP64 oracle on a two-species
model trained with the reference's QR solve."""
import numpy as np
import pytest
import scipy.linalg as sla

import flare_pp_gb300 as fg
from flare_pp_gb300 import synth
from oracle import predict as opred
from oracle.b2 import B2 as OB2, ClusterDescriptor as OCD
from oracle.geometry import Structure as OStructure
from oracle.kernel import NormalizedDotProduct as ONDP
from tests import fixtures

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def model():
    rc = 5.5
    ob = OB2("chebyshev", "quadratic", [0, rc], [], [2, 6, 3])
    frames = [synth.bcc_alloy((5, 5, 5), 910 + k) for k in range(2)]
    fit = fixtures.site_energy_model(ob, frames, 60, sigma=2.0, power=2, seed=3)
    ob.store_dervs = True        # the fit switched them off; envs_struc needs them
    kern = ONDP(2.0, 2)
    Kuu = kern.envs_envs(fit["sparse"], fit["sparse"])
    L_inv = sla.solve_triangular(np.linalg.cholesky(Kuu + 1e-8 * np.eye(len(Kuu))),
                                 np.eye(len(Kuu)), lower=True)
    gp, gb2 = fixtures.to_gpu_model((2, 6, 3, rc), fit["sparse"], fit["alpha"], 2.0, 2,
                                    R_inv=fit["R_inv"])
    gp.L_inv = L_inv
    return dict(ob=ob, fit=fit, kern=kern, L_inv=L_inv, gp=gp, rc=rc)


@pytest.mark.parametrize("reps,seed", [((6, 6, 6), 77), ((8, 7, 6), 78)])
def test_energy_uncertainty_matches_oracle(gpu_lib, model, reps, seed):
    rc, fit, kern = model["rc"], model["fit"], model["kern"]
    cell, sp, pos = synth.bcc_alloy(reps, seed)
    os_ = OStructure(cell, sp, pos, rc, [model["ob"]])
    dv = os_.descriptors[0]
    K = kern.envs_struc(fit["sparse"], dv)           # (n_sparse, 1 + 3N + 6)
    kE = K[:, 0]
    ref_e = kE @ fit["alpha"]
    ref_var = np.sum((fit["R_inv"].T @ kE) ** 2)
    # per atom: k(i, i) - |L_inv k(sparse, i)|^2, in atom order
    cd = OCD(dv)
    ks = kern.envs_envs(cd, fit["sparse"])           # (clusters, n_sparse)
    kself = np.diag(kern.envs_envs(cd, cd))
    q = np.einsum("ij,ij->j", model["L_inv"] @ ks.T, model["L_inv"] @ ks.T)
    ref_local_cluster = kself - q
    order = np.concatenate(dv.atom_indices)          # cluster -> atom
    ref_local = np.zeros(len(sp))
    ref_local[order] = ref_local_cluster
    gs = fg.Structure(cell, sp, pos, rc)
    e, var, local = model["gp"].predict_energy_uncertainty(gs)
    assert abs(e - ref_e) <= 1e-9 * max(1.0, np.abs(K[:, 0] * fit["alpha"]).sum())
    assert abs(var - ref_var) <= 1e-8 * max(ref_var, 1e-12)
    # differences of O(sigma^2) terms: compared on sigma^2's scale
    np.testing.assert_allclose(local, ref_local, rtol=0, atol=1e-8 * 4.0)
    # the same clusters as compute_cluster_uncertainties (cluster order)
    lv = model["gp"].compute_cluster_uncertainties(gs)[0] if model["gp"].L_inv is not None \
        else None
    np.testing.assert_allclose(local[order], lv, rtol=0, atol=1e-9 * 4.0)
