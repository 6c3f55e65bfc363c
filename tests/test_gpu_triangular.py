"""Variance products with triangular factors of several 128-column tiles.

The FP64-accurate tensor-core products skip the K blocks where a
lower-triangular operand (L_inv, R_inv^T) is zero; the skip only changes
anything once the sparse set spans more than one 128-wide output tile, so
these cases use 432 sparse environments (two species of 216) and random
triangular factors, against the same formulas in FP64 numpy:
predict_SOR (sparse_gp.cpp:630-649), compute_cluster_uncertainties
(sparse_gp.cpp:93-133) and the per-atom variances of
fpp_predict_energy_uncertainty, with L_inv dense below the diagonal and
block diagonal by species."""
import numpy as np
import pytest

import flare_pp_gb300 as fg
from flare_pp_gb300 import synth
from oracle.b2 import B2 as OB2, ClusterDescriptor as OCD
from oracle.geometry import Structure as OStructure
from oracle.kernel import NormalizedDotProduct as ONDP
from tests import fixtures

pytestmark = pytest.mark.gpu

RC = 5.5


@pytest.fixture(scope="module")
def case():
    ob = OB2("chebyshev", "quadratic", [0, RC], [], [2, 6, 3])
    cell, sp, pos = synth.bcc_alloy((6, 6, 6), 4401)
    sparse = OCD(OStructure(cell, sp, pos, RC, [ob]).descriptors[0])
    n = sparse.n_clusters
    rng = np.random.default_rng(4402)
    alpha = rng.normal(size=n)
    R_inv = np.triu(rng.normal(scale=0.05, size=(n, n))) + np.eye(n)
    L_inv = np.tril(rng.normal(scale=0.05, size=(n, n))) + np.eye(n)
    tcell, tsp, tpos = synth.bcc_alloy((4, 4, 4), 4403)
    dv = OStructure(tcell, tsp, tpos, RC, [ob]).descriptors[0]
    kern = ONDP(2.0, 2)
    return dict(ob=ob, sparse=sparse, n=n, alpha=alpha, R_inv=R_inv, L_inv=L_inv,
                kern=kern, K=kern.envs_struc(sparse, dv), dv=dv,
                test=(tcell, tsp, tpos))


def _gpu_model(c, L_inv=None):
    gp, _ = fixtures.to_gpu_model((2, 6, 3, RC), c["sparse"], c["alpha"], 2.0, 2,
                                  R_inv=c["R_inv"])
    if L_inv is not None:
        gp.L_inv = L_inv
    return gp


def _explained(c, L_inv):
    """|L_inv k_c|^2 per test cluster, cluster order, and the cluster -> atom map."""
    cd = OCD(c["dv"])
    ks = c["kern"].envs_envs(cd, c["sparse"])
    Q = L_inv @ ks.T
    return np.einsum("ij,ij->j", Q, Q), np.concatenate(c["dv"].atom_indices), cd, ks


def test_sor_variance_upper_R_inv(gpu_lib, case):
    assert case["n"] > 256
    gp = _gpu_model(case)
    gs = fg.Structure(*case["test"], RC)
    gp.predict_SOR(gs)
    K = case["K"]
    np.testing.assert_allclose(gs.mean_efs, K.T @ case["alpha"], rtol=0,
                               atol=1e-10 * np.abs(K.T @ case["alpha"]).max())
    vs = K.T @ case["R_inv"]
    ref = np.einsum("ij,ij->i", vs, vs)
    np.testing.assert_allclose(gs.variance_efs, ref, rtol=0, atol=1e-11 * np.abs(ref).max())


@pytest.mark.parametrize("blocks", [False, True], ids=["dense", "species_blocks"])
def test_local_variances_lower_L_inv(gpu_lib, case, blocks):
    L_inv = case["L_inv"].copy()
    if blocks:
        off = list(case["sparse"].cumulative_type_count) + [case["n"]]
        for a in range(2):
            for b in range(2):
                if a != b:
                    L_inv[off[a]:off[a + 1], off[b]:off[b + 1]] = 0.0
    q, order, cd, ks = _explained(case, L_inv)
    kself = np.diag(case["kern"].envs_envs(cd, cd))
    gp = _gpu_model(case, L_inv)
    gs = fg.Structure(*case["test"], RC)
    e, var, local = gp.predict_energy_uncertainty(gs)
    ref = np.zeros(len(order))
    ref[order] = kself - q
    np.testing.assert_allclose(local, ref, rtol=0, atol=1e-11 * np.abs(q).max())
    kE = case["K"][:, 0]
    v_ref = np.sum((case["R_inv"].T @ kE) ** 2)
    assert abs(var - v_ref) <= 1e-10 * v_ref
    # compute_cluster_uncertainties: the host-L_inv route, cluster order
    lv = gp.compute_cluster_uncertainties(gs)[0]
    np.testing.assert_allclose(lv, kself - q, rtol=0, atol=1e-11 * np.abs(q).max())
