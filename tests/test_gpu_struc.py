"""Structure-structure kernels on the GPU against the oracle
(NormalizedDotProduct::struc_struc / self_kernel_struc,
normalized_dot_product.cpp:212-578) and the DTC variance that uses them
(sparse_gp.cpp:651-680)."""
import numpy as np
import pytest

import flare_pp_gb300 as fg
from oracle.b2 import B2 as OB2
from oracle.b3 import B3 as OB3
from oracle.geometry import Structure as OStructure
from oracle.kernel import NormalizedDotProduct as ONDP

pytestmark = pytest.mark.gpu


def _pair():
    rng = np.random.default_rng(21)
    cell = np.array([[6.8, 0.2, 0.0], [0.1, 6.6, 0.2], [0.0, -0.3, 7.0]])
    pos = rng.uniform(0, 6.5, size=(10, 3))
    sp = rng.integers(0, 2, size=10)
    cell2 = cell * 1.02
    pos2 = pos[:8] * 1.01 + rng.normal(scale=0.1, size=(8, 3))
    sp2 = sp[:8].copy()
    return (cell, sp, pos), (cell2, sp2, pos2)


def _descs(kind):
    if kind == "B3":
        return (OB3("chebyshev", "quadratic", [0, 3.8], [], [2, 2, 2]),
                fg.B3("chebyshev", "quadratic", [0, 3.8], [], [2, 2, 2]))
    cut = np.array([[3.8, 3.4], [3.4, 3.6]])
    return (OB2("chebyshev", "quadratic", [0, 3.8], [], [2, 3, 2], cut),
            fg.B2("chebyshev", "quadratic", [0, 3.8], [], [2, 3, 2], cut))


@pytest.mark.parametrize("kind", ["B2", "B3"])
@pytest.mark.parametrize("power", [1, 2])
def test_struc_struc_and_self_kernel(gpu_lib, kind, power):
    (c1, s1, p1), (c2, s2, p2) = _pair()
    ob, gb = _descs(kind)
    o1 = OStructure(c1, s1, p1, 4.0, [ob]).descriptors[0]
    o2 = OStructure(c2, s2, p2, 4.0, [ob]).descriptors[0]
    g1 = fg.Structure(c1, s1, p1, 4.0, [gb]).descriptors[0]
    g2 = fg.Structure(c2, s2, p2, 4.0, [gb]).descriptors[0]
    ok, gk = ONDP(1.4, power), fg.NormalizedDotProduct(1.4, power)
    K_ref = ok.struc_struc(o1, o2)
    K = gk.struc_struc(g1, g2)
    scale = np.abs(K_ref).max()
    np.testing.assert_allclose(K, K_ref, rtol=0, atol=1e-10 * scale)
    d_ref = ok.self_kernel_struc(o1)
    d = gk.self_kernel_struc(g1)
    np.testing.assert_allclose(d, d_ref, rtol=0, atol=1e-10 * np.abs(d_ref).max())
    # symmetry of the covariance (K(a, b) = K(b, a)^T)
    Kt = gk.struc_struc(g2, g1)
    np.testing.assert_allclose(Kt, K.T, rtol=0, atol=1e-10 * scale)


def test_struc_struc_sum_rule_against_envs_struc(gpu_lib):
    # ctests/test_kernels.cpp:35-75: summing the environment kernel over the
    # environments of a structure gives the structure's energy row
    (c1, s1, p1), _ = _pair()
    ob, gb = _descs("B2")
    g1 = fg.Structure(c1, s1, p1, 4.0, [gb]).descriptors[0]
    gk = fg.NormalizedDotProduct(1.4, 2)
    K = gk.struc_struc(g1, g1)
    envs = fg.ClusterDescriptor(g1)
    Ke = gk.envs_struc(envs, g1)
    np.testing.assert_allclose(Ke.sum(0), K[0], rtol=0, atol=1e-10 * np.abs(K[0]).max())


def test_predict_dtc_matches_oracle(gpu_lib):
    """SparseGP::predict_DTC (sparse_gp.cpp:651-680) after a GPU training
    solve, against the oracle's DTC on the same training set."""
    from flare_pp_gb300 import synth
    from tests import fixtures
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
    cell, sp, pos = synth.fcc_al_108(101, 5)
    # a smaller test cell keeps the self kernel's pair-pair matrix small
    keep = np.arange(40)
    os_ = OStructure(cell, sp[keep], pos[keep], 5.0, [m["b2"]])
    ogp.predict_DTC(os_)
    gs = fg.Structure(cell, sp[keep], pos[keep], 5.0, [b2])
    gp.predict_DTC(gs)
    # the training system [Lambda^1/2 Kuf^T; L^T] has condition ~1e10 here
    # (sigma_e = 1e-3): Kuf equal to ~1e-15 gives alpha equal to ~1e-8 (the
    # oracle's own Kuf by stored derivatives vs by the adjoint route differ
    # the same way), and predictions to ~1e-7 relative
    scale = np.abs(os_.mean_efs).max()
    np.testing.assert_allclose(gs.mean_efs, os_.mean_efs, rtol=0, atol=1e-6 * scale)
    np.testing.assert_allclose(gs.variance_efs, os_.variance_efs, rtol=1e-4,
                               atol=1e-6 * np.abs(os_.variance_efs).max())


def test_batched_kuf_training_matches_oracle(gpu_lib):
    """Training on an uneven batch of strained two-species FCC cells (the
    batched-Kuf workload at a size the oracle trains in seconds): Kuf from
    fpp_kuf_batched, Kuu, the QR solve and alpha against the oracle's
    update_matrices_QR (sparse_gp.cpp:576-610); one structure trains on a
    subset of its atoms' forces (add_training_structure's atom_indices)."""
    from flare_pp_gb300 import synth
    from oracle.sparse_gp import SparseGP as OSGP
    rc = 5.0
    cells = synth.fcc_batch(n_structures=5, seed=404, lo=16, hi=48)
    ob = OB2("chebyshev", "quadratic", [0, rc], [], [2, 6, 3])
    gb = fg.B2("chebyshev", "quadratic", [0, rc], [], [2, 6, 3])
    ogp = OSGP([ONDP(2.0, 2)], 0.001, 0.05, 0.006)
    ggp = fg.SparseGP([fg.NormalizedDotProduct(2.0, 2)], 0.001, 0.05, 0.006)
    rng = np.random.default_rng(9)
    ostr, gstr = [], []
    for k, (cell, sp, pos) in enumerate(cells):
        e, f, st, _ = synth.lennard_jones(cell, pos)
        os_ = OStructure(cell, sp, pos, rc, [ob])
        gs = fg.Structure(cell, sp, pos, rc, [gb])
        for s in (os_, gs):
            s.energy, s.forces, s.stresses = np.array([e]), f.reshape(-1), st
        atoms = (-1,) if k != 2 else tuple(range(0, len(sp), 3))
        ogp.add_training_structure(os_, list(atoms))
        ggp.add_training_structure(gs, atoms)
        ostr.append(os_)
        gstr.append(gs)
    for k in range(len(cells)):
        n = len(cells[k][1])
        atoms = sorted(rng.choice(n, min(6, n), replace=False).tolist())
        ogp.add_specific_environments(ostr[k], atoms)
        ggp.add_specific_environments(gstr[k], atoms)
    ogp.update_matrices_QR()
    ggp.update_matrices_QR()
    np.testing.assert_allclose(ggp.Kuu, ogp.Kuu_mat, rtol=0,
                               atol=1e-10 * np.abs(ogp.Kuu_mat).max())
    np.testing.assert_allclose(ggp.Kuf, ogp.Kuf_mat, rtol=0,
                               atol=1e-9 * np.abs(ogp.Kuf_mat).max())
    np.testing.assert_allclose(ggp.y, ogp.y, rtol=0, atol=0)
    np.testing.assert_allclose(ggp.alpha, ogp.alpha, rtol=0,
                               atol=1e-5 * np.abs(ogp.alpha).max())


def test_local_uncertainties_match_oracle(gpu_lib):
    """SparseGP::compute_cluster_uncertainties / predict_local_uncertainties
    (sparse_gp.cpp:93-133, 682-702) after a GPU training solve, against the
    oracle on the same model."""
    from flare_pp_gb300 import synth
    from tests import fixtures
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
    cell, sp, pos = synth.fcc_al_108(101, 5)
    os_ = OStructure(cell, sp, pos, 5.0, [m["b2"]])
    ref = ogp.compute_cluster_uncertainties(os_)[0]
    gs = fg.Structure(cell, sp, pos, 5.0)
    gp.predict_local_uncertainties(gs)
    got = gs.local_uncertainties[0]
    # a difference of two O(sigma^2) terms: compare on sigma^2's scale
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-7 * 4.0)
    assert np.all(got > -1e-8)


def test_batched_kuf_full_size(gpu_lib):
    """The batched-Kuf workload at full size: 256 strained (+-3 %), rattled
    (0.1 A) two-species FCC cells of 32-512 atoms (69,380 atoms, 209,932 E/F/S
    labels), N = 8, lmax = 3, rc 5.0, 1000 sparse environments.  Kuf is
    assembled by one persistent adjoint launch over all structures' atoms
    (autotuned tiles) and the QR solve runs on the GPU.  Checked (a) column
    by column against the oracle's envs_struc (normalized_dot_product.cpp:
    115-210) for six structures (the three smallest and three drawn at
    random), with the same sparse set, (b) through the normal equations of
    the solve, (Kuu + jitter I + Kuf Lambda Kuf^T) alpha = Kuf Lambda y, and
    (c) alpha against the oracle's QR solve (sparse_gp.cpp:576-610, numpy /
    scipy on the host) of the same Kuu, Kuf, y and noise."""
    from flare_pp_gb300 import synth
    from oracle.b2 import ClusterDescriptor as OCD
    rc = 5.0
    cells = synth.fcc_batch(n_structures=256, seed=404, lo=32, hi=512)
    gb = fg.B2("chebyshev", "quadratic", [0, rc], [], [2, 8, 3])
    gb.store_dervs = False
    gp = fg.SparseGP([fg.NormalizedDotProduct(2.0, 2)], 0.001, 0.05, 0.006)
    strucs = []
    for cell, sp, pos in cells:
        e, f, st, _ = synth.lennard_jones(cell, pos)
        s = fg.Structure(cell, sp, pos, rc, [gb])
        s.energy, s.forces, s.stresses = np.array([e]), f.reshape(-1), st
        gp.add_training_structure(s)
        strucs.append(s)
    rng = np.random.default_rng(404)
    allc = [(k, a) for k, (_, sp, _) in enumerate(cells) for a in range(len(sp))]
    pick = rng.choice(len(allc), 1000, replace=False)
    for k in range(len(cells)):
        atoms = sorted(allc[p][1] for p in pick if allc[p][0] == k)
        if atoms:
            gp.add_specific_environments(strucs[k], atoms)
    import time
    t0 = time.perf_counter()
    gp.update_matrices_QR()
    print(f"full-size training (Kuu, Kuf of 256 structures, GPU QR): "
          f"{time.perf_counter() - t0:.2f} s, Kuf launch (ks, threads, ms, items) "
          f"{gp.kuf_launch()}")
    assert all(v > 0 for v in gp.kuf_tiles())
    n_lab = sum(1 + 3 * len(sp) + 6 for _, sp, _ in cells)
    assert gp.Kuf.shape == (1000, n_lab) and len(gp.y) == n_lab
    # (a) three structures against the oracle, same sparse set
    sd = gp.sparse_descriptors[0]
    osd = OCD()
    osd.initialize_cluster(sd.n_types, sd.n_descriptors)
    osd.descriptors = [np.array(d) for d in sd.descriptors]
    osd.descriptor_norms = [np.array(n) for n in sd.descriptor_norms]
    osd.n_clusters_by_type = list(sd.n_clusters_by_type)
    osd.cumulative_type_count = list(sd.cumulative_type_count)
    osd.n_clusters = sd.n_clusters
    ob = OB2("chebyshev", "quadratic", [0, rc], [], [2, 8, 3])
    offs = np.concatenate([[0], np.cumsum([1 + 3 * len(sp) + 6 for _, sp, _ in cells])])
    pick6 = list(np.argsort([len(sp) for _, sp, _ in cells], kind="stable")[:3])
    pick6 += list(np.random.default_rng(7).choice(256, 3, replace=False))
    for k in pick6:
        cell, sp, pos = cells[k]
        os_ = OStructure(cell, sp, pos, rc, [ob])
        ref = ONDP(2.0, 2).envs_struc(osd, os_.descriptors[0])
        got = gp.Kuf[:, offs[k]:offs[k + 1]]
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-9 * np.abs(ref).max())
    # (b) the normal equations of the solve
    nv, a = gp.noise_vector, gp.alpha
    b = gp.Kuf @ (nv * gp.y)
    Aa = gp.Kuu @ a + gp.Kuu_jitter * a + gp.Kuf @ (nv * (gp.Kuf.T @ a))
    a_norm = np.sum(nv * np.einsum("ij,ij->j", gp.Kuf, gp.Kuf)) + np.linalg.norm(gp.Kuu)
    assert np.linalg.norm(Aa - b) <= 1e-10 * a_norm * np.linalg.norm(a)
    # (c) alpha against the oracle's QR solve of the same system
    import scipy.linalg as sla
    n = gp.Kuu.shape[0]
    L = np.linalg.cholesky(gp.Kuu + gp.Kuu_jitter * np.eye(n))
    sq = np.sqrt(nv)
    A = np.vstack([sq[:, None] * gp.Kuf.T, L.T])
    Q, R = np.linalg.qr(A, mode="reduced")
    a_ref = sla.solve_triangular(R, Q.T @ np.concatenate([sq * gp.y, np.zeros(n)]))
    np.testing.assert_allclose(gp.alpha, a_ref, rtol=0, atol=1e-6 * np.abs(a_ref).max())
