"""The oracle against the reference's golden vectors and the reference's own
self-consistency tests (ctests/test_y_grad.cpp, test_radial.cpp,
test_kernels.cpp sum rules and finite differences, tests/test_lammps.py
beta-form == kernel-form)."""
import os

import numpy as np
import pytest

from oracle import basis, predict
from oracle.b2 import B2, ClusterDescriptor
from oracle.geometry import Structure
from oracle.kernel import NormalizedDotProduct
from flare_pp_gb300 import synth
from tests import fixtures

GOLD = os.path.join(os.path.dirname(__file__), "golden", "l0_golden.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def test_real_harmonics_match_reference(gold):
    v = gold["Y_vecs"]
    Y, Yx, Yy, Yz = basis.real_sph_harm(v[:, 0], v[:, 1], v[:, 2], 10)
    for mine, ref in ((Y, gold["Y"]), (Yx, gold["Yx"]), (Yy, gold["Yy"]),
                      (Yz, gold["Yz"])):
        np.testing.assert_allclose(mine, ref, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("cut", ["quadratic", "cosine"])
def test_radial_matches_reference(gold, cut):
    p = gold["rad_pts"]
    r = np.linalg.norm(p, axis=1)
    g = basis.calculate_radial(p[:, 0], p[:, 1], p[:, 2], r, float(gold["rad_rc"]),
                               int(gold["rad_N"]), float(gold["rad_r1"]), cut)
    for k in range(4):
        np.testing.assert_allclose(g[k], gold[f"g_{cut}"][k], rtol=1e-13, atol=1e-13)


def test_harmonics_fd_and_addition_theorem():
    # ctests/test_y_grad.cpp: FD gradient (1e-6) and sum_m Y_lm^2 = (2l+1)/4pi
    x, y, z, d = 2.16, 7.12, -3.14, 1e-6
    Y, Yx, Yy, Yz = basis.real_sph_harm(np.array([x]), np.array([y]), np.array([z]), 10)
    for k, G in enumerate((Yx, Yy, Yz)):
        e = np.zeros(3)
        e[k] = d
        Yp = basis.real_sph_harm(np.array([x + e[0]]), np.array([y + e[1]]),
                                 np.array([z + e[2]]), 10)[0]
        Ym = basis.real_sph_harm(np.array([x - e[0]]), np.array([y - e[1]]),
                                 np.array([z - e[2]]), 10)[0]
        np.testing.assert_allclose((Yp - Ym) / (2 * d), G, atol=1e-8)
    for l in range(11):
        s = np.sum(Y[0, l * l:(l + 1) ** 2] ** 2)
        assert abs(s - (2 * l + 1) / (4 * np.pi)) < 1e-12


def _small_two_species():
    rng = np.random.default_rng(7)
    cell = np.array([[7.0, 0.2, 0.0], [0.3, 6.5, 0.1], [0.0, -0.4, 7.2]])
    pos = rng.uniform(0, 6.5, size=(12, 3))
    sp = rng.integers(0, 2, size=12)
    return cell, sp, pos


def test_neighbor_list_contract():
    cell, sp, pos = _small_two_species()
    s = Structure(cell, sp, pos, 4.0)
    # symmetric pair relation with exactly negated vectors
    key = {}
    off = s.cumulative_neighbor_count
    for i in range(s.noa):
        for p in range(off[i], off[i + 1]):
            key[(i, s.structure_indices[p], tuple(s.relative_positions[p, 1:]))] = p
    for (i, j, v) in list(key):
        assert (j, i, tuple(-np.array(v))) in key
    # order: j ascending within each atom
    for i in range(s.noa):
        js = s.structure_indices[off[i]:off[i + 1]]
        assert np.all(np.diff(js) >= 0)
    assert np.all(s.relative_positions[:, 0] < 4.0)
    assert np.all(s.relative_positions[:, 0] > 0)


def test_stored_derivative_vs_adjoint_and_sum_rules():
    cell, sp, pos = _small_two_species()
    rc = 4.0
    cut = np.array([[4.0, 3.5], [3.5, 3.8]])
    b2 = B2("chebyshev", "quadratic", [0, rc], [], [2, 3, 2], cut)
    s = Structure(cell, sp, pos, rc, [b2])
    dv = s.descriptors[0]
    kern = NormalizedDotProduct(1.5, 2)
    envs = ClusterDescriptor(dv)
    K = kern.envs_struc(envs, dv)
    KK = kern.struc_struc(dv, dv)
    # ctests/test_kernels.cpp:35-75 sum rules
    np.testing.assert_allclose(K.sum(0), KK[0], atol=1e-8)
    assert abs(kern.envs_envs(envs, envs).sum() - KK[0, 0]) < 1e-8
    # kernel form without stored derivatives == K^T alpha
    alpha = np.random.default_rng(3).normal(size=envs.n_clusters)
    st = fixtures.settings(2, 3, 2, rc, cut)
    kf = predict.kernel_form(s, st, envs, alpha, 1.5, 2)
    np.testing.assert_allclose(kf["mean_efs"], K.T @ alpha, rtol=1e-10, atol=1e-10)


def test_kernel_force_finite_difference():
    # ctests/test_kernels.cpp:140-786: E/F kernel vs central differences
    cell, sp, pos = _small_two_species()
    rc = 4.0
    b2 = B2("chebyshev", "quadratic", [0, rc], [], [2, 3, 2])
    s = Structure(cell, sp, pos, rc, [b2])
    kern = NormalizedDotProduct(1.0, 2)
    envs = ClusterDescriptor(s.descriptors[0])
    K = kern.envs_struc(envs, s.descriptors[0])
    d = 1e-4
    for a in (0, 5):
        for c in range(3):
            pp, pm = pos.copy(), pos.copy()
            pp[a, c] += d
            pm[a, c] -= d
            ep = kern.envs_struc(envs, Structure(cell, sp, pp, rc, [b2]).descriptors[0])[:, 0]
            em = kern.envs_struc(envs, Structure(cell, sp, pm, rc, [b2]).descriptors[0])[:, 0]
            np.testing.assert_allclose(-(ep - em) / (2 * d), K[:, 1 + 3 * a + c], atol=1e-4)


def test_beta_form_equals_kernel_form():
    # tests/test_lammps.py:31-106 at 1e-6 (here far tighter)
    m = fixtures.config1_model(n_frames=2, n_sparse=20)
    cell, sp, pos = synth.fcc_al_108(101, 5)
    s = Structure(cell, sp, pos, m["rc"], [m["b2"]])
    gp = m["gp"]
    gp.predict_mean(s)
    beta = m["kernel"].compute_map_coeff_pow2(gp.sparse_descriptors[0], gp.alpha)
    B = predict.unpack_beta(beta, s.descriptors[0].n_descriptors)
    bf = predict.beta_form(s, m["settings"], B)
    assert abs(bf["energy"] - s.mean_efs[0]) < 1e-8
    np.testing.assert_allclose(bf["forces"].ravel(), s.mean_efs[1:-6], atol=1e-8)
    np.testing.assert_allclose(bf["stress"], s.mean_efs[-6:], atol=1e-8)


def test_qr_solve_matches_scipy():
    m = fixtures.config1_model(n_frames=2, n_sparse=20)
    gp = m["gp"]
    # alpha is the least-squares solution of the stacked system
    Kuu, Kuf = gp.Kuu_mat, gp.Kuf_mat
    L = np.linalg.cholesky(Kuu + 1e-8 * np.eye(Kuu.shape[0]))
    sq = np.sqrt(gp.noise_vector)
    A = np.vstack([sq[:, None] * Kuf.T, L.T])
    b = np.concatenate([sq * gp.y, np.zeros(Kuu.shape[0])])
    import scipy.linalg as sla
    ref = sla.lstsq(A, b)[0]
    np.testing.assert_allclose(gp.alpha, ref, rtol=1e-6, atol=1e-6 * np.abs(ref).max())


# ---------------------------------------------------------------- B3 ----
from oracle import b3 as ob3  # noqa: E402


@pytest.mark.parametrize("lmax", [0, 1, 2, 3, 4])
def test_b3_wigner_tables_match_reference(gold, lmax):
    # descriptors/wigner3j.cpp compute_coeffs, including the 57 entries of its
    # lmax = 4 table that evaluate to 0
    tab = np.zeros((lmax + 1) ** 6)
    tab[gold[f"w3j_{lmax}_idx"]] = gold[f"w3j_{lmax}_val"]
    np.testing.assert_allclose(ob3.w3j_table(lmax), tab, rtol=0, atol=1e-15)


def test_complex_harmonics_match_reference(gold):
    v = gold["Y_vecs"]
    Y = ob3.complex_sph_harm(v[:, 0], v[:, 1], v[:, 2], 6)
    for mine, key in zip(Y, ("Yc", "Ycx", "Ycy", "Ycz")):
        ref = gold[key][:, 0::2] + 1j * gold[key][:, 1::2]
        np.testing.assert_allclose(mine, ref, rtol=1e-12, atol=1e-12)


def _b3_structure(rot=None, shift=None):
    rng = np.random.default_rng(11)
    cell = np.array([[6.6, 0.1, 0.0], [0.2, 6.9, 0.0], [0.0, 0.3, 7.1]])
    pos = rng.uniform(0, 6.5, size=(10, 3))
    sp = rng.integers(0, 2, size=10)
    if shift is not None:
        pos = pos + shift
    if rot is not None:
        cell, pos = cell @ rot.T, pos @ rot.T
    return cell, sp, pos


def test_b3_rotation_invariance():
    # ctests/test_descriptor.cpp:9-48 (1e-10)
    d = ob3.B3("chebyshev", "quadratic", [0, 3.8], [], [2, 3, 3])
    cell, sp, pos = _b3_structure()
    p0 = Structure(cell, sp, pos, 4.0, [d]).descriptors[0]
    a, b = 0.7, 1.1
    Rz = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    Rx = np.array([[1, 0, 0], [0, np.cos(b), -np.sin(b)], [0, np.sin(b), np.cos(b)]])
    cell, sp, pos = _b3_structure(rot=Rx @ Rz)
    p1 = Structure(cell, sp, pos, 4.0, [d]).descriptors[0]
    for s in range(2):
        np.testing.assert_allclose(p1.descriptors[s], p0.descriptors[s], atol=1e-10)


def test_b3_kernel_route_and_finite_difference():
    d = ob3.B3("chebyshev", "quadratic", [0, 3.8], [], [2, 2, 2])
    cell, sp, pos = _b3_structure()
    s = Structure(cell, sp, pos, 4.0, [d])
    dv = s.descriptors[0]
    kern = NormalizedDotProduct(1.3, 2)
    envs = ClusterDescriptor(dv)
    K = kern.envs_struc(envs, dv)
    alpha = np.random.default_rng(4).normal(size=envs.n_clusters)
    st = fixtures.settings_b3(2, 2, 2, 3.8)
    kf = predict.kernel_form(s, st, envs, alpha, 1.3, 2)
    # adjoint route (no stored derivatives) == stored-derivative route
    np.testing.assert_allclose(kf["mean_efs"], K.T @ alpha, rtol=1e-9, atol=1e-9)
    # forces are -dE/dx (central differences)
    h = 1e-5
    for a in (0, 7):
        for c in range(3):
            pp, pm = pos.copy(), pos.copy()
            pp[a, c] += h
            pm[a, c] -= h
            ep = predict.kernel_form(Structure(cell, sp, pp, 4.0), st, envs, alpha, 1.3, 2)
            em = predict.kernel_form(Structure(cell, sp, pm, 4.0), st, envs, alpha, 1.3, 2)
            fd = -(ep["energy"] - em["energy"]) / (2 * h)
            assert abs(fd - kf["forces"][a, c]) < 1e-6
    # beta form == kernel form (tests/test_lammps.py:97-102)
    beta = kern.compute_map_coeff_pow2(envs, alpha)
    B = predict.unpack_beta(beta, dv.n_descriptors)
    bf = predict.beta_form(s, st, B)
    assert abs(bf["energy"] - kf["energy"]) < 1e-9
    np.testing.assert_allclose(bf["forces"], kf["forces"], atol=1e-9)
    np.testing.assert_allclose(bf["stress"], kf["stress"], atol=1e-9)


@pytest.mark.parametrize("lmax", [3, 4])
def test_b3_c_oracle_matches_numpy(lmax):
    from oracle import cfast
    d = ob3.B3("chebyshev", "quadratic", [0, 3.8], [], [2, 2, lmax])
    cell, sp, pos = _b3_structure()
    s = Structure(cell, sp, pos, 4.0, [d])
    envs = ClusterDescriptor(s.descriptors[0])
    alpha = np.random.default_rng(5).normal(size=envs.n_clusters)
    beta = NormalizedDotProduct(1.3, 2).compute_map_coeff_pow2(envs, alpha)
    B = predict.unpack_beta(beta, s.descriptors[0].n_descriptors)
    st = fixtures.settings_b3(2, 2, lmax, 3.8)
    ref = predict.beta_form(Structure(cell, sp, pos, 4.0), st, B)
    got = cfast.beta_form(cell, sp, pos, st, B, n_threads=2)
    assert abs(got["energy"] - ref["energy"]) < 1e-10 * max(1, abs(ref["energy"]))
    np.testing.assert_allclose(got["forces"], ref["forces"], atol=1e-9)
    np.testing.assert_allclose(got["stress"], ref["stress"], atol=1e-10)
    np.testing.assert_allclose(got["atom_energies"], ref["atom_energies"], atol=1e-10)
