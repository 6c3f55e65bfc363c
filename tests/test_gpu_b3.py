"""B3 on the GPU against the oracle (src/flare_pp/descriptors/b3.cpp).

FP64: descriptors, norms and stored derivatives (1e-10 relative), SparseGP
mean and SOR variance through the kernel form, the mapped-beta form.
Mixed: energy within 1e-6 eV/atom and forces within 1e-4 eV/A of the FP64
oracle, the same gates as B2.
"""
import numpy as np
import pytest

import flare_pp_gb300 as fg
from flare_pp_gb300 import synth
from oracle import predict as opred
from oracle.b3 import B3 as OB3
from oracle.geometry import Structure as OStructure
from oracle.kernel import NormalizedDotProduct as ONDP
from oracle.sparse_gp import SparseGP as OSGP
from tests import fixtures

pytestmark = pytest.mark.gpu

E_GATE = 1e-6   # eV / atom
F_GATE = 1e-4   # eV / A


def _structure():
    rng = np.random.default_rng(11)
    cell = np.array([[6.6, 0.1, 0.0], [0.2, 6.9, 0.0], [0.0, 0.3, 7.1]])
    pos = rng.uniform(0, 6.5, size=(12, 3))
    sp = rng.integers(0, 2, size=12)
    return cell, sp, pos


@pytest.mark.parametrize("settings", [[2, 3, 3], [1, 4, 4], [2, 2, 0], [2, 2, 1]],
                         ids=lambda s: "ns%d_N%d_l%d" % tuple(s))
def test_b3_descriptors_and_derivatives(gpu_lib, settings):
    cell, sp, pos = _structure()
    if settings[0] == 1:
        sp = np.zeros_like(sp)
    ob = OB3("chebyshev", "quadratic", [0, 3.8], [], settings)
    gb = fg.B3("chebyshev", "quadratic", [0, 3.8], [], settings)
    od = OStructure(cell, sp, pos, 4.0, [ob]).descriptors[0]
    gd = fg.Structure(cell, sp, pos, 4.0, [gb]).descriptors[0]
    assert gd.n_descriptors == od.n_descriptors
    for s in range(settings[0]):
        scale = max(1.0, np.abs(od.descriptors[s]).max())
        np.testing.assert_allclose(gd.descriptors[s], od.descriptors[s], rtol=0,
                                   atol=1e-10 * scale)
        np.testing.assert_allclose(gd.descriptor_norms[s], od.descriptor_norms[s],
                                   rtol=1e-10, atol=1e-12)
        np.testing.assert_array_equal(gd.neighbor_counts[s], od.neighbor_counts[s])
        np.testing.assert_array_equal(gd.neighbor_indices[s], od.neighbor_indices[s])
        dscale = max(1.0, np.abs(od.descriptor_force_dervs[s]).max())
        np.testing.assert_allclose(gd.descriptor_force_dervs[s],
                                   od.descriptor_force_dervs[s], rtol=0, atol=1e-10 * dscale)
        np.testing.assert_allclose(gd.descriptor_force_dots[s], od.descriptor_force_dots[s],
                                   rtol=0, atol=1e-10 * dscale * scale)


@pytest.fixture(scope="module")
def b3m():
    """FCC Al, 108 atoms, B3 N=4 lmax=3 at rc 5.0 (the shape of the 1M-atom
    B3 workload at a size the oracle runs in seconds), 60 sparse
    environments fitted to Lennard-Jones site energies."""
    rc = 5.0
    ob = OB3("chebyshev", "quadratic", [0, rc], [], [1, 4, 3])
    frames = [synth.fcc_al_108(505, k) for k in range(2)]
    fit = fixtures.site_energy_model(ob, frames, 60, sigma=2.0, power=2)
    ggp, gb = fixtures.to_gpu_model((1, 4, 3, rc), fit["sparse"], fit["alpha"], 2.0, 2,
                                    fit["R_inv"], kind="B3")
    cell, sp, pos = synth.fcc_al_108(505, 5)
    ob.store_dervs = True
    os_ = OStructure(cell, sp, pos, rc, [ob])
    ogp = OSGP([ONDP(2.0, 2)], 0.001, 0.05, 0.006)
    ogp.sparse_descriptors = [fit["sparse"]]
    ogp.alpha = fit["alpha"]
    ogp.R_inv = fit["R_inv"]
    ogp.predict_SOR(os_)
    st = fixtures.settings_b3(1, 4, 3, rc)
    beta = ONDP(2.0, 2).compute_map_coeff_pow2(fit["sparse"], fit["alpha"])
    B = opred.unpack_beta(beta, os_.descriptors[0].n_descriptors)
    bf = opred.beta_form(OStructure(cell, sp, pos, rc), st, B)
    gs = fg.Structure(cell, sp, pos, rc)
    return dict(ggp=ggp, gs=gs, os=os_, bf=bf, beta=beta, noa=len(sp))


def test_b3_predict_mean_and_sor(gpu_lib, b3m):
    ggp, gs, os_ = b3m["ggp"], b3m["gs"], b3m["os"]
    ggp.predict_mean(gs)
    scale = np.abs(os_.mean_efs).max()
    np.testing.assert_allclose(gs.mean_efs, os_.mean_efs, rtol=0, atol=1e-10 * scale)
    ggp.predict_SOR(gs)
    np.testing.assert_allclose(gs.mean_efs, os_.mean_efs, rtol=0, atol=1e-10 * scale)
    np.testing.assert_allclose(gs.variance_efs[0], os_.variance_efs[0], rtol=1e-5)
    np.testing.assert_allclose(gs.variance_efs[1:], os_.variance_efs[1:], rtol=1e-7,
                               atol=1e-9 * np.abs(os_.variance_efs).max())


def test_b3_mapped_fp64_and_mixed(gpu_lib, b3m):
    ggp, gs, bf = b3m["ggp"], b3m["gs"], b3m["bf"]
    e, f, s = ggp.predict_mapped(gs, "fp64")
    np.testing.assert_allclose(ggp.mapping_coefficients, b3m["beta"], rtol=0,
                               atol=1e-10 * np.abs(b3m["beta"]).max())
    assert abs(e - bf["energy"]) < 1e-9 * abs(bf["energy"])
    np.testing.assert_allclose(f, bf["forces"], rtol=0, atol=1e-9)
    np.testing.assert_allclose(s, bf["stress"], rtol=0, atol=1e-10)
    e, f, s = ggp.predict_mapped(gs, "mixed")
    n = b3m["noa"]
    err_e = abs(e - bf["energy"]) / n
    err_f = np.abs(f - bf["forces"]).max()
    print(f"B3 mixed: energy err/atom {err_e:.3e}, max force err {err_f:.3e}, "
          f"stress err {np.abs(s - bf['stress']).max():.3e}")
    assert err_e < E_GATE
    assert err_f < F_GATE


def test_b3_mixed_n6_lmax3(gpu_lib):
    """The settings of the 1M-atom B3 workload (N=6, lmax=3, one species),
    whose FP32 single-bond and pair stages are compiled for that shape: the
    mixed mapped form against the oracle's beta form on 108 atoms."""
    rc = 5.0
    ob = OB3("chebyshev", "quadratic", [0, rc], [], [1, 6, 3])
    frames = [synth.fcc_al_108(505, k) for k in range(2)]
    fit = fixtures.site_energy_model(ob, frames, 40, sigma=2.0, power=2)
    ggp, _ = fixtures.to_gpu_model((1, 6, 3, rc), fit["sparse"], fit["alpha"], 2.0, 2,
                                   fit["R_inv"], kind="B3")
    cell, sp, pos = synth.fcc_al_108(505, 5)
    st = fixtures.settings_b3(1, 6, 3, rc)
    beta = ONDP(2.0, 2).compute_map_coeff_pow2(fit["sparse"], fit["alpha"])
    B = opred.unpack_beta(beta, fit["sparse"].n_descriptors)
    bf = opred.beta_form(OStructure(cell, sp, pos, rc), st, B)
    gs = fg.Structure(cell, sp, pos, rc)
    e, f, s = ggp.predict_mapped(gs, "mixed")
    assert abs(e - bf["energy"]) / len(sp) < E_GATE
    assert np.abs(f - bf["forces"]).max() < F_GATE
