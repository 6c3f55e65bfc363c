"""Edge cases of the prediction path against the oracle: the cosine cutoff,
atoms whose environment is empty (|p|^2 < 1e-8, skipped as in
pair_flare.cpp:135 and normalized_dot_product.cpp:156-170), a species with
no atoms in the structure, and power 1 through the mapped form."""
import numpy as np
import pytest

import flare_pp_gb300 as fg
from oracle import predict as opred
from oracle.b2 import B2 as OB2, ClusterDescriptor as OCD
from oracle.geometry import Structure as OStructure
from oracle.kernel import NormalizedDotProduct as ONDP
from tests import fixtures

pytestmark = pytest.mark.gpu


def _model(cut_fn, power, ns=2, seed=3):
    """A small sparse set with random weights (the oracle's own envs)."""
    rng = np.random.default_rng(seed)
    cell = np.array([[8.0, 0.3, 0.0], [0.1, 7.6, 0.2], [0.0, -0.2, 8.2]])
    pos = rng.uniform(0, 7.5, size=(24, 3))
    sp = rng.integers(0, ns, size=24)
    ob = OB2("chebyshev", cut_fn, [0, 4.0], [], [ns, 4, 3])
    od = OStructure(cell, sp, pos, 4.0, [ob]).descriptors[0]
    sparse = OCD(od)
    alpha = rng.normal(size=sparse.n_clusters)
    return ob, sparse, alpha


def _gpu(sparse, alpha, cut_fn, power, ns=2):
    import flare_pp_gb300 as fg
    b2 = fg.B2("chebyshev", cut_fn, [0.0, 4.0], [], [ns, 4, 3])
    cd = fg.ClusterDescriptor()
    cd.initialize_cluster(ns, sparse.n_descriptors)
    cd.descriptors = [np.array(d) for d in sparse.descriptors]
    cd.descriptor_norms = [np.array(n) for n in sparse.descriptor_norms]
    cd.cutoff_values = [np.array(c) for c in sparse.cutoff_values]
    cd.n_clusters_by_type = list(sparse.n_clusters_by_type)
    cd.cumulative_type_count = list(sparse.cumulative_type_count)
    cd.n_clusters = sparse.n_clusters
    gp = fg.SparseGP([fg.NormalizedDotProduct(1.5, power)], 0.001, 0.05, 0.006)
    gp.set_model(b2, cd, alpha)
    return gp


def _test_structure(ns=2, lone=True, seed=8):
    """A dilute cell: a cluster of atoms plus (optionally) one atom farther
    than the cutoff from every other, so its environment is empty."""
    rng = np.random.default_rng(seed)
    cell = np.diag([14.0, 13.0, 15.0])
    pos = rng.uniform(0.5, 6.0, size=(18, 3))
    sp = rng.integers(0, ns, size=18)
    if lone:
        pos = np.vstack([pos, [10.5, 10.0, 11.0]])
        sp = np.concatenate([sp, [0]])
    return cell, sp, pos


@pytest.mark.parametrize("cut_fn", ["quadratic", "cosine"])
@pytest.mark.parametrize("power", [1, 2])
def test_empty_environment_and_cutoffs(gpu_lib, cut_fn, power):
    ob, sparse, alpha = _model(cut_fn, power)
    gp = _gpu(sparse, alpha, cut_fn, power)
    cell, sp, pos = _test_structure()
    st = fixtures.settings(2, 4, 3, 4.0, cutoff_function=cut_fn)
    ref = opred.kernel_form(OStructure(cell, sp, pos, 4.0), st, sparse, alpha, 1.5, power)
    gs = fg.Structure(cell, sp, pos, 4.0)
    gp.predict_mean(gs)
    scale = max(1.0, np.abs(ref["mean_efs"]).max())
    np.testing.assert_allclose(gs.mean_efs, ref["mean_efs"], rtol=0, atol=1e-10 * scale)
    # the lone atom: no energy, no force
    assert ref["atom_energies"][-1] == 0.0
    assert np.all(gs.mean_efs[1 + 3 * (len(sp) - 1):1 + 3 * len(sp)] == 0.0)
    # mapped form (FP64 and mixed) on the same structure
    e, f, s = gp.predict_mapped(gs, "fp64")
    assert abs(e - ref["energy"]) < 1e-9 * max(1.0, abs(ref["energy"]))
    np.testing.assert_allclose(f, ref["forces"], rtol=0, atol=1e-9 * scale)
    e, f, s = gp.predict_mapped(gs, "mixed")
    assert abs(e - ref["energy"]) / len(sp) < 1e-6
    assert np.abs(f - ref["forces"]).max() < 1e-4


def test_species_absent_from_structure(gpu_lib):
    # a two-species model on a structure with only species 1
    ob, sparse, alpha = _model("quadratic", 2)
    gp = _gpu(sparse, alpha, "quadratic", 2)
    cell, sp, pos = _test_structure(lone=False)
    sp = np.ones_like(sp)
    st = fixtures.settings(2, 4, 3, 4.0)
    ref = opred.kernel_form(OStructure(cell, sp, pos, 4.0), st, sparse, alpha, 1.5, 2)
    gs = fg.Structure(cell, sp, pos, 4.0)
    gp.predict_mean(gs)
    scale = max(1.0, np.abs(ref["mean_efs"]).max())
    np.testing.assert_allclose(gs.mean_efs, ref["mean_efs"], rtol=0, atol=1e-10 * scale)
    # This structure (species 1 only, no species-0 neighbours) is far from the
    # sparse set's mean: centred there, the tensor cores' truncating FP32
    # accumulation of beta delta would leave ~1.3e-6 eV/atom (a CPU emulation
    # of that accumulation gives the same figure).  By default the mixed form
    # centres each species on the first structure it evaluates, so the first
    # call already meets the gate.
    e, f, s = gp.predict_mapped(gs, "mixed")
    assert abs(e - ref["energy"]) / len(sp) < 1e-6
    assert np.abs(f - ref["forces"]).max() < 1e-4
    # an explicit recentre on the same structure gives the same centre
    gp.center_mixed_on(gs)
    e2, f2, s2 = gp.predict_mapped(gs, "mixed")
    assert abs(e2 - ref["energy"]) / len(sp) < 1e-7
    assert abs(e2 - e) <= 1e-9 * max(1.0, abs(e))
    assert np.abs(f - ref["forces"]).max() < 1e-4
