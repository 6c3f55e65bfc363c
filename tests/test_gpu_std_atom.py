"""The compute flare/std/atom on the GPU (fpp_std_atom_compute through
ComputeFlareStdAtom) against the oracle's restatement of
compute_flare_std_atom.cpp:98-207, on LAMMPS-shaped arrays with ghost atoms.

Both coefficient routes are exercised through their files: the L_inverse +
sparse-descriptor pair (power 1 and 2) and the variance map (power 1, computed
on the GPU by fpp_model_compute_varmap).  std is compared on the variance
scale, s |s| (var = 1 - O(1) terms), to 1e-10, and as std to 1e-6."""
import numpy as np
import pytest

import flare_pp_gb300 as fg
from flare_pp_gb300 import potential, synth
from oracle import predict as opred
from oracle.geometry import Structure as OStructure
from tests import fixtures

pytestmark = pytest.mark.gpu

HYPS_NOISE = [0.001, 0.05, 0.006]


def _write_L_inv_files(m, tmp_path):
    fl, fs = tmp_path / f"Linv{m['power']}.txt", tmp_path / f"sparse{m['power']}.txt"
    hyps = [m["sigma"]] + HYPS_NOISE
    potential.write_L_inverse(fl, m["L_inv"], m["power"], hyps, 2, 4, 2, m["cutoffs"])
    potential.write_sparse_descriptors(fs, m["sd"].descriptors, m["sd"].descriptor_norms)
    return str(fl), str(fs)


def _frame(m, seed=707):
    cell, sp, pos = synth.bcc_alloy((3, 3, 3), seed)
    return cell, sp, pos, OStructure(cell, sp, pos, m["rc"])


def _per_atom(std_all, owner, noa):
    """Local entries (the ghosts carry 0)."""
    assert np.all(std_all[noa:] == 0.0)
    return std_all[:noa]


def _close(got, ref):
    np.testing.assert_allclose(got * np.abs(got), ref * np.abs(ref), rtol=0, atol=1e-10)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-6)


@pytest.mark.parametrize("power", [1, 2])
def test_L_inv_form_matches_oracle(gpu_lib, tmp_path, power):
    m = fixtures.std_atom_model(power=power)
    comp = fg.ComputeFlareStdAtom(*_write_L_inv_files(m, tmp_path))
    assert not comp.use_map
    cell, sp, pos, os_ = _frame(m)
    x, t, il, nn, nb, owner = fixtures.lammps_arrays(cell, sp, pos, m["rc"])
    got = _per_atom(comp.compute_peratom(x, t, il, nn, nb), owner, len(sp))
    ref = opred.std_atom(os_, m["settings"], m["sigma"], power=power, L_inv=m["L_inv"],
                         sparse_normed=m["sparse_normed"])
    assert np.abs(ref).max() > 1e-3
    _close(got, ref)


def test_variance_map_matches_oracle_and_L_inv_form(gpu_lib, tmp_path):
    m = fixtures.std_atom_model(power=1)
    nd = m["sd"].n_descriptors
    # the map from the GPU (SparseGP::write_varmap_coefficients' route)
    b2 = fg.B2("chebyshev", "quadratic", [0.0, m["rc"]], [], [2, 4, 2], m["cutoffs"])
    gp = fg.SparseGP([fg.NormalizedDotProduct(m["sigma"], 1)], *HYPS_NOISE)
    sd = fg.ClusterDescriptor()
    sd.initialize_cluster(2, nd)
    sd.descriptors = [np.array(d) for d in m["sd"].descriptors]
    sd.descriptor_norms = [np.array(n) for n in m["sd"].descriptor_norms]
    sd.n_clusters_by_type = list(m["sd"].n_clusters_by_type)
    sd.cumulative_type_count = list(m["sd"].cumulative_type_count)
    sd.n_clusters = m["sd"].n_clusters
    gp.set_model(b2, sd, np.zeros(sd.n_clusters), L_inv=m["L_inv"])
    fv = tmp_path / "varmap.txt"
    gp.write_varmap_coefficients(str(fv), "test")
    ref_map = opred.varmap_coefficients(m["sd"], m["Kuu_inverse"], m["sigma"], 1)
    np.testing.assert_allclose(gp.varmap_coeffs, ref_map, rtol=0,
                               atol=1e-11 * np.abs(ref_map).max())
    comp = fg.ComputeFlareStdAtom(str(fv))
    assert comp.use_map
    cell, sp, pos, os_ = _frame(m)
    x, t, il, nn, nb, owner = fixtures.lammps_arrays(cell, sp, pos, m["rc"])
    got = _per_atom(comp.compute_peratom(x, t, il, nn, nb), owner, len(sp))
    ref = opred.std_atom(os_, m["settings"], m["sigma"], varmap=ref_map.reshape(2, nd, nd))
    _close(got, ref)
    # the two routes of the compute agree for a power-1 kernel
    fl, fs = _write_L_inv_files(m, tmp_path)
    other = fg.ComputeFlareStdAtom(fl, fs).compute_peratom(x, t, il, nn, nb)[:len(sp)]
    _close(other, got)
    # and the L_inv route is the cluster variance of
    # SparseGP::compute_cluster_uncertainties over sigma^2
    gs = fg.Structure(cell, sp, pos, m["rc"])
    var = gp.compute_cluster_uncertainties(gs)[0]
    order = np.concatenate([np.nonzero(sp == s)[0] for s in range(2)])
    np.testing.assert_allclose(var / m["sigma"] ** 2, (other * np.abs(other))[order],
                               rtol=0, atol=1e-10)


def test_unlisted_and_empty_atoms_are_zero(gpu_lib, tmp_path):
    m = fixtures.std_atom_model(power=2)
    comp = fg.ComputeFlareStdAtom(*_write_L_inv_files(m, tmp_path))
    cell, sp, pos, os_ = _frame(m)
    x, t, il, nn, nb, owner = fixtures.lammps_arrays(cell, sp, pos, m["rc"])
    # only the first 20 local atoms in ilist: the others stay 0
    k = 20
    nn_k = nn[:k]
    nb_k = nb[:int(nn_k.sum())]
    got = comp.compute_peratom(x, t, il[:k], nn_k, nb_k, nlocal=len(sp))
    full = comp.compute_peratom(x, t, il, nn, nb)
    # the same atoms (cuBLAS may block a GEMM of fewer rows differently)
    np.testing.assert_allclose(got[:k], full[:k], rtol=1e-12, atol=0)
    assert np.all(got[k:] == 0.0)
    # an atom with no neighbors inside the cutoff has an empty environment
    x1 = np.array([[0.0, 0.0, 0.0], [9.0, 0.0, 0.0]])
    out = comp.compute_peratom(x1, np.array([1, 2]), np.array([0]), np.array([1]),
                               np.array([1]), nlocal=2)
    np.testing.assert_array_equal(out, [0.0, 0.0])


def test_std_errors(gpu_lib, tmp_path):
    from flare_pp_gb300._lib import FlareGpuError
    m = fixtures.std_atom_model(power=2)
    comp = fg.ComputeFlareStdAtom(*_write_L_inv_files(m, tmp_path))
    with pytest.raises(FlareGpuError, match="power 1 only"):
        comp.model.compute_varmap()
    comp.use_map = True  # no map on this model
    with pytest.raises(FlareGpuError, match="variance map not set"):
        comp.compute_peratom(np.zeros((1, 3)), np.array([1]), np.array([0]),
                             np.array([0]), np.zeros(0, dtype=np.int32))
    comp.use_map = False
    with pytest.raises(FlareGpuError, match="atom type"):
        comp.compute_peratom(np.zeros((1, 3)), np.array([3]), np.array([0]),
                             np.array([0]), np.zeros(0, dtype=np.int32))
