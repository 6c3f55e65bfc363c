"""The compute flare/std/atom on the CPU: its coefficient files (writers of
sparse_gp.cpp:1208-1404, readers of compute_flare_std_atom.cpp:345-664) and the
oracle's two forms of the uncertainty, which agree for a power-1 kernel."""
import numpy as np
import pytest

from flare_pp_gb300 import potential, synth
from oracle import predict as opred
from oracle.geometry import Structure as OStructure
from tests import fixtures


@pytest.fixture(scope="module")
def m1():
    return fixtures.std_atom_model(power=1)


def _test_structure(m, seed=707):
    cell, sp, pos = synth.bcc_alloy((3, 3, 3), seed)
    return OStructure(cell, sp, pos, m["rc"])


def test_varmap_and_L_inv_forms_agree_for_power_1(m1):
    vm = opred.varmap_coefficients(m1["sd"], m1["Kuu_inverse"], m1["sigma"], 1)
    nd = m1["sd"].n_descriptors
    s = _test_structure(m1)
    a = opred.std_atom(s, m1["settings"], m1["sigma"], varmap=vm.reshape(2, nd, nd))
    b = opred.std_atom(s, m1["settings"], m1["sigma"], power=1, L_inv=m1["L_inv"],
                       sparse_normed=m1["sparse_normed"])
    np.testing.assert_allclose(a * np.abs(a), b * np.abs(b), rtol=0, atol=1e-10)
    assert np.abs(b).max() > 1e-3       # not trivially zero
    assert opred.varmap_coefficients(m1["sd"], m1["Kuu_inverse"], 1.5, 2) is None


def test_varmap_file_round_trip(m1, tmp_path):
    vm = opred.varmap_coefficients(m1["sd"], m1["Kuu_inverse"], m1["sigma"], 1)
    fn = tmp_path / "varmap.txt"
    hyps = [m1["sigma"], 0.001, 0.05, 0.006]
    potential.write_varmap(fn, vm, hyps, 2, 4, 2, m1["cutoffs"])
    lines = open(fn).read().splitlines()
    assert lines[1] == "4" and lines[4].split() == ["2", "4", "2", str(vm.shape[1])]
    assert lines[6].split() == ["4.50", "4.00", "4.00", "4.20"]
    assert len(lines[7].split()) == 5
    r = potential.read_varmap(fn)
    np.testing.assert_array_equal(r["varmap"].reshape(2, -1), vm)
    np.testing.assert_array_equal(r["hyps"], hyps)
    np.testing.assert_array_equal(r["cutoffs"], m1["cutoffs"])
    bad = tmp_path / "bad.txt"
    potential.write_varmap(bad, vm[:, :-1], hyps, 2, 4, 2, m1["cutoffs"])
    with pytest.raises(ValueError, match="Beta size"):
        potential.read_varmap(bad)


def test_L_inverse_and_sparse_descriptor_files_round_trip(m1, tmp_path):
    sd = m1["sd"]
    fl, fs = tmp_path / "Linv.txt", tmp_path / "sparse.txt"
    hyps = [m1["sigma"], 0.001, 0.05, 0.006]
    potential.write_L_inverse(fl, m1["L_inv"], 1, hyps, 2, 4, 2, m1["cutoffs"])
    potential.write_sparse_descriptors(fs, sd.descriptors, sd.descriptor_norms)
    r = potential.read_L_inverse(fl)
    n = sd.n_clusters
    assert (r["power"], r["n_kernels"], r["n_clusters"]) == (1, 1, n)
    np.testing.assert_array_equal(r["L_inv"], np.tril(m1["L_inv"]))
    rows = potential.read_sparse_descriptors(fs, sd.n_descriptors, n)
    for s in range(2):
        np.testing.assert_array_equal(rows[s], m1["sparse_normed"][s])
    # five numbers per line; each species block ends its line
    body = open(fs).read().splitlines()
    assert body[1] == "1" and body[2].split() == ["0", str(n), "2"]
    assert all(len(l.split()) <= 5 for l in body[4:])
    with pytest.raises(ValueError, match="n_clusters"):
        potential.read_sparse_descriptors(fs, sd.n_descriptors, n + 1)


def test_sparse_descriptor_file_writes_zero_rows_for_empty_environments(tmp_path):
    D = [np.array([[3.0, 4.0], [0.0, 0.0]]), np.zeros((0, 2))]
    nrm = [np.array([5.0, 0.0]), np.zeros(0)]
    fn = tmp_path / "s.txt"
    potential.write_sparse_descriptors(fn, D, nrm)
    rows = potential.read_sparse_descriptors(fn, 2)
    np.testing.assert_array_equal(rows[0], [[0.6, 0.8], [0.0, 0.0]])
    assert rows[1].shape == (0, 2)
