"""The oracle's Structure, B2 DescriptorValues and NormalizedDotProduct
kernels against the reference's own code.

tests/golden/struc_kernel_golden.npz holds outputs of the reference's
structure.cpp (neighbor list: counts, order, neighbor species, relative
positions, wrapped positions, sweep), descriptors/b2.cpp + descriptor.cpp
(DescriptorValues per species, including the stored force derivatives) and
kernels/normalized_dot_product.cpp (envs_envs, envs_struc, struc_struc,
self_kernel_struc at power 1 and 2), compiled unmodified against small Eigen
and nlohmann_json stand-ins (tests/golden/make_golden.py).  The cases
(tests/fixtures.struc_cases) include a triclinic cell that needs two sweeps, a
single atom, and species-dependent cutoffs.  Integer outputs must match
exactly; floating-point outputs to 1e-13 of their scale (the stand-in's 3 x 3
inverse and products may round differently from Eigen's).
"""
import os

import numpy as np
import pytest

from oracle.b2 import B2, ClusterDescriptor
from oracle.geometry import Structure
from oracle.kernel import NormalizedDotProduct
from tests import fixtures

GOLD = os.path.join(os.path.dirname(__file__), "golden", "struc_kernel_golden.npz")
CASES = fixtures.struc_cases()


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _close(mine, ref, rel=1e-13):
    mine, ref = np.asarray(mine, dtype=float), np.asarray(ref, dtype=float)
    assert mine.shape == ref.shape, (mine.shape, ref.shape)
    if ref.size:
        scale = max(np.abs(ref).max(), 1e-300)
        np.testing.assert_allclose(mine, ref, rtol=0, atol=rel * scale)


def _proj(m, seed=4242):
    r = np.random.default_rng(seed).normal(size=(m.shape[1], 4))
    return m @ r


def _structure(name, with_b2=True):
    cell, sp, pos, rc, (ns, N, lmax), cut = CASES[name]
    calc = [B2("chebyshev", "quadratic", [0.0, rc], [], [ns, N, lmax], np.asarray(cut))] \
        if with_b2 else []
    return Structure(cell, sp, pos, rc, calc)


@pytest.mark.parametrize("name", sorted(CASES))
def test_neighbor_list_matches_reference(gold, name):
    o = _structure(name, with_b2=False)
    k = f"struc/{name}/"
    assert o.sweep == int(gold[k + "sweep"][0])
    for f in ("neighbor_count", "cumulative_neighbor_count", "structure_indices",
              "neighbor_species"):
        np.testing.assert_array_equal(np.asarray(getattr(o, f)), gold[k + f], err_msg=f)
    _close(o.relative_positions, gold[k + "relative_positions"])
    _close(o.wrapped_positions, gold[k + "wrapped_positions"])
    v = gold[k + "volume"][0]
    assert abs(o.volume - v) <= 1e-13 * v


@pytest.mark.parametrize("name", sorted(CASES))
def test_b2_descriptor_values_match_reference(gold, name):
    o = _structure(name)
    dv = o.descriptors[0]
    ns = CASES[name][4][0]
    for s in range(ns):
        k = f"dv/{name}/{s}/"
        for f in ("neighbor_counts", "cumulative_neighbor_counts", "atom_indices",
                  "neighbor_indices"):
            np.testing.assert_array_equal(np.asarray(getattr(dv, f)[s]), gold[k + f],
                                          err_msg=f)
        _close(dv.descriptors[s], gold[k + "descriptors"])
        _close(dv.descriptor_norms[s], gold[k + "descriptor_norms"])
        _close(dv.descriptor_force_dots[s], gold[k + "descriptor_force_dots"])
        _close(dv.cutoff_values[s], gold[k + "cutoff_values"])
        _close(dv.neighbor_coordinates[s], gold[k + "neighbor_coordinates"])
        fd = np.asarray(dv.descriptor_force_dervs[s])
        _close(fd[:48], gold[k + "force_dervs_rows"])
        if len(fd):
            _close(_proj(fd), gold[k + "force_dervs_proj"], 1e-12)


@pytest.mark.parametrize("sigma,power", fixtures.KERNEL_HYPS)
def test_kernels_match_reference(gold, sigma, power):
    strucs = {n: _structure(n) for n in {n for n, _ in fixtures.KERNEL_SPARSE}
              | set(fixtures.KERNEL_STRUCS)}
    cd = ClusterDescriptor()
    for n, cl in fixtures.KERNEL_SPARSE:
        cd.add_clusters_by_type(strucs[n].descriptors[0], cl)
    a = strucs[fixtures.KERNEL_STRUCS[0]].descriptors[0]
    b = strucs[fixtures.KERNEL_STRUCS[1]].descriptors[0]
    k = NormalizedDotProduct(sigma, power)
    key = f"kernel/{{}}/{sigma}/{power}"
    _close(k.envs_envs(cd, cd), gold[key.format("envs_envs")])
    _close(k.envs_struc(cd, b), gold[key.format("envs_struc")])
    _close(np.asarray(k.self_kernel_struc(b)).reshape(-1, 1),
           gold[key.format("self_kernel_struc")].reshape(-1, 1))
    if key.format("struc_struc") + "/throws" in gold.files:
        # the reference throws std::invalid_argument here (power < 2 and a
        # zero normalized dot product, normalized_dot_product.cpp:285-288)
        with pytest.raises(ValueError):
            k.struc_struc(a, b)
    else:
        _close(k.struc_struc(a, b), gold[key.format("struc_struc")])
