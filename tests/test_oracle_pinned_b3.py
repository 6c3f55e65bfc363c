"""The oracle's B3 DescriptorValues and the NormalizedDotProduct kernels on B3
descriptors against the reference's own descriptors/b3.cpp (with
descriptor.cpp, structure.cpp, y_grad.cpp's complex harmonics and the
wigner3j.cpp tables), compiled unmodified against small Eigen and
nlohmann_json stand-ins (tests/golden/make_golden.py -> b3_golden.npz).
Cases (tests/fixtures.b3_cases): one and two species, lmax 2, 3 and 4 (the
lmax = 4 table with the reference's integer-division zeros), a triclinic cell
needing two sweeps.  Integers exactly, floating point to 1e-12 of scale."""
import os

import numpy as np
import pytest

from oracle.b2 import ClusterDescriptor
from oracle.b3 import B3
from oracle.geometry import Structure
from oracle.kernel import NormalizedDotProduct
from tests import fixtures

GOLD = os.path.join(os.path.dirname(__file__), "golden", "b3_golden.npz")
CASES = fixtures.b3_cases()


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _close(mine, ref, rel=1e-12):
    mine, ref = np.asarray(mine, dtype=float), np.asarray(ref, dtype=float)
    assert mine.shape == ref.shape, (mine.shape, ref.shape)
    if ref.size:
        scale = max(np.abs(ref).max(), 1e-300)
        np.testing.assert_allclose(mine, ref, rtol=0, atol=rel * scale)


def _proj(m, seed=4242):
    r = np.random.default_rng(seed).normal(size=(m.shape[1], 4))
    return m @ r


def _structure(name):
    cell, sp, pos, rc, (ns, N, lmax) = CASES[name]
    return Structure(cell, sp, pos, rc, [B3("chebyshev", "quadratic", [0.0, rc], [],
                                            [ns, N, lmax])])


@pytest.mark.parametrize("name", sorted(CASES))
def test_b3_descriptor_values_match_reference(gold, name):
    dv = _structure(name).descriptors[0]
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
        fd = np.asarray(dv.descriptor_force_dervs[s])
        _close(fd[:48], gold[k + "force_dervs_rows"])
        if len(fd):
            _close(_proj(fd), gold[k + "force_dervs_proj"], 1e-11)


@pytest.mark.parametrize("sigma,power", fixtures.KERNEL_HYPS)
def test_b3_kernels_match_reference(gold, sigma, power):
    strucs = {n: _structure(n) for n in {n for n, _ in fixtures.B3_KERNEL_SPARSE}
              | set(fixtures.B3_KERNEL_STRUCS)}
    cd = ClusterDescriptor()
    for n, cl in fixtures.B3_KERNEL_SPARSE:
        cd.add_clusters_by_type(strucs[n].descriptors[0], cl)
    a = strucs[fixtures.B3_KERNEL_STRUCS[0]].descriptors[0]
    b = strucs[fixtures.B3_KERNEL_STRUCS[1]].descriptors[0]
    k = NormalizedDotProduct(sigma, power)
    key = f"kernel/{{}}/{sigma}/{power}"
    _close(k.envs_envs(cd, cd), gold[key.format("envs_envs")])
    _close(k.envs_struc(cd, b), gold[key.format("envs_struc")])
    _close(np.asarray(k.self_kernel_struc(b)).reshape(-1, 1),
           gold[key.format("self_kernel_struc")].reshape(-1, 1))
    if key.format("struc_struc") + "/throws" in gold.files:
        with pytest.raises(ValueError):
            k.struc_struc(a, b)
    else:
        _close(k.struc_struc(a, b), gold[key.format("struc_struc")])
