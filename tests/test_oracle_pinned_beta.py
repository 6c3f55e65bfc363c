"""The oracle's pair-style math against the reference's own code.

tests/golden/beta_form_golden.npz holds outputs of the reference's
lammps_plugins/lammps_descriptor.cpp (single_bond_multiple_cutoffs,
B2_descriptor, compute_energy_and_u), compiled unmodified and driven by the
per-atom loop of pair_flare.cpp:95-180 over LAMMPS arrays with ghost atoms
(tests/golden/make_golden.py).  The cases (tests/fixtures.BETA_CASES) cover
one and two species, power 1 and 2, a species-dependent cutoff matrix and the
N = 12, lmax = 4 shape of the 32k-atom workload.  Both oracle forms are
checked: the numpy restatement (oracle/predict.py) and the C restatement
(oracle/c/flare_oracle.c) that the GPU parity tests and the CPU baseline use.
"""
import os

import numpy as np
import pytest

from oracle import predict as opred
from oracle.b2 import compute_b2, single_bond_multiple_cutoffs
from oracle.geometry import Structure as OStructure
from tests import fixtures

GOLD = os.path.join(os.path.dirname(__file__), "golden", "beta_form_golden.npz")
CASES = sorted(fixtures.BETA_CASES)


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _close(mine, ref, rel):
    scale = max(np.abs(ref).max(), 1e-300)
    np.testing.assert_allclose(mine, ref, rtol=0, atol=rel * scale)


def _flare_stress_from_virial(vir, volume):
    # flare order xx, xy, xz, yy, yz, zz from LAMMPS xx, yy, zz, xy, xz, yz;
    # sigma = -(1/V) sum f r_ij = (1/V) sum del f with del = -r_ij
    v = np.asarray(vir)
    return np.array([v[0], v[3], v[4], v[1], v[5], v[2]]) / volume


@pytest.mark.parametrize("name", CASES)
def test_numpy_oracle_matches_reference_pair_style(gold, name):
    cell, sp, pos, st, beta, power = fixtures.beta_case(name)
    o = OStructure(cell, sp, pos, float(np.max(st["cutoffs"])))
    r = opred.beta_form(o, st, beta, power)
    _close(r["atom_energies"], gold[f"{name}/atom_energies"], 1e-11)
    _close(r["forces"], gold[f"{name}/forces"], 1e-11)
    _close(r["virial"], gold[f"{name}/virial"], 1e-11)


@pytest.mark.parametrize("name", CASES)
def test_c_oracle_matches_reference_pair_style(gold, name):
    from oracle import cfast
    cell, sp, pos, st, beta, power = fixtures.beta_case(name)
    r = cfast.beta_form(cell, sp, pos, st, beta, power=power)
    _close(r["atom_energies"], gold[f"{name}/atom_energies"], 1e-11)
    _close(r["forces"], gold[f"{name}/forces"], 1e-11)
    vol = abs(np.linalg.det(np.asarray(cell)))
    _close(r["stress"], _flare_stress_from_virial(gold[f"{name}/virial"], vol), 1e-11)


@pytest.mark.parametrize("name", CASES)
def test_oracle_single_bond_b2_and_u_match_reference(gold, name):
    cell, sp, pos, st, beta, power = fixtures.beta_case(name)
    ns, N, lmax = st["n_species"], st["N"], st["lmax"]
    o = OStructure(cell, sp, pos, float(np.max(st["cutoffs"])))
    sbd = single_bond_multiple_cutoffs(o, ns, N, lmax, st["r1"], st["cutoffs"],
                                       st["cutoff_function"], store_dervs=False)
    c = sbd["c"]
    b2 = compute_b2(c, ns, N, lmax)
    p, norms = b2["p"], b2["norms"]
    rec = gold[f"{name}/rec_single_bond"].shape[0]
    idx = np.arange(rec)           # the listed atoms are 0..noa-1 in order
    _close(c[idx], gold[f"{name}/rec_single_bond"], 1e-12)
    _close(p[idx], gold[f"{name}/rec_b2"], 1e-12)
    # E_i and u of compute_energy_and_u (lammps_descriptor.cpp:250-304)
    q = norms[idx] ** 2
    w = np.zeros((rec, p.shape[1]))
    E = np.zeros(rec)
    for k, i in enumerate(idx):
        B = beta[int(sp[i])]
        if power == 2:
            bp = B @ p[i]
            E[k] = p[i] @ bp / q[k]
            w[k] = 2 * (bp - E[k] * p[i]) / q[k]
        else:
            E[k] = p[i] @ B / np.sqrt(q[k])
            w[k] = B / np.sqrt(q[k]) - E[k] * p[i] / q[k]
    u = opred.b2_adjoint(c[idx], w, ns, N, lmax)
    _close(E, gold[f"{name}/rec_energy"], 1e-11)
    _close(u, gold[f"{name}/rec_u"], 1e-11)
