"""Mapped-beta potential files written by the reference.

The reference ships two potential files in the older layout (no power line,
one cutoff for every species pair): lammps_plugins/test_compute/Si.txt (one
species, N = 8, lmax = 4, quadratic cutoff) and beta.txt (two species, N = 3,
lmax = 3, cosine cutoff).  flare_pp_gb300.potential.read_potential reads
them; the oracle's pair style evaluated with their coefficients matches the
reference's own pair-style math (lammps_descriptor.cpp, compiled into
oracle/_ref/libflare_ref.so) on a rattled diamond-silicon cell.  Those checks
need the reference tree ($FLARE_PP_REFERENCE, default /root/reference) and
skip without it; the layout check below runs everywhere.
"""
import ctypes
import os

import numpy as np
import pytest

from flare_pp_gb300.potential import read_potential
from oracle import predict as opred
from oracle.geometry import Structure as OStructure
from tests import fixtures

REF = os.environ.get("FLARE_PP_REFERENCE", "/root/reference")
TC = os.path.join(REF, "lammps_plugins", "test_compute")
REF_LIB = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                       "oracle", "_ref", "libflare_ref.so")


def test_older_layout_is_read(tmp_path):
    fn = tmp_path / "old.txt"
    beta = np.arange(1, 1 + 2 * 21, dtype=float).reshape(2, 21) * 1e-3   # n_d = 6
    with open(fn, "w") as f:
        f.write("DATE: x CONTRIBUTOR: y\nchebyshev\n2 1 1 21\ncosine\n4.50\n")
        for row in beta:
            for k in range(0, 21, 5):
                f.write(" ".join(f"{v:.16e}" for v in row[k:k + 5]) + "\n")
    p = read_potential(fn)
    assert p["legacy"] and p["power"] == 2 and p["cutoff_function"] == "cosine"
    assert p["n_species"] == 2 and p["n_max"] == 1 and p["l_max"] == 1
    np.testing.assert_array_equal(p["cutoffs"], np.full(4, 4.5))
    np.testing.assert_array_equal(p["beta"], beta)


def _diamond_si(reps=2, rattle=0.1, seed=17, n_species=1):
    a = 5.431
    base = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                     [.25, .25, .25], [.25, .75, .75], [.75, .25, .75], [.75, .75, .25]])
    cells = np.array([[i, j, k] for i in range(reps) for j in range(reps) for k in range(reps)])
    pos = ((cells[:, None, :] + base[None, :, :]).reshape(-1, 3)) * a
    rng = np.random.default_rng(seed)
    pos = pos + rng.normal(scale=rattle, size=pos.shape)
    sp = rng.integers(0, n_species, len(pos))
    return np.eye(3) * a * reps, sp, pos


def _reference_pair_style(cell, sp, pos, st, beta, power):
    lib = ctypes.CDLL(REF_LIB)
    D, I = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
    cut = np.ascontiguousarray(st["cutoffs"], dtype=np.float64)
    x, types, ilist, numneigh, nbrs, owner = fixtures.lammps_arrays(cell, sp, pos,
                                                                    float(cut.max()))
    x = np.ascontiguousarray(x, dtype=np.float64)
    types, ilist, numneigh, nbrs = (np.ascontiguousarray(v, dtype=np.int32)
                                    for v in (types, ilist, numneigh, nbrs))
    noa, nall = len(sp), len(x)
    off = np.zeros(noa + 1, dtype=np.int32)
    off[1:] = np.cumsum(numneigh)
    B = np.ascontiguousarray(np.stack(beta), dtype=np.float64)
    f, eat, vir = np.zeros((nall, 3)), np.zeros(nall), np.zeros(6)
    z = np.zeros(1)
    rc = lib.ref_pair_flare(nall, x.ctypes.data_as(D), types.ctypes.data_as(I), noa,
                            ilist.ctypes.data_as(I), numneigh.ctypes.data_as(I),
                            off.ctypes.data_as(I), nbrs.ctypes.data_as(I), st["n_species"],
                            st["N"], st["lmax"], ctypes.c_double(0.0), cut.ctypes.data_as(D),
                            st["cutoff_function"].encode(), power, B.ctypes.data_as(D),
                            f.ctypes.data_as(D), eat.ctypes.data_as(D),
                            vir.ctypes.data_as(D), 0, z.ctypes.data_as(D),
                            z.ctypes.data_as(D), z.ctypes.data_as(D), z.ctypes.data_as(D))
    assert rc == 0
    F = np.zeros((noa, 3))
    np.add.at(F, owner, f)
    return eat[:noa], F, vir


@pytest.mark.parametrize("name,n_species", [("Si.txt", 1), ("beta.txt", 2)])
def test_reference_potential_files(name, n_species):
    fn = os.path.join(TC, name)
    if not os.path.exists(fn):
        pytest.skip("the reference tree is not present")
    p = read_potential(fn)
    assert p["legacy"] and p["power"] == 2 and p["n_species"] == n_species
    n_rad = p["n_species"] * p["n_max"]
    n_d = n_rad * (n_rad + 1) // 2 * (p["l_max"] + 1)
    assert p["beta"].shape == (n_species, n_d * (n_d + 1) // 2)
    ns = p["n_species"]
    st = fixtures.settings(ns, p["n_max"], p["l_max"], float(p["cutoffs"].max()),
                           cutoffs=p["cutoffs"].reshape(ns, ns),
                           cutoff_function=p["cutoff_function"])
    B = opred.unpack_beta(p["beta"], n_d)
    cell, sp, pos = _diamond_si(n_species=ns)
    mine = opred.beta_form(OStructure(cell, sp, pos, float(p["cutoffs"].max())), st, B)
    assert np.isfinite(mine["energy"]) and np.abs(mine["forces"]).max() > 0
    if not os.path.exists(REF_LIB):
        pytest.skip("oracle/_ref/libflare_ref.so not built")
    eat, F, vir = _reference_pair_style(cell, sp, pos, st, B, 2)
    scale = lambda a: 1e-11 * max(np.abs(a).max(), 1e-300)
    np.testing.assert_allclose(mine["atom_energies"], eat, rtol=0, atol=scale(eat))
    np.testing.assert_allclose(mine["forces"], F, rtol=0, atol=scale(F))
    np.testing.assert_allclose(mine["virial"], vir, rtol=0, atol=scale(vir))
