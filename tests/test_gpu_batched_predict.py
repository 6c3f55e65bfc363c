"""fpp_predict_mapped_batched: a batch of uneven structures (a few to a few
hundred atoms, two species, strained and rattled FCC cells) predicted in one
pass of the mapped form equals the structure-by-structure prediction (FP64:
to FP64 rounding; mixed: to the mixed form's own reproducibility), and the
FP64 energies, forces and stresses equal the oracle's beta form."""
import time

import numpy as np
import pytest

import flare_pp_gb300 as fg
from flare_pp_gb300 import synth
from oracle import predict as opred
from oracle.b2 import B2 as OB2
from oracle.geometry import Structure as OStructure
from oracle.kernel import NormalizedDotProduct as ONDP
from tests import fixtures

pytestmark = pytest.mark.gpu

RC = 5.0


@pytest.fixture(scope="module")
def setup():
    ob = OB2("chebyshev", "quadratic", [0, RC], [], [2, 6, 3])
    frames = [synth.bcc_alloy((5, 5, 5), 950 + k, a=3.4) for k in range(2)]
    fit = fixtures.site_energy_model(ob, frames, 60, sigma=2.0, power=2, seed=6)
    gp, gb = fixtures.to_gpu_model((2, 6, 3, RC), fit["sparse"], fit["alpha"], 2.0, 2)
    cells = synth.fcc_batch(n_structures=24, seed=808, lo=4, hi=256)
    strucs = [fg.Structure(c, sp, p, RC) for c, sp, p in cells]
    return dict(gp=gp, fit=fit, cells=cells, strucs=strucs)


@pytest.mark.parametrize("precision,tol_e,tol_f", [("fp64", 1e-12, 1e-11),
                                                   ("mixed", 1e-7, 1e-5)])
def test_batched_equals_per_structure(gpu_lib, setup, precision, tol_e, tol_f):
    gp, strucs = setup["gp"], setup["strucs"]
    E, F, S = gp.predict_mapped_batched(strucs, precision)
    for k, s in enumerate(strucs):
        e, f, st = gp.predict_mapped(s, precision)
        assert abs(E[k] - e) <= tol_e * max(1.0, abs(e)), (k, E[k], e)
        np.testing.assert_allclose(F[k], f, rtol=0, atol=tol_f * max(1.0, np.abs(f).max()))
        np.testing.assert_allclose(S[k], st, rtol=0, atol=tol_f * max(1e-3, np.abs(st).max()))


def test_batched_fp64_matches_oracle(gpu_lib, setup):
    gp, fit, cells, strucs = setup["gp"], setup["fit"], setup["cells"], setup["strucs"]
    E, F, S = gp.predict_mapped_batched(strucs, "fp64")
    st = fixtures.settings(2, 6, 3, RC)
    B = opred.unpack_beta(ONDP(2.0, 2).compute_map_coeff_pow2(fit["sparse"], fit["alpha"]),
                          fit["sparse"].n_descriptors)
    for k in (0, 7, 23):
        cell, sp, pos = cells[k]
        ref = opred.beta_form(OStructure(cell, sp, pos, RC), st, B)
        assert abs(E[k] - ref["energy"]) <= 1e-10 * max(1.0, abs(ref["energy"]))
        np.testing.assert_allclose(F[k], ref["forces"], rtol=0,
                                   atol=1e-9 * max(1.0, np.abs(ref["forces"]).max()))
        np.testing.assert_allclose(S[k], ref["stress"], rtol=0,
                                   atol=1e-9 * max(1e-3, np.abs(ref["stress"]).max()))


def test_batched_timing(gpu_lib, setup):
    gp, strucs = setup["gp"], setup["strucs"]
    gp.predict_mapped_batched(strucs, "mixed")
    t0 = time.perf_counter()
    for _ in range(5):
        gp.predict_mapped_batched(strucs, "mixed")
    tb = (time.perf_counter() - t0) / 5
    t0 = time.perf_counter()
    for _ in range(5):
        for s in strucs:
            gp.predict_mapped(s, "mixed")
    ts = (time.perf_counter() - t0) / 5
    n = sum(s.noa for s in strucs)
    print(f"batched mapped prediction of {len(strucs)} structures ({n} atoms): "
          f"{1e3 * tb:.2f} ms batched, {1e3 * ts:.2f} ms one by one")


def test_batched_b3_equals_per_structure(gpu_lib):
    """A single-species B3 model (N = 4, lmax = 3): the packed batch runs the
    B3 forward and adjoint kernels unchanged."""
    from oracle.b3 import B3 as OB3
    ob = OB3("chebyshev", "quadratic", [0, RC], [], [1, 4, 3])
    frames = [synth.fcc_al_108(515, k) for k in range(2)]
    fit = fixtures.site_energy_model(ob, frames, 40, sigma=2.0, power=2, seed=8)
    gp, _ = fixtures.to_gpu_model((1, 4, 3, RC), fit["sparse"], fit["alpha"], 2.0, 2,
                                  kind="B3")
    rng = np.random.default_rng(3)
    strucs = []
    for k in range(6):
        cell, sp, pos = synth.fcc_al_108(516, k)
        keep = np.sort(rng.choice(len(sp), 20 + 15 * k, replace=False)) if k % 2 else \
            np.arange(len(sp))
        strucs.append(fg.Structure(cell, sp[keep], pos[keep], RC))
    for precision, tol_e, tol_f in (("fp64", 1e-12, 1e-11), ("mixed", 1e-7, 1e-5)):
        E, F, S = gp.predict_mapped_batched(strucs, precision)
        for k, s in enumerate(strucs):
            e, f, st = gp.predict_mapped(s, precision)
            assert abs(E[k] - e) <= tol_e * max(1.0, abs(e)), (precision, k)
            np.testing.assert_allclose(F[k], f, rtol=0,
                                       atol=tol_f * max(1.0, np.abs(f).max()))
            np.testing.assert_allclose(S[k], st, rtol=0,
                                       atol=tol_f * max(1e-3, np.abs(st).max()))


def test_batched_edge_structures(gpu_lib, setup):
    """Empty structures and a single atom whose neighbors are all its own
    periodic images, packed between ordinary cells: each structure's result
    equals its own prediction (an empty one: zero energy, no forces)."""
    gp, strucs = setup["gp"], setup["strucs"]
    empty = fg.Structure(np.eye(3) * 8.0, np.zeros(0, np.int32), np.zeros((0, 3)), RC)
    single = fg.Structure(np.eye(3) * 3.0, np.array([1], np.int32),
                          np.array([[0.3, 0.2, 0.1]]), RC)
    batch = [empty, strucs[0], single, strucs[5], empty]
    for precision, tol in (("fp64", 1e-11), ("mixed", 1e-5)):
        E, F, S = gp.predict_mapped_batched(batch, precision)
        assert E[0] == 0.0 and E[4] == 0.0
        assert F[0].shape == (0, 3) and F[4].shape == (0, 3)
        for k in (1, 2, 3):
            e, f, st = gp.predict_mapped(batch[k], precision)
            assert abs(E[k] - e) <= tol * max(1.0, abs(e)), (precision, k, E[k], e)
            np.testing.assert_allclose(F[k], f, rtol=0, atol=tol * max(1.0, np.abs(f).max()))
            np.testing.assert_allclose(S[k], st, rtol=0, atol=tol * max(1e-3, np.abs(st).max()))
