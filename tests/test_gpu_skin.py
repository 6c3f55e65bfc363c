"""Neighbor reuse within a skin (fpp_structure_set_skin): over an MD-like
sequence of small displacements, with an atom crossing the periodic boundary
while the list is reused, the mapped prediction through the reused list
equals the prediction on a fresh structure whose list is built at the cutoff
(FP64: 1e-10 relative; mixed: within the mixed form's own reproducibility),
the list is rebuilt only when an atom has moved more than skin / 2, and the
kernel-form mean (FP64) agrees as well."""
import numpy as np
import pytest

import flare_pp_gb300 as fg
from flare_pp_gb300 import synth
from oracle.b2 import B2 as OB2
from tests import fixtures

pytestmark = pytest.mark.gpu

RC = 5.0
SKIN = 0.6


@pytest.fixture(scope="module")
def model():
    ob = OB2("chebyshev", "quadratic", [0, RC], [], [2, 6, 3])
    frames = [synth.bcc_alloy((5, 5, 5), 930 + k) for k in range(2)]
    fit = fixtures.site_energy_model(ob, frames, 60, sigma=2.0, power=2, seed=5)
    gp, _ = fixtures.to_gpu_model((2, 6, 3, RC), fit["sparse"], fit["alpha"], 2.0, 2)
    return gp


def _trajectory(n_steps=8, seed=41):
    cell, sp, pos = synth.bcc_alloy((6, 6, 6), seed)
    rng = np.random.default_rng(seed)
    # atom 0 sits just inside the cell's lower x face and walks out of it
    pos = pos.copy()
    pos[0, 0] = 0.02
    frames = [pos]
    for k in range(n_steps):
        step = rng.normal(scale=0.02, size=pos.shape)
        step[0] = [-0.05, 0.0, 0.0]
        pos = pos + step
        frames.append(pos)
    return cell, sp, frames


def _compare(gp, reused, fresh, prec, tol_e, tol_f):
    e1, f1, s1 = gp.predict_mapped(reused, prec)
    e2, f2, s2 = gp.predict_mapped(fresh, prec)
    n = reused.noa
    assert abs(e1 - e2) / n <= tol_e, (prec, e1, e2)
    assert np.abs(f1 - f2).max() <= tol_f, (prec, np.abs(f1 - f2).max())
    assert np.abs(s1 - s2).max() <= tol_f, (prec, np.abs(s1 - s2).max())


def test_reused_list_matches_fresh_builds(gpu_lib, model):
    cell, sp, frames = _trajectory()
    s = fg.Structure(cell, sp, frames[0], RC)
    s.set_skin(SKIN)
    b0, r0, cut = s.neighbor_stats()
    assert cut == pytest.approx(RC + SKIN)
    start = frames[0]
    for k, pos in enumerate(frames[1:], 1):
        s.set_positions(pos)
        fresh = fg.Structure(cell, sp, pos, RC)
        _compare(model, s, fresh, "fp64", 1e-12, 1e-10)
        _compare(model, s, fresh, "mixed", 1e-6, 1e-4)
        moved = np.linalg.norm(pos - start, axis=1).max()
        b, r, _ = s.neighbor_stats()
        if moved > SKIN / 2:   # a rebuild happened at or before this step
            start = pos
        assert b + r == b0 + r0 + k
    b, r, _ = s.neighbor_stats()
    assert r >= 3 and b >= b0 + 1   # reused on most steps, rebuilt when needed
    # atom 0 left the cell through its x face while the list was reused
    assert frames[-1][0, 0] < 0


def test_rebuild_after_large_move_and_skin_off(gpu_lib, model):
    cell, sp, frames = _trajectory(n_steps=2, seed=43)
    s = fg.Structure(cell, sp, frames[0], RC)
    s.set_skin(SKIN)
    b0, r0, _ = s.neighbor_stats()
    far = frames[0].copy()
    far[5] += [SKIN, 0.0, 0.0]            # one atom beyond skin / 2
    s.set_positions(far)
    b, r, _ = s.neighbor_stats()
    assert (b, r) == (b0 + 1, r0)
    fresh = fg.Structure(cell, sp, far, RC)
    _compare(model, s, fresh, "fp64", 1e-12, 1e-10)
    s.set_skin(0.0)
    b1, r1, cut = s.neighbor_stats()
    assert cut == pytest.approx(RC)
    s.set_positions(frames[1])
    b2, r2, _ = s.neighbor_stats()
    assert (b2, r2) == (b1 + 1, r1)
    np.testing.assert_array_equal(s.neighbor_count,
                                  fg.Structure(cell, sp, frames[1], RC).neighbor_count)


def test_kernel_form_through_reused_list(gpu_lib, model):
    cell, sp, frames = _trajectory(n_steps=3, seed=47)
    s = fg.Structure(cell, sp, frames[0], RC)
    s.set_skin(SKIN)
    for pos in frames[1:]:
        s.set_positions(pos)
    assert s.neighbor_stats()[1] >= 1
    fresh = fg.Structure(cell, sp, frames[-1], RC)
    model.predict_mean(s)
    model.predict_mean(fresh)
    scale = np.abs(fresh.mean_efs).max()
    np.testing.assert_allclose(s.mean_efs, fresh.mean_efs, rtol=0, atol=1e-10 * scale)
