"""Neighbor rebuilds of one structure handle across set_positions calls.

The pair compaction of a rebuild is queued into the pair buffers of the
previous build before the host has read the new pair total; it writes nothing
and is launched again when the total outgrew those buffers (they keep an
eighth of headroom).  Three rebuilds cover both paths: a compression that
raises the pair count 1.7-fold (relaunch), the original positions again (fewer
pairs: the queued compaction stands) and a small displacement (the same).
After each, the neighbor list (counts, order, indices, species and the FP64
pair vectors of structure.cpp:52-118) equals that of a fresh structure at the
same positions bit for bit, and so do the mapped predictions."""
import numpy as np
import pytest

import flare_pp_gb300 as fg
from flare_pp_gb300 import synth
from oracle.b2 import B2 as OB2
from tests import fixtures

pytestmark = pytest.mark.gpu

RC = 5.0


@pytest.fixture(scope="module")
def model():
    ob = OB2("chebyshev", "quadratic", [0, RC], [], [2, 6, 3])
    frames = [synth.bcc_alloy((5, 5, 5), 950 + k) for k in range(2)]
    fit = fixtures.site_energy_model(ob, frames, 60, sigma=2.0, power=2, seed=7)
    gp, _ = fixtures.to_gpu_model((2, 6, 3, RC), fit["sparse"], fit["alpha"], 2.0, 2)
    return gp


def _same_lists(a, b):
    assert a.n_neighbors == b.n_neighbors
    np.testing.assert_array_equal(a.neighbor_count, b.neighbor_count)
    np.testing.assert_array_equal(a.cumulative_neighbor_count, b.cumulative_neighbor_count)
    np.testing.assert_array_equal(a.structure_indices, b.structure_indices)
    np.testing.assert_array_equal(a.neighbor_species, b.neighbor_species)
    np.testing.assert_array_equal(a.relative_positions, b.relative_positions)


def _same_predictions(gp, a, b):
    for prec in ("fp64", "mixed"):
        e1, f1, s1 = gp.predict_mapped(a, prec)
        e2, f2, s2 = gp.predict_mapped(b, prec)
        assert e1 == e2, prec
        np.testing.assert_array_equal(f1, f2)
        np.testing.assert_array_equal(s1, s2)


def test_rebuilds_grow_and_shrink(gpu_lib, model):
    cell, sp, pos = synth.bcc_alloy((6, 6, 6), 951)
    s = fg.Structure(cell, sp, pos, RC)
    n0 = s.n_neighbors
    centre = 0.5 * np.sum(np.asarray(cell), axis=0)
    squeezed = centre + 0.7 * (pos - centre)   # 1.7x the pairs
    rng = np.random.default_rng(952)
    nudged = pos + rng.normal(scale=0.01, size=pos.shape)
    for new, grows in ((squeezed, True), (pos, False), (nudged, False)):
        s.set_positions(new)
        fresh = fg.Structure(cell, sp, new, RC)
        if grows:
            assert s.n_neighbors > 1.2 * n0   # beyond the eighth of headroom
        _same_lists(s, fresh)
        _same_predictions(model, s, fresh)
