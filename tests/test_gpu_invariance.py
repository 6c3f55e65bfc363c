"""Size-independent properties of the GPU path (the reference's own checks,
ctests/test_descriptor.cpp:9-48, rotation invariance at 1e-10): B2 and B3
descriptors of a rotated structure (cell and positions rotated together) equal
the unrotated ones; the mapped prediction's energy is invariant under rotation
and translation, its forces rotate with the structure and its stress as
R sigma R^T (FP64 to 1e-10; the mixed form to its own tolerance)."""
import numpy as np
import pytest

import flare_pp_gb300 as fg
from flare_pp_gb300 import synth
from oracle.b2 import B2 as OB2
from tests import fixtures

pytestmark = pytest.mark.gpu

RC = 5.0


def _rotation(a=0.7, b=1.1, c=-0.4):
    Rz = np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])
    Rx = np.array([[1, 0, 0], [0, np.cos(b), -np.sin(b)], [0, np.sin(b), np.cos(b)]])
    Ry = np.array([[np.cos(c), 0, np.sin(c)], [0, 1, 0], [-np.sin(c), 0, np.cos(c)]])
    return Ry @ Rx @ Rz


def _small_structure(rot=None):
    rng = np.random.default_rng(11)
    cell = np.array([[6.6, 0.1, 0.0], [0.2, 6.9, 0.0], [0.0, 0.3, 7.1]])
    pos = rng.uniform(0, 6.5, size=(10, 3))
    sp = rng.integers(0, 2, size=10).astype(np.int32)
    if rot is not None:
        cell, pos = cell @ rot.T, pos @ rot.T
    return cell, sp, pos


@pytest.mark.parametrize("kind", ["B2", "B3"])
def test_descriptors_rotation_invariant(gpu_lib, kind):
    make = fg.B3 if kind == "B3" else fg.B2
    d = make("chebyshev", "quadratic", [0, 3.8], [], [2, 3, 3])
    p0 = fg.Structure(*_small_structure(), 4.0, [d]).descriptors[0]
    p1 = fg.Structure(*_small_structure(_rotation()), 4.0, [d]).descriptors[0]
    for s in range(2):
        np.testing.assert_allclose(p1.descriptors[s], p0.descriptors[s], rtol=0, atol=1e-10)
        np.testing.assert_allclose(p1.descriptor_norms[s], p0.descriptor_norms[s], rtol=1e-12)


@pytest.fixture(scope="module")
def model():
    ob = OB2("chebyshev", "quadratic", [0, RC], [], [2, 6, 3])
    frames = [synth.bcc_alloy((5, 5, 5), 960 + k, a=3.4) for k in range(2)]
    fit = fixtures.site_energy_model(ob, frames, 60, sigma=2.0, power=2, seed=9)
    gp, _ = fixtures.to_gpu_model((2, 6, 3, RC), fit["sparse"], fit["alpha"], 2.0, 2)
    return gp


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-4)])
def test_mapped_prediction_rotates_and_translates(gpu_lib, model, precision, tol):
    cell, sp, pos = synth.bcc_alloy((5, 5, 5), 961, a=3.4)
    cell = np.asarray(cell, float)
    R = _rotation()
    e0, f0, s0 = model.predict_mapped(fg.Structure(cell, sp, pos, RC), precision)
    # rotation: cell and positions together
    e1, f1, s1 = model.predict_mapped(fg.Structure(cell @ R.T, sp, pos @ R.T, RC), precision)
    # translation by a vector that moves atoms across the cell faces
    t = np.array([1.3, -0.7, 2.9])
    e2, f2, s2 = model.predict_mapped(fg.Structure(cell, sp, pos + t, RC), precision)
    n = len(sp)
    fs = max(1.0, np.abs(f0).max())
    assert abs(e1 - e0) / n <= tol and abs(e2 - e0) / n <= tol, (e0, e1, e2)
    np.testing.assert_allclose(f1, f0 @ R.T, rtol=0, atol=tol * fs)
    np.testing.assert_allclose(f2, f0, rtol=0, atol=tol * fs)
    # stress in flare order xx xy xz yy yz zz
    def full(s):
        return np.array([[s[0], s[1], s[2]], [s[1], s[3], s[4]], [s[2], s[4], s[5]]])
    ss = max(1e-3, np.abs(s0).max())
    np.testing.assert_allclose(full(s1), R @ full(s0) @ R.T, rtol=0, atol=tol * ss)
    np.testing.assert_allclose(s2, s0, rtol=0, atol=tol * ss)
