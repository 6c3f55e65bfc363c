"""Host-side checks that need no GPU: the C ABI library loads and exports
every declared symbol; argument errors are reported before any device work;
potential files round-trip."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "flare_pp_gb300.h")).read()
    return sorted(set(re.findall(r"\b(fpp_[A-Za-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from flare_pp_gb300 import build, _lib
    build.build()
    return _lib.lib()


def test_exports_every_declared_symbol(lib):
    names = _declared()
    assert "fpp_pair_compute" in names and "fpp_predict_mapped" in names
    raw = ctypes.CDLL(os.path.join(ROOT, "flare_pp_gb300", "libflare_pp_gb300.so"))
    for n in names:
        assert hasattr(raw, n), n
    from flare_pp_gb300._lib import SIGNATURES
    assert sorted(SIGNATURES) == names


def test_version(lib):
    assert lib.fpp_version() == 1


def test_b2_argument_errors(lib):
    from flare_pp_gb300 import _lib
    h = ctypes.c_void_p()
    rh = np.array([0.0, 5.0])
    ds = np.array([1, 8, 3], dtype=np.int32)
    rc = lib.fpp_b2_create(b"bessel", b"quadratic", rh.ctypes.data, 2, None, 0,
                           ds.ctypes.data, None, ctypes.byref(h))
    assert rc == _lib.FPP_ERR_UNSUPPORTED
    assert b"bessel" in lib.fpp_last_error()
    ds2 = np.array([1, 8, 12], dtype=np.int32)
    rc = lib.fpp_b2_create(b"chebyshev", b"quadratic", rh.ctypes.data, 2, None, 0,
                           ds2.ctypes.data, None, ctypes.byref(h))
    assert rc == _lib.FPP_ERR_CAPACITY
    rc = lib.fpp_b2_create(b"chebyshev", b"quadratic", rh.ctypes.data, 2, None, 0,
                           ds.ctypes.data, None, ctypes.byref(h))
    assert rc == 0
    n = ctypes.c_int32()
    assert lib.fpp_b2_n_descriptors(h, ctypes.byref(n)) == 0
    assert n.value == 8 * 9 // 2 * 4
    lib.fpp_b2_destroy(h)


def test_structure_rejects_bad_input_before_device_work(lib):
    from flare_pp_gb300 import _lib
    h = ctypes.c_void_p()
    cell = np.eye(3) * 10
    sp = np.zeros(2, dtype=np.int32)
    pos = np.array([[0.0, 0, 0], [np.nan, 1, 1]])
    rc = lib.fpp_structure_create(cell.ctypes.data, sp.ctypes.data, pos.ctypes.data,
                                  2, 5.0, None, ctypes.byref(h))
    assert rc == _lib.FPP_ERR_NUMERIC
    pos[1, 0] = 1.0
    rc = lib.fpp_structure_create(cell.ctypes.data, sp.ctypes.data, pos.ctypes.data,
                                  2, -1.0, None, ctypes.byref(h))
    assert rc == _lib.FPP_ERR_INVALID
    sp[0] = -3
    rc = lib.fpp_structure_create(cell.ctypes.data, sp.ctypes.data, pos.ctypes.data,
                                  2, 5.0, None, ctypes.byref(h))
    assert rc == _lib.FPP_ERR_INVALID


def test_potential_file_round_trip(tmp_path):
    from flare_pp_gb300.potential import read_potential, write_potential
    ns, N, lmax = 2, 3, 2
    n_d = (ns * N) * (ns * N + 1) // 2 * (lmax + 1)
    beta = np.random.default_rng(1).normal(size=(ns, n_d * (n_d + 1) // 2))
    fn = tmp_path / "pot.txt"
    write_potential(fn, beta, 2, ns, N, lmax, np.full((ns, ns), 4.5))
    p = read_potential(fn)
    assert p["power"] == 2 and p["n_species"] == 2 and p["beta_size"] == beta.shape[1]
    np.testing.assert_allclose(p["beta"], beta, rtol=1e-15)
    np.testing.assert_allclose(p["cutoffs"], 4.5)
    bad = tmp_path / "bad.txt"
    write_potential(bad, beta[:, :-1], 2, ns, N, lmax, np.full((ns, ns), 4.5))
    with pytest.raises(ValueError):
        read_potential(bad)


def test_std_atom_argument_errors(lib):
    """The compute flare/std/atom entry points check their arguments before
    any device work: a model without coefficients, the power-1 restriction of
    the variance map, a missing output."""
    from flare_pp_gb300 import _lib
    h = ctypes.c_void_p()
    rh = np.array([0.0, 5.0])
    ds = np.array([1, 4, 2], dtype=np.int32)
    assert lib.fpp_b2_create(b"chebyshev", b"quadratic", rh.ctypes.data, 2, None, 0,
                             ds.ctypes.data, None, ctypes.byref(h)) == 0
    m = ctypes.c_void_p()
    assert lib.fpp_model_create(h, 1.5, 2.0, ctypes.byref(m)) == 0
    x = np.zeros((1, 3))
    t = np.ones(1, dtype=np.int32)
    il = np.zeros(1, dtype=np.int32)
    nn = np.zeros(1, dtype=np.int32)
    out = np.zeros(1)
    for use_map, msg in ((1, b"variance map"), (0, b"L_inv")):
        rc = lib.fpp_std_atom_compute(m, 1, 1, x.ctypes.data, t.ctypes.data, 1,
                                      il.ctypes.data, nn.ctypes.data, None, use_map,
                                      out.ctypes.data, None)
        assert rc == _lib.FPP_ERR_INVALID and msg in lib.fpp_last_error()
    assert lib.fpp_model_compute_varmap(m, None, None) == _lib.FPP_ERR_UNSUPPORTED
    assert b"power 1 only" in lib.fpp_last_error()
    assert lib.fpp_model_set_L_inv(m, 3, out.ctypes.data) == _lib.FPP_ERR_INVALID
    assert lib.fpp_model_set_varmap(m, None) == _lib.FPP_ERR_INVALID
    lib.fpp_model_destroy(m)
    lib.fpp_b2_destroy(h)


def test_new_entry_points_reject_bad_arguments(lib):
    """The tensor-core FP64 GEMM, batched prediction, neighbor skin and Kuf
    instrumentation entry points report argument errors before device work."""
    from flare_pp_gb300 import _lib
    A = np.zeros((4, 8))
    C = np.zeros((4, 4))
    # negative sizes, leading dimensions below K / N
    assert lib.fpp_dgemm_nt(-1, 4, 8, A.ctypes.data, 8, A.ctypes.data, 8, C.ctypes.data, 4,
                            0, None) == _lib.FPP_ERR_INVALID
    assert lib.fpp_dgemm_nt(4, 4, 8, A.ctypes.data, 4, A.ctypes.data, 8, C.ctypes.data, 4,
                            0, None) == _lib.FPP_ERR_INVALID
    assert lib.fpp_dgemm_nt(4, 4, 8, A.ctypes.data, 8, A.ctypes.data, 8, C.ctypes.data, 2,
                            0, None) == _lib.FPP_ERR_INVALID
    assert lib.fpp_dgemm_nt(4, 4, 8, None, 8, A.ctypes.data, 8, C.ctypes.data, 4,
                            0, None) == _lib.FPP_ERR_INVALID
    # empty products need no device: M = 0 is a no-op, K = 0 writes zeros
    assert lib.fpp_dgemm_nt(0, 4, 8, None, 8, None, 8, None, 4, 0, None) == 0
    C[:] = 7.0
    assert lib.fpp_dgemm_nt(4, 4, 0, A.ctypes.data, 1, A.ctypes.data, 1, C.ctypes.data, 4,
                            0, None) == 0
    assert (C == 0).all()
    # batched prediction, skin, Kuf statistics
    assert lib.fpp_predict_mapped_batched(None, None, 1, 0, None, None, None, None) == \
        _lib.FPP_ERR_INVALID
    assert lib.fpp_structure_set_skin(None, 0.5, None) == _lib.FPP_ERR_INVALID
    assert lib.fpp_structure_neighbor_stats(None, None, None, None) == _lib.FPP_ERR_INVALID
    assert lib.fpp_model_kuf_tiles(None, None, None, None, None) == _lib.FPP_ERR_INVALID
