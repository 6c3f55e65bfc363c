"""The allocation-free B2 entry point, through the C ABI.

fpp_b2_descriptors_noalloc exists for callers that may not allocate device
memory when they need descriptors: an MD engine whose memory pool owns the
GPU (nothing may be cudaMalloc'd behind its back), or a loop with a fixed
memory budget.  Its scratch is a fixed array inside the library, shared by
every call and keeping the last call's contents.  These checks run it twice in
a row on different structures and compare each result with the regular
fpp_b2_compute entry point (FP64, relative 1e-12), so that a call reading the
previous call's scratch would show up; they check that a warm call leaves the
device's free memory unchanged, and the size limit.  The file is collected
last on purpose and also passes on its own.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_inputs(structure, b2):
    import torch
    nb = structure._neighbors()
    cnt, off = nb["neighbor_count"], nb["cumulative_neighbor_count"]
    rel = nb["relative_positions"]
    nsp = nb["neighbor_species"]
    dev = torch.device("cuda")
    t = dict(species=torch.tensor(np.asarray(structure.species, np.int32), device=dev),
             offsets=torch.tensor(off.astype(np.int32), device=dev),
             rel=torch.tensor(rel, dtype=torch.float64, device=dev).contiguous(),
             nbr_species=torch.tensor(nsp.astype(np.int32), device=dev))
    return t


def _noalloc(lib, b2, structure):
    import torch
    t = _device_inputs(structure, b2)
    n = structure.noa
    desc = torch.full((n, b2.n_descriptors), np.nan, dtype=torch.float64, device="cuda")
    norms = torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
    rc = lib.fpp_b2_descriptors_noalloc(
        b2._h, n, t["species"].data_ptr(), t["offsets"].data_ptr(), t["rel"].data_ptr(),
        t["nbr_species"].data_ptr(), desc.data_ptr(), norms.data_ptr(), None)
    assert rc == 0, lib.fpp_last_error()
    torch.cuda.synchronize()
    return desc.cpu().numpy(), norms.cpu().numpy()


def _regular(lib, b2, structure):
    from flare_pp_gb300._lib import ptr
    n = structure.noa
    desc = np.zeros((n, b2.n_descriptors))
    norms = np.zeros(n)
    assert lib.fpp_b2_compute(b2._h, structure.handle, ptr(desc), ptr(norms), None, None,
                              None, None, None, None) == 0
    return desc, norms


def test_noalloc_matches_regular_entry_point_twice():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("needs a CUDA device")
    import flare_pp_gb300 as fg
    from flare_pp_gb300 import synth, _lib
    lib = _lib.lib()
    cut = np.array([[5.5, 5.0], [5.0, 5.2]])
    b2 = fg.B2("chebyshev", "quadratic", [0.0, 5.5], [], [2, 6, 3], cut)
    cases = [synth.bcc_alloy((4, 4, 4), 11), synth.bcc_alloy((5, 4, 3), 12)]
    for cell, sp, pos in cases:          # two calls in a row, different inputs
        s = fg.Structure(cell, sp, pos, 5.5)
        d0, n0 = _regular(lib, b2, s)
        d1, n1 = _noalloc(lib, b2, s)
        np.testing.assert_allclose(d1, d0, rtol=0, atol=1e-12 * np.abs(d0).max())
        np.testing.assert_allclose(n1, n0, rtol=1e-12)


def test_noalloc_warm_call_leaves_free_memory_unchanged():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("needs a CUDA device")
    import flare_pp_gb300 as fg
    from flare_pp_gb300 import synth, _lib
    lib = _lib.lib()
    b2 = fg.B2("chebyshev", "quadratic", [0.0, 5.5], [], [2, 6, 3])
    cell, sp, pos = synth.bcc_alloy((4, 4, 4), 13)
    s = fg.Structure(cell, sp, pos, 5.5)
    t = _device_inputs(s, b2)
    n = s.noa
    desc = torch.empty((n, b2.n_descriptors), dtype=torch.float64, device="cuda")
    norms = torch.empty((n,), dtype=torch.float64, device="cuda")

    def call():
        rc = lib.fpp_b2_descriptors_noalloc(
            b2._h, n, t["species"].data_ptr(), t["offsets"].data_ptr(), t["rel"].data_ptr(),
            t["nbr_species"].data_ptr(), desc.data_ptr(), norms.data_ptr(), None)
        assert rc == 0, lib.fpp_last_error()
        torch.cuda.synchronize()

    call()                                   # first call: one-time set-up, module load
    free0, _ = torch.cuda.mem_get_info()
    call()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("needs a CUDA device")
    import flare_pp_gb300 as fg
    from flare_pp_gb300 import _lib
    lib = _lib.lib()
    b2 = fg.B2("chebyshev", "quadratic", [0.0, 5.0], [], [2, 12, 4])   # 600 per atom
    dummy = torch.zeros(64, dtype=torch.float64, device="cuda")
    rc = lib.fpp_b2_descriptors_noalloc(b2._h, 2000, dummy.data_ptr(), dummy.data_ptr(),
                                        dummy.data_ptr(), dummy.data_ptr(),
                                        dummy.data_ptr(), dummy.data_ptr(), None)
    assert rc == _lib.FPP_ERR_CAPACITY
    assert b"at most" in lib.fpp_last_error()
