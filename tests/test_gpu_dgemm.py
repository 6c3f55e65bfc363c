"""fpp_dgemm_nt, the FP64-accurate C = A B^T on the fp16 tensor cores (exact
5-bit digit planes, FP32 level sums exact below 2^24, FP64 recombination),
against numpy's FP64 matmul.

Bound checked: |C - A B^T| <= 2^-50 * K^(1/2) * max|a_i| * max|b_j| + 2^-50 *
(|A| |B|^T), i.e. the digit truncation (55 bits of each operand relative to
its row's largest entry, random-walk over K) plus numpy's own FP64 rounding.
Integer inputs (exactly representable products and sums) must come out
bit-exact."""
import ctypes

import numpy as np
import pytest

from flare_pp_gb300._lib import check

pytestmark = pytest.mark.gpu


def dgemm(lib, A, B):
    A = np.ascontiguousarray(A, dtype=np.float64)
    B = np.ascontiguousarray(B, dtype=np.float64)
    M, K = A.shape
    N = B.shape[0]
    C = np.full((M, N), np.nan)
    check(lib.fpp_dgemm_nt(M, N, K, A.ctypes.data, K, B.ctypes.data, K, C.ctypes.data, N,
                           0, None))
    return C


def within_bound(C, A, B):
    ref = A @ B.T
    K = A.shape[1]
    ra = np.abs(A).max(axis=1)[:, None]
    rb = np.abs(B).max(axis=1)[None, :]
    bound = 2.0 ** -50 * (np.sqrt(K) * ra * rb + np.abs(A) @ np.abs(B).T) + 1e-300
    err = np.abs(C - ref)
    return float((err / bound).max()), float(err.max())


@pytest.mark.parametrize("M,N,K", [(1, 1, 1), (130, 70, 50), (257, 300, 1000),
                                   (128, 128, 1536), (200, 129, 1537), (96, 160, 4000)])
def test_random_matches_fp64(gpu_lib, M, N, K):
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    A = rng.normal(size=(M, K))
    B = rng.normal(size=(N, K)) * 10.0 ** rng.uniform(-3, 3, size=(N, 1))
    C = dgemm(gpu_lib, A, B)
    ratio, err = within_bound(C, A, B)
    assert np.isfinite(C).all()
    assert ratio <= 1.0, (ratio, err)


def test_unit_rows_like_descriptors(gpu_lib):
    """Normalised descriptor rows (non-negative and mixed-sign) at the
    kernel-form shape: z = dhat . phat in [-1, 1] to ~1e-15."""
    rng = np.random.default_rng(5)
    P = np.abs(rng.normal(size=(1000, 1500)))
    P /= np.linalg.norm(P, axis=1, keepdims=True)
    D = rng.normal(size=(700, 1500))
    D /= np.linalg.norm(D, axis=1, keepdims=True)
    Z = dgemm(gpu_lib, P, D)
    ref = P @ D.T
    assert np.abs(Z - ref).max() < 2e-15


def test_integers_are_exact(gpu_lib):
    rng = np.random.default_rng(11)
    A = rng.integers(-2 ** 20, 2 ** 20, size=(300, 700)).astype(np.float64)
    B = rng.integers(-2 ** 20, 2 ** 20, size=(260, 700)).astype(np.float64)
    C = dgemm(gpu_lib, A, B)
    np.testing.assert_array_equal(C, A @ B.T)      # |sums| < 2^50: exact in FP64


def test_zero_rows_and_padding(gpu_lib):
    rng = np.random.default_rng(3)
    A = rng.normal(size=(70, 33))
    A[5] = 0.0
    B = rng.normal(size=(45, 33))
    B[[0, 44]] = 0.0
    C = dgemm(gpu_lib, A, B)
    assert (C[5] == 0).all() and (C[:, 0] == 0).all() and (C[:, 44] == 0).all()
    ratio, _ = within_bound(C, A, B)
    assert ratio <= 1.0


def test_rate_at_kernel_form_shape(gpu_lib):
    """One species block of the 32k variance workload: 16384 atoms x 2000
    sparse environments x n_d 1500, device-resident; prints the FP64-
    equivalent rate (the measured cuBLAS DGEMM rate of this GPU is 1.10
    TFLOP/s)."""
    import torch
    M, N, K = 16384, 2000, 1500
    g = torch.Generator(device="cuda").manual_seed(0)
    A = torch.rand(M, K, dtype=torch.float64, device="cuda", generator=g)
    B = torch.rand(N, K, dtype=torch.float64, device="cuda", generator=g) - 0.5
    C = torch.empty(M, N, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    def run():
        check(gpu_lib.fpp_dgemm_nt(M, N, K, A.data_ptr(), K, B.data_ptr(), K, C.data_ptr(), N,
                                   1, s))
    run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(3):
        run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 3
    ref = A[:256] @ B.T
    err = (C[:256] - ref).abs().max().item()
    print(f"fpp_dgemm_nt {M}x{N}x{K}: {ms:.2f} ms, {2 * M * N * K / ms / 1e9:.1f} "
          f"TFLOP/s FP64-equivalent; max |C - torch FP64| on 256 rows {err:.2e}")
    assert err < 1e-12
