"""The split GEMM entry point that allocates nothing
(fglsgpu_split_gemm_noalloc), checked against the allocating entry point
(fglsgpu_selftest_split_gemm) through the C ABI.

It exists for callers that may not allocate device memory themselves, e.g.
code running under a framework that owns the whole device through its own
memory pool: they hand in device buffers, and the kernel's scratch comes from
a fixed array inside the library.  Two calls in a row with different shapes
check that the shared array's leftovers from the first call do not leak into
the second.  This file is collected last so that a failure here stops a
run only after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(A, X, slices):
    import torch
    from fgls_gb300.engine import OK, lib
    M, K = A.shape
    N = X.shape[1]
    dA = torch.from_numpy(np.ascontiguousarray(A)).cuda()                # row-major M x K
    dX = torch.from_numpy(np.asfortranarray(X).T.copy()).cuda()          # column-major K x N
    dC = torch.full((N, M), np.nan, dtype=torch.float64, device="cuda")   # column-major M x N
    torch.cuda.synchronize()
    rc = lib().fglsgpu_split_gemm_noalloc(M, K, N, slices, C.c_void_p(dA.data_ptr()), C.c_void_p(dX.data_ptr()),
                                          C.c_void_p(dC.data_ptr()), None)
    assert rc == OK
    return dC.cpu().numpy().T


def test_noalloc_matches_allocating_entry_point_twice():
    from fgls_gb300.engine import split_gemm_selftest
    rng = np.random.default_rng(42)
    cases = [(256, 2048, 512, 9), (77, 300, 129, 6)]  # maximum sizes, then a smaller ragged call
    for M, K, N, S in cases:
        A = rng.standard_normal((M, K)) * np.exp(rng.uniform(-3, 3, size=(M, 1)))
        X = rng.integers(0, 3, size=(K, N)).astype(np.float64)
        ref = split_gemm_selftest(A, X, S)
        got = _noalloc(A, X, S)
        assert np.all(np.isfinite(got))
        # same kernels and arithmetic: identical bits (tolerance 0)
        np.testing.assert_array_equal(got, ref)
        assert np.all(np.abs(got - A @ X) <= 2.0 ** (-5 * S + 4) * (np.abs(A) @ X) + 1e-300)  # 5-bit digits


def test_noalloc_rejects_sizes_beyond_its_array():
    from fgls_gb300.engine import EINVAL, lib
    L = lib()
    for M, K, N, S in [(257, 64, 64, 2), (64, 2049, 64, 2), (64, 64, 513, 2), (64, 64, 64, 10)]:
        assert L.fglsgpu_split_gemm_noalloc(M, K, N, S, C.c_void_p(1), C.c_void_p(1), C.c_void_p(1), None) == EINVAL
