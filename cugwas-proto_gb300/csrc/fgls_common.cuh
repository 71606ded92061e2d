// Shared definitions for the GB300 FGLS engine (sm_103a).
//
// All matrices are column-major FP64 unless stated otherwise, as in the
// reference's on-disk layout (Phi n x n, XL n x wXL, XR blocks n x (x*wXR)).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "fgls_gb300.h"

namespace fgls {

// Device status word written by kernels that can fail on data (a non-SPD
// p x p system, a non-converging iteration, a bounded wait that expired).
// The first failure wins (atomicCAS on code).  Host reads it after a sync.
struct DevStatus {
  int code;      // FGLSGPU_OK or an FGLSGPU_E* code
  int info;      // LAPACK-style info (order of the failing minor, iteration count, ...)
  long long idx; // failing item (SNP index within the block, trait, row ...)
};

__device__ __forceinline__ void set_status(DevStatus* st, int code, int info, long long idx) {
  if (st && atomicCAS(&st->code, FGLSGPU_OK, code) == FGLSGPU_OK) {
    st->info = info;
    st->idx = idx;
  }
}

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Kernel launchers (host side, defined in the .cu files).  All are
// asynchronous on `s` and return cudaError_t of the launch.

// C = alpha * op(A) * op(B) + beta * C   (FP64, column-major, op = N or T)
cudaError_t dgemm(cudaStream_t s, bool transA, bool transB, int M, int N, int K, double alpha,
                  const double* A, long long lda, const double* B, long long ldb, double beta,
                  double* C, long long ldc);
// The same product with K split over CTAs when M x N has too few 64 x 64
// tiles to fill the GPU (partials in work, work_elems doubles, then summed in
// a fixed order); falls back to dgemm when splitting does not apply.
cudaError_t dgemm_splitk(cudaStream_t s, bool transA, bool transB, int M, int N, int K, double alpha,
                         const double* A, long long lda, const double* B, long long ldb, double beta, double* C,
                         long long ldc, double* work, long long work_elems);
// Lower-triangle-only variant (C n x n lower, tiles strictly above the
// diagonal are skipped; entries above the diagonal inside diagonal tiles
// are written too and must be ignored by the caller).
cudaError_t dgemm_lower(cudaStream_t s, bool transA, bool transB, int N, int K, double alpha,
                        const double* A, long long lda, const double* B, long long ldb,
                        double beta, double* C, long long ldc);

// In-place lower Cholesky of the n x n matrix A (only the lower triangle is
// read or written).  If `scale_alpha` is non-null the factored matrix is
// alpha*A + beta*I (the reference's M = h*s*Phi + (1-h)*s*I), built from
// Src's lower triangle into A first.  Returns cudaSuccess or a launch error;
// a non-positive pivot is reported through `st` (info = 1-based column).
cudaError_t dpotrf_lower(cudaStream_t s, int n, double* A, long long lda, DevStatus* st);
cudaError_t build_shifted(cudaStream_t s, int n, const double* Src, long long lds, double alpha,
                          double beta, double* A, long long lda);

// X := L^{-1} X   (L n x n lower, non-unit; X n x nrhs).  Blocked: diagonal
// blocks solved in shared memory, off-diagonal updates through dgemm.
cudaError_t dtrsm_llnn(cudaStream_t s, int n, int nrhs, const double* L, long long ldl, double* X,
                       long long ldx);

}  // namespace fgls

#define FGLS_CUDA_TRY(expr)                                  \
  do {                                                       \
    cudaError_t _e = (expr);                                 \
    if (_e != cudaSuccess) return _e;                        \
  } while (0)
