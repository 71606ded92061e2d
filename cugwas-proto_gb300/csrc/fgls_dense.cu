// FP64 dense kernels for the plain (all-FP64) path: tiled DGEMM, blocked
// lower Cholesky (the reference's dpotrf of M, src/fgls_chol.c:252-271) and
// blocked lower-triangular solve X := L^-1 X (the reference's per-block
// dtrsm, src/fgls_chol.c:365-368 and cublasDtrsm in
// src/fgls_chol_gpu.c:543-555).
//
// GB300 executes FP64 at a small fraction of its FP32/tensor rate, so these
// kernels are FP64-issue-bound by design: tiles are sized to keep the FP64
// pipe fed from shared memory, not to chase memory bandwidth.
#include <algorithm>

#include "fgls_common.cuh"
#include "fgls_kernels.cuh"

namespace fgls {

namespace {

constexpr int GM = 64, GN = 64, GK = 16;  // DGEMM CTA tile
constexpr int GT = 256;                   // threads: 16 x 16, 4 x 4 outputs each

// op(A)(i, k) for column-major A
__device__ __forceinline__ double ldA(const double* A, long long lda, bool tA, int i, int k) {
  return tA ? A[k + (long long)i * lda] : A[i + (long long)k * lda];
}

template <bool TA, bool TB, bool LOWER>
__global__ void __launch_bounds__(GT) dgemm_kernel(int M, int N, int K, double alpha,
                                                   const double* __restrict__ A, long long lda,
                                                   const double* __restrict__ B, long long ldb,
                                                   double beta, double* __restrict__ C,
                                                   long long ldc) {
  const int bi = blockIdx.x, bj = blockIdx.y;
  if (LOWER && bj > bi) return;  // tile strictly above the diagonal (square C, GM == GN)
  if (gridDim.z > 1) {
    // split K: slice z of the K range into its own M x N partial (ldc = M)
    const int kc = (K + (int)gridDim.z - 1) / (int)gridDim.z;
    const int k0 = (int)blockIdx.z * kc;
    K = max(0, min(K - k0, kc));
    A += TA ? (long long)k0 : (long long)k0 * lda;
    B += TB ? (long long)k0 * ldb : (long long)k0;
    C += (long long)blockIdx.z * ldc * N;
  }
  const int i0 = bi * GM, j0 = bj * GN;
  __shared__ double As[2][GK][GM + 1];
  __shared__ double Bs[2][GK][GN + 1];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int b = 0; b < 4; b++) acc[a][b] = 0.0;

  // each thread loads 4 A and 4 B elements per k-tile
  double ra[4], rb[4];
  auto load_regs = [&](int k0) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
      int e = tid + r * GT;  // 0..1023 over a GM x GK tile
      int ii, kk;
      if (!TA) { ii = e % GM; kk = e / GM; } else { kk = e % GK; ii = e / GK; }
      int gi = i0 + ii, gk = k0 + kk;
      ra[r] = (gi < M && gk < K) ? ldA(A, lda, TA, gi, gk) : 0.0;
      int jj, kb;
      if (!TB) { kb = e % GK; jj = e / GK; } else { jj = e % GN; kb = e / GN; }
      int gj = j0 + jj, gkb = k0 + kb;
      double v = 0.0;
      if (gj < N && gkb < K) v = TB ? B[gj + (long long)gkb * ldb] : B[gkb + (long long)gj * ldb];
      rb[r] = v;
    }
  };
  auto store_smem = [&](int buf) {
#pragma unroll
    for (int r = 0; r < 4; r++) {
      int e = tid + r * GT;
      int ii, kk;
      if (!TA) { ii = e % GM; kk = e / GM; } else { kk = e % GK; ii = e / GK; }
      As[buf][kk][ii] = ra[r];
      int jj, kb;
      if (!TB) { kb = e % GK; jj = e / GK; } else { jj = e % GN; kb = e / GN; }
      Bs[buf][kb][jj] = rb[r];
    }
  };

  const int nk = (K + GK - 1) / GK;
  if (nk > 0) {
    load_regs(0);
    store_smem(0);
  }
  __syncthreads();
  for (int kt = 0; kt < nk; kt++) {
    const int buf = kt & 1;
    if (kt + 1 < nk) load_regs((kt + 1) * GK);
#pragma unroll
    for (int k = 0; k < GK; k++) {
      double a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; r++) a[r] = As[buf][k][ty + 16 * r];
#pragma unroll
      for (int c = 0; c < 4; c++) b[c] = Bs[buf][k][tx + 16 * c];
#pragma unroll
      for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[r][c] = fma(a[r], b[c], acc[r][c]);
    }
    if (kt + 1 < nk) store_smem(buf ^ 1);
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; r++) {
    int gi = i0 + ty + 16 * r;
    if (gi >= M) continue;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      int gj = j0 + tx + 16 * c;
      if (gj >= N) continue;
      double* cp = C + gi + (long long)gj * ldc;
      double v = alpha * acc[r][c];
      if (beta != 0.0) v = fma(beta, *cp, v);
      *cp = v;
    }
  }
}

template <bool LOWER>
cudaError_t launch_dgemm(cudaStream_t s, bool tA, bool tB, int M, int N, int K, double alpha,
                         const double* A, long long lda, const double* B, long long ldb,
                         double beta, double* C, long long ldc) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  dim3 grid(ceil_div(M, GM), ceil_div(N, GN));
  if (!tA && !tB) dgemm_kernel<false, false, LOWER><<<grid, GT, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  else if (!tA && tB) dgemm_kernel<false, true, LOWER><<<grid, GT, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  else if (tA && !tB) dgemm_kernel<true, false, LOWER><<<grid, GT, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  else dgemm_kernel<true, true, LOWER><<<grid, GT, 0, s>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  note_launch();
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Diagonal-block kernels (NB = 128).
// ---------------------------------------------------------------------------
constexpr int NB = 128;       // block size of potrf / trsm
constexpr int SCB = 64;       // RHS columns per CTA in the diagonal solve
constexpr int DT = 256;       // threads of the diagonal kernels

// Factor the kb x kb diagonal block at A (lower, in place) in shared memory.
__global__ void __launch_bounds__(DT) potf2_kernel(int kb, double* A, long long lda, int col0,
                                                   DevStatus* st) {
  extern __shared__ double sm[];
  double* Ls = sm;  // [NB][NB+1], Ls[c * (NB+1) + r] = A(r, c)
  const int ld = NB + 1;
  for (int e = threadIdx.x; e < kb * kb; e += DT) {
    int r = e % kb, c = e / kb;
    Ls[c * ld + r] = (r >= c) ? A[r + (long long)c * lda] : 0.0;
  }
  __syncthreads();
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < kb; j++) {
    double d = Ls[j * ld + j];
    if (!(d > 0.0)) {
      if (threadIdx.x == 0 && !bad) {
        bad = 1;
        set_status(st, FGLSGPU_ENOTSPD, col0 + j + 1, -1);
      }
    }
    double piv = sqrt(d);
    __syncthreads();
    // scale column j below the diagonal
    for (int r = j + 1 + threadIdx.x; r < kb; r += DT) Ls[j * ld + r] /= piv;
    __syncthreads();
    if (threadIdx.x == 0) Ls[j * ld + j] = piv;
    // rank-1 update of the trailing lower triangle
    const int rem = kb - j - 1;
    for (int e = threadIdx.x; e < rem * rem; e += DT) {
      int r = j + 1 + e % rem, c = j + 1 + e / rem;
      if (r >= c) Ls[c * ld + r] -= Ls[j * ld + r] * Ls[j * ld + c];
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < kb * kb; e += DT) {
    int r = e % kb, c = e / kb;
    if (r >= c) A[r + (long long)c * lda] = Ls[c * ld + r];
  }
}

// Forward substitution with the kb x kb lower block L on a set of right-hand
// sides.  RHS element (i, c) lives at X[i*si + c*sc]; i < kb runs over the
// block's rows, c < nrhs over the right-hand sides.  Used for
//   TRSM:  X := L^-1 X        (si = 1, sc = ldx)
//   POTRF: P := P L^-T        (rows of the panel are the RHS: si = lda, sc = 1)
template <int SCB>
__global__ void __launch_bounds__(DT) diag_solve_kernel(int kb, const double* L, long long ldl,
                                                        double* X, long long si, long long sc,
                                                        int nrhs) {
  constexpr int G = DT / SCB;      // row groups (a power of two)
  extern __shared__ double sm[];
  const int ldL = NB + 1;
  double* Ls = sm;                 // [NB][NB+1] column-major
  double* Xs = sm + NB * ldL;      // [SCB][NB+1]: Xs[c * ldL + i]
  const int c0 = blockIdx.x * SCB;
  const int nc = min(SCB, nrhs - c0);
  for (int e = threadIdx.x; e < kb * kb; e += DT) {
    int r = e % kb, c = e / kb;
    Ls[c * ldL + r] = (r >= c) ? L[r + (long long)c * ldl] : 0.0;
  }
  if (si == 1) {
    for (int e = threadIdx.x; e < kb * nc; e += DT) {
      int i = e % kb, c = e / kb;
      Xs[c * ldL + i] = X[i + (long long)(c0 + c) * sc];
    }
  } else {
    for (int e = threadIdx.x; e < kb * nc; e += DT) {
      int c = e % nc, i = e / nc;
      Xs[c * ldL + i] = X[(long long)i * si + (long long)(c0 + c) * sc];
    }
  }
  __syncthreads();
  const int c = threadIdx.x % SCB;   // my column
  const int g = threadIdx.x / SCB;   // my row group
  for (int j = 0; j < kb; j++) {
    double xj = 0.0;
    if (c < nc) xj = Xs[c * ldL + j] / Ls[j * ldL + j];
    __syncthreads();
    if (c < nc) {
      if (g == (j & (G - 1))) Xs[c * ldL + j] = xj;
      for (int i = j + 1 + ((g - (j + 1)) & (G - 1)); i < kb; i += G) Xs[c * ldL + i] -= Ls[j * ldL + i] * xj;
    }
    __syncthreads();
  }
  if (si == 1) {
    for (int e = threadIdx.x; e < kb * nc; e += DT) {
      int i = e % kb, cc = e / kb;
      X[i + (long long)(c0 + cc) * sc] = Xs[cc * ldL + i];
    }
  } else {
    for (int e = threadIdx.x; e < kb * nc; e += DT) {
      int cc = e % nc, i = e / nc;
      X[(long long)i * si + (long long)(c0 + cc) * sc] = Xs[cc * ldL + i];
    }
  }
}

constexpr size_t POTF2_SMEM = sizeof(double) * NB * (NB + 1);
constexpr size_t DSOLVE_SMEM = sizeof(double) * (NB + SCB) * (NB + 1);
constexpr int SCB_NARROW = 16;  // RHS per CTA when few right-hand sides (e.g. the 512-wide L^-1 panels)
constexpr size_t DSOLVE_SMEM_NARROW = sizeof(double) * (NB + SCB_NARROW) * (NB + 1);

// X := L_kk^-1 X for nrhs right-hand sides: 64 per CTA, or 16 when that
// leaves fewer CTAs than half the SMs (the solve is FP64-issue-bound per SM)
void launch_diag_solve(cudaStream_t s, int kb, const double* L, long long ldl, double* X, long long si,
                       long long sc, int nrhs) {
  if (ceil_div(nrhs, SCB) < 76)
    diag_solve_kernel<SCB_NARROW><<<ceil_div(nrhs, SCB_NARROW), DT, DSOLVE_SMEM_NARROW, s>>>(kb, L, ldl, X, si,
                                                                                           sc, nrhs);
  else
    diag_solve_kernel<SCB><<<ceil_div(nrhs, SCB), DT, DSOLVE_SMEM, s>>>(kb, L, ldl, X, si, sc, nrhs);
}

__global__ void build_shifted_kernel(int n, const double* __restrict__ S, long long lds, double alpha,
                                     double beta, double* __restrict__ A, long long lda) {
  long long total = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    int r = (int)(e % n), c = (int)(e / n);
    if (r < c) continue;
    double v = alpha * S[r + (long long)c * lds];
    if (r == c) v += beta;
    A[r + (long long)c * lda] = v;
  }
}

bool g_attr_done = false;
cudaError_t ensure_attrs() {
  if (g_attr_done) return cudaSuccess;
  FGLS_CUDA_TRY(cudaFuncSetAttribute(potf2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)POTF2_SMEM));
  FGLS_CUDA_TRY(cudaFuncSetAttribute(diag_solve_kernel<SCB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)DSOLVE_SMEM));
  FGLS_CUDA_TRY(cudaFuncSetAttribute(diag_solve_kernel<SCB_NARROW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)DSOLVE_SMEM_NARROW));
  g_attr_done = true;
  return cudaSuccess;
}

}  // namespace

cudaError_t dgemm(cudaStream_t s, bool tA, bool tB, int M, int N, int K, double alpha,
                  const double* A, long long lda, const double* B, long long ldb, double beta,
                  double* C, long long ldc) {
  return launch_dgemm<false>(s, tA, tB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
}

namespace {
// C = alpha * sum_z P_z + beta * C, z ascending (P_z: M x N, ld M)
__global__ void splitk_reduce_kernel(int M, int N, int splits, const double* __restrict__ P, double alpha,
                                     double beta, double* __restrict__ C, long long ldc) {
  const long long total = (long long)M * N;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    double v = 0.0;
    for (int z = 0; z < splits; z++) v += P[e + (long long)z * total];
    const int i = (int)(e % M), j = (int)(e / M);
    double* c = C + i + (long long)j * ldc;
    *c = beta != 0.0 ? fma(beta, *c, alpha * v) : alpha * v;
  }
}
}  // namespace

cudaError_t dgemm_splitk(cudaStream_t s, bool tA, bool tB, int M, int N, int K, double alpha, const double* A,
                         long long lda, const double* B, long long ldb, double beta, double* C, long long ldc,
                         double* work, long long work_elems) {
  if (M <= 0 || N <= 0) return cudaSuccess;
  const int tiles = ceil_div(M, GM) * ceil_div(N, GN);
  int splits = std::min(ceil_div(2 * 152, tiles), K / 512);
  if ((long long)M * N > 0) splits = (int)std::min<long long>(splits, work_elems / ((long long)M * N));
  if (tiles >= 152 || splits < 2 || !work)
    return launch_dgemm<false>(s, tA, tB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  dim3 grid(ceil_div(M, GM), ceil_div(N, GN), splits);
  if (!tA && !tB) dgemm_kernel<false, false, false><<<grid, GT, 0, s>>>(M, N, K, 1.0, A, lda, B, ldb, 0.0, work, M);
  else if (!tA && tB) dgemm_kernel<false, true, false><<<grid, GT, 0, s>>>(M, N, K, 1.0, A, lda, B, ldb, 0.0, work, M);
  else if (tA && !tB) dgemm_kernel<true, false, false><<<grid, GT, 0, s>>>(M, N, K, 1.0, A, lda, B, ldb, 0.0, work, M);
  else dgemm_kernel<true, true, false><<<grid, GT, 0, s>>>(M, N, K, 1.0, A, lda, B, ldb, 0.0, work, M);
  const long long total = (long long)M * N;
  splitk_reduce_kernel<<<(int)std::min<long long>((total + 255) / 256, 152LL * 16), 256, 0, s>>>(M, N, splits, work,
                                                                                                alpha, beta, C, ldc);
  note_launch(2);
  return cudaGetLastError();
}

cudaError_t dgemm_lower(cudaStream_t s, bool tA, bool tB, int N, int K, double alpha,
                        const double* A, long long lda, const double* B, long long ldb,
                        double beta, double* C, long long ldc) {
  return launch_dgemm<true>(s, tA, tB, N, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
}

cudaError_t build_shifted(cudaStream_t s, int n, const double* Src, long long lds, double alpha,
                          double beta, double* A, long long lda) {
  long long total = (long long)n * n;
  int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 16);
  build_shifted_kernel<<<blocks, 256, 0, s>>>(n, Src, lds, alpha, beta, A, lda);
  note_launch();
  return cudaGetLastError();
}

cudaError_t dpotrf_lower(cudaStream_t s, int n, double* A, long long lda, DevStatus* st) {
  FGLS_CUDA_TRY(ensure_attrs());
  for (int k = 0; k < n; k += NB) {
    const int kb = std::min(NB, n - k);
    double* Akk = A + k + (long long)k * lda;
    potf2_kernel<<<1, DT, POTF2_SMEM, s>>>(kb, Akk, lda, k, st);
    note_launch();
    FGLS_CUDA_TRY(cudaGetLastError());
    const int rest = n - k - kb;
    if (rest > 0) {
      double* P = A + (k + kb) + (long long)k * lda;  // rest x kb panel
      // P := P L_kk^-T  (each panel row is a right-hand side)
      launch_diag_solve(s, kb, Akk, lda, P, lda, 1, rest);
      note_launch();
      FGLS_CUDA_TRY(cudaGetLastError());
      double* T = A + (k + kb) + (long long)(k + kb) * lda;
      FGLS_CUDA_TRY(dgemm_lower(s, false, true, rest, kb, -1.0, P, lda, P, lda, 1.0, T, lda));
    }
  }
  return cudaSuccess;
}

cudaError_t dtrsm_llnn(cudaStream_t s, int n, int nrhs, const double* L, long long ldl, double* X,
                       long long ldx) {
  if (nrhs <= 0) return cudaSuccess;
  FGLS_CUDA_TRY(ensure_attrs());
  for (int k = 0; k < n; k += NB) {
    const int kb = std::min(NB, n - k);
    const double* Lkk = L + k + (long long)k * ldl;
    double* Xk = X + k;
    launch_diag_solve(s, kb, Lkk, ldl, Xk, 1, ldx, nrhs);
    note_launch();
    FGLS_CUDA_TRY(cudaGetLastError());
    const int rest = n - k - kb;
    if (rest > 0)
      FGLS_CUDA_TRY(dgemm(s, false, false, rest, nrhs, kb, -1.0, L + (k + kb) + (long long)k * ldl,
                          ldl, Xk, ldx, 1.0, X + k + kb, ldx));
  }
  return cudaSuccess;
}

}  // namespace fgls
