// FP64 symmetric eigendecomposition Phi = Z diag(W) Z^T on the device,
// replacing the reference's one-off dsyevr('V','A','L') (src/fgls_eigen.c:
// 861-893).  W ascending, Z orthonormal columns.
//
// Algorithm (all FP64, no vendor library):
//  1. Householder reduction to tridiagonal form on the full symmetric matrix
//     (A := H A H per column; per step: reflector, column-wise A v by one warp
//     per column, rank-2 update).  Memory-bound: ~3 passes over the trailing
//     matrix per column.
//  2. Q = H_0 H_1 ... H_{n-3} formed explicitly by backward accumulation.
//  3. Eigenpairs of the tridiagonal by divide and conquer (fgls_dc.cu):
//     eigenvalues ascending, eigenvectors V of T.
//  4. Z = Q V (DGEMM).
#include <algorithm>
#include <cfloat>
#include <cstdio>
#include <cstdlib>

#include "fgls_common.cuh"
#include "fgls_kernels.cuh"

namespace fgls {

namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ double block_sum(double v, double* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    double s = (l < (int)(blockDim.x >> 5)) ? red[l] : 0.0;
    s = warp_sum(s);
    if (l == 0) red[32] = s;
  }
  __syncthreads();
  return red[32];
}

// Fill the strict upper triangle from the lower one (A symmetric in full storage).
__global__ void symmetrize_kernel(int n, double* A, long long lda) {
  const long long total = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    int r = (int)(e % n), c = (int)(e / n);
    if (r < c) A[r + (long long)c * lda] = A[c + (long long)r * lda];
  }
}

// Householder reflector for column k (one CTA).  v (length m = n-k-1, v[0]=1)
// to vbuf; v[1:] also stored in A[k+2:, k]; d[k], e[k], tau[k].
__global__ void __launch_bounds__(256) householder_kernel(int n, int k, double* A, long long lda, double* d,
                                                          double* e, double* tau, double* vbuf) {
  __shared__ double red[33];
  const int m = n - k - 1;
  const double* x = A + (k + 1) + (long long)k * lda;
  double s = 0.0;
  for (int i = 1 + threadIdx.x; i < m; i += blockDim.x) s += x[i] * x[i];
  const double xnorm2 = block_sum(s, red);
  const double alpha = x[0];
  double beta, t, scal;
  if (xnorm2 == 0.0) {
    t = 0.0;
    beta = alpha;
    scal = 0.0;
  } else {
    beta = -copysign(sqrt(alpha * alpha + xnorm2), alpha);
    t = (beta - alpha) / beta;
    scal = 1.0 / (alpha - beta);
  }
  double* xs = A + (k + 1) + (long long)k * lda;
  for (int i = 1 + threadIdx.x; i < m; i += blockDim.x) {
    double v = x[i] * scal;
    vbuf[i] = v;
    xs[i] = v;
  }
  if (threadIdx.x == 0) {
    vbuf[0] = 1.0;
    d[k] = A[k + (long long)k * lda];
    e[k] = beta;
    tau[k] = t;
  }
}

// p[j] = tau * sum_i A[k+1+i, k+1+j] v[i]   (one warp per column j)
__global__ void __launch_bounds__(256) colwise_dot_kernel(int m, const double* A, long long lda,
                                                          const double* v, const double* tau_ptr,
                                                          double* p) {
  const int j = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (j >= m) return;
  const double* col = A + (long long)j * lda;
  double s = 0.0;
  for (int i = lane; i < m; i += 32) s = fma(col[i], v[i], s);
  s = warp_sum(s);
  if (lane == 0) p[j] = (tau_ptr ? *tau_ptr : 1.0) * s;
}

// w = p - (tau/2)(p^T v) v  (one CTA, in place in p)
__global__ void __launch_bounds__(256) tridiag_w_kernel(int m, const double* v, const double* tau_ptr,
                                                        double* p) {
  __shared__ double red[33];
  double s = 0.0;
  for (int i = threadIdx.x; i < m; i += blockDim.x) s += p[i] * v[i];
  s = block_sum(s, red);
  const double g = -0.5 * (*tau_ptr) * s;
  __syncthreads();
  for (int i = threadIdx.x; i < m; i += blockDim.x) p[i] += g * v[i];
}

// A[i, j] -= v_i w_j + w_i v_j over the m x m trailing matrix
__global__ void syr2_kernel(int m, double* A, long long lda, const double* v, const double* w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const double vi = v[i], wi = w[i];
  for (int j = blockIdx.y; j < m; j += gridDim.y) {
    double* a = A + i + (long long)j * lda;
    *a -= vi * w[j] + wi * v[j];
  }
}

// Q[i, j] -= tau v_i w_j over the m x m block (rank-1, w = Q^T v)
__global__ void rank1_kernel(int m, double* Q, long long ldq, const double* v, const double* w,
                             const double* tau_ptr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const double tv = (*tau_ptr) * v[i];
  for (int j = blockIdx.y; j < m; j += gridDim.y) Q[i + (long long)j * ldq] -= tv * w[j];
}

__global__ void tridiag_tail_kernel(int n, const double* A, long long lda, double* d, double* e) {
  if (n >= 2) {
    d[n - 2] = A[(n - 2) + (long long)(n - 2) * lda];
    e[n - 2] = A[(n - 1) + (long long)(n - 2) * lda];
  }
  d[n - 1] = A[(n - 1) + (long long)(n - 1) * lda];
  e[n - 1] = 0.0;
}

__global__ void identity_kernel(int n, double* Q, long long ldq) {
  const long long total = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    int r = (int)(e % n), c = (int)(e / n);
    Q[r + (long long)c * ldq] = (r == c) ? 1.0 : 0.0;
  }
}

// gather v_k (v[0] = 1, v[1:] = A[k+2:, k]) into vbuf
__global__ void load_v_kernel(int n, int k, const double* A, long long lda, double* vbuf) {
  const int m = n - k - 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
    vbuf[i] = (i == 0) ? 1.0 : A[(k + 1 + i) + (long long)k * lda];
}

int grid_for(long long total) { return (int)std::min<long long>((total + 255) / 256, 152LL * 32); }

}  // namespace

size_t eig_workspace_bytes(int n) {
  // d, e, tau, vbuf, p (n each) + n ints of scratch
  return sizeof(double) * (size_t)n * 5 + sizeof(int) * (size_t)n + 256;
}

cudaError_t dsyev_device(cudaStream_t s, int n, const double* Phi, long long ldp, double* A, double* Z,
                         double* W, void* work, int* fail_out, long long* launches) {
  double* d = (double*)work;
  double* e = d + n;
  double* tau = e + n;
  double* vbuf = tau + n;
  double* p = vbuf + n;
  int* rank = (int*)(p + n);
  long long nl = 0;
  // FGLS_EIG_TIMING=1 prints the phase times (CUDA events on s) to stderr
  const bool timing = getenv("FGLS_EIG_TIMING") != nullptr;
  cudaEvent_t ev[5];
  if (timing)
    for (auto& x : ev) cudaEventCreate(&x);
  auto mark = [&](int i) {
    if (timing) cudaEventRecord(ev[i], s);
  };
  mark(0);
  // A := Phi (lower) symmetrized
  FGLS_CUDA_TRY(cudaMemcpy2DAsync(A, sizeof(double) * n, Phi, sizeof(double) * ldp, sizeof(double) * n, n,
                                  cudaMemcpyDeviceToDevice, s));
  symmetrize_kernel<<<grid_for((long long)n * n), 256, 0, s>>>(n, A, n);
  nl++;
  FGLS_CUDA_TRY(cudaGetLastError());
  // 1. tridiagonalization
  for (int k = 0; k + 2 < n; k++) {
    const int m = n - k - 1;
    householder_kernel<<<1, 256, 0, s>>>(n, k, A, n, d, e, tau, vbuf);
    double* Asub = A + (k + 1) + (long long)(k + 1) * n;
    colwise_dot_kernel<<<ceil_div(m, 8), 256, 0, s>>>(m, Asub, n, vbuf, tau + k, p);
    tridiag_w_kernel<<<1, 256, 0, s>>>(m, vbuf, tau + k, p);
    dim3 g2(ceil_div(m, 256), std::min(m, 512));
    syr2_kernel<<<g2, 256, 0, s>>>(m, Asub, n, vbuf, p);
    nl += 4;
  }
  tridiag_tail_kernel<<<1, 1, 0, s>>>(n, A, n, d, e);
  nl++;
  FGLS_CUDA_TRY(cudaGetLastError());
  mark(1);
  // 2. Q = H_0 ... H_{n-3}
  identity_kernel<<<grid_for((long long)n * n), 256, 0, s>>>(n, Z, n);
  nl++;
  for (int k = n - 3; k >= 0; k--) {
    const int m = n - k - 1;
    load_v_kernel<<<ceil_div(m, 256), 256, 0, s>>>(n, k, A, n, vbuf);
    double* Qsub = Z + (k + 1) + (long long)(k + 1) * n;
    colwise_dot_kernel<<<ceil_div(m, 8), 256, 0, s>>>(m, Qsub, n, vbuf, nullptr, p);
    dim3 g2(ceil_div(m, 256), std::min(m, 512));
    rank1_kernel<<<g2, 256, 0, s>>>(m, Qsub, n, vbuf, p, tau + k);
    nl += 3;
  }
  FGLS_CUDA_TRY(cudaGetLastError());
  mark(2);
  // 3. eigenpairs of T by divide and conquer (fgls_dc.cu) into A (free now)
  void* dcw = nullptr;
  FGLS_CUDA_TRY(cudaMalloc(&dcw, dc_workspace_bytes(n)));
  int* dfail = rank;  // n ints of scratch; first used as the failure flag
  FGLS_CUDA_TRY(cudaMemsetAsync(dfail, 0, sizeof(int), s));
  cudaError_t rc = dc_tridiag_eig(s, n, d, e, W, A, dcw, dfail, &nl);
  mark(3);
  // 4. Z = Q T-eigenvectors, through a scratch matrix of the workspace
  double* T = (double*)dcw;
  if (rc == cudaSuccess) rc = dgemm(s, false, false, n, n, n, 1.0, Z, n, A, n, 0.0, T, n);
  if (rc == cudaSuccess)
    rc = cudaMemcpyAsync(Z, T, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToDevice, s);
  int hfail = 0;
  if (rc == cudaSuccess) rc = cudaMemcpyAsync(&hfail, dfail, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (rc == cudaSuccess) rc = cudaStreamSynchronize(s);
  cudaFree(dcw);
  FGLS_CUDA_TRY(rc);
  *fail_out = hfail;
  mark(4);
  if (timing) {
    cudaEventSynchronize(ev[4]);
    float t[4];
    for (int i = 0; i < 4; i++) cudaEventElapsedTime(&t[i], ev[i], ev[i + 1]);
    fprintf(stderr, "[fgls eig n=%d] tridiagonal %.1f ms, form Q %.1f ms, divide-and-conquer %.1f ms, back-transform %.1f ms\n",
            n, t[0], t[1], t[2], t[3]);
    for (auto& x : ev) cudaEventDestroy(x);
  }
  if (launches) *launches += nl;
  note_launch(nl);
  return cudaSuccess;
}

}  // namespace fgls
