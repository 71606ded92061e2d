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
//  3. Implicit QL with Wilkinson shifts on the tridiagonal (the EISPACK
//     tql2 / tqli iteration) with an absolute deflation test |e_m| <= eps*|T|.
//     The scalar recurrence of each sweep runs in one thread and records its
//     Givens rotations; a second kernel applies the sweep's rotation chain to
//     every row of Z in parallel (one thread per row, coalesced by column).
//  4. Sort ascending, permuting the columns of Z.
#include <algorithm>
#include <cfloat>

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

struct QLState {
  int l;      // first not yet converged index
  int lo, hi; // rotation range of the last sweep (applied hi down to lo)
  int nrot;   // rotations recorded by the last sweep (0: none)
  int iter;   // sweeps spent on the current l
  int done;
  int fail;
  int sweeps;
  double anorm;
};

__global__ void ql_init_kernel(int n, const double* d, const double* e, QLState* q) {
  double a = 0.0;
  for (int i = 0; i < n; i++) {
    double r = fabs(d[i]) + fabs(e[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0);
    a = fmax(a, r);
  }
  q->l = 0;
  q->lo = q->hi = 0;
  q->nrot = 0;
  q->iter = 0;
  q->done = (n <= 1);
  q->fail = 0;
  q->sweeps = 0;
  q->anorm = a;
}

// One implicit QL sweep (scalar, single thread); records rotations in c/s.
__global__ void ql_sweep_kernel(int n, double* d, double* e, double* cs, double* sn, QLState* q) {
  q->nrot = 0;
  if (q->done) return;
  const double tol = DBL_EPSILON * q->anorm;
  int l = q->l;
  while (l < n) {
    int m;
    for (m = l; m < n - 1; m++)
      if (fabs(e[m]) <= tol) break;
    if (m == l) {
      l++;
      q->iter = 0;
      continue;
    }
    if (q->iter >= 64) {
      q->fail = 1;
      q->done = 1;
      q->l = l;
      return;
    }
    q->iter++;
    q->sweeps++;
    double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
    double r = hypot(g, 1.0);
    g = d[m] - d[l] + e[l] / (g + copysign(r, g));
    double s = 1.0, c = 1.0, p = 0.0;
    int i;
    int cnt = 0;
    for (i = m - 1; i >= l; i--) {
      double f = s * e[i];
      double b = c * e[i];
      r = hypot(f, g);
      e[i + 1] = r;
      if (r == 0.0) {
        d[i + 1] -= p;
        e[m] = 0.0;
        break;
      }
      s = f / r;
      c = g / r;
      g = d[i + 1] - p;
      r = (d[i] - g) * s + 2.0 * c * b;
      p = s * r;
      d[i + 1] = g + p;
      g = c * r - b;
      cs[i] = c;
      sn[i] = s;
      cnt++;
    }
    q->hi = m - 1;
    q->lo = m - cnt;
    q->nrot = cnt;
    if (!(r == 0.0 && i >= l)) {
      d[l] -= p;
      e[l] = g;
      e[m] = 0.0;
    }
    q->l = l;
    return;
  }
  q->l = n;
  q->done = 1;
}

// Apply the recorded rotation chain to every row of Z (column-major n x n).
__global__ void ql_apply_kernel(int n, double* Z, long long ldz, const double* cs, const double* sn,
                                const QLState* q) {
  const int nrot = q->nrot;
  if (nrot == 0) return;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int hi = q->hi, lo = q->lo;
  double carry = Z[r + (long long)(hi + 1) * ldz];
  for (int i = hi; i >= lo; i--) {
    const double zi = Z[r + (long long)i * ldz];
    const double c = cs[i], s = sn[i];
    Z[r + (long long)(i + 1) * ldz] = s * zi + c * carry;
    carry = c * zi - s * carry;
  }
  Z[r + (long long)lo * ldz] = carry;
}

// rank of each eigenvalue (ascending, ties by index), then gather
__global__ void rank_kernel(int n, const double* d, int* rank) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double di = d[i];
  int rk = 0;
  for (int j = 0; j < n; j++) {
    const double dj = d[j];
    rk += (dj < di) || (dj == di && j < i);
  }
  rank[i] = rk;
}

__global__ void permute_kernel(int n, const double* d, const int* rank, const double* Zin, long long ldi,
                               double* W, double* Zout, long long ldo) {
  const long long total = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    int r = (int)(e % n), c = (int)(e / n);
    int rc = rank[c];
    Zout[r + (long long)rc * ldo] = Zin[r + (long long)c * ldi];
    if (r == 0) W[rc] = d[c];
  }
}

int grid_for(long long total) { return (int)std::min<long long>((total + 255) / 256, 152LL * 32); }

}  // namespace

size_t eig_workspace_bytes(int n) {
  // d, e, tau, vbuf, p, cs, sn (n each) + rank (n ints) + QLState
  return sizeof(double) * (size_t)n * 7 + sizeof(int) * (size_t)n + 256;
}

cudaError_t dsyev_device(cudaStream_t s, int n, const double* Phi, long long ldp, double* A, double* Z,
                         double* W, void* work, int* fail_out, long long* launches) {
  double* d = (double*)work;
  double* e = d + n;
  double* tau = e + n;
  double* vbuf = tau + n;
  double* p = vbuf + n;
  double* cs = p + n;
  double* sn = cs + n;
  int* rank = (int*)(sn + n);
  QLState* q = (QLState*)(((uintptr_t)(rank + n) + 63) & ~(uintptr_t)63);
  long long nl = 0;
  // A := Phi (lower) symmetrized; use Z as the scratch copy target first
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
  // 3. implicit QL with rotations applied to Z
  ql_init_kernel<<<1, 1, 0, s>>>(n, d, e, q);
  nl++;
  QLState hq;
  const long long max_sweeps = 64LL * n + 64;
  long long it = 0;
  for (;;) {
    for (int b = 0; b < 128; b++, it++) {
      ql_sweep_kernel<<<1, 1, 0, s>>>(n, d, e, cs, sn, q);
      ql_apply_kernel<<<ceil_div(n, 128), 128, 0, s>>>(n, Z, n, cs, sn, q);
      nl += 2;
    }
    FGLS_CUDA_TRY(cudaGetLastError());
    FGLS_CUDA_TRY(cudaMemcpyAsync(&hq, q, sizeof(QLState), cudaMemcpyDeviceToHost, s));
    FGLS_CUDA_TRY(cudaStreamSynchronize(s));
    if (hq.done || it > max_sweeps) break;
  }
  *fail_out = (hq.fail || !hq.done) ? 1 : 0;
  // 4. sort ascending; A is free again and receives the permuted Z, copied back
  rank_kernel<<<ceil_div(n, 256), 256, 0, s>>>(n, d, rank);
  permute_kernel<<<grid_for((long long)n * n), 256, 0, s>>>(n, d, rank, Z, n, W, A, n);
  nl += 2;
  FGLS_CUDA_TRY(cudaGetLastError());
  FGLS_CUDA_TRY(cudaMemcpyAsync(Z, A, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToDevice, s));
  if (launches) *launches += nl;
  note_launch(nl);
  return cudaSuccess;
}

}  // namespace fgls
