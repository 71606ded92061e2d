// FP64 symmetric eigendecomposition Phi = Z diag(W) Z^T on the device,
// replacing the reference's one-off dsyevr('V','A','L') (src/fgls_eigen.c:
// 861-893).  W ascending, Z orthonormal columns.
//
// Algorithm (all FP64, no vendor library):
//  1. Householder reduction to tridiagonal form on the lower triangle
//     (A := H A H per column; per step: reflector, A v by 32 x 32 lower
//     tiles with a fixed-order reduction, rank-2 update of the lower
//     triangle).  Memory-bound: ~1.5 passes over the trailing matrix per column.
//  2. Eigenpairs of the tridiagonal by divide and conquer (fgls_dc.cu):
//     eigenvalues ascending, eigenvectors V of T.
//  3. Z = H_0 H_1 ... H_{n-3} V applied in blocks of 256 reflectors in
//     compact-WY form (Y, T from tau and Y^T Y): DGEMMs only.
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



__global__ void tridiag_tail_kernel(int n, const double* A, long long lda, double* d, double* e) {
  if (n >= 2) {
    d[n - 2] = A[(n - 2) + (long long)(n - 2) * lda];
    e[n - 2] = A[(n - 1) + (long long)(n - 2) * lda];
  }
  d[n - 1] = A[(n - 1) + (long long)(n - 1) * lda];
  e[n - 1] = 0.0;
}



int grid_for(long long total) { return (int)std::min<long long>((total + 255) / 256, 152LL * 32); }

// Symmetric matrix-vector product on the lower triangle only, in 32 x 32
// tiles: CTA (I, J), I >= J, adds A_IJ v_J to row block I and, below the
// diagonal, A_IJ^T v_I to row block J, each as its own partial vector
// part[(R * nt + K) * 32 + r] (R = the receiving row block, K = the other
// one; every slot is written exactly once), so that the reduction is a fixed
// order sum: deterministic, no atomics.  Reads m^2/2 elements instead of m^2.
constexpr int ST = 32;
__global__ void __launch_bounds__(256) symv_tiles_kernel(int m, const double* __restrict__ A, long long lda,
                                                         const double* __restrict__ v, double* __restrict__ part) {
  const int I = blockIdx.y, J = blockIdx.x;
  if (J > I) return;
  const int nt = gridDim.x;
  __shared__ double a[ST][ST + 1];  // a[c][r] = A[I*32 + r, J*32 + c]
  __shared__ double vr[ST], vc[ST];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int c = ty; c < ST; c += 8) {
    const int gr = I * ST + tx, gc = J * ST + c;
    a[c][tx] = (gr < m && gc < m) ? A[gr + (long long)gc * lda] : 0.0;
  }
  if (ty == 0) {
    vc[tx] = (J * ST + tx < m) ? v[J * ST + tx] : 0.0;
    vr[tx] = (I * ST + tx < m) ? v[I * ST + tx] : 0.0;
  }
  __syncthreads();
  __shared__ double red[8][ST];
  if (I == J) {
    // diagonal tile: the symmetric block from its lower part
    double s = 0.0;
    for (int c = ty; c < ST; c += 8) s += (tx >= c ? a[c][tx] : a[tx][c]) * vc[c];
    red[ty][tx] = s;
    __syncthreads();
    if (ty == 0) {
      double t = 0.0;
#pragma unroll
      for (int q = 0; q < 8; q++) t += red[q][tx];
      part[((long long)I * nt + J) * ST + tx] = t;
    }
    return;
  }
  double s = 0.0;  // row r = tx of A_IJ v_J
  for (int c = ty; c < ST; c += 8) s += a[c][tx] * vc[c];
  red[ty][tx] = s;
  __syncthreads();
  if (ty == 0) {
    double t = 0.0;
#pragma unroll
    for (int q = 0; q < 8; q++) t += red[q][tx];
    part[((long long)I * nt + J) * ST + tx] = t;
  }
  __syncthreads();
  s = 0.0;  // column c = tx of A_IJ^T v_I
  for (int r = ty; r < ST; r += 8) s += a[tx][r] * vr[r];
  red[ty][tx] = s;
  __syncthreads();
  if (ty == 0) {
    double t = 0.0;
#pragma unroll
    for (int q = 0; q < 8; q++) t += red[q][tx];
    part[((long long)J * nt + I) * ST + tx] = t;
  }
}

// p[i] = tau * sum_K part[(i/32 * nt + K) * 32 + i%32], K ascending
__global__ void symv_reduce_kernel(int m, int nt, const double* __restrict__ part, const double* __restrict__ tau_ptr,
                                   double* __restrict__ p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const double* q = part + ((long long)(i / ST) * nt) * ST + (i % ST);
  double s = 0.0;
  for (int K = 0; K < nt; K++) s += q[(long long)K * ST];
  p[i] = *tau_ptr * s;
}

// A[i, j] -= v_i w_j + w_i v_j on the lower triangle (i >= j) of the trailing matrix
__global__ void syr2_lower_kernel(int m, double* A, long long lda, const double* v, const double* w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const double vi = v[i], wi = w[i];
  for (int j = blockIdx.y; j <= i; j += gridDim.y) {
    double* a = A + i + (long long)j * lda;
    *a -= vi * w[j] + wi * v[j];
  }
}

// Y (mr x nb, ld mr): reflectors b .. b+nb-1 as explicit columns over rows
// b+1 .. n-1: column c is zero above row c, 1 at row c, A[b+c+1+i, b+c] below.
__global__ void build_y_kernel(int n, int b, int nb, const double* __restrict__ A, long long lda,
                               double* __restrict__ Y) {
  const int mr = n - b - 1;
  const long long total = (long long)mr * nb;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e % mr), c = (int)(e / mr);
    double v = 0.0;
    if (r == c) v = 1.0;
    else if (r > c) v = A[(b + 1 + r) + (long long)(b + c) * lda];
    Y[e] = v;
  }
}

// Compact-WY factor T (nb x nb upper, ld nb, nb <= 256) of
// H_b ... H_{b+nb-1} = I - Y T Y^T from tau and G = Y^T Y (forward,
// columnwise): T_ii = tau_i, T[0:i, i] = -tau_i T[0:i, 0:i] G[0:i, i].  One
// CTA of 256 threads, column by column.
__global__ void __launch_bounds__(256) larft_kernel(int nb, const double* __restrict__ tau, const double* G,
                                                    double* T) {
  __shared__ double g[256];
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) T[e] = 0.0;
  __syncthreads();
  for (int i = 0; i < nb; i++) {
    const double ti = tau[i];
    if (threadIdx.x < i) g[threadIdx.x] = G[threadIdx.x + (long long)i * nb];
    __syncthreads();
    if (threadIdx.x < i) {
      const int r = threadIdx.x;
      double acc = 0.0;
      for (int q = 0; q < i; q++)  // all threads read column q together (coalesced); T upper: rows r <= q
        if (q >= r) acc += T[r + (long long)q * nb] * g[q];
      T[r + (long long)i * nb] = -ti * acc;
    }
    if (threadIdx.x == 0) T[i + (long long)i * nb] = ti;
    __syncthreads();
  }
}

}  // namespace

size_t eig_workspace_bytes(int n) {
  // d, e, tau, vbuf, p (n each) + n ints of scratch + symv partials (nt^2 x 32)
  const size_t nt = (size_t)(n + ST - 1) / ST;
  return sizeof(double) * ((size_t)n * 5 + nt * nt * ST) + sizeof(int) * (size_t)n + 256;
}

cudaError_t dsyev_device(cudaStream_t s, int n, const double* Phi, long long ldp, double* A, double* Z,
                         double* W, void* work, int* fail_out, long long* launches) {
  double* d = (double*)work;
  double* e = d + n;
  double* tau = e + n;
  double* vbuf = tau + n;
  double* p = vbuf + n;
  int* rank = (int*)(p + n);
  double* part = (double*)(((uintptr_t)(rank + n) + 15) & ~(uintptr_t)15);  // symv partials
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
    const int nt = ceil_div(m, ST);
    symv_tiles_kernel<<<dim3(nt, nt), 256, 0, s>>>(m, Asub, n, vbuf, part);
    symv_reduce_kernel<<<ceil_div(m, 256), 256, 0, s>>>(m, nt, part, tau + k, p);
    tridiag_w_kernel<<<1, 256, 0, s>>>(m, vbuf, tau + k, p);
    dim3 g2(ceil_div(m, 256), std::min(m, 512));
    syr2_lower_kernel<<<g2, 256, 0, s>>>(m, Asub, n, vbuf, p);
    nl += 5;
  }
  tridiag_tail_kernel<<<1, 1, 0, s>>>(n, A, n, d, e);
  nl++;
  FGLS_CUDA_TRY(cudaGetLastError());
  mark(1);
  mark(2);  // (no explicit Q: the reflectors are applied to the eigenvectors below)
  // 3. eigenpairs of T by divide and conquer (fgls_dc.cu) into Z; A keeps the reflectors
  // one workspace for the divide and conquer, then for the back-transform
  // (Y: n x NBT, G, T: NBT x NBT, W, W2: NBT x n)
  constexpr int NBT = 256;
  const size_t bt_bytes = sizeof(double) * ((size_t)3 * NBT * n + (size_t)2 * NBT * NBT);
  void* dcw = nullptr;
  FGLS_CUDA_TRY(cudaMalloc(&dcw, std::max(dc_workspace_bytes(n), bt_bytes)));
  int* dfail = rank;  // n ints of scratch; first used as the failure flag
  FGLS_CUDA_TRY(cudaMemsetAsync(dfail, 0, sizeof(int), s));
  cudaError_t rc = dc_tridiag_eig(s, n, d, e, W, Z, dcw, dfail, &nl);
  mark(3);
  // 4. Z := H_0 H_1 ... H_{n-3} Z, blocks of NB reflectors from the last one
  //    in compact-WY form (I - Y T Y^T): three DGEMMs per block, 2 n^3 flops
  //    in all -- what a DGEMM with an explicit Q costs, without forming Q.
  {
    constexpr int NB = NBT;  // wide blocks: the Y^T Z product has NB/64 x n/64 output tiles
    double* Yb = (double*)dcw;         // n x NB
    double* G = Yb + (size_t)n * NB;   // NB x NB
    double* Tm = G + (size_t)NB * NB;  // NB x NB
    double* Wb = Tm + (size_t)NB * NB; // NB x n
    double* W2 = Wb + (size_t)NB * n;  // NB x n
    const int nref = n - 2;            // reflectors 0 .. n-3
    for (int b = nref > 0 ? ((nref - 1) / NB) * NB : -1; b >= 0 && rc == cudaSuccess; b -= NB) {
      const int nb = std::min(NB, nref - b);
      const int mr = n - b - 1;
      double* Zs = Z + (b + 1);  // rows b+1 .. n-1, all n columns (ld n)
      build_y_kernel<<<grid_for((long long)mr * nb), 256, 0, s>>>(n, b, nb, A, n, Yb);
      rc = dgemm(s, true, false, nb, nb, mr, 1.0, Yb, mr, Yb, mr, 0.0, G, nb);
      if (rc == cudaSuccess) {
        larft_kernel<<<1, 256, 0, s>>>(nb, tau + b, G, Tm);
        rc = dgemm(s, true, false, nb, n, mr, 1.0, Yb, mr, Zs, n, 0.0, Wb, nb);
      }
      if (rc == cudaSuccess) rc = dgemm(s, false, false, nb, n, nb, 1.0, Tm, nb, Wb, nb, 0.0, W2, nb);
      if (rc == cudaSuccess) rc = dgemm(s, false, false, mr, n, nb, -1.0, Yb, mr, W2, nb, 1.0, Zs, n);
      nl += 2;
    }
  }
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
    fprintf(stderr, "[fgls eig n=%d] tridiagonal %.1f ms, divide-and-conquer %.1f ms, back-transform %.1f ms\n", n,
            t[0], t[2], t[3]);
    for (auto& x : ev) cudaEventDestroy(x);
  }
  if (launches) *launches += nl;
  note_launch(nl);
  return cudaSuccess;
}

}  // namespace fgls
