// FP64 symmetric eigendecomposition Phi = Z diag(W) Z^T on the device,
// replacing the reference's one-off dsyevr('V','A','L') (src/fgls_eigen.c:
// 861-893).  W ascending, Z orthonormal columns.
//
// Algorithm (all FP64, no vendor library):
//  1. Householder reduction to tridiagonal form on the lower triangle
//     (A := H A H per column).  Each column's rank-2 update is deferred by
//     one step: step k first applies update k-1 to column k (reflector
//     kernel), then one pass over the trailing matrix applies update k-1 and
//     forms A v_k by 32 x 32 lower tiles with a fixed-order reduction.
//     Memory-bound: one read and one write of the trailing lower triangle
//     per column.
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

// Per column k the work is three launches, all spread over the SMs (a
// single CTA would be bound by one SM's FP64 rate):
//   tridiag_col_kernel   w_{k-1} = p + g v from the previous step's p, v and
//                        partial dots; the pending update of step k-1 applied
//                        to column k; partial sums of squares of column k
//   tridiag_step_kernel  the reflector v_k from those sums (every CTA derives
//                        the same scalars), then one pass over the trailing
//                        matrix: pending update and A v_k
//   tridiag_p_kernel     p_k = tau_k A v_k from the tile partials, partial
//                        dots p_k^T v_k
constexpr int RT = 256;  // rows per CTA of the row kernels

// Scalars of the Householder reflector of x (x[0] = alpha, |x[1:]|^2 = xnorm2):
// beta, tau and the scale of x[1:] into v[1:].
__device__ __forceinline__ void reflector(double alpha, double xnorm2, double& beta, double& tau, double& scal) {
  if (xnorm2 == 0.0) {
    tau = 0.0;
    beta = alpha;
    scal = 0.0;
  } else {
    beta = -copysign(sqrt(alpha * alpha + xnorm2), alpha);
    tau = (beta - alpha) / beta;
    scal = 1.0 / (alpha - beta);
  }
}

// Column k (rows k+1 .. n-1, i = 0 .. m-1).  With k > 0: g = -(tau_{k-1}/2)
// sum(dpart) (p^T v of step k-1, fixed order), w_{k-1} = p + g v into wprev
// (index 0 = row k), x_i = A[k+1+i, k] - (v[1+i] w[0] + w[1+i] v[0]) written
// back, d[k] = A[k, k] - 2 v[0] w[0], and v_{k-1}[1:] stored below the
// subdiagonal of column k-1.  Partial sums of x_i^2 (i >= 1) to npart.
__global__ void __launch_bounds__(RT) tridiag_col_kernel(int n, int k, double* A, long long lda, double* d,
                                                         const double* __restrict__ tau,
                                                         const double* __restrict__ pprev,
                                                         const double* __restrict__ vprev,
                                                         double* __restrict__ wprev,
                                                         const double* __restrict__ dpart, int ndp,
                                                         double* __restrict__ npart) {
  __shared__ double red[33];
  const int m = n - k - 1;
  const int i = blockIdx.x * RT + threadIdx.x;
  const bool upd = k > 0;
  double* x = A + (k + 1) + (long long)k * lda;
  double sq = 0.0;
  __shared__ double dot_s;
  if (upd && threadIdx.x == 0) {
    double dot = 0.0;
    for (int c = 0; c < ndp; c++) dot += dpart[c];
    dot_s = dot;
  }
  __syncthreads();
  if (upd) {
    const double g = -0.5 * tau[k - 1] * dot_s;
    const double v0 = vprev[0];
    const double w0 = pprev[0] + g * v0;
    if (i < m) {
      const double vi = vprev[1 + i];
      const double wi = pprev[1 + i] + g * vi;
      wprev[1 + i] = wi;
      const double xi = x[i] - (vi * w0 + wi * v0);
      x[i] = xi;
      if (i >= 1) sq = xi * xi;
      A[(k + 1 + i) + (long long)(k - 1) * lda] = vi;  // reflector k-1, row k+1+i
    }
    if (i == 0) {
      wprev[0] = w0;
      d[k] = A[k + (long long)k * lda] - 2.0 * v0 * w0;
    }
  } else {
    if (i < m && i >= 1) sq = x[i] * x[i];
    if (i == 0) d[k] = A[k + (long long)k * lda];
  }
  sq = block_sum(sq, red);
  if (threadIdx.x == 0) npart[blockIdx.x] = sq;
}

// The last 2 x 2 block.  n >= 3: w of step n-3 from its p, v and partial
// dots, its reflector stored (A[n-1, n-3]), and its pending update applied.
__global__ void tridiag_tail_kernel(int n, double* A, long long lda, double* d, double* e, const double* tau,
                                    const double* p, const double* v, const double* dpart, int ndp) {
  if (n >= 3) {
    double dot = 0.0;
    for (int c = 0; c < ndp; c++) dot += dpart[c];
    const double g = -0.5 * tau[n - 3] * dot;
    const double v0 = v[0], v1 = v[1];
    const double w0 = p[0] + g * v0, w1 = p[1] + g * v1;
    A[(n - 1) + (long long)(n - 3) * lda] = v1;
    d[n - 2] = A[(n - 2) + (long long)(n - 2) * lda] - 2.0 * v0 * w0;
    e[n - 2] = A[(n - 1) + (long long)(n - 2) * lda] - (v1 * w0 + w1 * v0);
    d[n - 1] = A[(n - 1) + (long long)(n - 1) * lda] - 2.0 * v1 * w1;
  } else if (n == 2) {
    d[0] = A[0];
    e[0] = A[1];
    d[1] = A[1 + lda];
  } else {
    d[0] = A[0];
  }
  e[n - 1] = 0.0;
}

int grid_for(long long total) { return (int)std::min<long long>((total + 255) / 256, 152LL * 32); }

// One pass over the trailing lower triangle (m x m, 32 x 32 tiles) per
// column: apply the pending rank-2 update A -= vo wo^T + wo vo^T (vo, wo:
// the previous step's vectors shifted to this trailing matrix; nullptr at
// step 0) and form A v with the updated values.  v is the reflector of
// column x (x[0] = alpha, rows below: the updated column), derived by every
// CTA from the same fixed-order sum of npart; CTAs Jc = 0 store it (vout),
// CTA (0, 0) stores tau and e.  CTA (Jc, I) takes the lower tiles (I, J), J
// in [Jc*SS, min(Jc*SS + SS, I + 1)).  Row block I's partial of A v from the
// strip goes to slot (I, Jc), and the below-diagonal tiles' A_IJ^T v_I to
// slot (J, I) (> J), each written exactly once: part[(R * nt + K) * 32 + r].
// The reduction sums them in a fixed order (deterministic, no atomics).
constexpr int ST = 32;
constexpr int SS = 4;
__global__ void __launch_bounds__(256) tridiag_step_kernel(int m, double* __restrict__ A, long long lda,
                                                           const double* __restrict__ vo,
                                                           const double* __restrict__ wo,
                                                           const double* __restrict__ x,
                                                           const double* __restrict__ npart, int nnp,
                                                           double* __restrict__ vout, double* __restrict__ tau_out,
                                                           double* __restrict__ e_out, double* __restrict__ part) {
  const int I = blockIdx.y, Jc = blockIdx.x, J0 = Jc * SS;
  if (J0 > I) return;
  __shared__ double scal_s;
  if (threadIdx.x == 0) {
    double xn2 = 0.0;
    for (int c = 0; c < nnp; c++) xn2 += npart[c];
    double beta, tau, scal;
    reflector(x[0], xn2, beta, tau, scal);
    scal_s = scal;
    if (blockIdx.x == 0 && blockIdx.y == 0) {
      *tau_out = tau;
      *e_out = beta;
    }
  }
  __syncthreads();
  const double scal = scal_s;
  // v_i: 1 at i = 0, x_i * scal below, 0 past the matrix
  auto vval = [&](int i) { return i < m ? (i == 0 ? 1.0 : x[i] * scal) : 0.0; };
  const int J1 = min(J0 + SS, I + 1);
  const int nt = gridDim.y;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  __shared__ double a[ST][ST + 1];  // a[c][r] = A[I*32 + r, J*32 + c]
  __shared__ double vr[ST], vor[ST], wor[ST], vc[ST], voc[ST], woc[ST];
  __shared__ double red[8][ST];
  const bool upd = vo != nullptr;
  const int gr = I * ST + tx;
  if (ty == 0) {
    const double vi = vval(gr);
    vr[tx] = vi;
    if (Jc == 0 && gr < m) vout[gr] = vi;
    vor[tx] = (upd && gr < m) ? vo[gr] : 0.0;
    wor[tx] = (upd && gr < m) ? wo[gr] : 0.0;
  }
  double rs = 0.0;  // row tx of this strip's A_I. v, over this thread's columns
  for (int J = J0; J < J1; J++) {
    __syncthreads();  // the previous tile's shared reads are done
    if (ty == 1) {
      const int gc = J * ST + tx;
      vc[tx] = vval(gc);
      voc[tx] = (upd && gc < m) ? vo[gc] : 0.0;
      woc[tx] = (upd && gc < m) ? wo[gc] : 0.0;
    }
    __syncthreads();
    for (int c = ty; c < ST; c += 8) {
      const int gc = J * ST + c;
      double av = 0.0;
      if (gr < m && gc < m && (I != J || tx >= c)) {
        double* pa = A + gr + (long long)gc * lda;
        av = *pa;
        if (upd) {
          // two FMAs (FP64 issue rate bounds this pass)
          av = fma(-vor[tx], woc[c], av);
          av = fma(-wor[tx], voc[c], av);
          *pa = av;
        }
      }
      a[c][tx] = av;
    }
    __syncthreads();
    if (I == J) {
      // diagonal tile: the symmetric block from its lower part
      for (int c = ty; c < ST; c += 8) rs += (tx >= c ? a[c][tx] : a[tx][c]) * vc[c];
    } else {
      for (int c = ty; c < ST; c += 8) rs += a[c][tx] * vc[c];
      // column tx of A_IJ^T v_I: rows ty, ty+8, ... here, the eight partial
      // sums added by one thread (FP64 issue rate is the bound: no shuffles)
      double cs = 0.0;
      for (int r = ty; r < ST; r += 8) cs += a[tx][r] * vr[r];
      red[ty][tx] = cs;
      __syncthreads();
      if (ty == 0) {
        double t = 0.0;
#pragma unroll
        for (int q = 0; q < 8; q++) t += red[q][tx];
        part[((long long)J * nt + I) * ST + tx] = t;
      }
    }
  }
  __syncthreads();  // the last tile's column reduction has read red
  red[ty][tx] = rs;
  __syncthreads();
  if (ty == 0) {
    double t = 0.0;
#pragma unroll
    for (int q = 0; q < 8; q++) t += red[q][tx];
    part[((long long)I * nt + Jc) * ST + tx] = t;
  }
}

// p[i] = tau_k * sum of row block R = i / 32's slots (strip slots K = 0 ..
// R/SS, then tile slots K = R+1 .. nt-1).  One CTA per row block: thread
// (r, c) sums slots c, c+8, ... of row r, the eight partial sums are added in
// c order (fixed order); the CTA's p^T v goes to dpart[R].
__global__ void __launch_bounds__(256) tridiag_p_kernel(int m, int nt, const double* __restrict__ part,
                                                        const double* __restrict__ tau_ptr,
                                                        const double* __restrict__ v, double* __restrict__ p,
                                                        double* __restrict__ dpart) {
  __shared__ double red[8][ST];
  const int R = blockIdx.x;
  const int r = threadIdx.x & 31, c = threadIdx.x >> 5;
  const int i = R * ST + r;
  const int ns = R / SS + 1;          // strip slots 0 .. R/SS
  const int nslots = ns + (nt - R - 1);  // then tile slots R+1 .. nt-1
  const double* q = part + ((long long)R * nt) * ST + r;
  double sum = 0.0;
  for (int e = c; e < nslots; e += 8) {
    const int K = e < ns ? e : R + 1 + (e - ns);
    sum += q[(long long)K * ST];
  }
  red[c][r] = sum;
  __syncthreads();
  if (c == 0) {
    double t = 0.0;
#pragma unroll
    for (int u = 0; u < 8; u++) t += red[u][r];
    const double pi = i < m ? *tau_ptr * t : 0.0;
    if (i < m) p[i] = pi;
    double pv = i < m ? pi * v[i] : 0.0;
    pv = warp_sum(pv);
    if (r == 0) dpart[R] = pv;
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
  // d, e, tau, two v and two w buffers, p (n each), per-CTA dot and norm
  // partials (n / RT each) + n ints of scratch + symv partials (nt^2 x 32)
  const size_t nt = (size_t)(n + ST - 1) / ST;
  const size_t nr = (size_t)(n + RT - 1) / RT;
  return sizeof(double) * ((size_t)n * 8 + nt + nr + nt * nt * ST) + sizeof(int) * (size_t)n + 256;
}

cudaError_t dsyev_device(cudaStream_t s, int n, const double* Phi, long long ldp, double* A, double* Z,
                         double* W, void* work, int* fail_out, long long* launches) {
  double* d = (double*)work;
  double* e = d + n;
  double* tau = e + n;
  double* vb[2] = {tau + n, tau + 2 * (size_t)n};      // reflectors of even / odd steps
  double* wb[2] = {tau + 3 * (size_t)n, tau + 4 * (size_t)n};  // their w vectors
  double* pbuf = tau + 5 * (size_t)n;                  // p of the current step
  double* dpart = pbuf + n;                            // p^T v per 32-row block
  double* npart = dpart + (n + ST - 1) / ST;           // per-CTA sums of squares of the column
  int* rank = (int*)(npart + (n + RT - 1) / RT);
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
  int ndp = 0;  // CTAs of the previous step's p kernel
  for (int k = 0; k + 2 < n; k++) {
    const int m = n - k - 1;
    const int cur = k & 1, prv = cur ^ 1;
    const int nr = ceil_div(m, RT);
    tridiag_col_kernel<<<nr, RT, 0, s>>>(n, k, A, n, d, tau, pbuf, vb[prv], wb[prv], dpart, ndp, npart);
    double* Asub = A + (k + 1) + (long long)(k + 1) * n;
    const int nt = ceil_div(m, ST);
    const double* vo = k > 0 ? vb[prv] + 1 : nullptr;  // pending update of step k-1, shifted to rows k+1..
    const double* wo = k > 0 ? wb[prv] + 1 : nullptr;
    tridiag_step_kernel<<<dim3(ceil_div(nt, SS), nt), 256, 0, s>>>(m, Asub, n, vo, wo, A + (k + 1) + (long long)k * n,
                                                                    npart, nr, vb[cur], tau + k, e + k, part);
    tridiag_p_kernel<<<nt, 256, 0, s>>>(m, nt, part, tau + k, vb[cur], pbuf, dpart);
    ndp = nt;
    nl += 3;
  }
  tridiag_tail_kernel<<<1, 1, 0, s>>>(n, A, n, d, e, tau, pbuf, n >= 3 ? vb[(n - 3) & 1] : nullptr, dpart, ndp);
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
      // G = Y^T Y has only (nb/64)^2 output tiles: K split over the SMs, W2 as scratch
      rc = dgemm_splitk(s, true, false, nb, nb, mr, 1.0, Yb, mr, Yb, mr, 0.0, G, nb, W2, (long long)NB * n);
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
