// Adjoint (vector-Jacobian product) of the eigen variant, FP64, and the
// null-model REML log-likelihood with its h-gradient.
//
// Forward per SNP i, trait j in the eigenbasis (v_l = [ZtXL_l ; r_il],
// r_i = Z^T x_i, d_l = 1/(s h w_l + s (1-h))):
//     S = sum_l d_l v_l v_l^T,  b = sum_l d_l v_l ytil_l,  beta = S^-1 b.
// With a cotangent bbar per (i, j) and g = S^-1 bbar:
//   dL/dd_l     = (g^T v_l)(ytil_l - v_l^T beta)
//   dL/dh_j     = sum_i g^T (b_c - S_c beta),  S_c, b_c: the Gram blocks with
//                 weights c_l = dd_l/dh = -s (w_l - 1) d_l^2 (recomputed from R,
//                 never stored per SNP)
//   dL/dsigma_j = sum_i g^T (b_s - S_s beta),  weights dd_l/ds = -d_l/s
//                 (= -(1/s) g^T (b - S beta), zero up to rounding: beta does
//                 not depend on the overall scale of M)
//   dL/dy_j     = Z (d_j .* sum_i V_i g_i) = Z (d_j .* (ZtXL gL_j + R gR_j))
// Null-model REML (sigma given, constants dropped):
//   l(h) = -1/2 [ -sum_l log d_l + log det V_tl + sum_l d_l r0_l^2 ],
//   r0 = ZtY - ZtXL b_L, V_tl = sum d ZtXL ZtXL^T, b_L = V_tl^-1 sum d ZtXL ytil;
//   dl/dh = -1/2 [ -sum c_l/d_l + tr(V_tl^-1 V_tl^c) + sum c_l r0_l^2 ]
//   (the b_L term vanishes at the optimum).
#include <algorithm>

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

// k x k SPD (column-major): Cholesky in place (lower); false if not SPD
__device__ bool chol_small(int k, double* A) {
  for (int j = 0; j < k; j++) {
    double a = A[j + j * k];
    for (int q = 0; q < j; q++) a -= A[j + q * k] * A[j + q * k];
    if (!(a > 0.0)) return false;
    const double ljj = sqrt(a);
    A[j + j * k] = ljj;
    for (int i = j + 1; i < k; i++) {
      double v = A[i + j * k];
      for (int q = 0; q < j; q++) v -= A[i + q * k] * A[j + q * k];
      A[i + j * k] = v / ljj;
    }
  }
  return true;
}
__device__ void chol_solve_small(int k, const double* L, double* x) {
  for (int i = 0; i < k; i++) {
    double v = x[i];
    for (int q = 0; q < i; q++) v -= L[i + q * k] * x[q];
    x[i] = v / L[i + i * k];
  }
  for (int i = k - 1; i >= 0; i--) {
    double v = x[i];
    for (int q = i + 1; q < k; q++) v -= L[q + i * k] * x[q];
    x[i] = v / L[i + i * k];
  }
}

// Per trait (one CTA): derivative weights, weighted operands and top blocks
// for c = dd/dh and s = dd/dsigma, and the REML value and h-gradient.
//   W2[:, j]            = c_j,           W2[:, t + j] = s_j
//   AYLc[:, j]          = ZtY_j .* c_j,   AYLc[:, t + j*wXL + k] = ZtXL_k .* c_j   (same for AYLs)
//   topc[j] = {sum c ZtXL ytil (wXL), sum c ZtXL ZtXL^T (wXL^2)}  (same for tops)
__global__ void __launch_bounds__(256) adj_trait_kernel(int n, int t, int wXL, const double* __restrict__ W,
                                                        const double* __restrict__ hh, const double* __restrict__ ss,
                                                        const double* __restrict__ ZtXL, const double* __restrict__ ZtY,
                                                        const double* __restrict__ dinv, double* __restrict__ Wc,
                                                        double* __restrict__ AYLc, double* __restrict__ AYLs,
                                                        double* __restrict__ topc, double* __restrict__ tops,
                                                        double* __restrict__ reml) {
  const int j = blockIdx.x;
  __shared__ double red[33];
  __shared__ double V[FGLS_MAX_P * FGLS_MAX_P], Vc[FGLS_MAX_P * FGLS_MAX_P], bt[FGLS_MAX_P], bl[FGLS_MAX_P];
  const double s = ss[j];  // dd/dh needs only sigma and w: d = 1/(s (h w + 1 - h))
  const double* y = ZtY + (long long)j * n;
  const double* d = dinv + (long long)j * n;
  const int tw = wXL + wXL * wXL;
  for (int l = threadIdx.x; l < n; l += blockDim.x) {
    const double dl = d[l];
    const double c = -s * (W[l] - 1.0) * dl * dl;
    const double sg = -dl / s;
    Wc[l + (long long)j * n] = c;
    Wc[l + (long long)(t + j) * n] = sg;
    AYLc[l + (long long)j * n] = y[l] * c;
    AYLs[l + (long long)j * n] = y[l] * sg;
    for (int k = 0; k < wXL; k++) {
      AYLc[l + (long long)(t + j * wXL + k) * n] = ZtXL[l + (long long)k * n] * c;
      AYLs[l + (long long)(t + j * wXL + k) * n] = ZtXL[l + (long long)k * n] * sg;
    }
  }
  // top blocks for d (to rebuild b_L), c and s
  for (int which = 0; which < 3; which++) {
    for (int a = 0; a < wXL; a++) {
      double v = 0.0;
      for (int l = threadIdx.x; l < n; l += blockDim.x) {
        const double dl = d[l];
        const double wgt = which == 0 ? dl : (which == 1 ? -s * (W[l] - 1.0) * dl * dl : -dl / s);
        v += wgt * ZtXL[l + (long long)a * n] * y[l];
      }
      v = block_sum(v, red);
      if (threadIdx.x == 0) {
        if (which == 0) bt[a] = v;
        else if (which == 1) topc[(long long)j * tw + a] = v;
        else tops[(long long)j * tw + a] = v;
      }
      for (int b = 0; b <= a; b++) {
        double q = 0.0;
        for (int l = threadIdx.x; l < n; l += blockDim.x) {
          const double dl = d[l];
          const double wgt = which == 0 ? dl : (which == 1 ? -s * (W[l] - 1.0) * dl * dl : -dl / s);
          q += wgt * ZtXL[l + (long long)a * n] * ZtXL[l + (long long)b * n];
        }
        q = block_sum(q, red);
        if (threadIdx.x == 0) {
          if (which == 0) {
            V[a + b * wXL] = q;
            V[b + a * wXL] = q;
          } else {
            double* T = (which == 1 ? topc : tops) + (long long)j * tw + wXL;
            T[a + b * wXL] = q;
            T[b + a * wXL] = q;
            if (which == 1) {
              Vc[a + b * wXL] = q;
              Vc[b + a * wXL] = q;
            }
          }
        }
      }
    }
  }
  __syncthreads();
  __shared__ double logdet, trterm;
  __shared__ int ok;
  if (threadIdx.x == 0) {
    double L[FGLS_MAX_P * FGLS_MAX_P];
    for (int e = 0; e < wXL * wXL; e++) L[e] = V[e];
    ok = chol_small(wXL, L);
    logdet = 0.0;
    trterm = 0.0;
    if (ok) {
      for (int a = 0; a < wXL; a++) {
        logdet += 2.0 * log(L[a + a * wXL]);
        bl[a] = bt[a];
      }
      chol_solve_small(wXL, L, bl);
      // tr(V^-1 Vc) = sum_a (V^-1 Vc[:, a])_a
      for (int a = 0; a < wXL; a++) {
        double col[FGLS_MAX_P];
        for (int q = 0; q < wXL; q++) col[q] = Vc[q + a * wXL];
        chol_solve_small(wXL, L, col);
        trterm += col[a];
      }
    }
  }
  __syncthreads();
  double sl = 0.0, sq = 0.0, sc = 0.0, scr = 0.0;
  for (int l = threadIdx.x; l < n; l += blockDim.x) {
    const double dl = d[l];
    const double c = -s * (W[l] - 1.0) * dl * dl;
    double r = y[l];
    for (int a = 0; a < wXL; a++) r -= ZtXL[l + (long long)a * n] * bl[a];
    sl += log(dl);
    sq += dl * r * r;
    sc += c / dl;
    scr += c * r * r;
  }
  sl = block_sum(sl, red);
  sq = block_sum(sq, red);
  sc = block_sum(sc, red);
  scr = block_sum(scr, red);
  if (threadIdx.x == 0) {
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    reml[j] = ok ? -0.5 * (-sl + logdet + sq) : nan;
    reml[t + j] = ok ? -0.5 * (-sc + trterm + scr) : nan;
  }
}

// One thread per (SNP i, trait j): recompute beta from the d-Gram, g = S^-1 bbar,
// contributions g^T (b_w - S_w beta) for w = c (h) and s (sigma), and g itself.
template <int P>
__global__ void __launch_bounds__(128) adj_snp_kernel(int x, int t, int wXL, const double* __restrict__ top,
                                                      const double* __restrict__ GYL, const double* __restrict__ GR,
                                                      const double* __restrict__ topc, const double* __restrict__ GYLc,
                                                      const double* __restrict__ GRc, const double* __restrict__ tops,
                                                      const double* __restrict__ GYLs, const double* __restrict__ GRs,
                                                      const double* __restrict__ Bbar, long long bstride,
                                                      double* __restrict__ contrib, double* __restrict__ gout,
                                                      DevStatus* st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= x) return;
  const int tw0 = wXL + wXL * wXL + 1, tw = wXL + wXL * wXL;
  const long long ld = x;  // Gram layout of the FP64 path, wXR = 1
  double S[P][P], b[P];
  auto load = [&](const double* T, int stride, const double* G, const double* Gr, double (&SS)[P][P], double (&bb)[P]) {
    for (int a = 0; a < wXL; a++) {
      bb[a] = T[(long long)j * stride + a];
      for (int q = 0; q < wXL; q++) SS[a][q] = T[(long long)j * stride + wXL + a + q * wXL];
    }
    bb[wXL] = G[i + (long long)j * ld];
    for (int k = 0; k < wXL; k++) {
      const double v = G[i + (long long)(t + j * wXL + k) * ld];
      SS[wXL][k] = v;
      SS[k][wXL] = v;
    }
    SS[wXL][wXL] = Gr[i + (long long)j * ld];
  };
  load(top, tw0, GYL, GR, S, b);
  // Cholesky of S
  double L[P][P];
  int info = 0;
#pragma unroll
  for (int c = 0; c < P; c++) {
    double a = S[c][c];
#pragma unroll
    for (int q = 0; q < c; q++) a -= L[c][q] * L[c][q];
    if (!(a > 0.0) && info == 0) info = c + 1;
    L[c][c] = sqrt(a);
#pragma unroll
    for (int r = c + 1; r < P; r++) {
      double v = S[r][c];
#pragma unroll
      for (int q = 0; q < c; q++) v -= L[r][q] * L[c][q];
      L[r][c] = v / L[c][c];
    }
  }
  if (info) set_status(st, FGLSGPU_ENOTSPD, info, i);
  auto solve = [&](double (&v)[P]) {
#pragma unroll
    for (int r = 0; r < P; r++) {
      double s = v[r];
#pragma unroll
      for (int q = 0; q < r; q++) s -= L[r][q] * v[q];
      v[r] = s / L[r][r];
    }
#pragma unroll
    for (int r = P - 1; r >= 0; r--) {
      double s = v[r];
#pragma unroll
      for (int q = r + 1; q < P; q++) s -= L[q][r] * v[q];
      v[r] = s / L[r][r];
    }
  };
  double beta[P], g[P];
#pragma unroll
  for (int r = 0; r < P; r++) {
    beta[r] = b[r];
    g[r] = Bbar[(long long)j * bstride + (long long)i * P + r];
  }
  solve(beta);
  solve(g);
  double out[2];
#pragma unroll
  for (int w = 0; w < 2; w++) {
    double Sw[P][P], bw[P];
    if (w == 0) load(topc, tw, GYLc, GRc, Sw, bw);
    else load(tops, tw, GYLs, GRs, Sw, bw);
    double acc = 0.0;
#pragma unroll
    for (int r = 0; r < P; r++) {
      double v = bw[r];
#pragma unroll
      for (int q = 0; q < P; q++) v -= Sw[r][q] * beta[q];
      acc += g[r] * v;
    }
    out[w] = acc;
  }
  contrib[(long long)j * x + i] = out[0];
  contrib[(long long)(t + j) * x + i] = out[1];
#pragma unroll
  for (int r = 0; r < P; r++) gout[((long long)j * x + i) * P + r] = g[r];
}

// Per trait: deterministic sums over the block's SNPs of the h and sigma
// contributions and of g_L; gR (x x t) for the dy GEMM.
__global__ void __launch_bounds__(256) adj_reduce_kernel(int x, int t, int P, int wXL, const double* __restrict__ contrib,
                                                         const double* __restrict__ g, double* __restrict__ acc,
                                                         double* __restrict__ gR) {
  const int j = blockIdx.x;
  __shared__ double red[33];
  double sh = 0.0, ssg = 0.0;
  for (int i = threadIdx.x; i < x; i += blockDim.x) {
    sh += contrib[(long long)j * x + i];
    ssg += contrib[(long long)(t + j) * x + i];
    gR[i + (long long)j * x] = g[((long long)j * x + i) * P + wXL];
  }
  sh = block_sum(sh, red);
  ssg = block_sum(ssg, red);
  double gl[FGLS_MAX_P];
  for (int k = 0; k < wXL; k++) {
    double v = 0.0;
    for (int i = threadIdx.x; i < x; i += blockDim.x) v += g[((long long)j * x + i) * P + k];
    gl[k] = block_sum(v, red);
  }
  if (threadIdx.x == 0) {
    // acc layout: [dh (t) | dsigma (t) | gL (t x wXL)]
    acc[j] += sh;
    acc[t + j] += ssg;
    for (int k = 0; k < wXL; k++) acc[2 * t + j * wXL + k] += gl[k];
  }
}

// V2[:, j] = d_j .* (ZtXL gL_j + U[:, j])
__global__ void adj_ybar_kernel(int n, int t, int wXL, const double* __restrict__ dinv, const double* __restrict__ ZtXL,
                                const double* __restrict__ acc, const double* __restrict__ U, double* __restrict__ V2) {
  const long long total = (long long)n * t;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int l = (int)(e % n), j = (int)(e / n);
    double v = U[e];
    for (int k = 0; k < wXL; k++) v += ZtXL[l + (long long)k * n] * acc[2 * t + j * wXL + k];
    V2[e] = dinv[e] * v;
  }
}

}  // namespace

cudaError_t adjoint_traits(cudaStream_t s, int n, int t, int wXL, const double* W, const double* h,
                           const double* sigma, const double* ZtXL, const double* ZtY, const double* dinv,
                           double* Wc, double* AYLc, double* AYLs, double* topc, double* tops, double* reml) {
  adj_trait_kernel<<<t, 256, 0, s>>>(n, t, wXL, W, h, sigma, ZtXL, ZtY, dinv, Wc, AYLc, AYLs, topc, tops, reml);
  note_launch();
  return cudaGetLastError();
}

cudaError_t adjoint_snps(cudaStream_t s, int p, int x, int t, int wXL, const double* top, const double* GYL,
                         const double* GR, const double* topc, const double* GYLc, const double* GRc,
                         const double* tops, const double* GYLs, const double* GRs, const double* Bbar,
                         long long bstride, double* contrib, double* g, DevStatus* st) {
  dim3 grid(ceil_div(x, 128), t);
  switch (p) {
#define FGLS_ADJ_CASE(P)                                                                                   \
  case P:                                                                                                  \
    adj_snp_kernel<P><<<grid, 128, 0, s>>>(x, t, wXL, top, GYL, GR, topc, GYLc, GRc, tops, GYLs, GRs, Bbar, \
                                           bstride, contrib, g, st);                                       \
    break;
    FGLS_ADJ_CASE(2)
    FGLS_ADJ_CASE(3)
    FGLS_ADJ_CASE(4)
    FGLS_ADJ_CASE(5)
    FGLS_ADJ_CASE(6)
    FGLS_ADJ_CASE(7)
    FGLS_ADJ_CASE(8)
#undef FGLS_ADJ_CASE
    default:
      return cudaErrorInvalidValue;
  }
  note_launch();
  return cudaGetLastError();
}

cudaError_t adjoint_reduce(cudaStream_t s, int x, int t, int p, int wXL, const double* contrib, const double* g,
                           double* acc, double* gR) {
  adj_reduce_kernel<<<t, 256, 0, s>>>(x, t, p, wXL, contrib, g, acc, gR);
  note_launch();
  return cudaGetLastError();
}

cudaError_t adjoint_ybar(cudaStream_t s, int n, int t, int wXL, const double* dinv, const double* ZtXL,
                         const double* acc, const double* U, double* V2) {
  const long long total = (long long)n * t;
  const int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 32);
  adj_ybar_kernel<<<blocks, 256, 0, s>>>(n, t, wXL, dinv, ZtXL, acc, U, V2);
  note_launch();
  return cudaGetLastError();
}

}  // namespace fgls
