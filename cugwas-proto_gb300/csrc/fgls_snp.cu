// Per-trait and per-SNP kernels of the FGLS association:
//
//  * chol null model  (src/fgls_chol.c:273-325): B_t = XL~^T y~, V_tl = XL~^T XL~,
//    b_L = V_tl^-1 B_t, res_sigma = |y~ - XL~ b_L|^2 / (n - wXL)
//  * eigen null model (src/fgls_eigen.c:428-466 and :1085-1160) in the
//    eigenbasis with d_j(l) = 1 / (alpha_j W_l + beta_j)
//  * skinny Gram (src/fgls_chol.c:392-414): per SNP column x~, x~^T [y~ XL~]
//    and the wXR x wXR self products
//  * batched p x p solve (src/fgls_chol.c:416-438): potrf, two trsv, potri,
//    res_sigma scaling, square-root diagonal, one thread per (SNP, trait)
//    test in registers.
//
// Gram layout shared by both variants (col-major, ld = x*wXR rows):
//   GYL[(i*wXR+c) + j*ld]              = x~_{i,c}^T y~_j            (j < t)
//   GYL[(i*wXR+c) + (t + j*wXL+k)*ld]  = x~_{i,c}^T XL~_{j,k}
//   GR [((i*wXR+c)*wXR+d) + j*ldr]     = x~_{i,c}^T x~_{i,d}  (trait j weights)
// Per-trait "top" record TOP[j*topw + ...] = {B_t[wXL], V_tl[wXL*wXL], res_sigma}.
#include <algorithm>

#include "fgls_common.cuh"
#include "fgls_kernels.cuh"
#include "fgls_batch.cuh"

namespace fgls {

namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum for 256 threads; every thread gets the result.
__device__ double block_sum256(double v, double* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x < 32) {
    s = (l < (int)(blockDim.x >> 5)) ? red[l] : 0.0;
    s = warp_sum(s);
    if (l == 0) red[8] = s;
  }
  __syncthreads();
  return red[8];
}

// Small SPD solve (wXL <= FGLS_MAX_P) by unblocked lower Cholesky, single thread.
__device__ bool small_chol_solve(int k, const double* S, const double* b, double* x) {
  double L[FGLS_MAX_P * FGLS_MAX_P];
  for (int j = 0; j < k; j++) {
    double a = S[j + j * k];
    for (int q = 0; q < j; q++) a -= L[j + q * k] * L[j + q * k];
    if (!(a > 0.0)) return false;
    double ljj = sqrt(a);
    L[j + j * k] = ljj;
    for (int i = j + 1; i < k; i++) {
      double v = S[i + j * k];
      for (int q = 0; q < j; q++) v -= L[i + q * k] * L[j + q * k];
      L[i + j * k] = v / ljj;
    }
  }
  double z[FGLS_MAX_P];
  for (int i = 0; i < k; i++) {
    double v = b[i];
    for (int q = 0; q < i; q++) v -= L[i + q * k] * z[q];
    z[i] = v / L[i + i * k];
  }
  for (int i = k - 1; i >= 0; i--) {
    double v = z[i];
    for (int q = i + 1; q < k; q++) v -= L[q + i * k] * x[q];
    x[i] = v / L[i + i * k];
  }
  return true;
}

// chol null model, one CTA of 256 threads.  WY = [y~ | XL~] (n x (1+wXL), ld n).
__global__ void __launch_bounds__(256) null_model_chol_kernel(int n, int wXL, const double* __restrict__ WY,
                                                              double* __restrict__ top, DevStatus* st,
                                                              int trait) {
  __shared__ double red[16];
  __shared__ double S[FGLS_MAX_P * FGLS_MAX_P], bt[FGLS_MAX_P], bl[FGLS_MAX_P];
  const double* y = WY;
  const double* XLt = WY + n;
  for (int a = 0; a < wXL; a++) {
    double s = 0.0;
    for (int l = threadIdx.x; l < n; l += blockDim.x) s += XLt[l + (long long)a * n] * y[l];
    s = block_sum256(s, red);
    if (threadIdx.x == 0) bt[a] = s;
    for (int b = 0; b <= a; b++) {
      double q = 0.0;
      for (int l = threadIdx.x; l < n; l += blockDim.x)
        q += XLt[l + (long long)a * n] * XLt[l + (long long)b * n];
      q = block_sum256(q, red);
      if (threadIdx.x == 0) { S[a + b * wXL] = q; S[b + a * wXL] = q; }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!small_chol_solve(wXL, S, bt, bl)) set_status(st, FGLSGPU_ENOTSPD, -1, trait);
  }
  __syncthreads();
  // r = y~ - XL~ b_L  (= L^-1 (y - XL b_L), src/fgls_chol.c:318-324, by linearity)
  double s = 0.0;
  for (int l = threadIdx.x; l < n; l += blockDim.x) {
    double r = y[l];
    for (int a = 0; a < wXL; a++) r -= XLt[l + (long long)a * n] * bl[a];
    s += r * r;
  }
  s = block_sum256(s, red);
  if (threadIdx.x == 0) {
    const int tw = wXL + wXL * wXL + 1;
    double* T = top + (long long)trait * tw;
    for (int a = 0; a < wXL; a++) T[a] = bt[a];
    for (int e = 0; e < wXL * wXL; e++) T[wXL + e] = S[e];
    T[wXL + wXL * wXL] = s / (double)(n - wXL);
  }
}

// eigen per-trait weights and null model, one CTA per trait.
//   dinv[l + j*n] = 1 / (a_j W_l + b_j)       (Winv^2 of src/fgls_eigen.c:441)
//   AYL[:, j]              = ZtY[:, j] * dinv[:, j]
//   AYL[:, t + j*wXL + k]  = ZtXL[:, k] * dinv[:, j]
//   top[j] = {B_t, V_tl, res_sigma} with res_sigma from src/fgls_eigen.c:1085-1160
//   (Z^T (y - XL b) computed as ZtY - ZtXL b, the same vector by linearity).
__global__ void __launch_bounds__(256) eigen_trait_kernel(int n, int t, int wXL, const double* __restrict__ W,
                                                          const double* __restrict__ hh,
                                                          const double* __restrict__ ss,
                                                          const double* __restrict__ ZtXL,
                                                          const double* __restrict__ ZtY,
                                                          double* __restrict__ dinv, double* __restrict__ AYL,
                                                          double* __restrict__ top, DevStatus* st) {
  const int j = blockIdx.x;
  __shared__ double red[16];
  __shared__ double S[FGLS_MAX_P * FGLS_MAX_P], bt[FGLS_MAX_P], bl[FGLS_MAX_P];
  const double a = ss[j] * hh[j];
  const double b = ss[j] * (1.0 - hh[j]);
  const double* y = ZtY + (long long)j * n;
  for (int l = threadIdx.x; l < n; l += blockDim.x) {
    double winv = sqrt(1.0 / (a * W[l] + b));
    double d = winv * winv;
    dinv[l + (long long)j * n] = d;
    AYL[l + (long long)j * n] = y[l] * d;
    for (int k = 0; k < wXL; k++) AYL[l + (long long)(t + j * wXL + k) * n] = ZtXL[l + (long long)k * n] * d;
  }
  for (int p = 0; p < wXL; p++) {
    double s = 0.0;
    for (int l = threadIdx.x; l < n; l += blockDim.x) {
      double winv = sqrt(1.0 / (a * W[l] + b));
      s += (ZtXL[l + (long long)p * n] * winv) * (y[l] * winv);
    }
    s = block_sum256(s, red);
    if (threadIdx.x == 0) bt[p] = s;
    for (int q = 0; q <= p; q++) {
      double v = 0.0;
      for (int l = threadIdx.x; l < n; l += blockDim.x) {
        double winv = sqrt(1.0 / (a * W[l] + b));
        v += (ZtXL[l + (long long)p * n] * winv) * (ZtXL[l + (long long)q * n] * winv);
      }
      v = block_sum256(v, red);
      if (threadIdx.x == 0) { S[p + q * wXL] = v; S[q + p * wXL] = v; }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!small_chol_solve(wXL, S, bt, bl)) set_status(st, FGLSGPU_ENOTSPD, -1, j);
  }
  __syncthreads();
  double s = 0.0;
  for (int l = threadIdx.x; l < n; l += blockDim.x) {
    double r = y[l];
    for (int p = 0; p < wXL; p++) r -= ZtXL[l + (long long)p * n] * bl[p];
    double winv = sqrt(1.0 / (a * W[l] + b));
    r *= winv;
    s += r * r;
  }
  s = block_sum256(s, red);
  if (threadIdx.x == 0) {
    const int tw = wXL + wXL * wXL + 1;
    double* T = top + (long long)j * tw;
    for (int p = 0; p < wXL; p++) T[p] = bt[p];
    for (int e = 0; e < wXL * wXL; e++) T[wXL + e] = S[e];
    T[wXL + wXL * wXL] = s / (double)(n - wXL);
  }
}

// Skinny Gram for the chol variant (one trait).  X: n x (x*wXR) whitened SNP
// columns; C = [y~ | XL~] (n x (1+wXL)).  One warp per SNP (its wXR columns),
// 8 warps per CTA share a shared-memory copy of a 256-row chunk of C.
constexpr int SG_ROWS = 256;
__global__ void __launch_bounds__(256) gram_skinny_kernel(int n, int x, int wXL, int wXR,
                                                          const double* __restrict__ X, long long ldx,
                                                          const double* __restrict__ C,
                                                          double* __restrict__ GYL, double* __restrict__ GR) {
  __shared__ double Cs[SG_ROWS * (FGLS_MAX_P + 1)];
  const int nc = 1 + wXL;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int snp = blockIdx.x * 8 + warp;
  const bool active = snp < x;
  double acc_c[FGLS_MAX_WXR][FGLS_MAX_P + 1];
  double acc_r[FGLS_MAX_WXR][FGLS_MAX_WXR];
  for (int c = 0; c < FGLS_MAX_WXR; c++) {
    for (int q = 0; q <= FGLS_MAX_P; q++) acc_c[c][q] = 0.0;
    for (int d = 0; d < FGLS_MAX_WXR; d++) acc_r[c][d] = 0.0;
  }
  for (int l0 = 0; l0 < n; l0 += SG_ROWS) {
    const int rows = min(SG_ROWS, n - l0);
    __syncthreads();
    for (int e = threadIdx.x; e < rows * nc; e += blockDim.x) {
      int r = e % rows, q = e / rows;
      Cs[q * SG_ROWS + r] = C[(l0 + r) + (long long)q * n];
    }
    __syncthreads();
    if (!active) continue;
    for (int r = lane; r < rows; r += 32) {
      double xv[FGLS_MAX_WXR];
      for (int c = 0; c < wXR; c++) xv[c] = X[(l0 + r) + (long long)(snp * wXR + c) * ldx];
      for (int c = 0; c < wXR; c++) {
        for (int q = 0; q < nc; q++) acc_c[c][q] = fma(xv[c], Cs[q * SG_ROWS + r], acc_c[c][q]);
        for (int d = 0; d <= c; d++) acc_r[c][d] = fma(xv[c], xv[d], acc_r[c][d]);
      }
    }
  }
  if (!active) return;
  const long long ld = (long long)x * wXR;
  for (int c = 0; c < wXR; c++) {
    for (int q = 0; q < nc; q++) {
      double v = warp_sum(acc_c[c][q]);
      if (lane == 0) GYL[(snp * wXR + c) + q * ld] = v;
    }
    for (int d = 0; d <= c; d++) {
      double v = warp_sum(acc_r[c][d]);
      if (lane == 0) {
        GR[((long long)(snp * wXR + c)) * wXR + d] = v;
        GR[((long long)(snp * wXR + d)) * wXR + c] = v;
      }
    }
  }
}

// Q[:, (i*wXR+c)*wXR+d] = R[:, i*wXR+c] * R[:, i*wXR+d]  (eigen self-product
// operand; the GEMM Q^T dinv then yields GR for every trait).
__global__ void quad_products_kernel(int n, int x, int wXR, const double* __restrict__ R, long long ldr,
                                     double* __restrict__ Q, long long ldq) {
  const long long cols = (long long)x * wXR * wXR;
  const long long total = cols * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int l = (int)(e % n);
    const long long col = e / n;
    const int d = (int)(col % wXR);
    const long long ic = col / wXR;  // i*wXR + c
    const long long i = ic / wXR;
    Q[l + col * ldq] = R[l + ic * ldr] * R[l + (i * wXR + d) * ldr];
  }
}

// ---------------------------------------------------------------------------
// Batched p x p solve: one thread per (SNP, trait) test.
// ---------------------------------------------------------------------------
// 128 tests (SNPs i0 .. i0+127 of trait j) per CTA of 128 threads; `tag` is
// added to the pivot index of a non-SPD report.
template <int P>
__device__ __forceinline__ void solve_block(int x, int t, int wXL, const int j, const int i0,
                                            const double* __restrict__ top, const double* __restrict__ GYL,
                                            long long rsg, long long ldg, const double* __restrict__ GR, long long ldr,
                                            double* __restrict__ Bout, long long bstride, double* __restrict__ Vout,
                                            long long vstride, DevStatus* st, long long snp_base, int tag) {
  extern __shared__ double stage[];  // [128][P + P*P]
  const int wXR = P - wXL;
  const int i = i0 + threadIdx.x;
  const int tw = wXL + wXL * wXL + 1;
  const double* T = top + (long long)j * tw;
  const bool valid = i < x;
  double* out = stage + threadIdx.x * (P + P * P);
  if (wXL == P - 1) {
    // One genotype column per SNP (wXR = 1): the leading W x W block of S
    // (XL^T M^-1 XL) and b (XL^T M^-1 y) are the same for every SNP of trait
    // j, so thread 0 factors them once for the CTA.  The per-SNP work below
    // is the last row of the factor, the Schur complement pivot and the
    // rank-one terms, in the same operation order as the general path, so
    // both give the same bits.
    constexpr int W = P - 1;
    __shared__ double sL[W][W], sri[W], szt[W], sLi[W][W], sAi[W][W], srs;
    __shared__ int sinfo;
    if (threadIdx.x == 0) {
      double A[W][W], L[W][W], ri[W], Li[W][W], z[W];
      for (int a = 0; a < W; a++)
        for (int q = 0; q <= a; q++) A[a][q] = T[W + a + q * W];
      int info = 0;
#pragma unroll
      for (int c = 0; c < W; c++) {
        double v = A[c][c];
#pragma unroll
        for (int q = 0; q < c; q++) v -= L[c][q] * L[c][q];
        if (!(v > 0.0) && info == 0) info = c + 1;
        const double lcc = sqrt(v);
        L[c][c] = lcc;
        ri[c] = 1.0 / lcc;
#pragma unroll
        for (int r = c + 1; r < W; r++) {
          double u = A[r][c];
#pragma unroll
          for (int q = 0; q < c; q++) u -= L[r][q] * L[c][q];
          L[r][c] = u * ri[c];
        }
      }
#pragma unroll
      for (int r = 0; r < W; r++) {
        double v = T[r];
#pragma unroll
        for (int q = 0; q < r; q++) v -= L[r][q] * z[q];
        z[r] = v * ri[r];
      }
#pragma unroll
      for (int c = 0; c < W; c++) {
        Li[c][c] = ri[c];
#pragma unroll
        for (int r = c + 1; r < W; r++) {
          double v = 0.0;
#pragma unroll
          for (int q = c; q < r; q++) v -= L[r][q] * Li[q][c];
          Li[r][c] = v * ri[r];
        }
      }
#pragma unroll
      for (int c = 0; c < W; c++) {
        sri[c] = ri[c];
        szt[c] = z[c];
#pragma unroll
        for (int r = c; r < W; r++) {
          sL[r][c] = L[r][c];
          sLi[r][c] = Li[r][c];
          double v = 0.0;
#pragma unroll
          for (int q = r; q < W; q++) v += Li[q][r] * Li[q][c];
          sAi[r][c] = v;  // rows q < W of (Li^T Li)[r][c]
        }
      }
      srs = T[W + W * W];
      sinfo = info;
    }
    __syncthreads();
    if (valid) {
      const long long row = i;
      double l[W];
      const double cc = GR[row + (long long)j * ldr];
      const double yx = GYL[row * rsg + (long long)j * ldg];
#pragma unroll
      for (int c = 0; c < W; c++) l[c] = GYL[row * rsg + (long long)(t + j * W + c) * ldg];
      // last row of the factor: l = L_A^-1 s, pivot^2 = c - l^T l
#pragma unroll
      for (int c = 0; c < W; c++) {
        double v = l[c];
#pragma unroll
        for (int q = 0; q < c; q++) v -= l[q] * sL[c][q];
        l[c] = v * sri[c];
      }
      double dd = cc;
#pragma unroll
      for (int q = 0; q < W; q++) dd -= l[q] * l[q];
      int info = sinfo;
      if (!(dd > 0.0) && info == 0) info = P;
      if (info) set_status(st, FGLSGPU_ENOTSPD, tag + info, snp_base + i);
      const double rP = 1.0 / sqrt(dd);
      // forward and back substitution
      double zP = yx;
#pragma unroll
      for (int q = 0; q < W; q++) zP -= l[q] * szt[q];
      zP *= rP;
      const double bP = zP * rP;
      double beta[W];
#pragma unroll
      for (int r = W - 1; r >= 0; r--) {
        double v = szt[r];
#pragma unroll
        for (int q = r + 1; q < W; q++) v -= sL[q][r] * beta[q];
        v -= l[r] * bP;
        beta[r] = v * sri[r];
      }
      // last row of L^-1, then S^-1 = Li^T Li
      double lp[W];
#pragma unroll
      for (int c = 0; c < W; c++) {
        double v = 0.0;
#pragma unroll
        for (int q = c; q < W; q++) v -= l[q] * sLi[q][c];
        lp[c] = v * rP;
      }
      const double rs = srs;
#pragma unroll
      for (int r = 0; r < W; r++) out[r] = beta[r];
      out[W] = bP;
      double* vo = out + P;
#pragma unroll
      for (int c = 0; c < P; c++) {
#pragma unroll
        for (int r = 0; r < P; r++) {
          double v = 0.0;
          if (r >= c) {
            if (r < W)
              v = sAi[r][c] + lp[r] * lp[c];
            else if (c < W)
              v = rP * lp[c];
            else
              v = rP * rP;
            v *= rs;
            if (r == c) v = sqrt(v);
          }
          vo[r + c * P] = v;  // column-major, strict upper = 0
        }
      }
    }
  } else {
    double S[P][P];  // lower triangle used
    double b[P];
    if (valid) {
      for (int a = 0; a < wXL; a++) {
        b[a] = T[a];
        for (int q = 0; q <= a; q++) S[a][q] = T[wXL + a + q * wXL];
      }
      for (int c = 0; c < wXR; c++) {
        const long long row = (long long)i * wXR + c;
        b[wXL + c] = GYL[row * rsg + (long long)j * ldg];
        for (int k = 0; k < wXL; k++) S[wXL + c][k] = GYL[row * rsg + (long long)(t + j * wXL + k) * ldg];
        for (int d = 0; d <= c; d++) S[wXL + c][wXL + d] = GR[row * wXR + d + (long long)j * ldr];
      }
    }
    if (valid) {
      const double rs = T[wXL + wXL * wXL];
      // potrf (lower, unblocked).  One division per column (ri = 1 / L_cc),
      // multiplications elsewhere: FP64 division is a multi-instruction
      // sequence on GB300's narrow FP64 pipe, which bounds this kernel.
      double L[P][P], ri[P];
      int info = 0;
#pragma unroll
      for (int c = 0; c < P; c++) {
        double a = S[c][c];
#pragma unroll
        for (int q = 0; q < c; q++) a -= L[c][q] * L[c][q];
        if (!(a > 0.0) && info == 0) info = c + 1;
        const double lcc = sqrt(a);
        L[c][c] = lcc;
        ri[c] = 1.0 / lcc;
#pragma unroll
        for (int r = c + 1; r < P; r++) {
          double v = S[r][c];
#pragma unroll
          for (int q = 0; q < c; q++) v -= L[r][q] * L[c][q];
          L[r][c] = v * ri[c];
        }
      }
      if (info) set_status(st, FGLSGPU_ENOTSPD, tag + info, snp_base + i);
      // two triangular solves: L z = b, L^T beta = z
      double z[P];
#pragma unroll
      for (int r = 0; r < P; r++) {
        double v = b[r];
#pragma unroll
        for (int q = 0; q < r; q++) v -= L[r][q] * z[q];
        z[r] = v * ri[r];
      }
#pragma unroll
      for (int r = P - 1; r >= 0; r--) {
        double v = z[r];
#pragma unroll
        for (int q = r + 1; q < P; q++) v -= L[q][r] * z[q];
        z[r] = v * ri[r];
      }
      // potri: Li = L^-1 (lower), Sinv = Li^T Li (lower part)
      double Li[P][P];
#pragma unroll
      for (int c = 0; c < P; c++) {
        Li[c][c] = ri[c];
#pragma unroll
        for (int r = c + 1; r < P; r++) {
          double v = 0.0;
#pragma unroll
          for (int q = c; q < r; q++) v -= L[r][q] * Li[q][c];
          Li[r][c] = v * ri[r];
        }
      }
#pragma unroll
      for (int r = 0; r < P; r++) out[r] = z[r];
      double* vo = out + P;
#pragma unroll
      for (int c = 0; c < P; c++) {
#pragma unroll
        for (int r = 0; r < P; r++) {
          double v = 0.0;
          if (r >= c) {
#pragma unroll
            for (int q = r; q < P; q++) v += Li[q][r] * Li[q][c];
            v *= rs;
            if (r == c) v = sqrt(v);
          }
          vo[r + c * P] = v;  // column-major, strict upper = 0
        }
      }
    }
  }
  __syncthreads();
  // coalesced copy-out of this CTA's contiguous SNP range for trait j
  const int nv = min(128, x - i0);
  double* Bj = Bout + (long long)j * bstride + (long long)i0 * P;
  double* Vj = Vout + (long long)j * vstride + (long long)i0 * P * P;
  for (int e = threadIdx.x; e < nv * P; e += 128) Bj[e] = stage[(e / P) * (P + P * P) + (e % P)];
  for (int e = threadIdx.x; e < nv * P * P; e += 128)
    Vj[e] = stage[(e / (P * P)) * (P + P * P) + P + (e % (P * P))];
}

template <int P>
__global__ void __launch_bounds__(128) snp_solve_kernel(
    int x, int t, int wXL, const double* __restrict__ top, const double* __restrict__ GYL, long long rsg,
    long long ldg, const double* __restrict__ GR, long long ldr, double* __restrict__ Bout, long long bstride,
    double* __restrict__ Vout, long long vstride, DevStatus* st, long long snp_base) {
  solve_block<P>(x, t, wXL, blockIdx.y, blockIdx.x * 128, top, GYL, rsg, ldg, GR, ldr, Bout, bstride, Vout, vstride,
                 st, snp_base, 0);
}

// Batched cohorts: CTA b solves SNPs [128 (b % bpp), +128) of problem
// plist[b / bpp] (one trait of one cohort, wXR = 1); results go to the
// cohort's step outputs.  A non-SPD report carries (cohort + 1) << 8 + pivot.
template <int P>
__global__ void __launch_bounds__(128) snp_solve_grouped_kernel(const SolveProblem* __restrict__ probs,
                                                                const int* __restrict__ plist, int bpp,
                                                                const StepCohort* __restrict__ sc, DevStatus* st) {
  const SolveProblem pr = probs[plist[blockIdx.x / bpp]];
  const StepCohort c = sc[pr.cohort];
  const int i0 = (blockIdx.x % bpp) * 128;
  if (i0 >= c.x) return;
  solve_block<P>(c.x, 1, P - 1, 0, i0, pr.top, pr.gyl, pr.rsg, 1, pr.GR, 0, c.B + (long long)pr.trait * c.x * P, 0,
                 c.V + (long long)pr.trait * c.x * P * P, 0, st, c.snp_base, (pr.cohort + 1) << 8);
}

template <int P>
cudaError_t launch_solve(cudaStream_t s, int x, int t, int wXL, const double* top, const double* GYL,
                         long long rsg, long long ldg, const double* GR, long long ldr, double* B, long long bstride,
                         double* V, long long vstride, DevStatus* st, long long snp_base) {
  const size_t smem = sizeof(double) * 128 * (P + P * P);
  static bool attr = false;
  if (!attr) {
    FGLS_CUDA_TRY(cudaFuncSetAttribute(snp_solve_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  dim3 grid(ceil_div(x, 128), t);
  snp_solve_kernel<P><<<grid, 128, smem, s>>>(x, t, wXL, top, GYL, rsg, ldg, GR, ldr, B, bstride, V, vstride, st,
                                              snp_base);
  note_launch();
  return cudaGetLastError();
}

__global__ void u8_to_f64_kernel(const unsigned char* __restrict__ in, double* __restrict__ out, long long count) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < count;
       e += (long long)gridDim.x * blockDim.x)
    out[e] = (double)in[e];
}

// 2-bit packed hard calls, SNP-major like a PLINK .bed body: column c holds
// ceil(n/4) bytes, individual k in bits 2(k%4)..2(k%4)+1 of byte k/4.  Codes:
// 00 -> 2, 10 -> 1, 11 -> 0 (copies of the first allele), 01 = missing (status
// FGLSGPU_EINVAL with the individual and the SNP, value 0).  One CTA per
// column, one packed byte (four individuals) per thread and step.
__global__ void __launch_bounds__(256) unpack_2bit_kernel(const unsigned char* __restrict__ in, int n, int wXR,
                                                          unsigned char* __restrict__ out, DevStatus* st,
                                                          long long snp_base) {
  const long long c = blockIdx.x;
  const int bpc = (n + 3) / 4;
  const unsigned char* col = in + c * bpc;
  unsigned char* o = out + c * n;
  for (int b = threadIdx.x; b < bpc; b += blockDim.x) {
    const unsigned v = col[b];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int k = 4 * b + i;
      if (k >= n) break;
      const unsigned code = (v >> (2 * i)) & 3u;
      if (code == 1u) set_status(st, FGLSGPU_EINVAL, k, snp_base + c / wXR);
      o[k] = (unsigned char)(code == 0u ? 2 : (code == 2u ? 1 : 0));
    }
  }
}

}  // namespace

std::atomic<long long> g_launches{0};

cudaError_t unpack_2bit(cudaStream_t s, const unsigned char* in, int n, long long cols, int wXR, unsigned char* out,
                        DevStatus* st, long long snp_base) {
  if (cols <= 0) return cudaSuccess;
  unpack_2bit_kernel<<<(unsigned)cols, 256, 0, s>>>(in, n, wXR, out, st, snp_base);
  note_launch();
  return cudaGetLastError();
}

cudaError_t u8_to_f64(cudaStream_t s, const unsigned char* in, double* out, long long count) {
  int blocks = (int)std::min<long long>((count + 255) / 256, 152LL * 32);
  if (blocks <= 0) return cudaSuccess;
  u8_to_f64_kernel<<<blocks, 256, 0, s>>>(in, out, count);
  note_launch();
  return cudaGetLastError();
}

cudaError_t null_model_chol(cudaStream_t s, int n, int wXL, const double* WY, double* top, DevStatus* st,
                            int trait) {
  null_model_chol_kernel<<<1, 256, 0, s>>>(n, wXL, WY, top, st, trait);
  note_launch();
  return cudaGetLastError();
}

cudaError_t eigen_traits(cudaStream_t s, int n, int t, int wXL, const double* W, const double* h,
                         const double* sigma, const double* ZtXL, const double* ZtY, double* dinv,
                         double* AYL, double* top, DevStatus* st) {
  eigen_trait_kernel<<<t, 256, 0, s>>>(n, t, wXL, W, h, sigma, ZtXL, ZtY, dinv, AYL, top, st);
  note_launch();
  return cudaGetLastError();
}

cudaError_t gram_skinny(cudaStream_t s, int n, int x, int wXL, int wXR, const double* X, long long ldx,
                        const double* C, double* GYL, double* GR) {
  gram_skinny_kernel<<<ceil_div(x, 8), 256, 0, s>>>(n, x, wXL, wXR, X, ldx, C, GYL, GR);
  note_launch();
  return cudaGetLastError();
}

cudaError_t quad_products(cudaStream_t s, int n, int x, int wXR, const double* R, long long ldr, double* Q,
                          long long ldq) {
  long long total = (long long)n * x * wXR * wXR;
  int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 32);
  quad_products_kernel<<<blocks, 256, 0, s>>>(n, x, wXR, R, ldr, Q, ldq);
  note_launch();
  return cudaGetLastError();
}

template <int P>
cudaError_t launch_solve_grouped(cudaStream_t s, const SolveProblem* probs, const int* plist, int count, int x_b,
                                 const StepCohort* sc, DevStatus* st) {
  const size_t smem = sizeof(double) * 128 * (P + P * P);
  FGLS_CUDA_TRY(
      cudaFuncSetAttribute(snp_solve_grouped_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int bpp = ceil_div(x_b, 128);
  snp_solve_grouped_kernel<P><<<count * bpp, 128, smem, s>>>(probs, plist, bpp, sc, st);
  note_launch();
  return cudaGetLastError();
}

cudaError_t snp_solve_grouped(cudaStream_t s, int p, const SolveProblem* probs, const int* plist, int count, int x_b,
                              const StepCohort* sc, DevStatus* st) {
  if (count <= 0) return cudaSuccess;
  switch (p) {
#define FGLS_P_CASE(P) \
  case P:              \
    return launch_solve_grouped<P>(s, probs, plist, count, x_b, sc, st);
    FGLS_P_CASE(2)
    FGLS_P_CASE(3)
    FGLS_P_CASE(4)
    FGLS_P_CASE(5)
    FGLS_P_CASE(6)
    FGLS_P_CASE(7)
    FGLS_P_CASE(8)
#undef FGLS_P_CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t snp_solve(cudaStream_t s, int p, int x, int t, int wXL, const double* top, const double* GYL,
                      long long rsg, long long ldg, const double* GR, long long ldr, double* B, long long bstride, double* V,
                      long long vstride, DevStatus* st, long long snp_base) {
  switch (p) {
#define FGLS_P_CASE(P) \
  case P:              \
    return launch_solve<P>(s, x, t, wXL, top, GYL, rsg, ldg, GR, ldr, B, bstride, V, vstride, st, snp_base);
    FGLS_P_CASE(2)
    FGLS_P_CASE(3)
    FGLS_P_CASE(4)
    FGLS_P_CASE(5)
    FGLS_P_CASE(6)
    FGLS_P_CASE(7)
    FGLS_P_CASE(8)
#undef FGLS_P_CASE
    default:
      return cudaErrorInvalidValue;
  }
}

}  // namespace fgls

// ---------------------------------------------------------------------------
// p-values of the SNP coefficients (no counterpart in the reference, which
// emits beta and V only): two-sided normal test on z = beta_k / SE_k,
// p = erfc(|z| / sqrt 2), for the wXR SNP columns k = wXL .. p-1 of every
// (trait, SNP).  B, V in the layouts written by snp_solve.
// ---------------------------------------------------------------------------
namespace fgls {
namespace {
__global__ void pvalues_kernel(int x, int t, int p, int wXL, const double* __restrict__ B, long long bstride,
                               const double* __restrict__ V, long long vstride, double* __restrict__ P,
                               long long pstride) {
  const int wXR = p - wXL;
  const long long total = (long long)x * t * wXR;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(e % wXR);
    const long long r = e / wXR;
    const int i = (int)(r % x), j = (int)(r / x);
    const int k = wXL + c;
    const double beta = B[(long long)j * bstride + (long long)i * p + k];
    const double se = V[(long long)j * vstride + (long long)i * p * p + k + k * p];  // diagonal = SE
    P[(long long)j * pstride + (long long)i * wXR + c] = erfc(fabs(beta / se) * 0.70710678118654752440);
  }
}
}  // namespace

namespace {
// SE_k = V_kk and p_k = erfc(|beta_k / SE_k| / sqrt 2) for every coefficient
__global__ void compact_kernel(int x, int t, int p, const double* __restrict__ B, long long bstride,
                               const double* __restrict__ V, long long vstride, double* __restrict__ SE,
                               double* __restrict__ P, long long cstride) {
  const long long total = (long long)x * t * p;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(e % p);
    const long long r = e / p;
    const int i = (int)(r % x), j = (int)(r / x);
    const double beta = B[(long long)j * bstride + (long long)i * p + k];
    const double se = V[(long long)j * vstride + (long long)i * p * p + k + k * p];
    SE[(long long)j * cstride + (long long)i * p + k] = se;
    P[(long long)j * cstride + (long long)i * p + k] = erfc(fabs(beta / se) * 0.70710678118654752440);
  }
}
}  // namespace

cudaError_t snp_compact(cudaStream_t s, int x, int t, int p, const double* B, long long bstride, const double* V,
                        long long vstride, double* SE, double* P, long long cstride) {
  const long long total = (long long)x * t * p;
  const int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 32);
  if (blocks <= 0) return cudaSuccess;
  compact_kernel<<<blocks, 256, 0, s>>>(x, t, p, B, bstride, V, vstride, SE, P, cstride);
  note_launch();
  return cudaGetLastError();
}

cudaError_t snp_pvalues(cudaStream_t s, int x, int t, int p, int wXL, const double* B, long long bstride,
                        const double* V, long long vstride, double* P, long long pstride) {
  const long long total = (long long)x * t * (p - wXL);
  const int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 32);
  if (blocks <= 0) return cudaSuccess;
  pvalues_kernel<<<blocks, 256, 0, s>>>(x, t, p, wXL, B, bstride, V, vstride, P, pstride);
  note_launch();
  return cudaGetLastError();
}
}  // namespace fgls
