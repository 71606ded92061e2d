// Null-model REML fit of the variance components (h_j, sigma_j) per trait,
// FP64, in the eigenbasis of Phi (Phi = Z diag(w) Z^T).
//
// The reference takes h and sigma as inputs (src/fgls_chol.c:139-145 reads
// h2_path and sigma2_path; src/fgls_chol.c:251-256 and src/fgls_eigen.c:1085-1160
// use them as M_j = sigma_j (h_j Phi + (1 - h_j) I)).  This kernel estimates
// them from the same eigenbasis operands the association uses
// (ZtXL = Z^T XL, ZtY = Z^T Y, w).
//
// With d_l = 1/(1 + h (w_l - 1)) (sigma = 1):
//   G = sum_l d_l x_l x_l^T,  g = sum_l d_l x_l ytil_l,  b = G^-1 g,
//   r = ytil - ZtXL b,        q = sum_l d_l r_l^2.
// sigma is profiled out in closed form, sigma_hat(h) = q / (n - wXL), and the
// profiled REML log-likelihood (constants dropped) is
//   l_p(h)  = -1/2 [ (n-wXL) log sigma_hat - sum_l log d_l + log det G + (n-wXL) ],
//   l_p'(h) = -1/2 [ (n-wXL) q_c / q - sum_l c_l / d_l + tr(G^-1 G_c) ],
// c_l = dd_l/dh = -(w_l - 1) d_l^2, G_c = sum c x x^T, q_c = sum c r^2 (the
// b-derivative of q vanishes because b minimises q).  At sigma = sigma_hat(h)
// these are the REML value and h-gradient of the adjoint's null model.
//
// Maximisation over [lo, hi] follows EMMA (Kang et al., Genetics 178:1709,
// 2008): l_p and l_p' on an even grid, every + -> - sign change of l_p'
// refined to a root by regula falsi with the Illinois modification, an
// endpoint taken when l_p' points out of the interval there, and the candidate
// with the largest l_p kept.
//
// One CTA per trait; every evaluation is two block-wide passes over the n
// eigen-coordinates (sums, then residual sums) with a fixed reduction order,
// so results are deterministic.
#include <cmath>

#include "fgls_common.cuh"
#include "fgls_kernels.cuh"

namespace fgls {

namespace {

constexpr int RF_THREADS = 256;
constexpr int RF_WARPS = RF_THREADS / 32;
constexpr int FGLS_REML_MAX_ITER = 100;  // regula falsi steps per bracket

// Block-wide sums of K per-thread values, fixed order (warp butterfly, then
// warps in index order).  out[] is shared; all threads return after it is set.
template <int K>
__device__ __forceinline__ void block_sums(double (&v)[K], double* red, double* out) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < K; k++) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) red[w * K + k] = x;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < K; k += RF_THREADS) {
    double s = 0.0;
    for (int q = 0; q < RF_WARPS; q++) s += red[q * K + k];
    out[k] = s;
  }
  __syncthreads();
}

struct RemlPoint {
  double ll, dll, sig;
  int ok;
};

template <int WX>
struct RemlShared {
  static constexpr int NG = WX * (WX + 1) / 2;
  static constexpr int K1 = 2 * NG + WX + 3;  // G, G_c, g, sum log d, sum c/d, bad count
  double red[RF_WARPS * K1];
  double sums[K1];
  double b[WX];
  double logdet, tr, sl, sc;
  int ok;
  RemlPoint pt;
};

// l_p, l_p' and sigma_hat at h for the trait whose columns are X (n x WX,
// ld n) and y.  Called by all threads; the result is in S.pt.
template <int WX>
__device__ void reml_point(int n, double h, const double* __restrict__ W, const double* __restrict__ X,
                           const double* __restrict__ y, RemlShared<WX>& S) {
  constexpr int NG = RemlShared<WX>::NG, K1 = RemlShared<WX>::K1;
  double acc[K1];
#pragma unroll
  for (int k = 0; k < K1; k++) acc[k] = 0.0;
  for (int l = threadIdx.x; l < n; l += RF_THREADS) {
    const double wm = W[l] - 1.0;
    const double den = fma(h, wm, 1.0);
    const double d = 1.0 / den;
    const double c = -wm * d * d;
    double x[WX];
#pragma unroll
    for (int a = 0; a < WX; a++) x[a] = X[l + (long long)a * n];
    const double yl = y[l];
    int k = 0;
#pragma unroll
    for (int a = 0; a < WX; a++)
#pragma unroll
      for (int b = 0; b <= a; b++, k++) {
        const double xx = x[a] * x[b];
        acc[k] = fma(d, xx, acc[k]);
        acc[NG + k] = fma(c, xx, acc[NG + k]);
      }
#pragma unroll
    for (int a = 0; a < WX; a++) acc[2 * NG + a] = fma(d * x[a], yl, acc[2 * NG + a]);
    acc[2 * NG + WX] -= log(den);      // log d
    acc[2 * NG + WX + 1] -= wm * d;    // c / d
    acc[2 * NG + WX + 2] += (den > 0.0 && den < INFINITY) ? 0.0 : 1.0;
  }
  block_sums<K1>(acc, S.red, S.sums);
  if (threadIdx.x == 0) {
    double G[WX * WX], L[WX * WX];
    int k = 0;
    for (int a = 0; a < WX; a++)
      for (int b = 0; b <= a; b++, k++) {
        G[a + b * WX] = G[b + a * WX] = S.sums[NG + k];  // G_c
        L[a + b * WX] = L[b + a * WX] = S.sums[k];       // G
      }
    bool ok = S.sums[2 * NG + WX + 2] == 0.0;
    // Cholesky of G in place (lower)
    for (int j = 0; ok && j < WX; j++) {
      double v = L[j + j * WX];
      for (int q = 0; q < j; q++) v -= L[j + q * WX] * L[j + q * WX];
      if (!(v > 0.0)) {
        ok = false;
        break;
      }
      const double ljj = sqrt(v);
      L[j + j * WX] = ljj;
      for (int i = j + 1; i < WX; i++) {
        double u = L[i + j * WX];
        for (int q = 0; q < j; q++) u -= L[i + q * WX] * L[j + q * WX];
        L[i + j * WX] = u / ljj;
      }
    }
    double logdet = 0.0, tr = 0.0;
    if (ok) {
      double bb[WX];
      for (int a = 0; a < WX; a++) {
        logdet += 2.0 * log(L[a + a * WX]);
        bb[a] = S.sums[2 * NG + a];
      }
      // b = G^-1 g, and tr(G^-1 G_c) column by column
      for (int col = -1; col < WX; col++) {
        double v[WX];
        for (int a = 0; a < WX; a++) v[a] = col < 0 ? bb[a] : G[a + col * WX];
        for (int i = 0; i < WX; i++) {
          double u = v[i];
          for (int q = 0; q < i; q++) u -= L[i + q * WX] * v[q];
          v[i] = u / L[i + i * WX];
        }
        for (int i = WX - 1; i >= 0; i--) {
          double u = v[i];
          for (int q = i + 1; q < WX; q++) u -= L[q + i * WX] * v[q];
          v[i] = u / L[i + i * WX];
        }
        if (col < 0)
          for (int a = 0; a < WX; a++) S.b[a] = v[a];
        else
          tr += v[col];
      }
    }
    S.logdet = logdet;
    S.tr = tr;
    S.sl = S.sums[2 * NG + WX];
    S.sc = S.sums[2 * NG + WX + 1];
    S.ok = ok;
  }
  __syncthreads();
  double acc2[2] = {0.0, 0.0};
  if (S.ok) {
    double bl[WX];
#pragma unroll
    for (int a = 0; a < WX; a++) bl[a] = S.b[a];
    for (int l = threadIdx.x; l < n; l += RF_THREADS) {
      const double wm = W[l] - 1.0;
      const double d = 1.0 / fma(h, wm, 1.0);
      double r = y[l];
#pragma unroll
      for (int a = 0; a < WX; a++) r = fma(-X[l + (long long)a * n], bl[a], r);
      const double dr2 = d * r * r;
      acc2[0] += dr2;
      acc2[1] = fma(-wm * d, dr2, acc2[1]);  // c r^2 = -(w - 1) d * d r^2
    }
  }
  block_sums<2>(acc2, S.red, S.sums);  // pass-1 sums are consumed by now
  if (threadIdx.x == 0) {
    const double nn = (double)(n - WX);
    const double q = S.sums[0], qc = S.sums[1];
    RemlPoint p;
    p.ok = S.ok && q > 0.0 && isfinite(q);
    p.sig = p.ok ? q / nn : NAN;
    p.ll = p.ok ? -0.5 * (nn * log(p.sig) - S.sl + S.logdet + nn) : -INFINITY;
    p.dll = p.ok ? -0.5 * (nn * qc / q - S.sc + S.tr) : NAN;
    S.pt = p;
  }
  __syncthreads();
}

template <int WX>
__global__ void __launch_bounds__(RF_THREADS)
    reml_fit_kernel(int n, int t, const double* __restrict__ W, const double* __restrict__ ZtXL,
                    const double* __restrict__ ZtY, double lo, double hi, int grid, double* __restrict__ out,
                    DevStatus* st) {
  __shared__ RemlShared<WX> S;
  __shared__ double gll[FGLS_REML_MAX_GRID], gdll[FGLS_REML_MAX_GRID], gsig[FGLS_REML_MAX_GRID];
  const int j = blockIdx.x;
  const double* y = ZtY + (long long)j * n;
  auto hk = [&](int k) { return k == grid - 1 ? hi : lo + (hi - lo) * ((double)k / (grid - 1)); };
  bool ok = true;
  for (int k = 0; k < grid && ok; k++) {
    reml_point<WX>(n, hk(k), W, ZtXL, y, S);
    ok = S.pt.ok;
    if (threadIdx.x == 0) {
      gll[k] = S.pt.ll;
      gdll[k] = S.pt.dll;
      gsig[k] = S.pt.sig;
    }
  }
  __syncthreads();
  double bh = NAN, bll = -INFINITY, bsig = NAN, bdll = NAN;
  if (ok) {
    if (!(gdll[0] > 0.0)) bh = lo, bll = gll[0], bsig = gsig[0], bdll = gdll[0];
    if (gdll[grid - 1] >= 0.0 && gll[grid - 1] > bll)
      bh = hi, bll = gll[grid - 1], bsig = gsig[grid - 1], bdll = gdll[grid - 1];
    for (int k = 0; k + 1 < grid && ok; k++) {
      if (!(gdll[k] > 0.0 && !(gdll[k + 1] > 0.0))) continue;
      // root of l_p' in [a, b] with fa > 0 >= fb: regula falsi, Illinois
      double a = hk(k), fa = gdll[k], b = hk(k + 1), fb = gdll[k + 1];
      double x = b, fx = fb, lx = gll[k + 1], sx = gsig[k + 1];
      int side = 0;
      for (int it = 0; it < FGLS_REML_MAX_ITER && fx != 0.0; it++) {
        double xn = (a * fb - b * fa) / (fb - fa);
        if (!(xn > a && xn < b)) xn = 0.5 * (a + b);
        reml_point<WX>(n, xn, W, ZtXL, y, S);
        if (!S.pt.ok) {
          ok = false;
          break;
        }
        x = xn, fx = S.pt.dll, lx = S.pt.ll, sx = S.pt.sig;
        if (fx > 0.0) {
          a = x, fa = fx;
          if (side < 0) fb *= 0.5;
          side = -1;
        } else {
          b = x, fb = fx;
          if (side > 0) fa *= 0.5;
          side = 1;
        }
        if (b - a <= 1e-15 + 2e-16 * fabs(x)) break;
      }
      if (ok && lx > bll) bh = x, bll = lx, bsig = sx, bdll = fx;
    }
  }
  if (threadIdx.x == 0) {
    if (!ok || !(bll > -INFINITY)) {
      bh = bsig = bll = bdll = NAN;
      set_status(st, FGLSGPU_ENOTSPD, -2, j);
    }
    out[j] = bh;
    out[t + j] = bsig;
    out[2 * t + j] = bll;
    out[3 * t + j] = bdll;
  }
}

}  // namespace

cudaError_t reml_fit(cudaStream_t s, int n, int t, int wXL, const double* W, const double* ZtXL, const double* ZtY,
                     double lo, double hi, int grid, double* out, DevStatus* st) {
  if (t <= 0) return cudaSuccess;
  if (n <= wXL || grid < 2 || grid > FGLS_REML_MAX_GRID || !(lo >= 0.0 && lo < hi && hi <= 1.0))
    return cudaErrorInvalidValue;
  switch (wXL) {
#define FGLS_REML_CASE(WX) \
  case WX:                  \
    reml_fit_kernel<WX><<<t, RF_THREADS, 0, s>>>(n, t, W, ZtXL, ZtY, lo, hi, grid, out, st); \
    break;
    FGLS_REML_CASE(1)
    FGLS_REML_CASE(2)
    FGLS_REML_CASE(3)
    FGLS_REML_CASE(4)
    FGLS_REML_CASE(5)
    FGLS_REML_CASE(6)
    FGLS_REML_CASE(7)
#undef FGLS_REML_CASE
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace fgls
