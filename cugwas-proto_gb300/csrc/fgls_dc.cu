// Divide-and-conquer eigensolver for the symmetric tridiagonal T (diagonal d,
// off-diagonal e, e[i] couples i and i+1): T = V diag(W) V^T, W ascending.
// Used by the device eigendecomposition of Phi after Householder reduction.
//
// Algorithm (Cuppen's method with Gu-Eisenstat eigenvectors, the scheme of
// LAPACK's dstedc, written for massive parallelism):
//  * tear: T = diag(T1', T2') + |b| u u^T at each split (u = e_k-1 + sign(b) e_k,
//    d[k-1], d[k] reduced by |b|), recursively down to leaves of <= 64 rows;
//  * leaves: implicit QL in one CTA per leaf (one thread runs the scalar
//    sweep, 64 threads apply each rotation chain to the leaf's rows);
//  * merge: z = Q^T u / sqrt2, rho = 2|b| > 0; sort the children's eigenvalues
//    (rank by binary search); deflate tiny |rho z_i| and close pairs (Givens,
//    sequential scan in one thread); secular equation 1 + rho sum z^2/(d - l)
//    for each surviving root by a pole-aware Newton iteration in its own
//    bisection bracket with the origin at the nearer pole (one warp per root); z
//    recomputed from the roots by the Loewner formula (one warp per root) so
//    that the eigenvectors are orthogonal to
//    working precision; eigenvectors u_k = z_i/(d_i - l_k) normalised (one
//    warp per root); new Q = Q_old[:, kept] * U by DGEMM; final rank sort.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "fgls_common.cuh"
#include "fgls_kernels.cuh"

namespace fgls {

namespace {

constexpr int LEAF = 64;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------- leaves
// One CTA (64 threads) per leaf: QL on the leaf's tridiagonal, eigenvectors
// into the diagonal block V[off.., off..] (ld n), eigenvalues sorted into W.
__global__ void __launch_bounds__(LEAF) dc_leaf_kernel(int n, const int* __restrict__ leaf_off,
                                                       const int* __restrict__ leaf_size, const double* __restrict__ d,
                                                       const double* __restrict__ e, double* __restrict__ W,
                                                       double* __restrict__ V, int* fail) {
  __shared__ double sd[LEAF], se[LEAF], cs[LEAF], sn[LEAF];
  __shared__ double Q[LEAF][LEAF + 1];  // Q[row][col]
  __shared__ int lo_s, hi_s, nrot_s, done_s;
  const int off = leaf_off[blockIdx.x], m = leaf_size[blockIdx.x];
  const int tid = threadIdx.x;
  if (tid < m) {
    sd[tid] = d[off + tid];
    se[tid] = (tid < m - 1) ? e[off + tid] : 0.0;
    for (int c = 0; c < m; c++) Q[tid][c] = (tid == c) ? 1.0 : 0.0;
  }
  __syncthreads();
  double anorm = 0.0;
  if (tid == 0) {
    for (int i = 0; i < m; i++)
      anorm = fmax(anorm, fabs(sd[i]) + fabs(se[i]) + (i > 0 ? fabs(se[i - 1]) : 0.0));
    done_s = 0;
  }
  int l = 0, iter = 0;
  for (int guard = 0; guard < 64 * LEAF + 64; guard++) {
    if (tid == 0) {
      nrot_s = 0;
      const double tol = DBL_EPSILON * anorm;
      while (l < m) {
        int mm;
        for (mm = l; mm < m - 1; mm++)
          if (fabs(se[mm]) <= tol) break;
        if (mm == l) {
          l++;
          iter = 0;
          continue;
        }
        if (iter++ >= 64) {
          atomicExch(fail, 1);
          l = m;
          break;
        }
        double g = (sd[l + 1] - sd[l]) / (2.0 * se[l]);
        double r = hypot(g, 1.0);
        g = sd[mm] - sd[l] + se[l] / (g + copysign(r, g));
        double s = 1.0, c = 1.0, p = 0.0;
        int i, cnt = 0;
        for (i = mm - 1; i >= l; i--) {
          double f = s * se[i], b = c * se[i];
          r = hypot(f, g);
          se[i + 1] = r;
          if (r == 0.0) {
            sd[i + 1] -= p;
            se[mm] = 0.0;
            break;
          }
          s = f / r;
          c = g / r;
          g = sd[i + 1] - p;
          r = (sd[i] - g) * s + 2.0 * c * b;
          p = s * r;
          sd[i + 1] = g + p;
          g = c * r - b;
          cs[i] = c;
          sn[i] = s;
          cnt++;
        }
        hi_s = mm - 1;
        lo_s = mm - cnt;
        nrot_s = cnt;
        if (!(r == 0.0 && i >= l)) {
          sd[l] -= p;
          se[l] = g;
          se[mm] = 0.0;
        }
        break;
      }
      if (l >= m) done_s = 1;
    }
    __syncthreads();
    if (nrot_s > 0 && tid < m) {
      double carry = Q[tid][hi_s + 1];
      for (int i = hi_s; i >= lo_s; i--) {
        const double zi = Q[tid][i];
        Q[tid][i + 1] = sn[i] * zi + cs[i] * carry;
        carry = cs[i] * zi - sn[i] * carry;
      }
      Q[tid][lo_s] = carry;
    }
    __syncthreads();
    if (done_s && nrot_s == 0) break;
  }
  // rank sort and write
  if (tid < m) {
    const double v = sd[tid];
    int rk = 0;
    for (int j = 0; j < m; j++) rk += (sd[j] < v) || (sd[j] == v && j < tid);
    W[off + rk] = v;
    for (int r = 0; r < m; r++) V[(off + r) + (long long)(off + rk) * n] = Q[r][tid];
  }
}

// ---------------------------------------------------------------- merge
struct MergeState {
  int K;      // surviving (non-deflated) roots
  int ndefl;  // deflated
  int nrot;   // deflation rotations
  double rho;
};

// z in node order, merged ascending order of the children's eigenvalues.
__global__ void dc_sort_kernel(int n, int off, int n1, int nn, double beta, const double* __restrict__ W,
                               const double* __restrict__ V, double* __restrict__ ds, double* __restrict__ zs,
                               int* __restrict__ perm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const double v = W[off + i];
  const double r2 = 0.70710678118654752440;
  double z;
  int rk;
  if (i < n1) {
    z = V[(off + n1 - 1) + (long long)(off + i) * n] * r2;
    // elements of the right child strictly smaller
    int lo = 0, hi = nn - n1;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (W[off + n1 + mid] < v) lo = mid + 1; else hi = mid;
    }
    rk = i + lo;
  } else {
    z = (beta >= 0.0 ? 1.0 : -1.0) * V[(off + n1) + (long long)(off + i) * n] * r2;
    // elements of the left child smaller or equal
    int lo = 0, hi = n1;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (W[off + mid] <= v) lo = mid + 1; else hi = mid;
    }
    rk = (i - n1) + lo;
  }
  ds[rk] = v;
  zs[rk] = z;
  perm[rk] = i;
}

// Sequential deflation scan, the dlaed2 criteria:
//   |rho z_j| <= tol            -> eigenpair (d_j, column j) kept as is
//   |(d_nj - d_pj) c s| <= tol  -> rotate columns pj, nj so that z_pj = 0
// Outputs kept roots (dk, zk, colk) in ascending order, deflated (dd, cold),
// and the rotation list (rc1, rc2, rcs, rsn) applied in order.  The scan is
// one thread's dependent chain; with STAGED its operands (d, z, perm) sit in
// shared memory (loaded and written back by the whole CTA), otherwise in
// global memory (merges too large for shared memory).  The kept roots are
// written over the scanned prefix (index K <= the current pair's first
// index, whose values are already consumed) and sorted there.
constexpr size_t DEFLATE_SMEM_MAX = 220 * 1024;  // dynamic shared memory of the staged scan (nn <= 11264)
template <bool STAGED>
__global__ void __launch_bounds__(256) dc_deflate_kernel(int nn, double rho, double* __restrict__ ds,
                                                         double* __restrict__ zs, int* __restrict__ perm,
                                                         double* __restrict__ dk, double* __restrict__ zk,
                                                         int* __restrict__ colk, double* __restrict__ dd,
                                                         int* __restrict__ cold, int* __restrict__ rc1,
                                                         int* __restrict__ rc2, double* __restrict__ rcs,
                                                         double* __restrict__ rsn, MergeState* st) {
  extern __shared__ double dsm[];
  __shared__ double red[2][32];
  double* sd = STAGED ? dsm : ds;
  double* sz = STAGED ? dsm + nn : zs;
  int* sp = STAGED ? (int*)(dsm + 2 * (size_t)nn) : perm;
  double dmax = 0.0, zmax = 0.0;
  for (int i = threadIdx.x; i < nn; i += blockDim.x) {
    const double dv = ds[i], zv = zs[i];
    if (STAGED) {
      sd[i] = dv;
      sz[i] = zv;
      sp[i] = perm[i];
    }
    dmax = fmax(dmax, fabs(dv));
    zmax = fmax(zmax, fabs(zv));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
    zmax = fmax(zmax, __shfl_xor_sync(0xffffffffu, zmax, o));
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = dmax;
    red[1][threadIdx.x >> 5] = zmax;
  }
  __syncthreads();
  __shared__ int Ks;
  if (threadIdx.x == 0) {
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
      dmax = fmax(dmax, red[0][w]);
      zmax = fmax(zmax, red[1][w]);
    }
    const double tol = 8.0 * DBL_EPSILON * fmax(dmax, rho * zmax);
    int K = 0, nd = 0, nr = 0;
    int pj = -1;
    for (int j = 0; j < nn; j++) {
      if (rho * fabs(sz[j]) <= tol) {
        dd[nd] = sd[j];
        cold[nd++] = sp[j];
        continue;
      }
      if (pj < 0) {
        pj = j;
        continue;
      }
      const double zp = sz[pj], zj = sz[j];
      const double t = sd[j] - sd[pj];
      // |t c s| <= tol with c = zj / tau, s = -zp / tau, tau^2 = zj^2 + zp^2,
      // tested without the square root and divisions (the scan is one
      // thread's FP64 dependency chain); c, s only for a rotation
      if (fabs(t * zj * zp) <= tol * (zj * zj + zp * zp)) {
        const double tau = hypot(zj, zp);
        const double c = zj / tau, sn = -zp / tau;
        // rotate: z_j <- tau, z_pj <- 0; columns (pj, j)
        sz[j] = tau;
        sz[pj] = 0.0;
        rc1[nr] = sp[pj];
        rc2[nr] = sp[j];
        rcs[nr] = c;
        rsn[nr] = sn;
        nr++;
        const double tt = sd[pj] * c * c + sd[j] * sn * sn;
        sd[j] = sd[pj] * sn * sn + sd[j] * c * c;
        sd[pj] = tt;
        dd[nd] = sd[pj];
        cold[nd++] = sp[pj];
        pj = j;
      } else {
        const double kd = sd[pj], kz = sz[pj];
        const int kc = sp[pj];
        sd[K] = kd;  // K <= pj: entries below pj are consumed
        sz[K] = kz;
        sp[K++] = kc;
        pj = j;
      }
    }
    if (pj >= 0) {
      const double kd = sd[pj], kz = sz[pj];
      const int kc = sp[pj];
      sd[K] = kd;
      sz[K] = kz;
      sp[K++] = kc;
    }
    // the rotations change the diagonal of kept entries already in place; the
    // kept list must stay ascending for the secular intervals
    for (int a = 1; a < K; a++) {
      const double dv = sd[a], zv = sz[a];
      const int cv = sp[a];
      int b = a - 1;
      while (b >= 0 && sd[b] > dv) {
        sd[b + 1] = sd[b];
        sz[b + 1] = sz[b];
        sp[b + 1] = sp[b];
        b--;
      }
      sd[b + 1] = dv;
      sz[b + 1] = zv;
      sp[b + 1] = cv;
    }
    st->K = K;
    st->ndefl = nd;
    st->nrot = nr;
    st->rho = rho;
    Ks = K;
  }
  __syncthreads();
  const int K = Ks;
  for (int i = threadIdx.x; i < K; i += blockDim.x) {
    dk[i] = sd[i];
    zk[i] = sz[i];
    colk[i] = sp[i];
  }
}

// Apply the deflation rotations to the node's columns (one thread per row).
__global__ void dc_rotate_kernel(int n, int off, int nn, const int* __restrict__ rc1, const int* __restrict__ rc2,
                                 const double* __restrict__ rcs, const double* __restrict__ rsn, int nr,
                                 double* __restrict__ V) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nn) return;
  double* row = V + (off + r);
  for (int k = 0; k < nr; k++) {
    double* a = row + (long long)(off + rc1[k]) * n;
    double* b = row + (long long)(off + rc2[k]) * n;
    const double c = rcs[k], s = rsn[k];
    const double x = *a, y = *b;
    // dlaed2: drot(q(:,pj), q(:,nj), c, s) -> pj' = c pj + s nj, nj' = c nj - s pj
    *a = c * x + s * y;
    *b = c * y - s * x;
  }
}

// Secular function at offset tau from the origin pole o, the K-term sums
// split over the 32 lanes of a warp (every lane returns the full sums):
//   f    = 1 + rho sum_j z_j^2 / (delta_j - tau)      (delta_j = d_j - d_o)
//   amag = 1 + rho sum_j |z_j^2 / (delta_j - tau)|    (rounding scale of f)
//   psi  = 1 + rho sum_{j != o} z_j^2 / (delta_j - tau),  dpsi = psi'
__device__ __forceinline__ void secular_warp(int K, const double* __restrict__ dk, const double* __restrict__ zk,
                                             int o, double rho, double tau, int lane, double& f, double& amag,
                                             double& psi, double& dpsi) {
  const double org = dk[o];
  double s = 0.0, sa = 0.0, so = 0.0, sp = 0.0;
  for (int j = lane; j < K; j += 32) {
    const double r = 1.0 / ((dk[j] - org) - tau);
    const double zr = zk[j] * r;
    const double term = zk[j] * zr;
    sa += fabs(term);
    if (j == o) {
      so += term;
    } else {
      s += term;
      sp += zr * zr;
    }
  }
  s = warp_sum(s);
  sa = warp_sum(sa);
  so = warp_sum(so);
  sp = warp_sum(sp);
  psi = 1.0 + rho * s;
  dpsi = rho * sp;
  f = psi + rho * so;
  amag = 1.0 + rho * sa;
}

// One warp per root k in (d_k, d_k+1) (last: (d_K, d_K + rho |z|^2)), the
// origin o at the nearer pole (the sign of f at the midpoint picks it).
// Iteration on tau in a bisection bracket [lo, hi] that shrinks with the sign
// of f at every iterate: each step keeps the origin's term -rho z_o^2 / tau
// exact and linearises the rest (psi), i.e. solves
//   psi(t) + psi'(t) (tau - t) - rho z_o^2 / tau = 0,
// a quadratic whose root on the origin's side is taken in its stable form
// (a pole-aware Newton step; LAPACK's dlaed4 uses refinements of the same
// idea).  Steps outside the bracket fall back to bisection.  Stops when |f|
// is below its rounding scale or the bracket is exhausted.  2-3 iterations
// per root on kinship spectra instead of ~55 of bisection.
__global__ void __launch_bounds__(256) dc_secular_kernel(int K, const double* __restrict__ dk,
                                                         const double* __restrict__ zk, double rho,
                                                         int* __restrict__ org_idx, double* __restrict__ tau_out) {
  const int k = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (k >= K) return;  // warp-uniform
  double zn = 0.0;
  for (int j = lane; j < K; j += 32) zn += zk[j] * zk[j];
  zn = warp_sum(zn);
  int o;
  double lo, hi;
  double f, amag, psi, dpsi;
  if (k < K - 1) {
    const double gap = dk[k + 1] - dk[k];
    secular_warp(K, dk, zk, k, rho, 0.5 * gap, lane, f, amag, psi, dpsi);
    if (f >= 0.0) {
      o = k;
      lo = 0.0;
      hi = 0.5 * gap;
    } else {
      o = k + 1;
      lo = -0.5 * gap;
      hi = 0.0;
    }
  } else {
    o = k;
    lo = 0.0;
    hi = rho * zn;
    // f(hi) > 0 is guaranteed in exact arithmetic; widen if rounding disagrees
    for (int w = 0; w < 8; w++) {
      secular_warp(K, dk, zk, k, rho, hi, lane, f, amag, psi, dpsi);
      if (f >= 0.0) break;
      hi *= 2.0;
    }
  }
  const double c = rho * zk[o] * zk[o];
  double t = 0.5 * (lo + hi);
  for (int it = 0; it < 200; it++) {
    if (!(t > lo && t < hi)) t = 0.5 * (lo + hi);
    if (t <= lo || t >= hi) break;  // bracket exhausted at working precision
    secular_warp(K, dk, zk, o, rho, t, lane, f, amag, psi, dpsi);
    if (fabs(f) <= 16.0 * DBL_EPSILON * amag) break;
    if (f < 0.0) lo = t; else hi = t;
    if (hi - lo <= 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi))) break;
    const double a = dpsi, b = psi - dpsi * t;
    const double sq = sqrt(b * b + 4.0 * a * c);
    double tn;
    if (o == k)  // root on the positive side of the origin
      tn = b > 0.0 ? 2.0 * c / (b + sq) : (-b + sq) / (2.0 * a);
    else
      tn = b < 0.0 ? -2.0 * c / (-b + sq) : (-b - sq) / (2.0 * a);
    t = (tn > lo && tn < hi && tn != t) ? tn : 0.5 * (lo + hi);
  }
  if (!(t > lo && t < hi)) t = 0.5 * (lo + hi);
  if (t == 0.0) t = (o == k) ? hi : lo;  // never exactly on the pole
  if (lane == 0) {
    org_idx[k] = o;
    tau_out[k] = t;
  }
}

// Loewner recomputation of z from the roots (one warp per i, the product
// split over the lanes):
//   z_i^2 = (l_i - d_i)/rho * prod_{j != i} (l_j - d_i)/(d_j - d_i)
__global__ void __launch_bounds__(256) dc_lowner_kernel(int K, const double* __restrict__ dk,
                                                        const double* __restrict__ zk,
                                                        const int* __restrict__ org_idx, const double* __restrict__ tau,
                                                        double rho, double* __restrict__ zh) {
  const int i = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= K) return;
  const double di = dk[i];
  double prod = 1.0;
  for (int j = lane; j < K; j += 32) {
    if (j == i) continue;
    const double num = (dk[org_idx[j]] - di) + tau[j];
    const double den = dk[j] - di;
    prod *= num / den;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) prod *= __shfl_xor_sync(0xffffffffu, prod, o);
  prod *= ((dk[org_idx[i]] - di) + tau[i]) / rho;
  if (lane == 0) zh[i] = copysign(sqrt(fmax(prod, 0.0)), zk[i]);
}

// U[:, k] = (z_i / (d_i - l_k))_i normalised; one warp per root k.
__global__ void dc_vectors_kernel(int K, const double* __restrict__ dk, const double* __restrict__ zh,
                                  const int* __restrict__ org_idx, const double* __restrict__ tau,
                                  double* __restrict__ U) {
  const int k = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (k >= K) return;
  const double dor = dk[org_idx[k]], tk = tau[k];
  double ss = 0.0;
  for (int i = lane; i < K; i += 32) {
    const double v = zh[i] / ((dk[i] - dor) - tk);
    U[i + (long long)k * K] = v;
    ss += v * v;
  }
  ss = warp_sum(ss);
  const double inv = 1.0 / sqrt(ss);
  for (int i = lane; i < K; i += 32) U[i + (long long)k * K] *= inv;
}

// G[:, c] = V_node[:, colk[c]]  (nn x K)
__global__ void dc_gather_kernel(int n, int off, int nn, int K, const int* __restrict__ colk,
                                 const double* __restrict__ V, double* __restrict__ G) {
  const long long total = (long long)nn * K;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e % nn);
    const int c = (int)(e / nn);
    G[e] = V[(off + r) + (long long)(off + colk[c]) * n];
  }
}

// Final order of the node: roots l_k = d_o + tau and deflated d; rank sort,
// then the node block of V from G2 (kept) or the old columns (deflated).
__global__ void dc_values_kernel(int K, int nd, const double* __restrict__ dk, const int* __restrict__ org_idx,
                                 const double* __restrict__ tau, const double* __restrict__ dd,
                                 double* __restrict__ vals) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < K) vals[i] = dk[org_idx[i]] + tau[i];
  else if (i < K + nd) vals[i] = dd[i - K];
}

__global__ void dc_rank_kernel(int nn, const double* __restrict__ vals, int* __restrict__ rank) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  const double v = vals[i];
  int rk = 0;
  for (int j = 0; j < nn; j++) rk += (vals[j] < v) || (vals[j] == v && j < i);
  rank[i] = rk;
}

// T[:, rank[q]] = (q < K) ? G2[:, q] : V_node[:, cold[q - K]]; W[off + rank[q]] = vals[q]
__global__ void dc_assemble_kernel(int n, int off, int nn, int K, const int* __restrict__ rank,
                                   const double* __restrict__ vals, const double* __restrict__ G2,
                                   const int* __restrict__ cold, const double* __restrict__ V, double* __restrict__ T,
                                   double* __restrict__ W) {
  const long long total = (long long)nn * nn;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e % nn);
    const int q = (int)(e / nn);
    const double v = (q < K) ? G2[r + (long long)q * nn] : V[(off + r) + (long long)(off + cold[q - K]) * n];
    T[r + (long long)rank[q] * nn] = v;
    if (r == 0) W[off + rank[q]] = vals[q];
  }
}

__global__ void dc_copyback_kernel(int n, int off, int nn, const double* __restrict__ T, double* __restrict__ V) {
  const long long total = (long long)nn * nn;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e % nn);
    const int c = (int)(e / nn);
    V[(off + r) + (long long)(off + c) * n] = T[e];
  }
}

__global__ void dc_tear_kernel(int ncut, const int* __restrict__ cut, const double* __restrict__ e,
                               double* __restrict__ d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncut) return;
  const int k = cut[i];  // split between k-1 and k
  const double b = fabs(e[k - 1]);
  atomicAdd(&d[k - 1], -b);  // a row can border two cuts only when leaves have size 1
  atomicAdd(&d[k], -b);
}

__global__ void zero_kernel(long long count, double* p) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < count;
       e += (long long)gridDim.x * blockDim.x)
    p[e] = 0.0;
}

int grid_for(long long total) { return (int)std::min<long long>((total + 255) / 256, 152LL * 32); }

struct Node {
  int off, size, n1;  // n1 == 0 for a leaf
};

void build(int off, int size, std::vector<Node>& post) {
  if (size <= LEAF) {
    post.push_back({off, size, 0});
    return;
  }
  const int n1 = size / 2;
  build(off, n1, post);
  build(off + n1, size - n1, post);
  post.push_back({off, size, n1});
}

}  // namespace

size_t dc_workspace_bytes(int n) {
  // vectors: ds zs dk zk dd tau zh vals rcs rsn (10 n doubles) + ints perm colk cold org rc1 rc2 rank leafoff
  // leafsize cut (10 n ints) + state + matrices U (n^2), G (n^2), G2 (n^2), T (n^2)
  return sizeof(double) * ((size_t)10 * n + 4 * (size_t)n * n) + sizeof(int) * (size_t)10 * n + 1024;
}

// d (n), e (n-1, e[n-1] unused) are modified.  On return W ascending and V the
// eigenvectors of T (n x n, ld n).
cudaError_t dc_tridiag_eig(cudaStream_t s, int n, double* d, double* e, double* W, double* V, void* work,
                           int* fail_dev, long long* launches) {
  FGLS_CUDA_TRY(cudaFuncSetAttribute(dc_deflate_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)DEFLATE_SMEM_MAX));
  double* ds = (double*)work;
  double* zs = ds + n;
  double* dk = zs + n;
  double* zk = dk + n;
  double* dd = zk + n;
  double* tau = dd + n;
  double* zh = tau + n;
  double* vals = zh + n;
  double* rcs = vals + n;
  double* rsn = rcs + n;
  double* U = rsn + n;
  double* G = U + (size_t)n * n;
  double* G2 = G + (size_t)n * n;
  double* T = G2 + (size_t)n * n;
  int* perm = (int*)(T + (size_t)n * n);
  int* colk = perm + n;
  int* cold = colk + n;
  int* orgi = cold + n;
  int* rc1 = orgi + n;
  int* rc2 = rc1 + n;
  int* rank = rc2 + n;
  int* leafoff = rank + n;
  int* leafsize = leafoff + n;
  int* cut = leafsize + n;
  MergeState* st = (MergeState*)(((uintptr_t)(cut + n) + 63) & ~(uintptr_t)63);
  long long nl = 0;

  std::vector<Node> post;
  build(0, n, post);
  std::vector<int> hoff, hsize, hcut;
  for (const Node& nd : post) {
    if (nd.n1 == 0) {
      hoff.push_back(nd.off);
      hsize.push_back(nd.size);
    } else {
      hcut.push_back(nd.off + nd.n1);
    }
  }
  // couplings of the merges, read before the tear changes nothing in e
  std::vector<double> hbeta(hcut.size());
  if (!hcut.empty()) {
    std::vector<double> he(n);
    FGLS_CUDA_TRY(cudaMemcpyAsync(he.data(), e, sizeof(double) * (n - 1 > 0 ? n - 1 : 1), cudaMemcpyDeviceToHost, s));
    FGLS_CUDA_TRY(cudaStreamSynchronize(s));
    for (size_t i = 0; i < hcut.size(); i++) hbeta[i] = he[hcut[i] - 1];
    FGLS_CUDA_TRY(cudaMemcpyAsync(cut, hcut.data(), sizeof(int) * hcut.size(), cudaMemcpyHostToDevice, s));
    dc_tear_kernel<<<ceil_div((long long)hcut.size(), 256), 256, 0, s>>>((int)hcut.size(), cut, e, d);
    nl++;
    // the torn couplings e[k-1] lie between two leaves: no leaf reads them
  }
  FGLS_CUDA_TRY(cudaMemcpyAsync(leafoff, hoff.data(), sizeof(int) * hoff.size(), cudaMemcpyHostToDevice, s));
  FGLS_CUDA_TRY(cudaMemcpyAsync(leafsize, hsize.data(), sizeof(int) * hsize.size(), cudaMemcpyHostToDevice, s));
  zero_kernel<<<grid_for((long long)n * n), 256, 0, s>>>((long long)n * n, V);
  dc_leaf_kernel<<<(int)hoff.size(), LEAF, 0, s>>>(n, leafoff, leafsize, d, e, W, V, fail_dev);
  nl += 2;
  FGLS_CUDA_TRY(cudaGetLastError());

  size_t ci = 0;
  MergeState hs;
  for (const Node& nd : post) {
    if (nd.n1 == 0) continue;
    const double beta = hbeta[ci++];
    const int nn = nd.size, off = nd.off;
    const double rho = 2.0 * fabs(beta);
    dc_sort_kernel<<<ceil_div(nn, 256), 256, 0, s>>>(n, off, nd.n1, nn, beta, W, V, ds, zs, perm);
    const size_t dsmem = (size_t)nn * (2 * sizeof(double) + sizeof(int));
    if (dsmem <= DEFLATE_SMEM_MAX)
      dc_deflate_kernel<true><<<1, 256, dsmem, s>>>(nn, rho, ds, zs, perm, dk, zk, colk, dd, cold, rc1, rc2, rcs,
                                                    rsn, st);
    else
      dc_deflate_kernel<false><<<1, 256, 0, s>>>(nn, rho, ds, zs, perm, dk, zk, colk, dd, cold, rc1, rc2, rcs,
                                                 rsn, st);
    nl += 2;
    FGLS_CUDA_TRY(cudaMemcpyAsync(&hs, st, sizeof(MergeState), cudaMemcpyDeviceToHost, s));
    FGLS_CUDA_TRY(cudaStreamSynchronize(s));
    const int K = hs.K, ndf = hs.ndefl;
    if (hs.nrot > 0) {
      dc_rotate_kernel<<<ceil_div(nn, 128), 128, 0, s>>>(n, off, nn, rc1, rc2, rcs, rsn, hs.nrot, V);
      nl++;
    }
    if (K > 0) {
      dc_secular_kernel<<<ceil_div(K, 8), 256, 0, s>>>(K, dk, zk, rho, orgi, tau);
      dc_lowner_kernel<<<ceil_div(K, 8), 256, 0, s>>>(K, dk, zk, orgi, tau, rho, zh);
      dc_vectors_kernel<<<ceil_div(K, 8), 256, 0, s>>>(K, dk, zh, orgi, tau, U);
      dc_gather_kernel<<<grid_for((long long)nn * K), 256, 0, s>>>(n, off, nn, K, colk, V, G);
      nl += 4;
      FGLS_CUDA_TRY(cudaGetLastError());
      FGLS_CUDA_TRY(dgemm(s, false, false, nn, K, K, 1.0, G, nn, U, K, 0.0, G2, nn));
    }
    dc_values_kernel<<<ceil_div(nn, 256), 256, 0, s>>>(K, ndf, dk, orgi, tau, dd, vals);
    dc_rank_kernel<<<ceil_div(nn, 256), 256, 0, s>>>(nn, vals, rank);
    dc_assemble_kernel<<<grid_for((long long)nn * nn), 256, 0, s>>>(n, off, nn, K, rank, vals, G2, cold, V, T, W);
    dc_copyback_kernel<<<grid_for((long long)nn * nn), 256, 0, s>>>(n, off, nn, T, V);
    nl += 4;
    FGLS_CUDA_TRY(cudaGetLastError());
  }
  if (launches) *launches += nl;
  note_launch(nl);
  return cudaSuccess;
}

}  // namespace fgls
