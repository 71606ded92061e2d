// Quadratic Gram terms of the split path in double-FP32 on the CUDA cores:
//
//   GR[i + j*ldg] = sum_l A[l,i] * D[l,j]
//
// A = R^2 as float pairs (hi, lo) written by the split-GEMM epilogue (SNP i
// at column i, row l = eigen coordinate), D = d_j(l) as float pairs (eigen
// weights 1/(a_j w_l + b_j)).  This is the reference's per-trait rescale
// followed by the x~^T x~ dot product (src/fgls_eigen.c:505-507 and
// 530-535), evaluated for all traits at once.  The chol variant's unit-weight
// term (src/fgls_chol.c:404-406) is summed by the split GEMM itself and
// finished by sqsum_combine / unit_gram_grouped (end of this file).
//
// Arithmetic.  All terms are non-negative (no cancellation).  Each product is
// error-free (p + pe = ah*dh exactly, by fma) and its cross terms ah*dl + al*dh
// go to the low accumulator.  The high accumulator starts at a power of two
// B_ij no smaller than any term (max_l ah[l,i] * max_l dh[l,j], rounded up), so
// every addition has |s| >= |p| and Fast2Sum (3 operations) is exact.  Every
// 64 rows the chunk (offset removed exactly) is folded into an outer (H, L)
// pair by TwoSum, so the FP32 low parts never sum more than 64 rounding
// errors of one chunk: relative error ~1e-14 at n = 10^4.  9 FP32 operations
// per term.
//
// Work decomposition.  CTA tile I SNPs x J traits (TY x TX threads, RI x RJ
// terms each), rows streamed in chunks of L through a double-buffered shared
// memory ring filled by cp.async (row-padded, conflict-free fills).  The tile
// shape is picked per call from a small menu to minimise trait padding (t=100
// runs 60 x 100 tiles, t=1 a 256 x 1 tile).  To fill all SMs the rows are
// split into KS contiguous ranges (a multiple of the 64-row fold) when the
// tile grid alone would leave a partial last wave; each range writes its
// (H, L) pair and a combine kernel adds the KS pairs in FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "fgls_common.cuh"
#include "fgls_kernels.cuh"
#include "fgls_selfgram.cuh"
#include "fgls_batch.cuh"

namespace fgls {

namespace {

constexpr int FOLD = 64;

// Knuth's TwoSum: s + e == a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

__device__ __forceinline__ float pow2_ceil(float v) {
  // smallest power of two >= v (v > 0, finite)
  return __int_as_float((__float_as_int(v) + 0x007FFFFF) & 0x7F800000);
}

__device__ __forceinline__ void cp_async8(void* dst, const void* src, int src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
               "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// amax[i] = max_l A[l, i].x  (one warp per column)
__global__ void colmax_kernel(int n, int x, const float2* __restrict__ A, long long lda, float* __restrict__ amax) {
  const int i = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= x) return;
  float m = 0.0f;
  for (int l = lane; l < n; l += 32) m = fmaxf(m, A[l + (long long)i * lda].x);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) amax[i] = m;
}

template <int TX, int TY, int RI, int RJ, int L>
constexpr int smem_bytes() {
  return 2 * (TY * RI + TX * RJ) * (L + 1) * (int)sizeof(float2);
}

template <int TX, int TY, int RI, int RJ, int L, int MINB>
__global__ void __launch_bounds__(TX* TY, MINB)
    quad_gram_kernel(int n, int x, int t, const float2* __restrict__ A, long long lda,
                     const float* __restrict__ amax, const float2* __restrict__ D, long long ldd,
                     const float* __restrict__ dmax, int rows_per_unit, float2* __restrict__ part,
                     double* __restrict__ GR, long long ldg) {
  constexpr int NT = TX * TY, I = TY * RI, J = TX * RJ, LP = L + 1, STAGE = (I + J) * LP;
  static_assert(FOLD % L == 0, "fold must be a multiple of the chunk");
  extern __shared__ float2 qsm[];
  const int i0 = blockIdx.x * I, j0 = blockIdx.y * J;
  const int lbeg = blockIdx.z * rows_per_unit;
  const int lend = min(n, lbeg + rows_per_unit);
  const int tid = threadIdx.x, tx = tid % TX, ty = tid / TX;

  auto load = [&](int buf, int l0) {
    float2* As = qsm + buf * STAGE;
    float2* Bs = As + I * LP;
    for (int e = tid; e < I * L; e += NT) {
      const int r = e / L, l = e % L;
      const bool ok = (l0 + l < lend) && (i0 + r < x);
      cp_async8(As + r * LP + l, ok ? A + (l0 + l) + (long long)(i0 + r) * lda : A, ok ? 8 : 0);
    }
    for (int e = tid; e < J * L; e += NT) {
      const int r = e / L, l = e % L;
      const bool ok = (l0 + l < lend) && (j0 + r < t);
      cp_async8(Bs + r * LP + l, ok ? D + (l0 + l) + (long long)(j0 + r) * ldd : D, ok ? 8 : 0);
    }
  };
  auto offset = [&](int a, int b) {
    const int i = i0 + ty + TY * a, j = j0 + tx + TX * b;
    const float bound = ((i < x) ? amax[i] : 0.0f) * ((j < t) ? dmax[j] : 0.0f);
    return bound > 0.0f ? pow2_ceil(bound) : 0.0f;
  };

  // inner (sh, sl): one 64-row chunk from the offset; outer (H, Lo): the fold
  float sh[RI][RJ], sl[RI][RJ], H[RI][RJ], Lo[RI][RJ];
#pragma unroll
  for (int a = 0; a < RI; a++)
#pragma unroll
    for (int b = 0; b < RJ; b++) {
      sh[a][b] = offset(a, b);
      sl[a][b] = H[a][b] = Lo[a][b] = 0.0f;
    }

  const int nch = (lend - lbeg + L - 1) / L;
  load(0, lbeg);
  cp_async_commit();
  for (int c = 0; c < nch; c++) {
    if (c + 1 < nch) load((c + 1) & 1, lbeg + (c + 1) * L);
    cp_async_commit();
    cp_async_wait1();
    __syncthreads();
    const float2* As = qsm + (c & 1) * STAGE;
    const float2* Bs = As + I * LP;
#pragma unroll 4
    for (int l = 0; l < L; l++) {
      float2 av[RI], bv[RJ];
#pragma unroll
      for (int a = 0; a < RI; a++) av[a] = As[(ty + TY * a) * LP + l];
#pragma unroll
      for (int b = 0; b < RJ; b++) bv[b] = Bs[(tx + TX * b) * LP + l];
#pragma unroll
      for (int a = 0; a < RI; a++)
#pragma unroll
        for (int b = 0; b < RJ; b++) {
          const float p = __fmul_rn(av[a].x, bv[b].x);
          const float pe = fmaf(av[a].x, bv[b].x, -p);
          float lo = fmaf(av[a].x, bv[b].y, sl[a][b]);
          lo = fmaf(av[a].y, bv[b].x, lo);
          const float s2 = __fadd_rn(sh[a][b], p);
          const float err = __fsub_rn(p, __fsub_rn(s2, sh[a][b]));
          sh[a][b] = s2;
          sl[a][b] = __fadd_rn(__fadd_rn(lo, pe), err);
        }
    }
    if (((c + 1) * L) % FOLD == 0 || c + 1 == nch) {
#pragma unroll
      for (int a = 0; a < RI; a++)
#pragma unroll
        for (int b = 0; b < RJ; b++) {
          const float off = offset(a, b);
          float hs, he, h2, e1;
          two_sum(sh[a][b], -off, hs, he);
          two_sum(H[a][b], hs, h2, e1);
          H[a][b] = h2;
          Lo[a][b] = __fadd_rn(Lo[a][b], __fadd_rn(__fadd_rn(e1, he), sl[a][b]));
          sh[a][b] = off;
          sl[a][b] = 0.0f;
        }
    }
    __syncthreads();  // the next iteration refills this buffer
  }
#pragma unroll
  for (int a = 0; a < RI; a++) {
    const int i = i0 + ty + TY * a;
    if (i >= x) continue;
#pragma unroll
    for (int b = 0; b < RJ; b++) {
      const int j = j0 + tx + TX * b;
      if (j >= t) continue;
      if (part)
        part[((long long)blockIdx.z * t + j) * x + i] = make_float2(H[a][b], Lo[a][b]);
      else
        GR[i + (long long)j * ldg] = (double)H[a][b] + (double)Lo[a][b];
    }
  }
}

// GR[i + j*ldg] = sum over the KS row ranges of the (H, L) pairs, in FP64
__global__ void quad_gram_combine_kernel(int x, int t, int ks, const float2* __restrict__ part,
                                         double* __restrict__ GR, long long ldg) {
  const long long total = (long long)x * t;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % x), j = (int)(e / x);
    double s = 0.0;
    for (int z = 0; z < ks; z++) {
      const float2 v = part[((long long)z * t + j) * x + i];
      s += (double)v.x + (double)v.y;
    }
    GR[i + (long long)j * ldg] = s;
  }
}

struct Variant {
  int I, J, threads, minb, smem;
  void (*kernel)(int, int, int, const float2*, long long, const float*, const float2*, long long, const float*, int,
                 float2*, double*, long long);
};

template <int TX, int TY, int RI, int RJ, int L, int MINB>
Variant make_variant() {
  return Variant{TY * RI, TX * RJ, TX * TY, MINB, smem_bytes<TX, TY, RI, RJ, L>(),
                 quad_gram_kernel<TX, TY, RI, RJ, L, MINB>};
}

const Variant* variants(int* count) {
  static const Variant v[] = {
      make_variant<20, 12, 5, 5, 32, 1>(),  // 60 x 100
      make_variant<16, 16, 4, 7, 32, 1>(),  // 64 x 112
      make_variant<16, 16, 4, 4, 32, 2>(),  // 64 x 64
      make_variant<8, 32, 4, 4, 32, 2>(),   // 128 x 32
      make_variant<2, 128, 2, 4, 16, 2>(),  // 256 x 8
      make_variant<1, 256, 1, 4, 16, 2>(),  // 256 x 4
      make_variant<1, 256, 1, 1, 16, 2>(),  // 256 x 1
  };
  *count = (int)(sizeof(v) / sizeof(v[0]));
  return v;
}

// Cost per (SNP, row): 9 FP32 operations per padded trait plus the re-read
// of the 8-byte R^2 pair once per trait tile (~4 operations per byte at the
// FP32 issue rate versus L2 bandwidth); ties go to the wider tile.
const Variant& pick(int t) {
  int nv;
  const Variant* v = variants(&nv);
  int best = 0;
  long long best_cost = -1;
  for (int k = 0; k < nv; k++) {
    const long long tiles = (t + v[k].J - 1) / v[k].J;
    const long long cost = 9 * tiles * v[k].J + 32 * tiles;
    if (best_cost < 0 || cost < best_cost || (cost == best_cost && v[k].J > v[best].J)) {
      best = k;
      best_cost = cost;
    }
  }
  return v[best];
}

constexpr int MAX_KS = 16;

// row ranges so that the CTAs fill whole waves (>= 90 % of the last wave)
int pick_ks(int n, long long units, int slots) {
  const int max_ks = std::max(1, std::min(MAX_KS, n / (2 * FOLD)));
  int best = 1;
  double best_eff = 0.0;
  for (int ks = 1; ks <= max_ks; ks++) {
    const double waves = (double)(units * ks) / slots;
    const double eff = waves / std::ceil(waves);
    if (eff >= 0.9 && waves >= 1.0) return ks;
    if (eff > best_eff + 1e-9) {
      best_eff = eff;
      best = ks;
    }
  }
  return best;
}

// Unit weights (chol: x~'x~ = sum_l R_l^2).  The split GEMM's last pass
// leaves, per SNP column i, the sums of R_l^2 over the 32-row groups
// g < ceil(n / 32) as float pairs at Q[i + g*ldq].  A CTA of 32 x 8 threads
// takes 32 columns: thread (c, k) adds the groups g = k, k + 8, ... of
// column c in double-FP32 (TwoSum of the high parts, Fast2Sum
// renormalisation), then thread (c, 0) adds the eight partial sums in k
// order and writes FP64: a fixed order, so the result is deterministic.  All
// terms are non-negative: relative error ~(groups / 8 + 13) * 2^-47 at most.
// A warp reads 32 consecutive columns of one group row (coalesced).
constexpr int GS_COLS = 32, GS_SPLIT = 8;

__device__ __forceinline__ void pair_acc(float& H, float& L, float vh, float vl) {
  float s, e;
  two_sum(H, vh, s, e);
  e = __fadd_rn(e, __fadd_rn(L, vl));
  H = __fadd_rn(s, e);
  L = __fsub_rn(e, __fsub_rn(H, s));
}

__device__ __forceinline__ void group_sums(const float2* __restrict__ Q, long long ldq, int groups, int x, int i0,
                                           double* __restrict__ GR) {
  __shared__ float2 part[GS_SPLIT][GS_COLS];
  const int c = threadIdx.x, k = threadIdx.y, i = i0 + c;
  float H = 0.0f, L = 0.0f;
  if (i < x)
    for (int g = k; g < groups; g += GS_SPLIT) {
      const float2 v = Q[i + (long long)g * ldq];
      pair_acc(H, L, v.x, v.y);
    }
  part[k][c] = make_float2(H, L);
  __syncthreads();
  if (k == 0 && i < x) {
    for (int q = 1; q < GS_SPLIT; q++) pair_acc(H, L, part[q][c].x, part[q][c].y);
    GR[i] = (double)H + (double)L;
  }
}

__global__ void __launch_bounds__(GS_COLS * GS_SPLIT) sqsum_combine_kernel(int n, int x, const float2* __restrict__ Q,
                                                                          long long ldq, double* __restrict__ GR) {
  group_sums(Q, ldq, (n + 31) >> 5, x, blockIdx.x * GS_COLS, GR);
}

// many problems in one launch: blockIdx.y = problem, SNPs of its cohort's step
__global__ void __launch_bounds__(GS_COLS * GS_SPLIT) unit_gram_grouped_kernel(
    const UnitGramProblem* __restrict__ probs, const StepCohort* __restrict__ sc) {
  const UnitGramProblem pr = probs[blockIdx.y];
  const int x = sc[pr.cohort].x;
  if ((int)blockIdx.x * GS_COLS >= x) return;  // whole CTA: no thread reaches the barrier
  group_sums(pr.Q, pr.ldq, (pr.n + 31) >> 5, x, blockIdx.x * GS_COLS, pr.GR);
}

}  // namespace

cudaError_t unit_gram_grouped(cudaStream_t s, const UnitGramProblem* dprobs, int count, const StepCohort* dsc,
                              int x_b) {
  if (count <= 0) return cudaSuccess;
  dim3 grid((x_b + GS_COLS - 1) / GS_COLS, count);
  unit_gram_grouped_kernel<<<grid, dim3(GS_COLS, GS_SPLIT), 0, s>>>(dprobs, dsc);
  note_launch();
  return cudaGetLastError();
}

cudaError_t sqsum_combine(cudaStream_t s, int n, int x, const float2* Q, long long ldq, double* GR) {
  if (x <= 0) return cudaSuccess;
  sqsum_combine_kernel<<<(x + GS_COLS - 1) / GS_COLS, dim3(GS_COLS, GS_SPLIT), 0, s>>>(n, x, Q, ldq, GR);
  note_launch();
  return cudaGetLastError();
}

size_t quad_gram_part_elems(int x, int t) { return (size_t)MAX_KS * t * x; }

cudaError_t quad_gram(cudaStream_t s, int n, int x, int t, const float2* A, long long lda, float* amax,
                      const float2* D, long long ldd, const float* dmax, float2* part, double* GR, long long ldg,
                      int sms) {
  if (x <= 0 || t <= 0 || n <= 0) return cudaSuccess;
  colmax_kernel<<<(x + 7) / 8, 256, 0, s>>>(n, x, A, lda, amax);
  note_launch();
  const Variant& v = pick(t);
  FGLS_CUDA_TRY(cudaFuncSetAttribute(v.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, v.smem));
  const long long units = (long long)((x + v.I - 1) / v.I) * ((t + v.J - 1) / v.J);
  int ks = part ? pick_ks(n, units, std::max(1, sms) * v.minb) : 1;
  int rows = (n + ks - 1) / ks;
  rows = (rows + FOLD - 1) / FOLD * FOLD;
  ks = (n + rows - 1) / rows;
  dim3 grid((x + v.I - 1) / v.I, (t + v.J - 1) / v.J, ks);
  v.kernel<<<grid, v.threads, v.smem, s>>>(n, x, t, A, lda, amax, D, ldd, dmax, rows, ks > 1 ? part : nullptr, GR,
                                           ldg);
  note_launch();
  if (ks > 1) {
    const long long total = (long long)x * t;
    const int blocks = (int)std::min<long long>((total + 255) / 256, 4096);
    quad_gram_combine_kernel<<<blocks, 256, 0, s>>>(x, t, ks, part, GR, ldg);
    note_launch();
  }
  return cudaGetLastError();
}

}  // namespace fgls
