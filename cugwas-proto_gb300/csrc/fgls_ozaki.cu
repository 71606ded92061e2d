// Split-precision (Ozaki-style) tensor-core path for the bulk GEMMs.
//
//   C[r, c] = sum_k A[r, k] * G[c, k]        A FP64 (rows of Z^T, U^T or L^-1),
//                                            G genotypes (0/1/2), K = n
//
// A is cut once per problem into S FP8 (E4M3) "digit" slices with a per-row
// power-of-two scale 2^e_r:
//   A[r, k] = 2^(e_r - 4) * sum_s d_s[r, k] * 2^(-5 s),   d_s integer in [-16, 16]
// (round-to-nearest digits: each slice carries 5 bits, truncation error
// <= 2^(e_r - 5 S)).  Even slices hold d_s, odd slices d_s / 32; both are
// exact in E4M3, and so are the genotypes (0/1/2).  One pass accumulates a
// slice pair into ONE FP32 accumulator:
//   v = sum_k (d_2p + d_2p+1 / 32) g_k = P_2p + P_2p+1 / 32.
// With round-to-nearest digits d_2p + d_2p+1 / 32 = w - r / 32 for the
// pair's leading remainder |w| <= 16 and the next one |r| <= 1/2, so
// |v| <= (32 + 1/32) K < 2^19 for K <= FUSED_KMAX = 16368: v and every
// partial sum are multiples of 2^-5 below 2^19, representable in FP32, and
// the accumulation is exact and bit-reproducible.  The kind::f8f6f4 MMA runs
// at twice the BF16 rate: 9 five-bit slices (45 bits) cost 4.5 BF16
// slice-equivalents where 6 eight-bit BF16 slices (48 bits) would cost 6
// (and eight-bit digits would need 29 bits for a fused pair).
//
// Kernel ozaki_gemm_kernel (persistent: one CTA per SM takes 128 x 256
// output tiles from a launch-wide counter, 10 warps):
//   warp 0      TMA producer: per K-step of 128 bytes (128 digits), two
//               A-slice tiles (128 x 128) and one genotype tile (256 x 128),
//               128B-swizzled, three 64 KB stages.
//   warp 1      allocates 512 TMEM columns and issues tcgen05.mma
//               (kind::f8f6f4, E4M3 x E4M3 -> F32, M=128 N=256 K=32): both
//               slices of pass p into accumulator p % 2 (columns
//               [256 (p % 2), 256 (p % 2) + 256)), so the MMAs of one pass run
//               while the epilogue drains the previous one.
//   warps 2-9   epilogue: tcgen05.ld the pass's accumulator, convert it
//               exactly to the int32 q = 32 v = P_2p * 32 + P_2p+1,
//               Horner-accumulate the passes in int64 in the output buffer
//               (V = V * 2^10 + q), and on the last pass write
//               V * 2^(e_r - 9 - 10 (passes-1)) as FP64.  |V| < 2^62 for S <= 9.
// Every mbarrier wait is bounded; on expiry the kernel raises an error flag,
// drains its own in-flight copies and MMAs (bounded), frees TMEM and exits.
//
// Consumers (fgls eigen / chol split path):
//   eigen: A = [Z^T ; U^T], U = Z * [ZtY .* d_j | ZtXL .* d_j] (n x t(1+wXL)):
//          rows [0, n) of C are R = Z^T X, rows [n, n + t(1+wXL)) are the
//          Gram terms x~^T y~_j and x~^T XL~_j directly (one-sided: the exact
//          genotypes are the other operand).  The quadratic terms
//          sum_l R_l^2 d_j(l) run on the tensor cores from base-32 E4M3
//          digits of R^2 and d_j (quadtc_kernel below, 33 <= t), else in
//          double-FP32 (error-free products and sums) on the CUDA cores:
//          quad_gram (fgls_selfgram.cu).
//   chol:  A = [L^-1 ; U^T], U = L^-T [y~ | XL~].  The quadratic term has
//          unit weights, |x~|^2 = sum_l R_l^2: the GEMM's last pass sums the
//          squares over each 32-row group in registers (no R^2 is written)
//          and sqsum_combine (fgls_selfgram.cu) adds the groups.
#include <cuda.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "fgls_common.cuh"
#include "fgls_kernels.cuh"
#include "fgls_ozaki.cuh"
#include "fgls_selfgram.cuh"
#include "fgls_batch.cuh"

namespace fgls {

namespace oz {

constexpr int BM = 128, BN = 256;
constexpr int A_TILE = BM * 128;  // 16 KB: 128 rows of 128 bytes
// Split GEMM ring (one-SM kernel): a K-step of 128 FP8 digits, 128-byte
// rows with 128B swizzle, three 64 KB stages of two A-slice tiles and one
// genotype tile.  64-byte rows (64B swizzle) allow six 32 KB stages in the
// same shared memory, and so more bytes in flight, but the MMAs read
// 64B-swizzled operands more slowly: with one accumulator per slice pair and
// double-buffered TMEM the split GEMM took 8.99 ms per launch with 128-byte
// rows and 9.17 ms with 64-byte rows (n = 10000, x_b = 16384; five 32 KB
// stages: 9.61 ms, seven: 9.13 ms).
struct GemmRing {
  static constexpr int ROW = 128;  // bytes (FP8 digits) of one K-step row
  static constexpr int STAGES = 3;
  static constexpr int A = BM * ROW;
  static constexpr int B = BN * ROW;
  static constexpr int STAGE = 2 * A + B;
  static constexpr int SMEM = STAGES * STAGE + 1024 + 256;
};
constexpr int GBK = GemmRing::ROW;  // digits per K-step (the tensor maps' box)
constexpr int SMEM_BYTES = GemmRing::SMEM;
constexpr int THREADS = 320;  // producer, MMA, 8 epilogue warps
constexpr int MAX_SLICES = 9;   // FP8 digit slices; |V| < 2^62 in the epilogue
constexpr int FUSED_KMAX = 16368;  // K of the FP8 split GEMM: (32 + 1/32) K < 2^19
constexpr int DEFAULT_SLICES = 9;
constexpr int KALIGN = 128;     // K padding of the FP8 operands (one 128-byte row)
constexpr int GROUP_M = 8;

// tcgen05.mma instruction descriptor, kind::f8f6f4: D=F32, A=B=E4M3
// (format 0), both K-major, N=256, M=128.
constexpr uint32_t IDESC = (1u << 4) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
constexpr uint64_t WAIT_NS = 2000000000ull;  // default limit of one wait: 2 s

// Bounded wait: false if the phase does not complete within `limit_ns` (the
// kernel-wide error word `err` then records `site`), or if this CTA or any
// other CTA of the launch (or an earlier launch since the host last cleared
// `err`) already gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag,
                                          int* err, int site, uint64_t limit_ns) {
  const uint64_t t0 = globaltimer_ns();
  for (uint32_t it = 0;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    // the clock after the first miss (a short limit takes effect at once)
    // and every 64; the error words, which cost a memory load, every 64
    const bool every = (it & 63) == 63;
    if (every && (*abort_flag || *(volatile int*)err)) {
      *abort_flag = 1;
      return false;
    }
    if ((every || it == 0) && globaltimer_ns() - t0 > limit_ns) {
      *abort_flag = 1;
      atomicCAS(err, 0, site);
      return false;
    }
  }
}

// Drain wait of a CTA pair's leader on the abort path: one deadline for all
// its stages (a stage may never complete when the peer gave up before its
// copies; the leader's own copies land within microseconds).
__device__ __forceinline__ void mbar_drain_until(uint64_t* bar, uint32_t parity, uint64_t deadline) {
  while (!mbar_try_wait(bar, parity) && globaltimer_ns() < deadline) {
  }
}

// Bounded drain wait used on the abort path only (always the default limit,
// so that no copy or MMA of this CTA outlives its shared memory or TMEM).
__device__ __forceinline__ void mbar_drain(uint64_t* bar, uint32_t parity) {
  const uint64_t t0 = globaltimer_ns();
  while (!mbar_try_wait(bar, parity) && globaltimer_ns() - t0 < WAIT_NS) {
  }
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)tm), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// 2-SM (cluster of two CTAs) forms.  `bar` below is a shared::cluster
// address, possibly of the peer CTA's barrier (mapa).
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_addr(const void* p, uint32_t rank) {  // the same variable in CTA `rank`
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}
// every thread of both CTAs (a superset of __syncthreads)
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait_cluster(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// a copy into this CTA's shared memory that completes on the barrier at
// cluster address `bar` (the pair leader's)
__device__ __forceinline__ void tma_load_2d_cg2(void* dst, const CUtensorMap* tm, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)tm), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

__device__ __forceinline__ uint64_t desc_sw128(const void* p) {
  const uint32_t a = smem_u32(p);
  uint64_t d = 0;
  d |= (uint64_t)((a & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                // leading byte offset (unused for SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;      // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                // descriptor version (sm_100 family)
  d |= (uint64_t)2 << 61;                // 128B swizzle
  return d;
}

__device__ __forceinline__ void mma_f8(uint32_t dt, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(dt),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
// 2-SM MMA (issued by the pair leader; operands from both CTAs' shared
// memory at the same offsets, accumulator in both CTAs' TMEM)
__device__ __forceinline__ void mma_f8_cg2(uint32_t dt, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::2.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(dt),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
      : "memory");
}
// arrive on the barrier at `bar`'s offset in each CTA of `mask` once the
// leader's 2-SM MMAs so far have completed
__device__ __forceinline__ void mma_commit_cg2(uint64_t* bar, uint16_t mask) {
  asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
                   smem_u32(bar)),
               "h"(mask)
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

struct GemmArgs {
  int M;            // valid rows of A
  int Mpad;         // rows per slice in the A tensor (multiple of BM)
  int N;            // valid genotype columns
  int Kpad;         // K padded to a multiple of BK
  int S;            // slices (1..MAX_SLICES)
  int tiles_m, tiles_n;
  int tri_rows;     // rows [0, tri_rows) of A are lower triangular in K (0: none)
  const double* row_scale;  // per row 2^(e_r - 9 - 10 (passes-1))
  double* C;        // output, column-major, ld = ldc (int64 between passes)
  long long ldc;
  int col0;         // first genotype column of this launch (TMA row offset of G)
  int sq_rows;      // rows [0, sq_rows): write (C^2) as an error-free float pair (hi, lo)
  int* err;         // first failing wait site (0 = ok)
  unsigned long long wait_ns;  // limit of one pipeline wait
  // Unit weights (chol variant): when set, rows [0, sq_rows) write no
  // squares; the last pass sums (C^2) over each 32-row group g instead, as a
  // float pair at sqsum[c + g * ldq] for output column c.
  float2* sqsum = nullptr;
  long long ldq = 0;
};

// Grouped launches: one problem per (cohort, trait), tiles listed by the host.
struct GroupedProblem {
  GemmArgs g;  // g.N is replaced by the cohort's columns of the launch
  int cohort;
  int pad;
};
struct GroupedTile {
  int prob, m_tile, n_tile, pad;
};

// q = 32 v for a float v that is a multiple of 2^-5 with |v| < 2^19 (a fused
// FP8 slice pair, P_2p + P_2p+1 / 32), exactly and without a conversion
// instruction: h = rint(v) through the 1.5 * 2^23 addend (|v| < 2^22: v +
// 1.5 * 2^23 lies in [2^23, 2^24), where the float's mantissa bits are the
// integer h + 2^22), the remainder l = v - h in [-1/2, 1/2] is exact, and
// 32 l is an integer in [-16, 16]; q = 32 h + 32 l, |q| < 2^24.
__device__ __forceinline__ int fused_pair_f2i(float v) {
  const float t = __fadd_rn(v, 12582912.0f);
  const float l = __fsub_rn(v, __fsub_rn(t, 12582912.0f));
  const float u = __fmaf_rn(l, 32.0f, 12582912.0f);
  return (int)(((uint32_t)__float_as_int(t) - 0x4B400000u) * 32u + ((uint32_t)__float_as_int(u) - 0x4B400000u));
}

// An integer |x| < 2^22 as a float, exactly, without a conversion
// instruction (the 1.5 * 2^23 addend read backwards).
__device__ __forceinline__ float exact_i2f(int x) { return __fsub_rn(__int_as_float(x + 0x4B400000), 12582912.0f); }

__device__ __forceinline__ void two_sum_g(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

// Exact int64 value V (|V| < 2^62) times a power-of-two scale, squared, as a
// float pair.  V = a 2^42 + b 2^21 + c with b, c in [0, 2^21) and |a| < 2^20:
// each part converts exactly by exact_i2f, two TwoSums give V = hi + lo to
// ~2^-48 (GB300 runs 64-bit integer <-> float conversions on its narrow FP64
// pipe, which made this the slowest step of the epilogue).  Then
// v = V*scale = vh + vl and v^2 ~= ah + al with ah = fl(vh^2),
// al = (vh^2 - ah) + 2 vh vl: relative error ~2^-47.
__device__ __forceinline__ float2 square_pair(long long V, float fscale) {
  const float fa = __fmul_rn(exact_i2f((int)(V >> 42)), 4398046511104.0f);        // a 2^42
  const float fb = __fmul_rn(exact_i2f((int)((V >> 21) & 0x1FFFFF)), 2097152.0f);  // b 2^21
  const float fc = exact_i2f((int)(V & 0x1FFFFF));
  float s, e1, t, e2;
  two_sum_g(fa, fb, s, e1);
  two_sum_g(s, fc, t, e2);
  const float lo0 = __fadd_rn(e1, e2);
  const float hi = __fadd_rn(t, lo0);  // Fast2Sum renormalisation (|t| >= |lo0|)
  const float lo = __fsub_rn(lo0, __fsub_rn(hi, t));
  const float vh = hi * fscale;
  const float vl = lo * fscale;
  const float ah = vh * vh;
  const float al = fmaf(vh, vh, -ah) + 2.0f * vh * vl;
  return make_float2(ah, al);
}

// One 128 x 256 output tile of a split GEMM as the three roles see it: its
// problem, position, valid columns this launch, and whether it is skipped
// (no valid columns).  The problem's arguments are read in place through
// args(prob) (kernel parameters or a table in global memory), never copied
// as a whole per tile: a per-tile copy of the argument struct made the
// compiler spill the epilogue.
struct TileRef {
  int prob, m_tile, n_tile, N;
  bool skip;
};

// Single problem: tile index -> (m_tile, n_tile) in grouped rasterization
// (GROUP_M row tiles share the column tiles resident in L2); for the
// triangular L^-1 operand the row order is reversed so that the longest
// tiles (row tile i has ~i + 1 K-blocks) come first.  In the 2-SM kernel a
// tile index names row tiles 2i (rank 0) and 2i + 1 (rank 1) over one
// column tile; with an odd tiles_m the last pair's second row tile lies past
// the operand and its rows are never written.
struct SingleTiles {
  const CUtensorMap* tmA;
  const CUtensorMap* tmB;
  const GemmArgs* g;  // kernel parameter
  int pair_rank;      // CTA rank in the 2-SM kernel's pair, -1: one CTA per tile
  static constexpr bool global_maps = false;
  __device__ __forceinline__ int units_m() const { return pair_rank >= 0 ? (g->tiles_m + 1) >> 1 : g->tiles_m; }
  __device__ __forceinline__ int count() const { return units_m() * g->tiles_n; }
  // uniform tiles are dealt statically; the triangular L^-1 operand's tiles
  // (row tile i has ~i + 1 K-blocks) from the counter
  __device__ __forceinline__ bool dynamic() const { return g->tri_rows > 0; }
  __device__ __forceinline__ const GemmArgs& args(int) const { return *g; }
  __device__ __forceinline__ int* err() const { return g->err; }
  __device__ __forceinline__ uint64_t wait_ns() const { return g->wait_ns; }
  __device__ __forceinline__ const CUtensorMap* mapA(int) const { return tmA; }
  __device__ __forceinline__ const CUtensorMap* mapB(int) const { return tmB; }
  __device__ __forceinline__ TileRef tile(int t) const {
    const int gm = pair_rank >= 0 ? GROUP_M / 2 : GROUP_M;  // row units (tiles or tile pairs) per group
    const int per_group = gm * g->tiles_n;
    const int first_m = (t / per_group) * gm;
    const int gsz = min(units_m() - first_m, gm);
    int mu = first_m + (t % per_group) % gsz;
    if (g->tri_rows > 0) mu = units_m() - 1 - mu;  // longest (lowest) rows of L^-1 first
    const int m_tile = pair_rank >= 0 ? 2 * mu + pair_rank : mu;
    return TileRef{0, m_tile, (t % per_group) / gsz, g->N, false};
  }
};

// Many independent problems: a host-built table of tiles (longest problems
// first); the valid columns of each cohort this launch are cols[cohort];
// tensor maps in global memory, written by the host before the launch.  In
// the 2-SM kernel an entry names a pair of row tiles (m_tile = pair index):
// rank r computes row tile 2 m_tile + r.
struct GroupedTiles {
  const GroupedTile* tiles;
  const GroupedProblem* probs;
  const CUtensorMap* maps;
  const int* cols;
  int ntiles;
  int pair_rank;  // CTA rank in the 2-SM kernel's pair, -1: one CTA per tile
  static constexpr bool global_maps = true;
  __device__ __forceinline__ int count() const { return ntiles; }
  __device__ __forceinline__ bool dynamic() const { return true; }
  __device__ __forceinline__ const GemmArgs& args(int prob) const { return probs[prob].g; }
  __device__ __forceinline__ int* err() const { return probs[0].g.err; }  // shared by all problems
  __device__ __forceinline__ uint64_t wait_ns() const { return probs[0].g.wait_ns; }
  __device__ __forceinline__ const CUtensorMap* mapA(int prob) const { return maps + 2 * prob; }
  __device__ __forceinline__ const CUtensorMap* mapB(int prob) const { return maps + 2 * prob + 1; }
  __device__ __forceinline__ TileRef tile(int i) const {
    const GroupedTile tl = tiles[i];
    const int N = cols[probs[tl.prob].cohort];
    const int m_tile = pair_rank >= 0 ? 2 * tl.m_tile + pair_rank : tl.m_tile;
    return TileRef{tl.prob, m_tile, tl.n_tile, N, tl.n_tile * BN >= N};
  }
};

// Sum of two float pairs of non-negative values: TwoSum of the high parts,
// the rounding error and both low parts into the low part.  No
// renormalisation: over the five rounds below the low part stays below
// ~2^-20 of the high part, so its own rounding costs ~2^-44 relative, and
// the combine kernel renormalises.
__device__ __forceinline__ void pair_add(float ah, float al, float bh, float bl, float& h, float& l) {
  float e;
  two_sum_g(ah, bh, h, e);
  l = __fadd_rn(e, __fadd_rn(al, bl));
}

// Column sums over a warp's 32 rows.  Five exchange-and-add rounds with
// lane offsets 16, 8, 4, 2, 1, each lane keeping the half of its columns
// named by its lane bit, leave the sum of column `lane` with that lane; the
// order of the additions is fixed.  The caller runs the first round (offset
// 16, 32 -> 16 columns) as it forms the values; this runs the other four on
// lane k's 16 partial sums (h[c], l[c]), leaving column `lane` in (h[0], l[0]).
__device__ __forceinline__ void warp_column_sums(float (&h)[16], float (&l)[16], int lane) {
#pragma unroll
  for (int o = 8; o >= 1; o >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int k = 0; k < o; k++) {
      const float sh = up ? h[k] : h[k + o], sl = up ? l[k] : l[k + o];
      const float kh = up ? h[k + o] : h[k], kl = up ? l[k + o] : l[k];
      const float rh = __shfl_xor_sync(0xffffffffu, sh, o), rl = __shfl_xor_sync(0xffffffffu, sl, o);
      pair_add(kh, kl, rh, rl, h[k], l[k]);
    }
  }
}

// One pass of the split GEMM's epilogue for one thread (one output row,
// `cend` columns of its half tile from `crow`, stride ldc): read the pass's
// accumulator (P_2p + P_2p+1 / 32) from TMEM at `tacc` 32 columns at a time,
// form the exact int32 q = 32 v = P_2p * 32 + P_2p+1, and fold it into the
// int64 partial sums in C (V = V * 2^10 + q), or on the last pass write V
// times the row scale (FP64, or squared as a float pair for rows `sq`).
// With `qrow` set (warp-uniform: the warp's 32-row group holds rows `sq` of a
// unit-weight problem) the last pass writes no squares: the warp sums them
// over its rows and lane k writes column c0 + k's sum to qrow[c0 + k] for
// the `qend` valid columns of the half tile; rows not `sq` still write FP64.
__device__ __forceinline__ void epilogue_pass(uint32_t tacc, int p, bool last, bool sq, double scale, float fscale,
                                              long long* crow, long long ldc, int cend, float2* qrow, int qend) {
  const int lane = threadIdx.x & 31;
  // The int64 partial sums live from one pass to the next (~50 us, while the
  // other CTAs stream ~0.5 GB of operand tiles through L2): stored with
  // evict-last priority and read back, their last use, with evict-first, so
  // that they stay in L2 instead of making a DRAM round trip.
  uint64_t pol_keep, pol_drop;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol_keep));
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol_drop));
#pragma unroll 1
  for (int ch = 0; ch < BN / 64; ch++) {
    const int c0 = ch * 32;
    long long prev[32];
    if (p > 0) {
      // all 32 partial sums in flight at once, before the TMEM reads
#pragma unroll
      for (int j = 0; j < 32; j++) {
        long long t = 0;
        if (c0 + j < cend)
          asm volatile("ld.global.cg.L2::cache_hint.b64 %0, [%1], %2;"
                       : "=l"(t)
                       : "l"(crow + (long long)(c0 + j) * ldc), "l"(pol_drop));
        prev[j] = t;
      }
    }
    uint32_t v[32];
    tmem_ld32(tacc + c0, v);
    tmem_ld_wait();
    if (last && qrow != nullptr) {
      // column j's square as a float pair (0 past cend; rows not sq write FP64)
      auto term = [&](int j) -> float2 {
        if (c0 + j >= cend) return make_float2(0.0f, 0.0f);
        const int qv = fused_pair_f2i(__uint_as_float(v[j]));
        const long long V = (p == 0) ? (long long)qv : prev[j] * 1024ll + (long long)qv;
        if (sq) return square_pair(V, fscale);
        *(double*)(crow + (long long)(c0 + j) * ldc) = (double)V * scale;
        return make_float2(0.0f, 0.0f);
      };
      float h[16], l[16];
      const bool up = (lane & 16) != 0;
#pragma unroll
      for (int k = 0; k < 16; k++) {  // the offset-16 round: columns k and k + 16
        const float2 a = term(k), b = term(k + 16);
        const float2 send = up ? a : b, keep = up ? b : a;
        const float rh = __shfl_xor_sync(0xffffffffu, send.x, 16), rl = __shfl_xor_sync(0xffffffffu, send.y, 16);
        pair_add(keep.x, keep.y, rh, rl, h[k], l[k]);
      }
      warp_column_sums(h, l, lane);
      if (c0 + lane < qend) qrow[c0 + lane] = make_float2(h[0], l[0]);
      continue;
    }
#pragma unroll
    for (int j = 0; j < 32; j++) {
      if (c0 + j >= cend) break;
      const int qv = fused_pair_f2i(__uint_as_float(v[j]));
      long long* cp = crow + (long long)(c0 + j) * ldc;
      const long long V = (p == 0) ? (long long)qv : prev[j] * 1024ll + (long long)qv;
      if (!last)
        asm volatile("st.global.L2::cache_hint.b64 [%0], %1, %2;" ::"l"(cp), "l"(V), "l"(pol_keep) : "memory");
      else if (sq)
        *(float2*)cp = square_pair(V, fscale);
      else
        *(double*)cp = (double)V * scale;
    }
  }
}

// The producer thread of each CTA picks its next tile and publishes the
// index to the CTA's MMA thread and epilogue warps through a small ring in
// shared memory (tq_full / tq_empty barriers); an index past the end (-1)
// tells them to stop.  Tiles of uneven cost (grouped problems, the
// triangular L^-1 operand) are taken from a launch-wide counter, so that
// tiles listed longest first balance like the hardware block scheduler would,
// without a CTA launch per tile; uniform tiles are dealt statically in
// rounds of gridDim.x, forward in even rounds and backward in odd ones
// (measured 2 % faster than the counter on the eigen operand).  The counter
// pair (next tile, finished CTAs) starts at zero; the last CTA to finish
// zeroes it again for the next launch on the stream, so no reset is enqueued.
constexpr int TQ = 4;                // tile-queue slots
constexpr int TQ_CONSUMERS = 1 + 8;  // the MMA thread and lane 0 of each epilogue warp

// Persistent one-SM split GEMM: each CTA takes tiles from the launch-wide
// counter (or a static deal) until none are left; per tile, (S + 1) / 2
// passes of two slices each, both into one 256-column accumulator, passes
// alternating between the two halves of TMEM so that the epilogue of one
// pass (epilogue_pass) runs under the MMAs of the next.
// Between tiles the producer keeps loading the next tile's operands, so a
// CTA never drains its ring, and TMEM is allocated and the barriers
// initialised once per CTA.  (Releasing TMEM before the C round trip, with
// q held in registers, measured slower: within 168 registers a thread keeps
// too few partial-sum loads in flight for the round trip to finish within
// one pass of MMAs.)
template <class Src>
__device__ __forceinline__ void gemm_persistent(const Src& src, int* tile_counter) {
  using R = GemmRing;
  constexpr int KB = R::ROW;  // FP8 digits per K-step
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + R::STAGES * R::STAGE);
  uint64_t* empty = full + R::STAGES;
  uint64_t* tfull = empty + R::STAGES;  // [2]: accumulator half ready for the epilogue
  uint64_t* tempty = tfull + 2;         // [2]: accumulator half drained
  uint64_t* drain = tempty + 2;
  uint64_t* tq_full = drain + 1;
  uint64_t* tq_empty = tq_full + TQ;
  volatile int* tq_id = (volatile int*)(tq_empty + TQ);
  uint32_t* tbase_slot = (uint32_t*)(tq_id + TQ);
  volatile int* abort_flag = (volatile int*)(tbase_slot + 1);
  static_assert((R::STAGES * 2 + 5 + 2 * TQ) * 8 + TQ * 4 + 8 <= 256, "barriers fit the 256-byte tail");

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = src.count();

  if (threadIdx.x == 0) {
    for (int s = 0; s < R::STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], THREADS - 64);
    }
    mbar_init(drain, 1);
    for (int s = 0; s < TQ; s++) {
      mbar_init(&tq_full[s], 1);
      mbar_init(&tq_empty[s], TQ_CONSUMERS);
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tbase_slot)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tbase_slot;

  if (warp == 0) {
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int issued[R::STAGES];
      uint32_t issued_phase[R::STAGES];
      for (int s = 0; s < R::STAGES; s++) issued[s] = 0;
      bool ok = true;
      int last_prob = -1;
      int tq = 0;
      uint32_t tqph = 0;
      const bool dyn = src.dynamic();
      int kdeal = 0;
#pragma unroll 1
      while (ok) {
        int it;
        if (dyn) {
          it = atomicAdd(tile_counter, 1);
        } else {
          const int base = kdeal * (int)gridDim.x;
          it = base >= ntiles ? ntiles
                              : base + ((kdeal & 1) ? (int)gridDim.x - 1 - (int)blockIdx.x : (int)blockIdx.x);
          kdeal++;
        }
        if (it >= ntiles) it = -1;
        // publish the tile to the MMA thread and the epilogue warps
        if (!mbar_wait(&tq_empty[tq], tqph ^ 1, abort_flag, src.err(), 5, src.wait_ns())) { ok = false; break; }
        tq_id[tq] = it;
        mbar_arrive(&tq_full[tq]);
        if (++tq == TQ) { tq = 0; tqph ^= 1; }
        if (it < 0) break;
        const TileRef T = src.tile(it);
        if (T.skip) continue;
        const GemmArgs& g = src.args(T.prob);
        const CUtensorMap* tmA = src.mapA(T.prob);
        const CUtensorMap* tmB = src.mapB(T.prob);
        if (Src::global_maps && T.prob != last_prob) {
          asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;" ::"l"((uint64_t)tmA) : "memory");
          asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;" ::"l"((uint64_t)tmB) : "memory");
          last_prob = T.prob;
        }
        const int m0 = T.m_tile * BM, n0 = T.n_tile * BN;
        const int passes = (g.S + 1) / 2;
        int nk = g.Kpad / KB;
        if (m0 + BM <= g.tri_rows) nk = min(nk, (m0 + BM + KB - 1) / KB);  // zero upper part of L^-1
#pragma unroll 1
        for (int p = 0; p < passes && ok; p++) {
          const int s0 = 2 * p, s1 = 2 * p + 1;
          const bool two = s1 < g.S;
#pragma unroll 1
          for (int kb = 0; kb < nk; kb++) {
            if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag, g.err, 1, g.wait_ns)) { ok = false; break; }
            issued[stage] = 0;
            uint8_t* sb = smem + stage * R::STAGE;
            mbar_expect_tx(&full[stage], (two ? 2 * R::A : R::A) + R::B);
            tma_load_2d(sb, tmA, kb * KB, s0 * g.Mpad + m0, &full[stage]);
            if (two) tma_load_2d(sb + R::A, tmA, kb * KB, s1 * g.Mpad + m0, &full[stage]);
            tma_load_2d(sb + 2 * R::A, tmB, kb * KB, g.col0 + n0, &full[stage]);
            issued[stage] = 1;
            issued_phase[stage] = phase;
            if (++stage == R::STAGES) { stage = 0; phase ^= 1; }
          }
        }
      }
      if (!ok) {
        // let this CTA's own copies land before the shared memory is released
        for (int s = 0; s < R::STAGES; s++)
          if (issued[s]) mbar_drain(&full[s], issued_phase[s]);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0, q = 0;  // q: passes issued by this CTA (accumulator half and phase)
      bool ok = true;
      bool any = false;
      int tq = 0;
      uint32_t tqph = 0;
#pragma unroll 1
      while (ok) {
        if (!mbar_wait(&tq_full[tq], tqph, abort_flag, src.err(), 6, src.wait_ns())) { ok = false; break; }
        const int it = tq_id[tq];
        mbar_arrive(&tq_empty[tq]);
        if (++tq == TQ) { tq = 0; tqph ^= 1; }
        if (it < 0) break;
        const TileRef T = src.tile(it);
        if (T.skip) continue;
        const GemmArgs& g = src.args(T.prob);
        const int m0 = T.m_tile * BM;
        const int passes = (g.S + 1) / 2;
        int nk = g.Kpad / KB;
        if (m0 + BM <= g.tri_rows) nk = min(nk, (m0 + BM + KB - 1) / KB);
#pragma unroll 1
        for (int p = 0; p < passes && ok; p++, q++) {
          const bool two = 2 * p + 1 < g.S;
          const uint32_t buf = q & 1, par = (q >> 1) & 1;  // accumulator half and its phase
          if (!mbar_wait(&tempty[buf], par ^ 1, abort_flag, g.err, 2, g.wait_ns)) { ok = false; break; }
          tc_fence_after();
          const uint32_t acc = tbase + 256 * buf;
#pragma unroll 1
          for (int kb = 0; kb < nk; kb++) {
            if (!mbar_wait(&full[stage], phase, abort_flag, g.err, 3, g.wait_ns)) { ok = false; break; }
            tc_fence_after();
            uint8_t* sb = smem + stage * R::STAGE;
            const uint64_t a0 = desc_sw128(sb), a1 = desc_sw128(sb + R::A), b = desc_sw128(sb + 2 * R::A);
#pragma unroll
            for (int kk = 0; kk < R::ROW / 32; kk++) {  // 32 FP8 digits per MMA
              const uint64_t koff = (uint64_t)((kk * 32) >> 4);
              mma_f8(acc, a0 + koff, b + koff, IDESC, (kb > 0 || kk > 0) ? 1u : 0u);
              if (two) mma_f8(acc, a1 + koff, b + koff, IDESC, 1u);  // adds to slice 2p's sum
            }
            any = true;
            mma_commit(&empty[stage]);
            if (++stage == R::STAGES) { stage = 0; phase ^= 1; }
          }
          if (!ok) break;
          mma_commit(&tfull[buf]);
        }
      }
      if (!ok && any) {
        // all MMAs issued by this thread complete before TMEM is released
        mma_commit(drain);
        mbar_drain(drain, 0);
      }
    }
    __syncwarp();
  } else {
    // epilogue: warps 2..9.  Warp w reads TMEM lane quarter w % 4 (the
    // quarter a warp may access is fixed by its rank modulo 4) and column
    // half (w - 2) / 4; thread = one output row.
    const int lq = warp & 3;
    const int cbeg = ((warp - 2) >> 2) * (BN / 2);
    const int row = lq * 32 + lane;
    const uint32_t ta = tbase + ((uint32_t)(lq * 32) << 16) + (uint32_t)cbeg;
    uint32_t q = 0;
    bool ok = true;
    int tq = 0;
    uint32_t tqph = 0;
#pragma unroll 1
    while (ok) {
      int it = 0, okq = 1;
      if (lane == 0) {
        okq = mbar_wait(&tq_full[tq], tqph, abort_flag, src.err(), 7, src.wait_ns()) ? 1 : 0;
        if (okq) {
          it = tq_id[tq];
          mbar_arrive(&tq_empty[tq]);
        }
      }
      okq = __shfl_sync(0xffffffffu, okq, 0);
      it = __shfl_sync(0xffffffffu, it, 0);
      if (!okq) { ok = false; break; }
      if (++tq == TQ) { tq = 0; tqph ^= 1; }
      if (it < 0) break;
      const TileRef T = src.tile(it);
      if (T.skip) continue;
      const GemmArgs& g = src.args(T.prob);
      const int m0 = T.m_tile * BM, n0 = T.n_tile * BN;
      const int r = m0 + row;
      const bool rvalid = r < g.M;
      const double scale = rvalid ? g.row_scale[r] : 0.0;
      const bool sq = r < g.sq_rows;
      const float fscale = (float)scale;  // power of two: exact while >= 2^-149
      const int ncols = rvalid ? min(BN, T.N - n0) : 0;  // valid columns of this tile for this row
      const int cend = min(BN / 2, ncols - cbeg);        // of this thread's half (may be <= 0)
      long long* crow = (long long*)(g.C + (long long)r + (long long)(g.col0 + n0 + cbeg) * g.ldc);
      // unit weights: this warp's 32-row group (rows r & ~31 ..) sums its squares
      float2* qrow = (g.sqsum != nullptr && (r & ~31) < g.sq_rows)
                         ? g.sqsum + (long long)(r >> 5) * g.ldq + (g.col0 + n0 + cbeg)
                         : nullptr;
      const int qend = min(BN / 2, min(BN, T.N - n0) - cbeg);
      const int passes = (g.S + 1) / 2;
#pragma unroll 1
      for (int p = 0; p < passes; p++, q++) {
        const bool last = p == passes - 1;
        const uint32_t buf = q & 1, par = (q >> 1) & 1;
        // pull this row's partial sums (written a pass ago) back into L2
        // while the pass's MMAs run, if the evict-last policy did not keep
        // them.  Only for uniform long-K tiles: with the short passes of the
        // triangular and grouped operands the instructions cost more than
        // they save (grouped cohorts: 29.5 against 27.9 ms per launch).
        if (p > 0 && !src.dynamic())
          for (int c = 0; c < cend; c++)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(crow + (long long)c * g.ldc));
        int okw = 1;
        if (lane == 0) okw = mbar_wait(&tfull[buf], par, abort_flag, g.err, 4, g.wait_ns) ? 1 : 0;
        okw = __shfl_sync(0xffffffffu, okw, 0);  // warp-uniform: tcgen05.ld is .sync.aligned
        if (!okw) { ok = false; break; }
        tc_fence_after();
        epilogue_pass(ta + 256 * buf, p, last, sq, scale, fscale, crow, g.ldc, cend, qrow, qend);
        tc_fence_before();
        mbar_arrive(&tempty[buf]);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(512) : "memory");
  // the last CTA out zeroes the counters for the next launch (every CTA has
  // then stopped fetching tiles)
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(tile_counter + 1, 1) == (int)gridDim.x - 1) {
      atomicExch(tile_counter, 0);
      atomicExch(tile_counter + 1, 0);
    }
  }
}

// Single problem: at most one CTA per SM (launch with min(tiles, SMs) CTAs);
// tile_counter: two ints, zero before the first launch.
__global__ void __launch_bounds__(THREADS, 1)
    ozaki_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                      const __grid_constant__ GemmArgs g, int* tile_counter) {
  const SingleTiles src{&tmA, &tmB, &g, -1};
  gemm_persistent(src, tile_counter);
}

// ---------------------------------------------------------------------------
// 2-SM split GEMM (FP8 digits): a cluster of two CTAs on two
// SMs computes 256 x 256 output tiles with tcgen05.mma.cta_group::2 (M =
// 256, N = 256, K = 32).  CTA rank r holds rows 128 r .. 128 r + 127 of the
// tile (its A-slice tiles in shared memory, its accumulators in TMEM) and
// genotype rows 128 r .. 128 r + 127; the MMAs, issued by rank 0 (the
// leader), read both CTAs' shared memory and write both CTAs' TMEM.  Each
// CTA's shared memory thus holds half of the genotype tile where the one-SM
// kernel holds all of it: a 48 KB stage (two 128 x 128 A-slice tiles and a
// 128 x 128 genotype half, 128-byte K rows, 128B swizzle) carries the
// operands of eight 128 x 256 x 32 MMAs per SM, against 64 KB in the one-SM
// kernel, so four stages fit and a quarter fewer operand bytes move per MMA.
//
// Barriers: full[s] lives in the leader only (both CTAs' copies complete on
// it; the leader arms it with both CTAs' bytes); empty[s] and tfull[b] live
// in both CTAs and are released by the leader's multicast commits;
// tempty[b] lives in the leader and counts one arrival per epilogue warp of
// both CTAs.  The leader's producer picks each tile (a static deal per
// cluster for uniform tiles, the launch-wide counter for the triangular L^-1
// operand and for grouped problems) and writes its index into both CTAs'
// tile queues (the peer's slot through distributed shared memory, then a
// remote arrive on the peer's tq_full); tq_empty lives in the leader and
// counts the slot's eighteen readers (the leader's MMA thread, the peer's
// producer, both CTAs' epilogue warps).  Every wait is bounded.
namespace p2 {
constexpr int ROW = 128;            // bytes (FP8 digits) per K-step row
constexpr int A = BM * ROW;         // 16 KB: one A-slice tile of this CTA
constexpr int B = (BN / 2) * ROW;   // 16 KB: this CTA's half of the genotype tile
constexpr int STAGE = 2 * A + B;    // 48 KB
constexpr int STAGES = 4;
constexpr int SMEM = STAGES * STAGE + 1024 + 256;
// kind::f8f6f4: D=F32, A=B=E4M3, K-major, N=256, M=256 (the pair)
constexpr uint32_t IDESC = (1u << 4) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(256 >> 4) << 24);
constexpr int EPI_WARPS = 8;
}  // namespace p2

template <class Src>
__device__ __forceinline__ void gemm_pair(const Src& src, int* tile_counter) {
  constexpr int ROW = p2::ROW, A = p2::A, B = p2::B, STAGE = p2::STAGE, STAGES = p2::STAGES;
  constexpr int EPI_WARPS = p2::EPI_WARPS;
  constexpr uint32_t IDESC = p2::IDESC;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES * STAGE);  // [STAGES], used in the leader
  uint64_t* empty = full + STAGES;                       // [STAGES]
  uint64_t* tfull = empty + STAGES;                      // [2]
  uint64_t* tempty = tfull + 2;                          // [2], used in the leader
  uint64_t* drain = tempty + 2;
  uint64_t* tq_full = drain + 1;                         // [TQ], both CTAs
  uint64_t* tq_empty = tq_full + TQ;                     // [TQ], used in the leader
  volatile int* tq_id = (volatile int*)(tq_empty + TQ);
  uint32_t* tbase_slot = (uint32_t*)(tq_id + TQ);
  volatile int* abort_flag = (volatile int*)(tbase_slot + 1);
  static_assert((STAGES * 2 + 5 + 2 * TQ) * 8 + TQ * 4 + 8 <= 256, "barriers fit the 256-byte tail");

  const uint32_t rank = (uint32_t)src.pair_rank;
  const bool lead = rank == 0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = src.count();
  const uint16_t BOTH = 0x3;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], 2 * EPI_WARPS);
    }
    mbar_init(drain, 1);
    for (int s = 0; s < TQ; s++) {
      mbar_init(&tq_full[s], 1);
      // consumers of a queue slot: the leader's MMA thread and both CTAs'
      // epilogue warps and the peer's producer
      mbar_init(&tq_empty[s], 2 * (1 + EPI_WARPS));
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {  // one warp of each CTA allocates the same columns in both
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tbase_slot)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  cluster_sync();  // both CTAs' barriers are initialised before either signals the other's
  tc_fence_after();
  const uint32_t tbase = *tbase_slot;
  const uint32_t lead_full = cluster_addr(full, 0);          // full[s] is 8 s bytes further
  const uint32_t lead_tq_empty = cluster_addr(tq_empty, 0);  // tq_empty[s] likewise
  int* err = src.err();
  const uint64_t wait_ns = src.wait_ns();

  // Bounded wait with cluster-scope acquire, for the tile-queue barriers:
  // their arrivals (and the queued index) may come from the other CTA.
  auto cwait = [&](uint64_t* bar, uint32_t par, int site) -> bool {
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t it = 0;; ++it) {
      if (mbar_try_wait_cluster(bar, par)) return true;
      const bool every = (it & 63) == 63;  // as in mbar_wait
      if (every && (*abort_flag || *(volatile int*)err)) {
        *abort_flag = 1;
        return false;
      }
      if ((every || it == 0) && globaltimer_ns() - t0 > wait_ns) {
        *abort_flag = 1;
        atomicCAS(err, 0, site);
        return false;
      }
    }
  };

  if (warp == 0) {
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int issued[STAGES];
      uint32_t issued_phase[STAGES];
      for (int s = 0; s < STAGES; s++) issued[s] = 0;
      bool ok = true;
      int tq = 0;
      uint32_t tqph = 0;
      int last_prob = -1;
      const bool dyn = src.dynamic();
      const int deal_id = (int)(blockIdx.x >> 1), deal_n = (int)(gridDim.x >> 1);
      int kdeal = 0;
      const uint32_t peer_tq_id = cluster_addr((const void*)tq_id, 1);
      const uint32_t peer_tq_full = cluster_addr(tq_full, 1);
#pragma unroll 1
      while (ok) {
        int it;
        if (lead) {
          // the leader picks the pair's next tile and publishes it to both CTAs
          if (dyn) {
            it = atomicAdd(tile_counter, 1);
          } else {
            const int base = kdeal * deal_n;
            it = base >= ntiles ? ntiles : base + ((kdeal & 1) ? deal_n - 1 - deal_id : deal_id);
            kdeal++;
          }
          if (it >= ntiles) it = -1;
          if (!cwait(&tq_empty[tq], tqph ^ 1, 5)) { ok = false; break; }
          tq_id[tq] = it;
          asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(peer_tq_id + 4u * (uint32_t)tq), "r"(it) : "memory");
          mbar_arrive(&tq_full[tq]);
          mbar_arrive_cluster(peer_tq_full + 8u * (uint32_t)tq);  // release: the index is visible first
        } else {
          if (!cwait(&tq_full[tq], tqph, 9)) { ok = false; break; }
          it = tq_id[tq];
          mbar_arrive_cluster(lead_tq_empty + 8u * (uint32_t)tq);
        }
        if (++tq == TQ) { tq = 0; tqph ^= 1; }
        if (it < 0) break;
        const TileRef T = src.tile(it);
        if (T.skip) continue;
        const GemmArgs& g = src.args(T.prob);
        const CUtensorMap* tmA = src.mapA(T.prob);
        const CUtensorMap* tmB = src.mapB(T.prob);
        if (Src::global_maps && T.prob != last_prob) {
          asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;" ::"l"((uint64_t)tmA) : "memory");
          asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;" ::"l"((uint64_t)tmB) : "memory");
          last_prob = T.prob;
        }
        const int m0 = T.m_tile * BM, n0 = T.n_tile * BN;
        const int passes = (g.S + 1) / 2;
        int nk = g.Kpad / ROW;
        // the pair's larger row tile decides the K extent of the zero-topped L^-1
        const int top = ((T.m_tile | 1) + 1) * BM;
        if (top <= g.tri_rows) nk = min(nk, (top + ROW - 1) / ROW);
#pragma unroll 1
        for (int p = 0; p < passes && ok; p++) {
          const int s0 = 2 * p, s1 = 2 * p + 1;
          const bool two = s1 < g.S;
#pragma unroll 1
          for (int kb = 0; kb < nk; kb++) {
            if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag, g.err, 1, g.wait_ns)) { ok = false; break; }
            issued[stage] = 0;
            uint8_t* sb = smem + stage * STAGE;
            const uint32_t fb = lead_full + 8u * (uint32_t)stage;
            if (lead) mbar_expect_tx(&full[stage], 2 * ((two ? 2 * A : A) + B));  // both CTAs' bytes
            tma_load_2d_cg2(sb, tmA, kb * ROW, s0 * g.Mpad + m0, fb);
            if (two) tma_load_2d_cg2(sb + A, tmA, kb * ROW, s1 * g.Mpad + m0, fb);
            tma_load_2d_cg2(sb + 2 * A, tmB, kb * ROW, g.col0 + n0 + (int)rank * (BN / 2), fb);
            issued[stage] = 1;
            issued_phase[stage] = phase;
            if (++stage == STAGES) { stage = 0; phase ^= 1; }
          }
        }
      }
      if (ok) {
        // every stage filled so far has been released by the leader's MMAs:
        // no multicast commit is still on its way to this CTA
#pragma unroll 1
        for (int i = 0; i < STAGES; i++) {
          if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag, err, 8, wait_ns)) break;
          if (++stage == STAGES) { stage = 0; phase ^= 1; }
        }
      } else if (lead) {
        // the leader's barrier tracks both CTAs' copies of every stage it armed
        const uint64_t deadline = globaltimer_ns() + WAIT_NS;
        for (int s = 0; s < STAGES; s++)
          if (issued[s]) mbar_drain_until(&full[s], issued_phase[s], deadline);
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && lead) {
      int stage = 0;
      uint32_t phase = 0, q = 0;
      bool ok = true;
      bool any = false;
      int tq = 0;
      uint32_t tqph = 0;
#pragma unroll 1
      while (ok) {
        if (!cwait(&tq_full[tq], tqph, 6)) { ok = false; break; }
        const int it = tq_id[tq];
        mbar_arrive(&tq_empty[tq]);
        if (++tq == TQ) { tq = 0; tqph ^= 1; }
        if (it < 0) break;
        const TileRef T = src.tile(it);
        if (T.skip) continue;
        const GemmArgs& g = src.args(T.prob);
        const int passes = (g.S + 1) / 2;
        int nk = g.Kpad / ROW;
        const int top = ((T.m_tile | 1) + 1) * BM;
        if (top <= g.tri_rows) nk = min(nk, (top + ROW - 1) / ROW);
#pragma unroll 1
        for (int p = 0; p < passes && ok; p++, q++) {
          const bool two = 2 * p + 1 < g.S;
          const uint32_t buf = q & 1, par = (q >> 1) & 1;
          // both CTAs' epilogues have drained this accumulator half
          {
            const uint64_t t0 = globaltimer_ns();
            uint32_t spin = 0;
            while (!mbar_try_wait_cluster(&tempty[buf], par ^ 1)) {
              const bool every = (spin & 63) == 63, first = spin == 0;  // as in mbar_wait
              spin++;
              if ((every && (*abort_flag || *(volatile int*)g.err)) ||
                  ((every || first) && globaltimer_ns() - t0 > g.wait_ns)) {
                *abort_flag = 1;
                atomicCAS(g.err, 0, 2);
                ok = false;
                break;
              }
            }
            if (!ok) break;
          }
          tc_fence_after();
          const uint32_t acc = tbase + 256 * buf;
#pragma unroll 1
          for (int kb = 0; kb < nk; kb++) {
            if (!mbar_wait(&full[stage], phase, abort_flag, g.err, 3, g.wait_ns)) { ok = false; break; }
            tc_fence_after();
            uint8_t* sb = smem + stage * STAGE;
            const uint64_t a0 = desc_sw128(sb), a1 = desc_sw128(sb + A), b = desc_sw128(sb + 2 * A);
#pragma unroll
            for (int kk = 0; kk < ROW / 32; kk++) {  // 32 FP8 digits per MMA
              const uint64_t koff = (uint64_t)((kk * 32) >> 4);
              mma_f8_cg2(acc, a0 + koff, b + koff, IDESC, (kb > 0 || kk > 0) ? 1u : 0u);
              if (two) mma_f8_cg2(acc, a1 + koff, b + koff, IDESC, 1u);  // adds to slice 2p's sum
            }
            any = true;
            mma_commit_cg2(&empty[stage], BOTH);  // the stage is free in both CTAs
            if (++stage == STAGES) { stage = 0; phase ^= 1; }
          }
          if (!ok) break;
          mma_commit_cg2(&tfull[buf], BOTH);
        }
      }
      if (!ok && any) {
        // all MMAs issued by this thread complete before TMEM is released
        mma_commit_cg2(drain, 0x1);
        mbar_drain(drain, 0);
      }
    }
    __syncwarp();
  } else {
    // epilogue: warps 2..9 of each CTA drain that CTA's 128 rows, as in the
    // one-SM kernel; one arrival per warp on the leader's tempty
    const int lq = warp & 3;
    const int cbeg = ((warp - 2) >> 2) * (BN / 2);
    const int row = lq * 32 + lane;
    const uint32_t ta = tbase + ((uint32_t)(lq * 32) << 16) + (uint32_t)cbeg;
    const uint32_t lead_tempty = cluster_addr(tempty, 0);
    uint32_t q = 0;
    bool ok = true;
    int tq = 0;
    uint32_t tqph = 0;
#pragma unroll 1
    while (ok) {
      int it = 0, okq = 1;
      if (lane == 0) {
        okq = cwait(&tq_full[tq], tqph, 7) ? 1 : 0;
        if (okq) {
          it = tq_id[tq];
          mbar_arrive_cluster(lead_tq_empty + 8u * (uint32_t)tq);
        }
      }
      okq = __shfl_sync(0xffffffffu, okq, 0);
      it = __shfl_sync(0xffffffffu, it, 0);
      if (!okq) { ok = false; break; }
      if (++tq == TQ) { tq = 0; tqph ^= 1; }
      if (it < 0) break;
      const TileRef T = src.tile(it);
      if (T.skip) continue;
      const GemmArgs& g = src.args(T.prob);
      const int m0 = T.m_tile * BM, n0 = T.n_tile * BN;
      const int r = m0 + row;
      const bool rvalid = r < g.M;
      const double scale = rvalid ? g.row_scale[r] : 0.0;
      const bool sq = r < g.sq_rows;
      const float fscale = (float)scale;
      const int ncols = rvalid ? min(BN, T.N - n0) : 0;
      const int cend = min(BN / 2, ncols - cbeg);
      long long* crow = (long long*)(g.C + (long long)r + (long long)(g.col0 + n0 + cbeg) * g.ldc);
      // unit weights: this warp's 32-row group (rows r & ~31 ..) sums its squares
      float2* qrow = (g.sqsum != nullptr && (r & ~31) < g.sq_rows)
                         ? g.sqsum + (long long)(r >> 5) * g.ldq + (g.col0 + n0 + cbeg)
                         : nullptr;
      const int qend = min(BN / 2, min(BN, T.N - n0) - cbeg);
      const int passes = (g.S + 1) / 2;
#pragma unroll 1
      for (int p = 0; p < passes; p++, q++) {
        const bool last = p == passes - 1;
        const uint32_t buf = q & 1, par = (q >> 1) & 1;
        if (p > 0 && !src.dynamic())  // as in the one-SM kernel
          for (int c = 0; c < cend; c++)
            asm volatile("prefetch.global.L2 [%0];" ::"l"(crow + (long long)c * g.ldc));
        int okw = 1;
        if (lane == 0) okw = mbar_wait(&tfull[buf], par, abort_flag, g.err, 4, g.wait_ns) ? 1 : 0;
        okw = __shfl_sync(0xffffffffu, okw, 0);
        if (!okw) { ok = false; break; }
        tc_fence_after();
        epilogue_pass(ta + 256 * buf, p, last, sq, scale, fscale, crow, g.ldc, cend, qrow, qend);
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive_cluster(lead_tempty + 8u * buf);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  // the leader's MMAs, which write both CTAs' TMEM, are complete (its MMA
  // thread drained or its epilogue consumed every pass) before either CTA
  // releases TMEM
  cluster_sync();
  tc_fence_after();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(512) : "memory");
  // neither CTA exits while the other may still signal its barriers or
  // copy into its shared memory.  After an expired wait the peer's copies of
  // a stage the leader never armed cannot be observed; both producers have
  // stopped issuing once both CTAs pass the cluster barrier, so a short
  // pause lets such copies land before the shared memory is released.
  cluster_sync();
  if (*abort_flag) {
    const uint64_t t0 = globaltimer_ns();
    while (globaltimer_ns() - t0 < 100000ull) {
    }
  }
  // the last CTA out zeroes the tile counters for the next launch (every CTA
  // has then stopped fetching tiles)
  if (threadIdx.x == 0 && tile_counter) {
    __threadfence();
    if (atomicAdd(tile_counter + 1, 1) == (int)gridDim.x - 1) {
      atomicExch(tile_counter, 0);
      atomicExch(tile_counter + 1, 0);
    }
  }
}

// 2-SM launches: clusters of two CTAs, one pair of SMs per cluster, at most
// as many clusters as fit at once.  Uniform tiles are dealt statically per
// cluster, those of the triangular L^-1 operand (and of grouped problems)
// taken from the launch-wide counter (two ints, zero before the first launch).
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(THREADS, 1)
    ozaki_gemm2_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmBh,
                       const __grid_constant__ GemmArgs g, int* tile_counter) {
  const SingleTiles src{&tmA, &tmBh, &g, (int)cluster_rank()};
  gemm_pair(src, tile_counter);
}

// Many independent problems over a table of row-tile pairs; genotype maps in
// 128-row boxes.
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(THREADS, 1)
    ozaki_grouped_gemm2_kernel(const GroupedTile* __restrict__ tiles, const GroupedProblem* __restrict__ probs,
                               const CUtensorMap* __restrict__ maps, const int* __restrict__ cols, int ntiles,
                               int* tile_counter) {
  const GroupedTiles src{tiles, probs, maps, cols, ntiles, (int)cluster_rank()};
  gemm_pair(src, tile_counter);
}

// Many independent problems in one persistent launch over a tile table;
// tiles past a problem's valid columns this launch are skipped by all roles.
__global__ void __launch_bounds__(THREADS, 1)
    ozaki_grouped_gemm_kernel(const GroupedTile* __restrict__ tiles, const GroupedProblem* __restrict__ probs,
                              const CUtensorMap* __restrict__ maps, const int* __restrict__ cols, int ntiles,
                              int* tile_counter) {
  const GroupedTiles src{tiles, probs, maps, cols, ntiles, -1};
  gemm_persistent(src, tile_counter);
}

// ---------------------------------------------------------------------------
// Quadratic Gram terms on the tensor cores (eigen, many traits):
//
//   GR[i + j*ldg] = sum_l R2[l,i] d_j(l),  R2 >= 0, d > 0.
//
// Both operands are cut into signed base-32 digits (5 bits, |digit| <= 16,
// exact in FP8 E4M3): a = R2 / sigma_i = sum_s alpha_s 32^-s,
// b = d / tau_j = sum_t delta_t 32^-t with sigma_i, tau_j powers of two such
// that a, b <= 1/2.  A digit product is at most 2^8, so a K-sum over
// K <= 65536 rows is an integer of at most 2^24: exact in the FP32 TMEM
// accumulator of the kind::f8f6f4 MMA (twice the BF16 rate).  Pairs with
// s + t <= L are kept (L = 12, 11 digits a side: the dropped pairs and the
// digit remainders stay below 2^-55 of sigma_i tau_j per row).  The epilogue
// scales each exact pair sum by 32^-(s+t) (exact) and accumulates it in a
// float pair by TwoSum (relative error ~2^-47), then multiplies by
// sigma_i tau_j in FP64.
//
// quadtc_kernel: persistent CTAs over (128 SNP rows x group of 112 traits,
// pass) units.  A pass holds one SNP digit s (A tile 128 x 128 bytes) and up
// to four trait digits t (B tiles 112 x 128 bytes, two per MMA as N = 224);
// TMEM accumulators at columns [0, 224) and [224, 448).  Same warp roles and
// bounded waits as ozaki_gemm_kernel.  Threads keep the running (hi, lo) sums
// of 56 traits.
// ---------------------------------------------------------------------------
constexpr int QT_STAGES = 3;                      // ring stages
constexpr int QT_TP = 112;                          // trait rows of the digit operand
constexpr int QT_KB = 128;                          // K-block: 128 one-byte digits (one 128B-swizzled row)
constexpr int QT_BT = QT_TP * QT_KB;                // 14 KB trait tile
constexpr int QT_STAGE = A_TILE + 4 * QT_BT;        // 72 KB
constexpr int QT_SMEM = QT_STAGES * QT_STAGE + 1024 + 256;
constexpr int QT_MAXPASS = 40;
// kind::f8f6f4 instruction descriptor: F32 accumulator, A and B E4M3 (format
// 0), K-major, N = 224, M = 128
constexpr uint32_t QT_IDESC = (1u << 4) | ((uint32_t)(224 >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
// the same with N = 112: one trait digit of a slot pair whose second slot is empty
constexpr uint32_t QT_IDESC1 = (1u << 4) | ((uint32_t)(QT_TP >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
static_assert(A_TILE == BM * QT_KB, "the SNP digit tile has the bytes of one 128-byte-row GEMM tile");

struct QuadPasses {
  int n;
  signed char s[QT_MAXPASS];     // SNP digit (1-based)
  signed char t[QT_MAXPASS][4];  // trait digits (1-based, 0 = empty slot)
};

struct QuadArgs {
  int x;          // valid SNP rows
  int t;          // valid traits
  int tgp;        // rows per trait digit plane: trait groups of QT_TP times QT_TP
  int Ncap;       // rows per SNP digit slice
  int Kq;         // digit row length (bytes, multiple of QT_KB)
  int groups;     // trait groups (tgp / QT_TP)
  int units;      // work units: tiles (128 SNPs x one trait group) x passes
  const int* aexp;  // per SNP: sigma_i = 2^aexp
  const int* dexp;  // per trait: tau_j = 2^dexp
  double* part;     // QT_SLOTS partial planes of Ncap x tgp (column-major, ld Ncap)
  int* err;
  unsigned long long wait_ns;  // limit of one pipeline wait
};

// Work units are dealt to the persistent CTAs in contiguous ranges, unit
// u = tile * passes + pass, tile = m_tile * groups + group.  A tile whose
// passes span several CTAs gets one partial plane per CTA (slot = CTA -
// first owner); quadtc_combine_kernel adds them in slot order.
constexpr int QT_SLOTS = 3;
__host__ __device__ __forceinline__ int qt_range_begin(int c, int units, int ctas) {
  return (int)(((long long)c * units) / ctas);
}
__host__ __device__ __forceinline__ int qt_owner(int u, int units, int ctas) {
  return (int)((((long long)u + 1) * ctas - 1) / units);
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}

__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}

// Partial plane of tile `tl` from this CTA (slot = this CTA - the tile's
// first owner): the thread's SNP row and 56 traits, scaled to FP64.
__device__ __forceinline__ void quadtc_flush(const QuadArgs& g, int tl, int np, int q, int lane, int jl,
                                             const float (&H)[56], const float (&L)[56]) {
  const int i = (tl / g.groups) * BM + q * 32 + lane;
  const int jh = (tl % g.groups) * QT_TP + jl;
  const int slot = (int)blockIdx.x - qt_owner(tl * np, g.units, gridDim.x);
  if (i >= g.x) return;
  const double si = ldexp(1.0, g.aexp[i]);
  double* P = g.part + (size_t)slot * g.Ncap * g.tgp;
#pragma unroll
  for (int c = 0; c < 56; c++) {
    const int j = jh + c;
    if (j < g.t) P[i + (size_t)j * g.Ncap] = ((double)H[c] + (double)L[c]) * si * ldexp(1.0, g.dexp[j]);
  }
}

__global__ void __launch_bounds__(THREADS, 1)
    quadtc_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmD,
                  const __grid_constant__ QuadPasses qp, const QuadArgs g) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + QT_STAGES * QT_STAGE);
  uint64_t* empty = full + QT_STAGES;
  uint64_t* tfull = empty + QT_STAGES;
  uint64_t* tempty = tfull + 1;
  uint64_t* drain = tempty + 1;
  uint32_t* tbase_slot = (uint32_t*)(drain + 1);
  volatile int* abort_flag = (volatile int*)(tbase_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = g.Kq / QT_KB;
  const int np = qp.n;
  const int u0 = qt_range_begin(blockIdx.x, g.units, gridDim.x);
  const int u1 = qt_range_begin(blockIdx.x + 1, g.units, gridDim.x);

  if (threadIdx.x == 0) {
    for (int s = 0; s < QT_STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(tfull, 1);
    mbar_init(tempty, THREADS - 64);
    mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tbase_slot)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = *tbase_slot;

  if (warp == 0) {
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int issued[QT_STAGES];
      uint32_t issued_phase[QT_STAGES];
      for (int s = 0; s < QT_STAGES; s++) issued[s] = 0;
      bool ok = true;
      for (int u = u0; u < u1 && ok; u++) {
        const int tile = u / np, p = u - tile * np;
        const int m0 = (tile / g.groups) * BM, grp = tile % g.groups;
        int nt = 0;
        for (int q = 0; q < 4; q++) nt += qp.t[p][q] > 0 ? 1 : 0;
        for (int kb = 0; kb < nk; kb++) {
          if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag, g.err, 11, g.wait_ns)) { ok = false; break; }
          issued[stage] = 0;
          uint8_t* sb = smem + stage * QT_STAGE;
          mbar_expect_tx(&full[stage], A_TILE + nt * QT_BT);
          tma_load_2d(sb, &tmA, kb * QT_KB, (qp.s[p] - 1) * g.Ncap + m0, &full[stage]);
          for (int q = 0; q < 4; q++)
            if (qp.t[p][q] > 0)
              tma_load_2d(sb + A_TILE + q * QT_BT, &tmD, kb * QT_KB, (qp.t[p][q] - 1) * g.tgp + grp * QT_TP,
                          &full[stage]);
          issued[stage] = 1;
          issued_phase[stage] = phase;
          if (++stage == QT_STAGES) { stage = 0; phase ^= 1; }
        }
      }
      if (!ok)
        for (int s = 0; s < QT_STAGES; s++)
          if (issued[s]) mbar_drain(&full[s], issued_phase[s]);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      bool ok = true, any = false;
      for (int u = u0; u < u1 && ok; u++) {
        const int lu = u - u0;
        const int p = u % np;
        const bool second = qp.t[p][2] > 0;
        // a slot pair with its second slot empty needs only the first slot's columns
        const uint32_t id01 = qp.t[p][1] > 0 ? QT_IDESC : QT_IDESC1;
        const uint32_t id23 = qp.t[p][3] > 0 ? QT_IDESC : QT_IDESC1;
        if (!mbar_wait(tempty, (lu & 1) ^ 1, abort_flag, g.err, 12, g.wait_ns)) { ok = false; break; }
        tc_fence_after();
        for (int kb = 0; kb < nk; kb++) {
          if (!mbar_wait(&full[stage], phase, abort_flag, g.err, 13, g.wait_ns)) { ok = false; break; }
          tc_fence_after();
          uint8_t* sb = smem + stage * QT_STAGE;
          const uint64_t a = desc_sw128(sb), b01 = desc_sw128(sb + A_TILE), b23 = desc_sw128(sb + A_TILE + 2 * QT_BT);
#pragma unroll
          for (int k = 0; k < QT_KB / 32; k++) {  // K = 32 one-byte digits (32 bytes) per MMA
            const uint64_t koff = (uint64_t)((k * 32) >> 4);
            const uint32_t acc = (kb > 0 || k > 0) ? 1u : 0u;
            mma_f8(tbase, a + koff, b01 + koff, id01, acc);
            if (second) mma_f8(tbase + 224, a + koff, b23 + koff, id23, acc);
          }
          any = true;
          mma_commit(&empty[stage]);
          if (++stage == QT_STAGES) { stage = 0; phase ^= 1; }
        }
        if (!ok) break;
        mma_commit(tfull);
      }
      if (!ok && any) {
        mma_commit(drain);
        mbar_drain(drain, 0);
      }
    }
    __syncwarp();
  } else {
    // epilogue: warp w reads TMEM lane quarter w % 4 (SNP rows) and the
    // trait half (w - 2) / 4 (56 traits) of the unit's trait group
    const int q = warp & 3;
    const int jl = ((warp - 2) >> 2) * 56;  // TMEM column offset within the group
    float H[56], L[56];
    bool done = true;
    for (int u = u0; u < u1 && done;) {
      const int tile = u / np;
      const int uend = min(u1, (tile + 1) * np);  // this CTA's passes of the tile
#pragma unroll
      for (int c = 0; c < 56; c++) H[c] = L[c] = 0.0f;
      for (; u < uend; u++) {
        const int lu = u - u0;
        const int p = u - tile * np;
        int ok = 1;
        if (lane == 0) ok = mbar_wait(tfull, lu & 1, abort_flag, g.err, 14, g.wait_ns) ? 1 : 0;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) { done = false; break; }
        tc_fence_after();
#pragma unroll 1
        for (int slot = 0; slot < 4; slot++) {
          const int tt = qp.t[p][slot];
          if (tt <= 0) continue;  // uniform across the CTA
          const float w = __int_as_float((127 - 5 * (qp.s[p] + tt)) << 23);  // 32^-(s+t)
          const uint32_t col = (uint32_t)((slot >> 1) * 224 + (slot & 1) * QT_TP + jl);
          const uint32_t ta = tbase + ((uint32_t)(q * 32) << 16) + col;
#pragma unroll
          for (int c8 = 0; c8 < 7; c8++) {
            uint32_t v[8];
            tmem_ld8(ta + c8 * 8, v);
            tmem_ld_wait();
#pragma unroll
            for (int e8 = 0; e8 < 8; e8++) {
              const float x = __fmul_rn(__uint_as_float(v[e8]), w);  // exact: integer times a power of two
              float s2, e;
              two_sum_f(H[c8 * 8 + e8], x, s2, e);
              H[c8 * 8 + e8] = s2;
              L[c8 * 8 + e8] = __fadd_rn(L[c8 * 8 + e8], e);
            }
          }
        }
        tc_fence_before();
        mbar_arrive(tempty);
      }
      if (done) quadtc_flush(g, tile, np, q, lane, jl, H, L);
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(512) : "memory");
}

// ---------------------------------------------------------------------------
// 2-SM tensor-core quadratic Gram: a cluster of two CTAs computes 256 SNP
// rows (rank r: rows 128 r .. 128 r + 127 of the pair tile) of one 112-trait
// group per unit, with tcgen05.mma.cta_group::2 (M = 256) issued by the
// leader.  An MMA over the slot pair (2q, 2q + 1) (N = 224) takes trait
// digit slot 2q + r from CTA r (112 rows); with the pair's second slot empty
// (N = 112) each CTA holds 56 rows of slot 2q.  Per CTA a stage is the SNP
// digit tile (16 KB) and two trait tiles (2 x 14 KB): 44 KB, five stages;
// the accumulator layout in each CTA's TMEM and the epilogue are those of
// quadtc_kernel.  Units are dealt to clusters in contiguous ranges; full[s]
// and tempty live in the leader, empty[s] and tfull in both CTAs.
// ---------------------------------------------------------------------------
constexpr int QT2_STAGES = 5;
constexpr int QT2_STAGE = A_TILE + 2 * QT_BT;  // 44 KB
constexpr int QT2_SMEM = QT2_STAGES * QT2_STAGE + 1024 + 256;
constexpr uint32_t QT2_IDESC = (1u << 4) | ((uint32_t)(224 >> 3) << 17) | ((uint32_t)(256 >> 4) << 24);
constexpr uint32_t QT2_IDESC1 = (1u << 4) | ((uint32_t)(QT_TP >> 3) << 17) | ((uint32_t)(256 >> 4) << 24);

// Partial plane of pair tile `tl` from this cluster (slot = this cluster -
// the tile's first owner): the thread's SNP row and 56 traits, scaled to FP64.
__device__ __forceinline__ void quadtc2_flush(const QuadArgs& g, int tl, int np, int rank, int q, int lane, int jl,
                                              const float (&H)[56], const float (&L)[56]) {
  const int i = (tl / g.groups) * (2 * BM) + rank * BM + q * 32 + lane;
  const int jh = (tl % g.groups) * QT_TP + jl;
  const int slot = (int)(blockIdx.x >> 1) - qt_owner(tl * np, g.units, gridDim.x >> 1);
  if (i >= g.x) return;
  const double si = ldexp(1.0, g.aexp[i]);
  double* P = g.part + (size_t)slot * g.Ncap * g.tgp;
#pragma unroll
  for (int c = 0; c < 56; c++) {
    const int j = jh + c;
    if (j < g.t) P[i + (size_t)j * g.Ncap] = ((double)H[c] + (double)L[c]) * si * ldexp(1.0, g.dexp[j]);
  }
}

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(THREADS, 1)
    quadtc2_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmD,
                   const __grid_constant__ CUtensorMap tmD56, const __grid_constant__ QuadPasses qp,
                   const QuadArgs g) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + QT2_STAGES * QT2_STAGE);  // [QT2_STAGES], used in the leader
  uint64_t* empty = full + QT2_STAGES;                           // [QT2_STAGES]
  uint64_t* tfull = empty + QT2_STAGES;
  uint64_t* tempty = tfull + 1;  // used in the leader
  uint64_t* drain = tempty + 1;
  uint32_t* tbase_slot = (uint32_t*)(drain + 1);
  volatile int* abort_flag = (volatile int*)(tbase_slot + 1);
  static_assert((QT2_STAGES * 2 + 3) * 8 + 8 <= 256, "barriers fit the 256-byte tail");

  const uint32_t rank = cluster_rank();
  const bool lead = rank == 0;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = g.Kq / QT_KB;
  const int np = qp.n;
  const int cid = (int)(blockIdx.x >> 1), ncl = (int)(gridDim.x >> 1);
  const int u0 = qt_range_begin(cid, g.units, ncl);
  const int u1 = qt_range_begin(cid + 1, g.units, ncl);
  const uint16_t BOTH = 0x3;

  if (threadIdx.x == 0) {
    for (int s = 0; s < QT2_STAGES; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(tfull, 1);
    mbar_init(tempty, 2 * 8);  // one arrival per epilogue warp of both CTAs
    mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {  // one warp of each CTA allocates the same columns in both
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tbase_slot)),
                 "r"(512)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  cluster_sync();
  tc_fence_after();
  const uint32_t tbase = *tbase_slot;
  const uint32_t lead_full = cluster_addr(full, 0);

  if (warp == 0) {
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int issued[QT2_STAGES];
      uint32_t issued_phase[QT2_STAGES];
      for (int s = 0; s < QT2_STAGES; s++) issued[s] = 0;
      bool ok = true;
      for (int u = u0; u < u1 && ok; u++) {
        const int tile = u / np, p = u - tile * np;
        const int m0 = (tile / g.groups) * (2 * BM) + (int)rank * BM, grp = tile % g.groups;
        // this CTA's bytes of a K-step: the SNP digit tile, then per slot
        // pair its slot 2q + rank (both slots present) or its 56-row half
        // of slot 2q (second slot empty)
        int bytes = A_TILE;
        for (int pq = 0; pq < 2; pq++)
          if (qp.t[p][2 * pq] > 0) bytes += qp.t[p][2 * pq + 1] > 0 ? QT_BT : QT_BT / 2;
        for (int kb = 0; kb < nk; kb++) {
          if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag, g.err, 11, g.wait_ns)) { ok = false; break; }
          issued[stage] = 0;
          uint8_t* sb = smem + stage * QT2_STAGE;
          const uint32_t fb = lead_full + 8u * (uint32_t)stage;
          if (lead) mbar_expect_tx(&full[stage], 2 * bytes);  // both CTAs' copies
          tma_load_2d_cg2(sb, &tmA, kb * QT_KB, (qp.s[p] - 1) * g.Ncap + m0, fb);
          for (int pq = 0; pq < 2; pq++) {
            const int t0 = qp.t[p][2 * pq], t1 = qp.t[p][2 * pq + 1];
            if (t0 <= 0) continue;
            uint8_t* db = sb + A_TILE + pq * QT_BT;
            if (t1 > 0)
              tma_load_2d_cg2(db, &tmD, kb * QT_KB, ((rank ? t1 : t0) - 1) * g.tgp + grp * QT_TP, fb);
            else
              tma_load_2d_cg2(db, &tmD56, kb * QT_KB, (t0 - 1) * g.tgp + grp * QT_TP + (int)rank * (QT_TP / 2),
                              fb);
          }
          issued[stage] = 1;
          issued_phase[stage] = phase;
          if (++stage == QT2_STAGES) { stage = 0; phase ^= 1; }
        }
      }
      if (ok) {
        // every stage filled so far has been released by the leader's MMAs:
        // no multicast commit is still on its way to this CTA
#pragma unroll 1
        for (int i = 0; i < QT2_STAGES; i++) {
          if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag, g.err, 15, g.wait_ns)) break;
          if (++stage == QT2_STAGES) { stage = 0; phase ^= 1; }
        }
      } else if (lead) {
        const uint64_t deadline = globaltimer_ns() + WAIT_NS;
        for (int s = 0; s < QT2_STAGES; s++)
          if (issued[s]) mbar_drain_until(&full[s], issued_phase[s], deadline);
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && lead) {
      int stage = 0;
      uint32_t phase = 0;
      bool ok = true, any = false;
      for (int u = u0; u < u1 && ok; u++) {
        const int lu = u - u0;
        const int p = u % np;
        const bool second = qp.t[p][2] > 0;
        const uint32_t id01 = qp.t[p][1] > 0 ? QT2_IDESC : QT2_IDESC1;
        const uint32_t id23 = qp.t[p][3] > 0 ? QT2_IDESC : QT2_IDESC1;
        {  // both CTAs' epilogues have drained the accumulators
          const uint64_t t0 = globaltimer_ns();
          uint32_t spin = 0;
          while (!mbar_try_wait_cluster(tempty, (lu & 1) ^ 1)) {
            const bool every = (spin & 63) == 63, first = spin == 0;  // as in mbar_wait
            spin++;
            if ((every && (*abort_flag || *(volatile int*)g.err)) ||
                ((every || first) && globaltimer_ns() - t0 > g.wait_ns)) {
              *abort_flag = 1;
              atomicCAS(g.err, 0, 12);
              ok = false;
              break;
            }
          }
          if (!ok) break;
        }
        tc_fence_after();
        for (int kb = 0; kb < nk; kb++) {
          if (!mbar_wait(&full[stage], phase, abort_flag, g.err, 13, g.wait_ns)) { ok = false; break; }
          tc_fence_after();
          uint8_t* sb = smem + stage * QT2_STAGE;
          const uint64_t a = desc_sw128(sb), b01 = desc_sw128(sb + A_TILE), b23 = desc_sw128(sb + A_TILE + QT_BT);
#pragma unroll
          for (int k = 0; k < QT_KB / 32; k++) {  // K = 32 one-byte digits per MMA
            const uint64_t koff = (uint64_t)((k * 32) >> 4);
            const uint32_t acc = (kb > 0 || k > 0) ? 1u : 0u;
            mma_f8_cg2(tbase, a + koff, b01 + koff, id01, acc);
            if (second) mma_f8_cg2(tbase + 224, a + koff, b23 + koff, id23, acc);
          }
          any = true;
          mma_commit_cg2(&empty[stage], BOTH);
          if (++stage == QT2_STAGES) { stage = 0; phase ^= 1; }
        }
        if (!ok) break;
        mma_commit_cg2(tfull, BOTH);
      }
      if (!ok && any) {
        mma_commit_cg2(drain, 0x1);
        mbar_drain(drain, 0);
      }
    }
    __syncwarp();
  } else {
    // epilogue: as in quadtc_kernel, over this CTA's 128 SNP rows
    const int q = warp & 3;
    const int jl = ((warp - 2) >> 2) * 56;
    const uint32_t lead_tempty = cluster_addr(tempty, 0);
    float H[56], L[56];
    bool done = true;
    for (int u = u0; u < u1 && done;) {
      const int tile = u / np;
      const int uend = min(u1, (tile + 1) * np);
#pragma unroll
      for (int c = 0; c < 56; c++) H[c] = L[c] = 0.0f;
      for (; u < uend; u++) {
        const int lu = u - u0;
        const int p = u - tile * np;
        int ok = 1;
        if (lane == 0) ok = mbar_wait(tfull, lu & 1, abort_flag, g.err, 14, g.wait_ns) ? 1 : 0;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) { done = false; break; }
        tc_fence_after();
#pragma unroll 1
        for (int slot = 0; slot < 4; slot++) {
          const int tt = qp.t[p][slot];
          if (tt <= 0) continue;
          const float w = __int_as_float((127 - 5 * (qp.s[p] + tt)) << 23);  // 32^-(s+t)
          const uint32_t col = (uint32_t)((slot >> 1) * 224 + (slot & 1) * QT_TP + jl);
          const uint32_t ta = tbase + ((uint32_t)(q * 32) << 16) + col;
#pragma unroll
          for (int c8 = 0; c8 < 7; c8++) {
            uint32_t v[8];
            tmem_ld8(ta + c8 * 8, v);
            tmem_ld_wait();
#pragma unroll
            for (int e8 = 0; e8 < 8; e8++) {
              const float x = __fmul_rn(__uint_as_float(v[e8]), w);
              float s2, e;
              two_sum_f(H[c8 * 8 + e8], x, s2, e);
              H[c8 * 8 + e8] = s2;
              L[c8 * 8 + e8] = __fadd_rn(L[c8 * 8 + e8], e);
            }
          }
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive_cluster(lead_tempty);
      }
      if (done) quadtc2_flush(g, tile, np, (int)rank, q, lane, jl, H, L);
    }
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync();  // the leader's MMAs into both CTAs' TMEM are complete
  tc_fence_after();
  if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(512) : "memory");
  cluster_sync();
  if (*abort_flag) {
    const uint64_t t0 = globaltimer_ns();
    while (globaltimer_ns() - t0 < 100000ull) {
    }
  }
}

// GR[i + j ldg] = sum over the CTAs (or CTA pairs) that covered tile
// (i / rows, j / 112) of their partial planes, in slot order (deterministic).
__global__ void __launch_bounds__(256) quadtc_combine_kernel(int x, int t, int Ncap, int tgp, int groups, int np,
                                                             int units, int ctas, int rows,
                                                             const double* __restrict__ part,
                                                             double* __restrict__ GR, long long ldg) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)x * t) return;
  const int i = (int)(idx % x), j = (int)(idx / x);
  const int tile = (i / rows) * groups + j / QT_TP;
  const int first = qt_owner(tile * np, units, ctas), last = qt_owner(tile * np + np - 1, units, ctas);
  double v = 0.0;
  for (int c = first; c <= last; c++) v += part[(size_t)(c - first) * Ncap * tgp + i + (size_t)j * Ncap];
  GR[i + (long long)j * ldg] = v;
}

// SNP digits: CTA per SNP column i of the R2 float pairs (rows l < n):
// sigma_i = 2^aexp[i] >= 2 max_l R2, then S signed base-32 digits of R2 / sigma_i
// as E4M3 bytes at Ad[(s*Ncap + i)*Kq + l].  Digits from the exact float-pair
// value: d = rint(hi), (hi, lo) = TwoSum(hi - d, lo), times 32.
__device__ __forceinline__ uint32_t e4m3_digit(float d) {  // |d| <= 16 an integer (or one / 32): exact
  return (uint32_t)__nv_cvt_float_to_fp8(d, __NV_SATFINITE, __NV_E4M3);
}
constexpr int QD_THREADS = 256;
__global__ void __launch_bounds__(QD_THREADS) snp_digits_kernel(int n, const float2* __restrict__ A, long long lda,
                                                              int S, int Ncap, int Kq, uint8_t* __restrict__ Ad,
                                                              int* __restrict__ aexp) {
  // 4 consecutive rows per thread: two 16-byte loads, one 4-byte store per
  // digit.  The column is read twice (maximum, then digits) and the second
  // read mostly misses L2 (~1200 columns in flight).  CTAs of 1024 threads
  // (two per SM) made the second read hit L2 but ran slower, as did staging
  // the column in shared memory and taking the maxima in the GEMM epilogue.
  const int i = blockIdx.x;
  const float4* a4 = (const float4*)(A + (long long)i * lda);  // lda even: 32-byte aligned groups of 4 pairs
  const int n4 = (n + 3) >> 2;
  __shared__ float red[32];
  float m = 0.0f;
  for (int g = threadIdx.x; g < n4; g += blockDim.x) {
    const float4 u = a4[2 * g], w = a4[2 * g + 1];  // pairs 4g .. 4g+3; rows >= n read C padding (ignored)
    const int l = 4 * g;
    if (l < n) m = fmaxf(m, u.x);
    if (l + 1 < n) m = fmaxf(m, u.z);
    if (l + 2 < n) m = fmaxf(m, w.x);
    if (l + 3 < n) m = fmaxf(m, w.z);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) red[0] = v;
  }
  __syncthreads();
  m = red[0];
  int e = 0;  // 2^e >= 2 m, so that R2 / sigma <= (1 + 2^-23) / 2 and every digit is <= 16
  if (m > 0.0f) {
    int ex;
    frexpf(m, &ex);  // m = f 2^ex, f in [0.5, 1)
    e = ex + 1;
  }
  if (threadIdx.x == 0) aexp[i] = e;
  const int se = 5 - e;  // scale 2^se, a normal float for |se| <= 126
  const bool scale_ok = se >= -126 && se <= 127;
  const float sc = scale_ok ? __int_as_float((127 + se) << 23) : 0.0f;
  for (int g = threadIdx.x; g < n4; g += blockDim.x) {
    const int l = 4 * g;
    const float4 u = a4[2 * g], w = a4[2 * g + 1];
    float vh[4] = {u.x, u.z, w.x, w.z}, vl[4] = {u.y, u.w, w.y, w.w};
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (l + k >= n) vh[k] = vl[k] = 0.0f;
      vh[k] = scale_ok ? vh[k] * sc : ldexpf(vh[k], se);
      vl[k] = scale_ok ? vl[k] * sc : ldexpf(vl[k], se);
    }
    for (int sd = 0; sd < S; sd++) {
      float d[4];
#pragma unroll
      for (int k = 0; k < 4; k++) {
        d[k] = rintf(vh[k]);
        const float r = __fsub_rn(vh[k], d[k]);  // exact
        float hs, he;
        if (sd == 0) {
          two_sum_f(r, vl[k], hs, he);  // the squared pair from the GEMM need not be normalised
        } else {
          // Fast2Sum: (vh, vl) is normalised here, |vl| <= ulp(vh) / 2, and r is
          // 0 or a multiple of ulp(vh), so |r| >= |vl| and the sum is exact
          hs = __fadd_rn(r, vl[k]);
          he = __fsub_rn(vl[k], __fsub_rn(hs, r));
        }
        vh[k] = hs * 32.0f;
        vl[k] = he * 32.0f;
      }
      // two digits per conversion instruction (|d| <= 16: exact in E4M3)
      const uint32_t lo = __nv_cvt_float2_to_fp8x2(make_float2(d[0], d[1]), __NV_SATFINITE, __NV_E4M3);
      const uint32_t hi = __nv_cvt_float2_to_fp8x2(make_float2(d[2], d[3]), __NV_SATFINITE, __NV_E4M3);
      *(uint32_t*)(Ad + ((long long)sd * Ncap + i) * Kq + l) = lo | (hi << 16);  // rows n..Kq-1 receive zeros
    }
  }
}

// Trait digits: CTA per trait j of d (FP64, d[l + j*n]): tau_j = 2^dexp[j] >=
// 2 max_l d, digits of d / tau_j in FP64 at Dd[(s*QT_TP + j)*Kpad + l].
__global__ void __launch_bounds__(256) trait_digits_kernel(int n, const double* __restrict__ d, int S, int tgp,
                                                           int Kq, uint8_t* __restrict__ Dd,
                                                           int* __restrict__ dexp) {
  const int j = blockIdx.x;
  const double* c = d + (long long)j * n;
  __shared__ double red[32];
  double m = 0.0;
  for (int l = threadIdx.x; l < n; l += blockDim.x) m = fmax(m, c[l]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) red[0] = v;
  }
  __syncthreads();
  m = red[0];
  const int e = m > 0.0 ? ilogb(m) + 2 : 0;  // 2^e >= 2 m
  if (threadIdx.x == 0) dexp[j] = e;
  for (int l = threadIdx.x; l < n; l += blockDim.x) {
    double v = ldexp(c[l], 5 - e);
    for (int s = 0; s < S; s++) {
      const double dd = rint(v);  // |dd| <= 16
      Dd[((long long)s * tgp + j) * Kq + l] = (uint8_t)e4m3_digit((float)dd);
      v = (v - dd) * 32.0;
    }
  }
}

// ---------------------------------------------------------------------------
// Slicing: row r of A (K-contiguous source, element k at src[k + r*lds]) ->
// S five-bit digit slices (E4M3 bytes; odd slices hold d / 32, the weight
// of a fused pair's second slice) at A[(s*Mpad + r)*Kpad + k], scale per row.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) slice_rows_kernel(int K, int rows, const double* __restrict__ src,
                                                         long long lds, int row_off, int S, int Mpad, int Kpad,
                                                         uint8_t* __restrict__ Aout, double* __restrict__ row_scale) {
  // five-bit digits |d| <= 16, exact in E4M3 (and so is d / 32)
  constexpr int LOG_BASE = 5;
  const int r = blockIdx.x;
  if (r >= rows) return;
  const double* a = src + (long long)r * lds;
  __shared__ double red[32];
  double mx = 0.0;
  for (int k = threadIdx.x; k < K; k += blockDim.x) mx = fmax(mx, fabs(a[k]));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) red[0] = v;
  }
  __syncthreads();
  mx = red[0];
  const int e = (mx > 0.0) ? ilogb(mx) + 1 : 0;  // max * 2^-e in [0.5, 1)
  const int passes = (S + 1) / 2;
  const int R = row_off + r;
  // V (Horner over slice pairs) times 2^(e + 1 - 2 LOG_BASE passes) is the row of C
  if (threadIdx.x == 0) row_scale[R] = ldexp(1.0, e + 1 - 2 * LOG_BASE * passes);
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    double v = ldexp(a[k], LOG_BASE - 1 - e);  // |v| < 2^(LOG_BASE - 1)
#pragma unroll 1
    for (int s = 0; s < S; s++) {
      const double d = rint(v);
      const long long at = ((long long)s * Mpad + R) * Kpad + k;
      Aout[at] = (uint8_t)e4m3_digit((s & 1) ? (float)d * 0.03125f : (float)d);
      v = (v - d) * (double)(1 << LOG_BASE);
    }
  }
}

// Genotype value (FP64 or byte) as an E4M3 byte; hard calls 0/1/2 are exact.
__device__ __forceinline__ uint8_t geno_f8(unsigned char v) {
  return (uint8_t)__nv_cvt_float_to_fp8((float)v, __NV_SATFINITE, __NV_E4M3);
}
__device__ __forceinline__ uint8_t geno_f8(double v) {
  return (uint8_t)__nv_cvt_float_to_fp8((float)v, __NV_SATFINITE, __NV_E4M3);
}
__device__ __forceinline__ uint16_t geno_f8x2(double a, double b) {
  return (uint16_t)__nv_cvt_float2_to_fp8x2(make_float2((float)a, (float)b), __NV_SATFINITE, __NV_E4M3);
}

// One CTA per genotype column (no 64-bit index division per element).  FP64
// columns that start on a 16-byte boundary move as 16-byte pairs into 2-byte
// E4M3 pairs; rows K .. Kpad-1 of G stay zero from its allocation.
template <typename T>
__global__ void __launch_bounds__(256) genotypes_f8_kernel(int K, int cols, const T* __restrict__ src,
                                                             long long lds, uint8_t* __restrict__ G,
                                                             int Kpad) {
  const long long c = blockIdx.x;
  const T* col = src + c * lds;
  uint8_t* g = G + c * Kpad;
  if constexpr (sizeof(T) == 8) {
    if (((uintptr_t)col & 15) == 0) {
      const double2* col2 = (const double2*)col;
      uint16_t* g2 = (uint16_t*)g;
      const int K2 = K >> 1;
      for (int k = threadIdx.x; k < K2; k += blockDim.x) {
        const double2 v = col2[k];
        g2[k] = geno_f8x2(v.x, v.y);
      }
      if ((K & 1) && threadIdx.x == 0) g[K - 1] = geno_f8(col[K - 1]);
      return;
    }
  }
  for (int k = threadIdx.x; k < K; k += blockDim.x) g[k] = geno_f8(col[k]);
}

// 2-bit packed genotype columns (SNP-major PLINK .bed body: ceil(K/4) bytes a
// column, codes 00 -> 2, 10 -> 1, 11 -> 0, 01 = missing) straight to the E4M3
// operand, four individuals per thread and step; a missing call sets the
// status word (FGLSGPU_EINVAL, individual, SNP) and enters as 0.
__global__ void __launch_bounds__(256) genotypes_packed_f8_kernel(int K, const uint8_t* __restrict__ src,
                                                                    uint8_t* __restrict__ G, int Kpad, int wXR,
                                                                    DevStatus* st, long long snp_base) {
  const long long c = blockIdx.x;
  const int bpc = (K + 3) / 4;
  const uint8_t* col = src + c * bpc;
  uint8_t* g = G + c * Kpad;
  const uint32_t e0 = geno_f8((unsigned char)0), e1 = geno_f8((unsigned char)1), e2 = geno_f8((unsigned char)2);
  for (int b = threadIdx.x; b < bpc; b += blockDim.x) {
    const uint32_t v = col[b];
    uint32_t w = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const uint32_t code = (v >> (2 * i)) & 3u;
      if (code == 1u && 4 * b + i < K) set_status(st, FGLSGPU_EINVAL, 4 * b + i, snp_base + c / wXR);
      w |= (code == 0u ? e2 : code == 2u ? e1 : e0) << (8 * i);
    }
    if (4 * b + 3 < K) {
      *(uint32_t*)(g + 4 * b) = w;  // Kpad is a multiple of 128: 4-byte aligned
    } else {
      for (int i = 0; 4 * b + i < K; i++) g[4 * b + i] = (uint8_t)(w >> (8 * i));
    }
  }
}

__global__ void eye_kernel(int n, double* A) {
  const long long total = (long long)n * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x)
    A[e] = (e % n == e / n) ? 1.0 : 0.0;
}

// B = A^T for n x n column-major, 32 x 32 tiles through shared memory
__global__ void transpose_kernel(int n, const double* __restrict__ A, double* __restrict__ B) {
  __shared__ double tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int r = bx + threadIdx.x, c = by + j;
    if (r < n && c < n) tile[j][threadIdx.x] = A[r + (long long)c * n];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int r = by + threadIdx.x, c = bx + j;
    if (r < n && c < n) B[r + (long long)c * n] = tile[threadIdx.x][j];
  }
}

// ---------------------------------------------------------------------------
// Weights of the quadratic Gram terms (fgls_selfgram.cu) as float pairs.
// ---------------------------------------------------------------------------
// unit weights (chol: |x~|^2)
// D (FP64 n x t) -> interleaved float pairs, and dmax[j] = max_l hi
__global__ void split_pairs_kernel(int n, int t, const double* __restrict__ d, float2* __restrict__ D,
                                   float* __restrict__ dmax) {
  const int j = blockIdx.x;
  float m = 0.0f;
  for (int l = threadIdx.x; l < n; l += blockDim.x) {
    const double v = d[l + (long long)j * n];
    const float h = (float)v;
    D[l + (long long)j * n] = make_float2(h, (float)(v - (double)h));
    m = fmaxf(m, h);
  }
  __shared__ float red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) m = fmaxf(m, red[w]);
    m = fmaxf(m, red[0]);
    dmax[j] = m;
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn get_encoder() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

// 2D tensor map of the split GEMM's E4M3 operands (A slices or genotypes):
// K innermost in rows of K bytes, box {GBK, box_rows}, 128B swizzle.
cudaError_t make_map(CUtensorMap* m, const void* base, long long K, long long rows, int box_rows) {
  EncodeTiledFn enc = get_encoder();
  if (!enc) return cudaErrorNotSupported;
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)K};
  cuuint32_t box[2] = {(cuuint32_t)GBK, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}
// 2D byte tensor map (FP8 digits), K innermost in rows of K bytes, box
// {QT_KB, box_rows}, 128B swizzle.
cudaError_t make_map_u8(CUtensorMap* m, const void* base, long long K, long long rows, int box_rows) {
  EncodeTiledFn enc = get_encoder();
  if (!enc) return cudaErrorNotSupported;
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)K};
  cuuint32_t box[2] = {(cuuint32_t)QT_KB, (cuuint32_t)box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims, strides, box, es,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

int grid_for(long long total) { return (int)std::min<long long>((total + 255) / 256, 152LL * 32); }

// CTAs of a persistent split-GEMM launch over `tiles` tiles: one per SM of
// the current device (each CTA holds all 512 TMEM columns and most of the
// shared memory), fewer when there are fewer tiles.
int persistent_grid(int tiles) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
      cudaSuccess || sms <= 0)
    sms = 1;
  return std::max(1, std::min(tiles, sms));
}

// Clusters of the 2-SM split GEMM (two CTAs, one per SM) that the current
// device holds at once, queried once per device; 0 if none can launch.
int pair_clusters() {
  static std::atomic<int> known[64];  // clusters + 1; 0: not queried yet
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  const int v = known[dev].load(std::memory_order_relaxed);
  if (v > 0) return v - 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2);
  cfg.blockDim = dim3(THREADS);
  cfg.dynamicSmemBytes = p2::SMEM;
  int n = 0;
  if (cudaFuncSetAttribute(ozaki_gemm2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, p2::SMEM) !=
          cudaSuccess ||
      cudaOccupancyMaxActiveClusters(&n, (void*)ozaki_gemm2_kernel, &cfg) != cudaSuccess) {
    (void)cudaGetLastError();
    n = 0;
  }
  known[dev].store(n + 1, std::memory_order_relaxed);
  return n;
}

}  // namespace oz

using namespace oz;

struct OzakiPlan {
  int n = 0, t = 0, wXL = 0, wXR = 0, x_b = 0, S = 0;
  int eigen = 0;
  int nU = 0;           // U rows appended below the n rows of Z^T / L^-1
  int M = 0, Mpad = 0;  // rows of A
  int Kpad = 0, Ncap = 0;
  uint8_t* A = nullptr;         // S x Mpad x Kpad E4M3 digit slices
  uint8_t* G = nullptr;         // Ncap x Kpad E4M3 genotypes
  double* scale = nullptr;      // Mpad
  double* C = nullptr;          // Mpad x Ncap (ld Mpad)
  double* U = nullptr;          // n x nU
  float2* D = nullptr;          // n x t weights as float pairs (eigen d_j; chol: ones)
  float* dmax = nullptr;        // t: max_l of the high part of D[:, j]
  float* amax = nullptr;        // Ncap: per-SNP max_l of the high part of R^2
  float2* part = nullptr;       // quadratic Gram partial sums over row ranges
  int sms = 0;                  // SM count of the device
  // tensor-core quadratic Gram (eigen, 33 <= t <= 112): digit operands
  bool tq = false;
  int SQ = 11;                    // digits per side built (trait digits); pairs with s + t <= SQ_run + 1
  int SQ_run = 11;                // digits per side in use (1..SQ)
  int Kq = 0;                     // digit row length (bytes): n rounded up to QT_KB
  int tgp = 0;                    // trait rows per digit plane (multiple of QT_TP)
  double* qpart = nullptr;        // QT_SLOTS x Ncap x tgp partial planes of the tensor-core Gram
  uint8_t* Adig = nullptr;        // SQ x Ncap x Kq SNP digits (E4M3)
  uint8_t* Ddig = nullptr;        // SQ x tgp x Kq trait digits (E4M3)
  int *aexp = nullptr, *dexp = nullptr;
  CUtensorMap mapAd, mapDd;
  CUtensorMap mapDd56;  // trait digits in 56-row boxes (2-SM quadratic Gram, one-digit slot pairs)
  QuadPasses qp;
  double* Linv = nullptr;       // chol: n x n, L^-1
  double* LinvT = nullptr;      // chol: n x n, (L^-1)^T (rows of L^-1 contiguous)
  float2* sqsum = nullptr;      // chol: Mpad/32 x Ncap sums of R^2 over 32-row groups (ld Ncap)
  int* err = nullptr;
  CUtensorMap mapA, mapB;
  CUtensorMap mapBh;                // genotypes in 128-row boxes (2-SM kernel); valid when has_mapBh
  bool has_mapBh = false;
  bool maps = false;
  int sub = 0;                      // SNPs per pipelined sub-block (multiple of BN)
  int S_run = 0;                    // slices the GEMM uses: the first S_run of the S built
  double* scale_run = nullptr;      // Mpad row scales for S_run slices (when S_run < S)
  unsigned long long wait_ns = WAIT_NS;  // limit of one wait in the tcgen05 kernels
};

// Passes of the tensor-core quadratic Gram for k digits a side: one SNP
// digit s with up to four trait digits t, s + t <= k + 1.  Round-to-nearest
// base-32 digits, so the first k of the SQ digits built are the k-digit cut.
static void quad_passes(OzakiPlan* p, int k) {
  p->SQ_run = k;
  memset(&p->qp, 0, sizeof(p->qp));
  for (int sd = 1; sd <= k; sd++)
    for (int t0 = 1; t0 <= k + 1 - sd; t0 += 4) {
      const int q0 = p->qp.n++;
      p->qp.s[q0] = (signed char)sd;
      for (int q = 0; q < 4; q++) p->qp.t[q0][q] = (signed char)(t0 + q <= k + 1 - sd ? t0 + q : 0);
    }
}

cudaError_t ozaki_create(OzakiPlan** out, int n, int t, int wXL, int wXR, int x_b, int slices, int eigen) {
  *out = nullptr;
  if (wXR != 1) return cudaErrorNotSupported;  // split path: one column per SNP
  if (n > FUSED_KMAX) return cudaErrorNotSupported;  // exactness bound of the FP32 accumulation
  OzakiPlan* p = new OzakiPlan();
  p->n = n;
  p->t = t;
  p->wXL = wXL;
  p->wXR = wXR;
  p->x_b = x_b;
  p->S = slices > 0 ? std::min(slices, MAX_SLICES) : DEFAULT_SLICES;
  p->S_run = p->S;
  p->eigen = eigen;
  p->nU = eigen ? t * (1 + wXL) : (1 + wXL);
  p->M = n + p->nU;
  p->Mpad = (p->M + BM - 1) / BM * BM;
  p->Kpad = (n + KALIGN - 1) / KALIGN * KALIGN;
  p->Ncap = (x_b + BN - 1) / BN * BN;
  cudaError_t r = cudaSuccess;
  auto chk = [&](cudaError_t e) {
    if (r == cudaSuccess) r = e;
  };
  chk(cudaMalloc(&p->A, (size_t)p->S * p->Mpad * p->Kpad));
  chk(cudaMalloc(&p->G, (size_t)p->Ncap * p->Kpad));
  chk(cudaMalloc(&p->scale, sizeof(double) * p->Mpad));
  chk(cudaMalloc(&p->scale_run, sizeof(double) * p->Mpad));
  chk(cudaMalloc(&p->C, sizeof(double) * (size_t)p->Mpad * p->Ncap));
  chk(cudaMalloc(&p->U, sizeof(double) * (size_t)n * p->nU));
  chk(cudaMalloc(&p->D, sizeof(float2) * (size_t)n * t));
  chk(cudaMalloc(&p->dmax, sizeof(float) * (size_t)t));
  chk(cudaMalloc(&p->amax, sizeof(float) * (size_t)p->Ncap));
  chk(cudaMalloc(&p->part, sizeof(float2) * quad_gram_part_elems(p->Ncap, t)));
  {
    int dev = 0;
    chk(cudaGetDevice(&dev));
    chk(cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, dev));
  }
  chk(cudaMalloc(&p->err, 3 * sizeof(int)));  // [wait error word, GEMM tile counter, finished CTAs]
  if (!eigen) chk(cudaMalloc(&p->Linv, sizeof(double) * (size_t)n * n));
  if (!eigen) chk(cudaMalloc(&p->LinvT, sizeof(double) * (size_t)n * n));
  if (!eigen) chk(cudaMalloc(&p->sqsum, sizeof(float2) * (size_t)(p->Mpad / 32) * p->Ncap));
  if (r == cudaSuccess) chk(cudaMemset(p->A, 0, (size_t)p->S * p->Mpad * p->Kpad));
  if (r == cudaSuccess) chk(cudaMemset(p->G, 0, (size_t)p->Ncap * p->Kpad));
  if (r == cudaSuccess) chk(cudaMemset(p->scale, 0, sizeof(double) * p->Mpad));
  if (r == cudaSuccess) chk(cudaMemset(p->err, 0, 3 * sizeof(int)));
  if (r == cudaSuccess) chk(make_map(&p->mapA, p->A, p->Kpad, (long long)p->S * p->Mpad, BM));
  if (r == cudaSuccess) chk(make_map(&p->mapB, p->G, p->Kpad, p->Ncap, BN));
  if (r == cudaSuccess) chk(make_map(&p->mapBh, p->G, p->Kpad, p->Ncap, BN / 2));
  if (r == cudaSuccess) p->has_mapBh = true;
  if (r == cudaSuccess) chk(cudaFuncSetAttribute(ozaki_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 SMEM_BYTES));
  p->sub = p->Ncap;  // one GEMM launch per block
  {
    const char* qe = getenv("FGLS_QUAD_TC");
    p->tq = eigen && t >= 33 && !(qe && qe[0] == '0');
  }
  if (p->tq && r == cudaSuccess) {
    p->tgp = (t + QT_TP - 1) / QT_TP * QT_TP;
    p->Kq = (n + QT_KB - 1) / QT_KB * QT_KB;
    const size_t na = (size_t)p->SQ * p->Ncap * p->Kq, nd = (size_t)p->SQ * p->tgp * p->Kq;
    chk(cudaMalloc(&p->Adig, na));
    chk(cudaMalloc(&p->Ddig, nd));
    chk(cudaMalloc(&p->aexp, sizeof(int) * p->Ncap));
    chk(cudaMalloc(&p->dexp, sizeof(int) * p->tgp));
    chk(cudaMalloc(&p->qpart, sizeof(double) * QT_SLOTS * (size_t)p->Ncap * p->tgp));
    if (r == cudaSuccess) chk(cudaMemset(p->Adig, 0, na));
    if (r == cudaSuccess) chk(cudaMemset(p->Ddig, 0, nd));
    if (r == cudaSuccess) chk(cudaMemset(p->dexp, 0, sizeof(int) * p->tgp));
    if (r == cudaSuccess) chk(make_map_u8(&p->mapAd, p->Adig, p->Kq, (long long)p->SQ * p->Ncap, BM));
    if (r == cudaSuccess) chk(make_map_u8(&p->mapDd, p->Ddig, p->Kq, (long long)p->SQ * p->tgp, QT_TP));
    if (r == cudaSuccess) chk(make_map_u8(&p->mapDd56, p->Ddig, p->Kq, (long long)p->SQ * p->tgp, QT_TP / 2));
    if (r == cudaSuccess)
      chk(cudaFuncSetAttribute(quadtc2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, QT2_SMEM));
    if (r == cudaSuccess)
      chk(cudaFuncSetAttribute(quadtc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, QT_SMEM));
    quad_passes(p, p->SQ);
  }
  // the memsets above ran on the legacy default stream, which does not order
  // against the caller's non-blocking streams: finish them before any launch
  if (r == cudaSuccess) chk(cudaDeviceSynchronize());
  if (r != cudaSuccess) {
    ozaki_destroy(p);
    return r;
  }
  p->maps = true;
  *out = p;
  return cudaSuccess;
}

void ozaki_destroy(OzakiPlan* p) {
  if (!p) return;
  void* ptrs[] = {p->A,    p->G,     p->scale, p->scale_run, p->C, p->U, p->D,    p->dmax, p->amax,
                  p->part, p->Linv,  p->LinvT, p->err,   p->Adig, p->Ddig, p->aexp, p->dexp, p->qpart,
                  p->sqsum};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  delete p;
}

namespace {

cudaError_t slice_operands(OzakiPlan* p, cudaStream_t s, const double* top, long long ldtop, int toprows) {
  // rows [0, toprows) from `top` (row r contiguous at top + r*ldtop), rows
  // [n, n + nU) from the columns of U.
  slice_rows_kernel<<<toprows, 256, 0, s>>>(p->n, toprows, top, ldtop, 0, p->S, p->Mpad, p->Kpad, p->A,
                                                    p->scale);
  note_launch();
  slice_rows_kernel<<<p->nU, 256, 0, s>>>(p->n, p->nU, p->U, p->n, p->n, p->S, p->Mpad, p->Kpad, p->A,
                                                  p->scale);
  note_launch();
  return cudaGetLastError();
}

cudaError_t run_gemm(OzakiPlan* p, cudaStream_t s, int col0, int x, int tri_rows, int sq_rows) {
  GemmArgs g;
  g.M = p->M;
  g.Mpad = p->Mpad;
  g.N = x;
  g.col0 = col0;
  g.sq_rows = sq_rows;
  g.Kpad = p->Kpad;
  // slices in use: S_run (1..S) once set, else all S built; rescaled row
  // scales exist only in plans made by ozaki_create
  const int S_run = (p->S_run > 0 && p->S_run <= p->S && p->scale_run) ? p->S_run : p->S;
  g.S = S_run;
  g.tiles_m = p->Mpad / BM;
  g.tiles_n = (x + BN - 1) / BN;
  g.tri_rows = tri_rows;
  g.row_scale = S_run == p->S ? p->scale : p->scale_run;
  g.C = p->C;
  g.ldc = p->Mpad;
  g.err = p->err;
  g.wait_ns = p->wait_ns;
  // chol (unit weights): the GEMM sums the squares of rows [0, n) per 32-row group
  g.sqsum = sq_rows > 0 ? p->sqsum : nullptr;
  g.ldq = p->Ncap;
  // the 2-SM kernel (pairs of row tiles share each genotype tile across two
  // SMs; the triangular L^-1 operand's pairs longest first from the counter),
  // else one CTA per tile
  const int pairs = ((g.tiles_m + 1) / 2) * g.tiles_n;
  const int clusters = p->has_mapBh ? pair_clusters() : 0;
  if (clusters > 0)
    ozaki_gemm2_kernel<<<2 * std::min(pairs, clusters), THREADS, p2::SMEM, s>>>(p->mapA, p->mapBh, g, p->err + 1);
  else
    ozaki_gemm_kernel<<<persistent_grid(g.tiles_m * g.tiles_n), THREADS, SMEM_BYTES, s>>>(p->mapA, p->mapB, g,
                                                                                          p->err + 1);
  note_launch();
  return cudaGetLastError();
}

template <typename T>
cudaError_t load_genotypes(OzakiPlan* p, cudaStream_t s, const T* X, int x) {
  if (x <= 0) return cudaSuccess;
  genotypes_f8_kernel<T><<<x, 256, 0, s>>>(p->n, x, X, p->n, p->G, p->Kpad);
  note_launch();
  return cudaGetLastError();
}

cudaError_t load_genotypes_packed(OzakiPlan* p, cudaStream_t s, const uint8_t* X2, int x, DevStatus* st,
                                  long long snp_base) {
  if (x <= 0) return cudaSuccess;
  genotypes_packed_f8_kernel<<<x, 256, 0, s>>>(p->n, X2, p->G, p->Kpad, p->wXR, st, snp_base);
  note_launch();
  return cudaGetLastError();
}

cudaError_t selfgram(OzakiPlan* p, cudaStream_t s, int col0, int xq, int t, double* GR, long long ldg) {
  if (p->sqsum) return sqsum_combine(s, p->n, xq, p->sqsum + col0, p->Ncap, GR + col0);
  const float2* A = (const float2*)(p->C + (long long)col0 * p->Mpad);
  if (!p->tq || col0 != 0)
    return quad_gram(s, p->n, xq, t, A, p->Mpad, p->amax + col0, p->D, p->n, p->dmax, p->part, GR + col0, ldg,
                     p->sms);
  snp_digits_kernel<<<xq, QD_THREADS, 0, s>>>(p->n, A, p->Mpad, p->SQ_run, p->Ncap, p->Kq, p->Adig, p->aexp);
  note_launch();
  QuadArgs g;
  g.x = xq;
  g.t = t;
  g.tgp = p->tgp;
  g.Ncap = p->Ncap;
  g.Kq = p->Kq;
  g.groups = p->tgp / QT_TP;
  g.aexp = p->aexp;
  g.dexp = p->dexp;
  g.part = p->qpart;
  g.err = p->err;
  g.wait_ns = p->wait_ns;
  // 2-SM: tiles of 256 SNP rows over CTA pairs; else 128 rows per CTA.
  // Persistent CTAs (pairs), at most one per SM, each with >= half a tile's
  // passes (so a tile spans at most QT_SLOTS of them)
  const int clusters = pair_clusters();
  const int rows = clusters > 0 ? 2 * BM : BM;
  g.units = (xq + rows - 1) / rows * g.groups * p->qp.n;
  const int cap = clusters > 0 ? clusters : p->sms;
  const int ctas = std::max(1, std::min(cap, g.units / ((p->qp.n + 1) / 2)));
  if (clusters > 0)
    quadtc2_kernel<<<2 * ctas, THREADS, QT2_SMEM, s>>>(p->mapAd, p->mapDd, p->mapDd56, p->qp, g);
  else
    quadtc_kernel<<<ctas, THREADS, QT_SMEM, s>>>(p->mapAd, p->mapDd, p->qp, g);
  note_launch();
  const long long cells = (long long)xq * t;
  quadtc_combine_kernel<<<(int)((cells + 255) / 256), 256, 0, s>>>(xq, t, p->Ncap, p->tgp, g.groups, p->qp.n,
                                                                    g.units, ctas, rows, p->qpart, GR, ldg);
  note_launch();
  return cudaGetLastError();
}

}  // namespace

cudaError_t ozaki_set_eigen(OzakiPlan* p, cudaStream_t s, const double* Z, const double* AYL, const double* dinv) {
  // U = Z * AYL (FP64, once per problem): x~^T y~_j = x^T U[:, j] etc.
  FGLS_CUDA_TRY(dgemm(s, false, false, p->n, p->nU, p->n, 1.0, Z, p->n, AYL, p->n, 0.0, p->U, p->n));
  // rows of Z^T are the columns of Z (contiguous): ld n
  FGLS_CUDA_TRY(slice_operands(p, s, Z, p->n, p->n));
  split_pairs_kernel<<<p->t, 256, 0, s>>>(p->n, p->t, dinv, p->D, p->dmax);
  note_launch();
  if (p->tq) {
    trait_digits_kernel<<<p->t, 256, 0, s>>>(p->n, dinv, p->SQ, p->tgp, p->Kq, p->Ddig, p->dexp);
    note_launch();
  }
  return cudaGetLastError();
}

// L^-1 (lower, FP64) by blocked TRSM on the identity.  Column panel
// [c0, c0 + w) of L^-1 is zero above row c0, so each panel solves only the
// trailing system L[c0:, c0:] X = I[c0:, c0:c0+w]: n^3/3 flops instead of n^3.
cudaError_t lower_inverse(cudaStream_t s, int n, const double* L, double* Linv) {
  eye_kernel<<<grid_for((long long)n * n), 256, 0, s>>>(n, Linv);
  note_launch();
  constexpr int W = 512;
  for (int c0 = 0; c0 < n; c0 += W) {
    const int w = std::min(W, n - c0);
    const long long off = (long long)c0 + (long long)c0 * n;
    FGLS_CUDA_TRY(dtrsm_llnn(s, n - c0, w, L + off, n, Linv + off, n));
  }
  return cudaGetLastError();
}

cudaError_t ozaki_set_chol(OzakiPlan* p, cudaStream_t s, const double* L, const double* WY) {
  const int n = p->n;
  // L^-1 by the FP64 blocked TRSM on the identity, then U = L^-T [y~ | XL~]
  FGLS_CUDA_TRY(lower_inverse(s, n, L, p->Linv));
  FGLS_CUDA_TRY(dgemm(s, true, false, n, p->nU, n, 1.0, p->Linv, n, WY, n, 0.0, p->U, n));
  // rows of L^-1 contiguous: transpose, then slice
  dim3 tg((n + 31) / 32, (n + 31) / 32);
  transpose_kernel<<<tg, dim3(32, 8), 0, s>>>(n, p->Linv, p->LinvT);
  note_launch();
  FGLS_CUDA_TRY(slice_operands(p, s, p->LinvT, n, n));
  return cudaGetLastError();
}

cudaError_t ozaki_block(OzakiPlan* p, cudaStream_t s, const GenoBlock& X, int x, double* GR, StageHook hook,
                        void* ctx) {
  const int t = p->eigen ? p->t : 1;
  const int tri = p->eigen ? 0 : p->n;
  auto mark = [&](int cls, int begin, cudaStream_t st) {
    if (hook) hook(ctx, cls, begin, st);
  };
  mark(FGLSGPU_PROF_GENOTYPES, 1, s);
  FGLS_CUDA_TRY(X.packed ? load_genotypes_packed(p, s, X.packed, x, X.st, X.snp_base)
                : X.u8     ? load_genotypes<unsigned char>(p, s, X.u8, x)
                           : load_genotypes<double>(p, s, X.f64, x));
  mark(FGLSGPU_PROF_GENOTYPES, 0, s);
  for (int x0 = 0; x0 < x; x0 += p->sub) {
    const int xq = std::min(p->sub, x - x0);
    mark(FGLSGPU_PROF_SPLIT_GEMM, 1, s);
    FGLS_CUDA_TRY(run_gemm(p, s, x0, xq, tri, p->n));
    mark(FGLSGPU_PROF_SPLIT_GEMM, 0, s);
    mark(FGLSGPU_PROF_SELFGRAM, 1, s);
    FGLS_CUDA_TRY(selfgram(p, s, x0, xq, t, GR, x));
    mark(FGLSGPU_PROF_SELFGRAM, 0, s);
  }
  return cudaSuccess;
}

double ozaki_flops_per_snp(const OzakiPlan* p) {
  // sliced tensor-core MMA operations actually issued per genotype column
  // (chol: the zero upper part of L^-1 is skipped by 64-column K blocks)
  double rows_k = (double)p->M * p->n;
  if (!p->eigen) rows_k = (double)p->nU * p->n + 0.5 * (double)p->n * p->n;
  return 2.0 * p->S_run * rows_k;
}

// Gram operand view of the last block's output: rows [n, n + nU) of C.
const double* ozaki_gram_rows(const OzakiPlan* p, long long* ld) {
  *ld = p->Mpad;
  return p->C + p->n;
}

int* ozaki_error_word(OzakiPlan* p) { return p->err; }

void ozaki_set_wait_limit(OzakiPlan* p, unsigned long long ns) { p->wait_ns = ns ? ns : WAIT_NS; }

// ---------------------------------------------------------------------------
// Batched cohorts: the split operand of one chol problem into caller buffers,
// grouped genotype conversion and the grouped split GEMM.
// ---------------------------------------------------------------------------
int split_rows_padded(int rows) { return (rows + BM - 1) / BM * BM; }
int split_k_padded(int n) { return (n + KALIGN - 1) / KALIGN * KALIGN; }
int split_cols_padded(int x) { return (x + BN - 1) / BN * BN; }

cudaError_t split_chol_operand(cudaStream_t s, int n, int wXL, const double* L, const double* WY, int S, int Mpad,
                               int Kpad, uint8_t* A, double* scale, double* Linv, double* LinvT, double* U) {
  const int nU = 1 + wXL;
  FGLS_CUDA_TRY(lower_inverse(s, n, L, Linv));
  FGLS_CUDA_TRY(dgemm(s, true, false, n, nU, n, 1.0, Linv, n, WY, n, 0.0, U, n));
  dim3 tg((n + 31) / 32, (n + 31) / 32);
  transpose_kernel<<<tg, dim3(32, 8), 0, s>>>(n, Linv, LinvT);
  note_launch();
  slice_rows_kernel<<<n, 256, 0, s>>>(n, n, LinvT, n, 0, S, Mpad, Kpad, A, scale);
  note_launch();
  slice_rows_kernel<<<nU, 256, 0, s>>>(n, nU, U, n, n, S, Mpad, Kpad, A, scale);
  note_launch();
  return cudaGetLastError();
}

namespace {
// per-row scale of an S-slice operand from that of the same digits cut at
// S_built slices: 2^(e + 1 - 10 passes) depends on the pass count only
__global__ void rescale_rows_kernel(int rows, const double* __restrict__ built, int bits, double* __restrict__ out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < rows) out[r] = ldexp(built[r], bits);
}

template <typename T>
__global__ void grouped_genotypes_kernel(const GenoCohort* __restrict__ gc, const StepCohort* __restrict__ sc) {
  const int c = blockIdx.y;
  const int x = sc[c].x, n = gc[c].n, Kpad = gc[c].Kpad;
  const T* __restrict__ src = (const T*)sc[c].X;
  uint8_t* __restrict__ G = gc[c].G;
  // columns strided over the CTAs of this cohort, rows over the threads; u8
  // columns that start on a 4-byte boundary move 4 calls per load (Kpad is a
  // multiple of 128, so the E4M3 column is 4-byte aligned)
  for (int col = blockIdx.x; col < x; col += gridDim.x) {
    const T* s = src + (long long)col * n;
    uint8_t* g = G + (long long)col * Kpad;
    if constexpr (sizeof(T) == 1) {
      if (((uintptr_t)s & 3) == 0) {
        const int n4 = n >> 2;
        for (int q = threadIdx.x; q < n4; q += blockDim.x) {
          const uchar4 v = ((const uchar4*)s)[q];
          ((uint32_t*)g)[q] = (uint32_t)geno_f8(v.x) | ((uint32_t)geno_f8(v.y) << 8) |
                              ((uint32_t)geno_f8(v.z) << 16) | ((uint32_t)geno_f8(v.w) << 24);
        }
        for (int k = 4 * n4 + threadIdx.x; k < n; k += blockDim.x) g[k] = geno_f8(s[k]);
        continue;
      }
    }
    for (int k = threadIdx.x; k < n; k += blockDim.x) g[k] = geno_f8(s[k]);
  }
}
}  // namespace

cudaError_t split_rescale_rows(cudaStream_t s, int rows, const double* built_scale, int S_built, int S,
                               double* scale) {
  const int dpass = (S_built + 1) / 2 - (S + 1) / 2;
  rescale_rows_kernel<<<(rows + 255) / 256, 256, 0, s>>>(rows, built_scale, 10 * dpass, scale);  // 10 bits a slice pair
  note_launch();
  return cudaGetLastError();
}

cudaError_t ozaki_set_run_slices(OzakiPlan* p, cudaStream_t s, int S) {
  S = std::max(1, std::min(S, p->S));
  p->S_run = S;
  if (S == p->S) return cudaSuccess;
  // the first S five-bit digits of each row are its S-digit cut; with fewer
  // slice pairs the Horner sum is 2^(10 (passes - passes_run)) smaller
  const int dpass = (p->S + 1) / 2 - (S + 1) / 2;
  rescale_rows_kernel<<<(p->Mpad + 255) / 256, 256, 0, s>>>(p->Mpad, p->scale, 10 * dpass, p->scale_run);
  note_launch();
  return cudaGetLastError();
}

int ozaki_quad_digits(const OzakiPlan* p) { return p && p->tq ? p->SQ_run : 0; }

void ozaki_set_quad_digits(OzakiPlan* p, int k) {
  if (!p || !p->tq) return;
  quad_passes(p, std::max(1, std::min(k, p->SQ)));
}

int ozaki_slices(const OzakiPlan* p, int* built) {
  if (built) *built = p->S;
  return p->S_run;
}

cudaError_t grouped_genotypes(cudaStream_t s, const GenoCohort* dgc, const StepCohort* dsc, int cohorts, bool u8) {
  dim3 grid(256, cohorts);
  if (u8)
    grouped_genotypes_kernel<unsigned char><<<grid, 256, 0, s>>>(dgc, dsc);
  else
    grouped_genotypes_kernel<double><<<grid, 256, 0, s>>>(dgc, dsc);
  note_launch();
  return cudaGetLastError();
}

struct GroupedGemm {
  int ntiles = 0, nprob = 0;
  bool pair = false;  // 2-SM kernel over row-tile pairs
  GroupedTile* tiles = nullptr;
  GroupedProblem* probs = nullptr;
  CUtensorMap* maps = nullptr;
  int* counter = nullptr;  // tile counter and finished CTAs of the persistent launch
};

cudaError_t grouped_gemm_create(GroupedGemm** out, const GroupedGemmDesc* d, int count, int x_b, int* err,
                                bool want_pair) {
  *out = nullptr;
  const bool pair = want_pair && pair_clusters() > 0;
  std::vector<GroupedProblem> probs(count);
  std::vector<CUtensorMap> maps(2 * (size_t)count);
  std::vector<int> order(count);
  std::vector<long long> work(count);
  for (int i = 0; i < count; i++) {
    GemmArgs& g = probs[i].g;
    g.M = d[i].M;
    g.Mpad = d[i].Mpad;
    g.N = x_b;
    g.Kpad = d[i].Kpad;
    g.S = d[i].S;
    g.tiles_m = d[i].Mpad / BM;
    g.tiles_n = (x_b + BN - 1) / BN;
    g.tri_rows = d[i].tri_rows;
    g.row_scale = d[i].scale;
    g.C = d[i].C;
    g.ldc = d[i].Mpad;
    g.col0 = 0;
    g.sq_rows = d[i].sq_rows;
    g.sqsum = d[i].Q;
    g.ldq = d[i].ldq;
    g.err = err;
    g.wait_ns = WAIT_NS;
    probs[i].cohort = d[i].cohort;
    probs[i].pad = 0;
    FGLS_CUDA_TRY(make_map(&maps[2 * i], d[i].A, d[i].Kpad, (long long)d[i].S_alloc * d[i].Mpad, BM));
    FGLS_CUDA_TRY(make_map(&maps[2 * i + 1], d[i].G, d[i].Kpad, d[i].Ncap, pair ? BN / 2 : BN));
    order[i] = i;
    work[i] = (long long)g.tiles_m * g.Kpad;
  }
  // longest problems first, so that the short ones fill the last waves
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work[a] > work[b]; });
  std::vector<GroupedTile> tiles;
  for (int i : order) {
    const GemmArgs& g = probs[i].g;
    // rows in units of tiles, or of tile pairs for the 2-SM kernel (an odd
    // last pair's second tile lies past the operand and is never written)
    const int units = pair ? (g.tiles_m + 1) / 2 : g.tiles_m;
    const int gm = pair ? GROUP_M / 2 : GROUP_M;
    for (int first = 0; first < units; first += gm) {
      const int gsz = std::min(gm, units - first);
      for (int nt = 0; nt < g.tiles_n; nt++)
        for (int m = 0; m < gsz; m++) tiles.push_back(GroupedTile{i, first + m, nt, 0});
    }
  }
  GroupedGemm* gg = new GroupedGemm();
  gg->pair = pair;
  gg->ntiles = (int)tiles.size();
  gg->nprob = count;
  cudaError_t r = cudaSuccess;
  auto chk = [&](cudaError_t e) {
    if (r == cudaSuccess) r = e;
  };
  chk(cudaMalloc(&gg->tiles, sizeof(GroupedTile) * tiles.size()));
  chk(cudaMalloc(&gg->probs, sizeof(GroupedProblem) * probs.size()));
  chk(cudaMalloc(&gg->maps, sizeof(CUtensorMap) * maps.size()));  // 256-byte aligned: >= the 64 a map needs
  chk(cudaMalloc(&gg->counter, 2 * sizeof(int)));
  if (r == cudaSuccess) chk(cudaMemset(gg->counter, 0, 2 * sizeof(int)));
  if (r == cudaSuccess) chk(cudaDeviceSynchronize());  // the memset is on the legacy default stream
  if (r == cudaSuccess)
    chk(cudaMemcpy(gg->tiles, tiles.data(), sizeof(GroupedTile) * tiles.size(), cudaMemcpyHostToDevice));
  if (r == cudaSuccess)
    chk(cudaMemcpy(gg->probs, probs.data(), sizeof(GroupedProblem) * probs.size(), cudaMemcpyHostToDevice));
  if (r == cudaSuccess)
    chk(cudaMemcpy(gg->maps, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice));
  if (r == cudaSuccess)
    chk(cudaFuncSetAttribute(ozaki_grouped_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             SMEM_BYTES));
  if (r == cudaSuccess && pair)
    chk(cudaFuncSetAttribute(ozaki_grouped_gemm2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, p2::SMEM));
  if (r != cudaSuccess) {
    grouped_gemm_destroy(gg);
    return r;
  }
  *out = gg;
  return cudaSuccess;
}

cudaError_t grouped_gemm_run(GroupedGemm* gg, cudaStream_t s, const int* dcols) {
  if (gg->ntiles == 0) return cudaSuccess;
  if (gg->pair)
    ozaki_grouped_gemm2_kernel<<<2 * std::min(gg->ntiles, pair_clusters()), THREADS, p2::SMEM, s>>>(
        gg->tiles, gg->probs, gg->maps, dcols, gg->ntiles, gg->counter);
  else
    ozaki_grouped_gemm_kernel<<<persistent_grid(gg->ntiles), THREADS, SMEM_BYTES, s>>>(
        gg->tiles, gg->probs, gg->maps, dcols, gg->ntiles, gg->counter);
  note_launch();
  return cudaGetLastError();
}

int grouped_gemm_tiles(const GroupedGemm* gg) { return gg ? gg->ntiles : 0; }

int grouped_gemm_tile_rows(const GroupedGemm* gg) { return gg && gg->pair ? 2 * BM : BM; }

void grouped_gemm_destroy(GroupedGemm* gg) {
  if (!gg) return;
  if (gg->tiles) cudaFree(gg->tiles);
  if (gg->probs) cudaFree(gg->probs);
  if (gg->maps) cudaFree(gg->maps);
  if (gg->counter) cudaFree(gg->counter);
  delete gg;
}

}  // namespace fgls

// Self-test of the split-precision GEMM on caller data (host pointers):
// C = A * X^T with A (M x K, row-major FP64) cut into S slices and X (K x N,
// column-major, integer values in [0, 2]).  C is M x N column-major.
extern "C" int fglsgpu_selftest_split_gemm(int M, int K, int N, int S, const double* A, const double* X,
                                           double* C) {
  using namespace fgls;
  using namespace fgls::oz;
  if (M <= 0 || K <= 0 || K > FUSED_KMAX || N <= 0 || S < 1 || S > MAX_SLICES) return FGLSGPU_EINVAL;
  OzakiPlan p;
  p.n = K;
  p.S = S;
  p.S_run = S;
  p.M = M;
  p.Mpad = (M + BM - 1) / BM * BM;
  p.Kpad = (K + KALIGN - 1) / KALIGN * KALIGN;
  p.Ncap = (N + BN - 1) / BN * BN;
  double *dA = nullptr, *dX = nullptr;
  cudaError_t r = cudaSuccess;
  auto chk = [&](cudaError_t e) {
    if (r == cudaSuccess) r = e;
  };
  cudaStream_t s = nullptr;
  chk(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  chk(cudaMalloc(&p.A, (size_t)S * p.Mpad * p.Kpad));
  chk(cudaMalloc(&p.G, (size_t)p.Ncap * p.Kpad));
  chk(cudaMalloc(&p.scale, sizeof(double) * p.Mpad));
  chk(cudaMalloc(&p.C, sizeof(double) * (size_t)p.Mpad * p.Ncap));
  chk(cudaMalloc(&p.err, 3 * sizeof(int)));
  chk(cudaMalloc(&dA, sizeof(double) * (size_t)M * K));
  chk(cudaMalloc(&dX, sizeof(double) * (size_t)K * N));
  if (r == cudaSuccess) chk(cudaMemset(p.A, 0, (size_t)S * p.Mpad * p.Kpad));
  if (r == cudaSuccess) chk(cudaMemset(p.G, 0, (size_t)p.Ncap * p.Kpad));
  if (r == cudaSuccess) chk(cudaMemset(p.scale, 0, sizeof(double) * p.Mpad));
  if (r == cudaSuccess) chk(cudaMemset(p.err, 0, 3 * sizeof(int)));
  if (r == cudaSuccess) chk(cudaMemcpy(dA, A, sizeof(double) * (size_t)M * K, cudaMemcpyHostToDevice));
  if (r == cudaSuccess) chk(cudaMemcpy(dX, X, sizeof(double) * (size_t)K * N, cudaMemcpyHostToDevice));
  if (r == cudaSuccess) chk(make_map(&p.mapA, p.A, p.Kpad, (long long)S * p.Mpad, BM));
  if (r == cudaSuccess) chk(make_map(&p.mapB, p.G, p.Kpad, p.Ncap, BN));
  if (r == cudaSuccess) chk(make_map(&p.mapBh, p.G, p.Kpad, p.Ncap, BN / 2));
  if (r == cudaSuccess) p.has_mapBh = true;
  if (r == cudaSuccess)
    chk(cudaFuncSetAttribute(ozaki_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES));
  if (r == cudaSuccess) {
    slice_rows_kernel<<<M, 256, 0, s>>>(K, M, dA, K, 0, S, p.Mpad, p.Kpad, p.A, p.scale);
    chk(cudaGetLastError());
  }
  if (r == cudaSuccess) chk(load_genotypes<double>(&p, s, dX, N));
  if (r == cudaSuccess) chk(run_gemm(&p, s, 0, N, 0, 0));
  if (r == cudaSuccess) chk(cudaStreamSynchronize(s));
  int herr = 0;
  if (r == cudaSuccess) chk(cudaMemcpy(&herr, p.err, sizeof(int), cudaMemcpyDeviceToHost));
  if (r == cudaSuccess)
    chk(cudaMemcpy2D(C, sizeof(double) * M, p.C, sizeof(double) * p.Mpad, sizeof(double) * M, N,
                     cudaMemcpyDeviceToHost));
  void* ptrs[] = {p.A, p.G, p.scale, p.C, p.err, dA, dX};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  p.A = nullptr; p.G = nullptr; p.scale = nullptr; p.C = nullptr; p.err = nullptr;
  if (s) cudaStreamDestroy(s);
  if (r != cudaSuccess) return FGLSGPU_ECUDA;
  return herr ? FGLSGPU_ETIMEOUT : FGLSGPU_OK;
}

// ---------------------------------------------------------------------------
// Split GEMM that allocates nothing.
//
// For callers that may not allocate device memory themselves: code that runs
// inside a framework which owns every byte of the device through its own
// pool (a raw cudaMalloc would bypass its accounting and can fail once the
// pool has reserved the memory), and code that must not change the device's
// memory footprint between steps.  They pass device buffers for the inputs
// and the output; the kernel's scratch (E4M3 slices of A, the E4M3 genotype
// operand, per-row scales, an error word and the GEMM's tile counters) lives
// in the file-scope array below,
// which every GPU that loads this library holds until the process exits.
//
// Limits (the array's size, 5.8 MB): M <= 256, K <= 2048, N <= 512,
// slices <= 9.  Every call shares the array and leaves its contents behind;
// calls that overlap on the GPU (several streams or threads at once) race on
// it and must be serialised by the caller.  The first call on a device looks
// up the array's device address (cudaGetSymbolAddress) with that device
// current; make that first call before any stream capture.  Every call reads
// the kernel's error word back and synchronizes `stream` before it returns.
// ---------------------------------------------------------------------------
namespace fgls {
namespace oz {
constexpr int NA_MAX_M = 256, NA_MAX_K = 2048, NA_MAX_N = 512, NA_MAX_S = MAX_SLICES;
constexpr size_t NA_A_BYTES = (size_t)NA_MAX_S * NA_MAX_M * NA_MAX_K;   // E4M3 slices
constexpr size_t NA_G_BYTES = (size_t)NA_MAX_N * NA_MAX_K;              // E4M3 genotypes
constexpr size_t NA_SCALE_BYTES = (size_t)NA_MAX_M * 8;                     // row scales
constexpr size_t NA_BYTES = NA_A_BYTES + NA_G_BYTES + NA_SCALE_BYTES + 256;  // + error word, tile counters
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

constexpr int NA_MAX_DEVICES = 64;
// device address of g_noalloc_scratch per device ordinal, set once; atomic
// because host threads may make their first call on a device concurrently
// (they then store the same address)
static std::atomic<void*> g_noalloc_addr[NA_MAX_DEVICES];
}  // namespace oz
}  // namespace fgls

extern "C" int fglsgpu_split_gemm_noalloc(int M, int K, int N, int slices, const double* dA, const double* dX,
                                          double* dC, void* stream) {
  using namespace fgls;
  using namespace fgls::oz;
  if (M <= 0 || M > NA_MAX_M || K <= 0 || K > NA_MAX_K || N <= 0 || N > NA_MAX_N || slices < 1 ||
      slices > NA_MAX_S || !dA || !dX || !dC)
    return FGLSGPU_EINVAL;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) return FGLSGPU_ENODEV;
  void* addr = g_noalloc_addr[dev].load(std::memory_order_acquire);
  if (!addr) {
    // set-up, once per device, with the device current: the host-side name of
    // the array is not a device address
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return FGLSGPU_ECUDA;
    if (cudaFuncSetAttribute(ozaki_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) !=
        cudaSuccess)
      return FGLSGPU_ECUDA;
    g_noalloc_addr[dev].store(ptr, std::memory_order_release);
    addr = ptr;
  }
  unsigned char* base = (unsigned char*)addr;
  OzakiPlan p;
  p.n = K;
  p.S = slices;
  p.S_run = slices;
  p.M = M;
  p.Mpad = (M + BM - 1) / BM * BM;
  p.Kpad = (K + KALIGN - 1) / KALIGN * KALIGN;
  p.Ncap = (N + BN - 1) / BN * BN;
  p.A = (uint8_t*)base;
  p.G = (uint8_t*)(base + NA_A_BYTES);
  p.scale = (double*)(base + NA_A_BYTES + NA_G_BYTES);
  p.err = (int*)(base + NA_A_BYTES + NA_G_BYTES + NA_SCALE_BYTES);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t r = cudaSuccess;
  auto chk = [&](cudaError_t e) {
    if (r == cudaSuccess) r = e;
  };
  // the array keeps the previous call's contents: zero what must start at zero
  // (slice and genotype padding, scales of padding rows, the error word)
  chk(cudaMemsetAsync(p.A, 0, (size_t)slices * p.Mpad * p.Kpad, s));
  chk(cudaMemsetAsync(p.G, 0, (size_t)p.Ncap * p.Kpad, s));
  chk(cudaMemsetAsync(p.scale, 0, sizeof(double) * p.Mpad, s));
  chk(cudaMemsetAsync(p.err, 0, 3 * sizeof(int), s));  // error word and the GEMM's tile counters
  if (r == cudaSuccess) chk(make_map(&p.mapA, p.A, p.Kpad, (long long)slices * p.Mpad, BM));
  if (r == cudaSuccess) chk(make_map(&p.mapB, p.G, p.Kpad, p.Ncap, BN));
  if (r == cudaSuccess) {
    slice_rows_kernel<<<M, 256, 0, s>>>(K, M, dA, K, 0, slices, p.Mpad, p.Kpad, p.A, p.scale);
    note_launch();
    chk(cudaGetLastError());
  }
  if (r == cudaSuccess) chk(load_genotypes<double>(&p, s, dX, N));
  if (r == cudaSuccess) {
    // the output doubles as the int64 accumulator between passes
    p.C = dC;
    GemmArgs g;
    g.M = M;
    g.Mpad = p.Mpad;
    g.N = N;
    g.Kpad = p.Kpad;
    g.S = slices;
    g.tiles_m = p.Mpad / BM;
    g.tiles_n = (N + BN - 1) / BN;
    g.tri_rows = 0;
    g.row_scale = p.scale;
    g.C = dC;
    g.ldc = M;
    g.col0 = 0;
    g.sq_rows = 0;
    g.err = p.err;
    g.wait_ns = WAIT_NS;
    ozaki_gemm_kernel<<<persistent_grid(g.tiles_m * g.tiles_n), THREADS, SMEM_BYTES, s>>>(p.mapA, p.mapB, g,
                                                                                          p.err + 1);
    note_launch();
    chk(cudaGetLastError());
  }
  int herr = 0;
  if (r == cudaSuccess) chk(cudaMemcpyAsync(&herr, p.err, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (r == cudaSuccess) chk(cudaStreamSynchronize(s));
  p.A = nullptr;
  p.G = nullptr;
  p.scale = nullptr;
  p.C = nullptr;
  p.err = nullptr;
  if (r != cudaSuccess) return FGLSGPU_ECUDA;
  return herr ? FGLSGPU_ETIMEOUT : FGLSGPU_OK;
}
