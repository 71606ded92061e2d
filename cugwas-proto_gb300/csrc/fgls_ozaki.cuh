// Split-precision ("Ozaki") tensor-core path: the FP64 operand of each bulk
// GEMM (Z^T, U = M^-1 [y XL] or L^-1) is cut into integer digit slices with a
// per-row power-of-two scale: five-bit digits stored as FP8 E4M3 (odd
// slices as d / 32); the genotype operand (0/1/2) is exact in E4M3 too.
// tcgen05.mma (kind::f8f6f4) accumulates each slice pair x genotype tile in
// one FP32 accumulator in TMEM (every partial sum is a multiple of 2^-5
// below 2^19, hence exact), and the epilogue recombines the pairs.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fgls {

struct OzakiPlan;

cudaError_t ozaki_create(OzakiPlan** out, int n, int t, int wXL, int wXR, int x_b, int slices, int eigen);
void ozaki_destroy(OzakiPlan* p);
// eigen: Z (n x n), AYL (n x t(1+wXL)), dinv (n x t)
cudaError_t ozaki_set_eigen(OzakiPlan* p, cudaStream_t s, const double* Z, const double* AYL, const double* dinv);
// chol: L (n x n lower), WY = [y~ | XL~] (n x (1+wXL)) of the selected trait
cudaError_t ozaki_set_chol(OzakiPlan* p, cudaStream_t s, const double* L, const double* WY);
// A genotype block on the device in one of three formats (exactly one
// pointer set): FP64 or bytes, n values per column, or 2-bit packed as a
// SNP-major PLINK .bed body (ceil(n/4) bytes per column; a missing call sets
// st to FGLSGPU_EINVAL with the individual and snp_base + SNP).
struct DevStatus;
struct GenoBlock {
  const double* f64 = nullptr;
  const unsigned char* u8 = nullptr;
  const unsigned char* packed = nullptr;
  DevStatus* st = nullptr;
  long long snp_base = 0;
};
// One genotype block (n x x): E4M3 operand build, the tcgen05 split GEMM
// C = [Z^T ; U^T] X (chol: [L^-1 ; U^T] X), and the quadratic Gram terms
// GR[i + j*x] = sum_l C[l,i]^2 d_j(l) (chol: d = 1), all on stream s.
// `hook(ctx, class, begin, stream)` brackets each stage (FGLSGPU_PROF_*
// classes) for timing; may be null.
typedef void (*StageHook)(void* ctx, int cls, int begin, cudaStream_t s);
cudaError_t ozaki_block(OzakiPlan* p, cudaStream_t s, const GenoBlock& X, int x, double* GR, StageHook hook,
                        void* ctx);
// sliced MMA operations per genotype column (2 * slices * rows * K)
double ozaki_flops_per_snp(const OzakiPlan* p);

// Rows [n, n + nU) of the last block's split GEMM output: the Gram terms
// x~^T y~_j, x~^T XL~_j; element (SNP i, q) at ptr[q + i * ld].
const double* ozaki_gram_rows(const OzakiPlan* p, long long* ld);
// The plan's device error word: the first pipeline-wait site of a tcgen05
// kernel that gave up (0 = none).  It stays set, and later launches of the
// plan abort, until the host reads and clears it.
int* ozaki_error_word(OzakiPlan* p);
// Use only the first S of the plan's digit slices in the GEMM (1..built;
// after the operands are set: the row scales are derived from theirs).
cudaError_t ozaki_set_run_slices(OzakiPlan* p, cudaStream_t s, int S);
// Slices in use; *built (may be null) receives the slices the operand holds.
int ozaki_slices(const OzakiPlan* p, int* built);
// base-32 digits a side of the tensor-core quadratic Gram in use (0 when the
// plan does not use it), and setting them (1..11; fewer digits, fewer passes)
int ozaki_quad_digits(const OzakiPlan* p);
void ozaki_set_quad_digits(OzakiPlan* p, int k);
// Limit of one pipeline wait in the plan's tcgen05 kernels (0: 2 s).
void ozaki_set_wait_limit(OzakiPlan* p, unsigned long long ns);

// ---- batched cohorts (fgls_batch.cu) -------------------------------------
struct StepCohort;
struct GenoCohort;
// padded sizes of a split operand with `rows` rows, K = n, x columns
int split_rows_padded(int rows);
int split_k_padded(int n);
int split_cols_padded(int x);
// [L^-1 ; (L^-T WY)^T] of one chol problem cut into S E4M3 five-bit digit slices at A
// (S x Mpad x Kpad) with row scales; Linv, LinvT (n x n) and U (n x (1+wXL))
// are caller scratch.
cudaError_t split_chol_operand(cudaStream_t s, int n, int wXL, const double* L, const double* WY, int S, int Mpad,
                               int Kpad, uint8_t* A, double* scale, double* Linv, double* LinvT, double* U);
// row scales of the first S slices of an operand cut into S_built slices
cudaError_t split_rescale_rows(cudaStream_t s, int rows, const double* built_scale, int S_built, int S,
                               double* scale);
// genotype blocks of all cohorts (per-step table) -> their E4M3 operands
cudaError_t grouped_genotypes(cudaStream_t s, const GenoCohort* dgc, const StepCohort* dsc, int cohorts, bool u8);

struct GroupedGemmDesc {
  const uint8_t* A;        // E4M3 five-bit digit slices (odd slices / 32), S_alloc x Mpad x Kpad
  int S, S_alloc, M, Mpad, Kpad, tri_rows, sq_rows;
  const double* scale;     // Mpad row scales for S slices
  const uint8_t* G;        // cohort E4M3 genotype operand, Ncap x Kpad
  int Ncap;
  double* C;               // Mpad x x_b output (ld Mpad)
  float2* Q;               // rows [0, sq_rows): sums of C^2 over 32-row groups, group g of column c
  long long ldq;           //   at Q[c + g*ldq] (no squares are written to C)
  int cohort;
};
struct GroupedGemm;
// One launch over all problems' tiles (x_b columns each at most); the
// columns of a launch come from dcols[cohort] (device ints).
// pair: 256 x 256 tiles over CTA pairs (2-SM MMAs, when the device launches
// clusters of two), else 128 x 256 tiles on one SM each
cudaError_t grouped_gemm_create(GroupedGemm** out, const GroupedGemmDesc* d, int count, int x_b, int* err,
                                bool pair);
// output tile rows of a grouped plan (256: CTA pairs, 128: one SM)
int grouped_gemm_tile_rows(const GroupedGemm* gg);
cudaError_t grouped_gemm_run(GroupedGemm* gg, cudaStream_t s, const int* dcols);
int grouped_gemm_tiles(const GroupedGemm* gg);
void grouped_gemm_destroy(GroupedGemm* gg);

}  // namespace fgls
