// Shared device-side tables of the batched-cohort path (fgls_batch.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fgls {

// Per cohort, rewritten before every step (one host->device copy).
struct StepCohort {
  const void* X;       // genotype block, SNP-major (SNP i at X + i*n), u8 or FP64
  double* B;           // results: trait j of SNP i at B + (j*x + i)*p
  double* V;           //          and V + (j*x + i)*p*p
  long long snp_base;  // index of the block's first SNP (error reports)
  int x;               // SNPs of this step (0: cohort idle)
  int pad;
};

// Per cohort, fixed: E4M3 genotype operand of the split GEMM.
struct GenoCohort {
  uint8_t* G;  // E4M3 genotypes, Ncap x Kpad, column c at G + c*Kpad
  int n, Kpad;
};

// Per (cohort, trait) problem, fixed.
struct UnitGramProblem {
  const float2* Q;  // sums of R^2 over 32-row groups: SNP i, group g at Q[i + g*ldq]
  long long ldq;
  double* GR;       // x_b results
  int n, cohort;
};

struct SolveProblem {
  const double* top;  // null model of the trait: b_T, S_TL, res_sigma
  const double* gyl;  // Gram rows of the split GEMM: SNP i at gyl + i*rsg, [x~'y~, x~'XL~]
  long long rsg;
  const double* GR;   // x~'x~ of SNP i at GR[i]
  int cohort, trait;
};

}  // namespace fgls
