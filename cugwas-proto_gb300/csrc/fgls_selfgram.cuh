// Quadratic Gram terms of the split path (fgls_selfgram.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace fgls {

// GR[i + j*ldg] = sum_{l<n} A[l + i*lda] * D[l + j*ldd] for i < x, j < t, with
// A and D float pairs (hi, lo) and the sum in double-FP32 (relative error
// ~1e-14).  amax (x floats) is scratch: per-column max of A.hi.  part may be
// null (no row split) or hold quad_gram_part_elems(x, t) pairs; sms = SM count.
cudaError_t quad_gram(cudaStream_t s, int n, int x, int t, const float2* A, long long lda, float* amax,
                      const float2* D, long long ldd, const float* dmax, float2* part, double* GR, long long ldg,
                      int sms);
size_t quad_gram_part_elems(int x, int t);

// Unit weights (chol): GR[i] = sum over the 32-row groups g < ceil(n/32) of
// the split GEMM's group sums of R^2, Q[i + g*ldq] (float pairs), for i < x.
cudaError_t sqsum_combine(cudaStream_t s, int n, int x, const float2* Q, long long ldq, double* GR);

struct UnitGramProblem;
struct StepCohort;
// x~'x~ = sum_l R_l^2 for every (problem, SNP < x of its cohort this step)
// from the problem's group sums, one launch (grid covers x_b SNPs per problem).
cudaError_t unit_gram_grouped(cudaStream_t s, const UnitGramProblem* dprobs, int count, const StepCohort* dsc,
                              int x_b);

}  // namespace fgls
