// Launchers of the engine's kernels (host side).  Every launcher enqueues on
// the given stream and returns the launch's cudaError_t.
#pragma once

#include <atomic>

#include "fgls_common.cuh"

#define FGLS_MAX_P 8    // p = wXL + wXR handled by the batched solve
#define FGLS_MAX_WXR 4  // SNP columns per SNP handled by the Gram kernels

namespace fgls {

// Count of kernels this library has launched (all engines, all devices).
extern std::atomic<long long> g_launches;
inline void note_launch(long long k = 1) { g_launches.fetch_add(k, std::memory_order_relaxed); }

// chol null model.  WY = [y~ | XL~] (n x (1 + wXL), ld n).  Writes the
// trait's top record {B_t[wXL], V_tl[wXL*wXL], res_sigma} at top + trait*topw.
cudaError_t null_model_chol(cudaStream_t s, int n, int wXL, const double* WY, double* top, DevStatus* st,
                            int trait);

// eigen per-trait weights dinv (n x t), AYL = [ZtY.*dinv | ZtXL.*dinv_j ...]
// (n x t(1+wXL)) and top records for all t traits.
cudaError_t eigen_traits(cudaStream_t s, int n, int t, int wXL, const double* W, const double* h,
                         const double* sigma, const double* ZtXL, const double* ZtY, double* dinv,
                         double* AYL, double* top, DevStatus* st);

// chol Gram of one block: X (n x x*wXR, ld ldx) against C = [y~ | XL~].
cudaError_t gram_skinny(cudaStream_t s, int n, int x, int wXL, int wXR, const double* X, long long ldx,
                        const double* C, double* GYL, double* GR);

// Q[:, (i*wXR+c)*wXR+d] = R[:, i*wXR+c] .* R[:, i*wXR+d]
cudaError_t quad_products(cudaStream_t s, int n, int x, int wXR, const double* R, long long ldr, double* Q,
                          long long ldq);

// Batched p x p solve of x SNPs x t traits (see fgls_snp.cu for layouts).
// Gram term (row, q) is read at GYL[row*rsg + q*ldg].
cudaError_t snp_solve(cudaStream_t s, int p, int x, int t, int wXL, const double* top, const double* GYL,
                      long long rsg, long long ldg, const double* GR, long long ldr, double* B, long long bstride, double* V,
                      long long vstride, DevStatus* st, long long snp_base);

// Eigendecomposition (fgls_eig.cu).  A and Z: n x n device scratch/outputs
// (ld n); work: eig_workspace_bytes(n).  *fail_out = 1 if QL did not converge.
size_t eig_workspace_bytes(int n);
cudaError_t dsyev_device(cudaStream_t s, int n, const double* Phi, long long ldp, double* A, double* Z,
                         double* W, void* work, int* fail_out, long long* launches);

// Divide-and-conquer eigensolver of the tridiagonal (d, e) (fgls_dc.cu):
// W ascending, V (n x n) eigenvectors; d, e are overwritten; fail_dev set
// to 1 if a leaf iteration did not converge.
size_t dc_workspace_bytes(int n);
cudaError_t dc_tridiag_eig(cudaStream_t s, int n, double* d, double* e, double* W, double* V, void* work,
                           int* fail_dev, long long* launches);

// Batched cohorts: solves of all problems with p predictors listed in plist
// (device ints into probs), x_b SNPs per problem at most, one launch.
struct SolveProblem;
struct StepCohort;
cudaError_t snp_solve_grouped(cudaStream_t s, int p, const SolveProblem* probs, const int* plist, int count, int x_b,
                              const StepCohort* sc, DevStatus* st);

// compact outputs: SE and p-value of every coefficient (layout of B)
cudaError_t snp_compact(cudaStream_t s, int x, int t, int p, const double* B, long long bstride, const double* V,
                        long long vstride, double* SE, double* P, long long cstride);

// 2-bit packed genotypes (PLINK .bed codes, ceil(n/4) bytes per column) -> bytes
cudaError_t unpack_2bit(cudaStream_t s, const unsigned char* in, int n, long long cols, int wXR, unsigned char* out,
                        DevStatus* st, long long snp_base);

// Two-sided normal p-values of the SNP coefficients from B and V (fgls_snp.cu).
cudaError_t snp_pvalues(cudaStream_t s, int x, int t, int p, int wXL, const double* B, long long bstride,
                        const double* V, long long vstride, double* P, long long pstride);

// Adjoint of the eigen variant (fgls_adjoint.cu); layouts in that file.
cudaError_t adjoint_traits(cudaStream_t s, int n, int t, int wXL, const double* W, const double* h,
                           const double* sigma, const double* ZtXL, const double* ZtY, const double* dinv,
                           double* Wc, double* AYLc, double* AYLs, double* topc, double* tops, double* reml);
cudaError_t adjoint_snps(cudaStream_t s, int p, int x, int t, int wXL, const double* top, const double* GYL,
                         const double* GR, const double* topc, const double* GYLc, const double* GRc,
                         const double* tops, const double* GYLs, const double* GRs, const double* Bbar,
                         long long bstride, double* contrib, double* g, DevStatus* st);
cudaError_t adjoint_reduce(cudaStream_t s, int x, int t, int p, int wXL, const double* contrib, const double* g,
                           double* acc, double* gR);
cudaError_t adjoint_ybar(cudaStream_t s, int n, int t, int wXL, const double* dinv, const double* ZtXL,
                         const double* acc, const double* U, double* V2);

// Null-model REML fit per trait over h in [lo, hi] (grid of `grid` points,
// 2 <= grid <= FGLS_REML_MAX_GRID, then root refinement of the h-gradient).
// out (4 x t): h, sigma_hat, profiled log-likelihood, its h-gradient there.
#define FGLS_REML_MAX_GRID 256
cudaError_t reml_fit(cudaStream_t s, int n, int t, int wXL, const double* W, const double* ZtXL, const double* ZtY,
                     double lo, double hi, int grid, double* out, DevStatus* st);

// Genotype conversion: FP64 or u8 hard calls -> FP64 (device to device).
cudaError_t u8_to_f64(cudaStream_t s, const unsigned char* in, double* out, long long count);

}  // namespace fgls
