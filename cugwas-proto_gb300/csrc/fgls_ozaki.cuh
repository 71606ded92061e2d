// Split-precision ("Ozaki") tensor-core path: the FP64 operand of each bulk
// GEMM (Z^T, U = M^-1 [y XL] or L^-1) is cut into BF16 integer slices with a
// per-row power-of-two scale; the genotype operand (0/1/2) is exact in BF16.
// tcgen05.mma multiplies slice x genotype tiles with FP32 accumulation in
// TMEM (every partial sum is an integer below 2^24, hence exact), and the
// epilogue recombines the slices in FP64.
#pragma once

#include <cuda_runtime.h>

namespace fgls {

struct OzakiPlan;

cudaError_t ozaki_create(OzakiPlan** out, int n, int t, int wXL, int wXR, int x_b, int slices, int eigen);
void ozaki_destroy(OzakiPlan* p);
// eigen: Z (n x n), AYL (n x t(1+wXL)), dinv (n x t)
cudaError_t ozaki_set_eigen(OzakiPlan* p, cudaStream_t s, const double* Z, const double* AYL, const double* dinv);
// chol: L (n x n lower)
cudaError_t ozaki_set_chol(OzakiPlan* p, cudaStream_t s, const double* L);
// eigen block: genotypes (FP64 or u8, n x x*wXR) -> GYL, GR (Gram layout of fgls_snp.cu)
cudaError_t ozaki_eigen_block(OzakiPlan* p, cudaStream_t s, const double* X, int x, double* GYL, double* GR);
cudaError_t ozaki_eigen_block_u8(OzakiPlan* p, cudaStream_t s, const unsigned char* X, int x, double* GYL,
                                 double* GR);
// chol block: Xout = L^-1 X (FP64, n x x*wXR)
cudaError_t ozaki_chol_block(OzakiPlan* p, cudaStream_t s, const double* X, int x, double* Xout);

}  // namespace fgls
