#include "fgls_ozaki.cuh"

namespace fgls {
struct OzakiPlan {
  int dummy;
};
cudaError_t ozaki_create(OzakiPlan** out, int, int, int, int, int, int, int) {
  *out = nullptr;
  return cudaErrorNotSupported;
}
void ozaki_destroy(OzakiPlan*) {}
cudaError_t ozaki_set_eigen(OzakiPlan*, cudaStream_t, const double*, const double*, const double*) {
  return cudaErrorNotSupported;
}
cudaError_t ozaki_set_chol(OzakiPlan*, cudaStream_t, const double*) { return cudaErrorNotSupported; }
cudaError_t ozaki_eigen_block(OzakiPlan*, cudaStream_t, const double*, int, double*, double*) {
  return cudaErrorNotSupported;
}
cudaError_t ozaki_eigen_block_u8(OzakiPlan*, cudaStream_t, const unsigned char*, int, double*, double*) {
  return cudaErrorNotSupported;
}
cudaError_t ozaki_chol_block(OzakiPlan*, cudaStream_t, const double*, int, double*) { return cudaErrorNotSupported; }
}  // namespace fgls
