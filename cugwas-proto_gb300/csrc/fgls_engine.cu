// The fglsgpu_* engine: device buffers, streams and the per-trait / per-block
// schedules of the two FGLS variants.
//
// chol  (src/fgls_chol.c:223-487):  per trait j: M_j = h s Phi + (1-h) s I on
//   the device, blocked FP64 potrf, [y~ | XL~] = L^-1 [y | XL], null model;
//   per SNP block: X~ = L^-1 XR_blk (blocked TRSM), skinny Gram, batched solve.
// eigen (src/fgls_eigen.c:38-677):  once: Phi = Z W Z^T (device FP64
//   eigensolver), Z^T XL, Z^T Y, per-trait weights d_j = 1/(a_j W + b_j) and
//   null models; per SNP block: R = Z^T XR_blk once for all traits, Gram
//   terms for all traits as GEMMs against d_j-weighted operands (the
//   reference's per-trait rescale of the block, src/fgls_eigen.c:505-507, is
//   folded into the small operand and never materialised), batched solve
//   over SNP x trait.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "fgls_common.cuh"
#include "fgls_kernels.cuh"
#include "fgls_ozaki.cuh"

using namespace fgls;

struct fglsgpu_engine {
  fglsgpu_config cfg{};
  int p = 0, topw = 0;
  cudaStream_t comp = nullptr, h2d = nullptr, d2h = nullptr;
  cudaEvent_t evH[2]{}, evC[2]{}, evD[2]{};
  // in-core operands
  double *dPhi = nullptr, *dL = nullptr, *dZ = nullptr, *dW = nullptr;
  double *dXL = nullptr, *dY = nullptr, *dh = nullptr, *dsig = nullptr;
  double *dWY = nullptr, *dZtXL = nullptr, *dZtY = nullptr, *ddinv = nullptr, *dAYL = nullptr;
  double* dtop = nullptr;
  void* deigwork = nullptr;
  // per-block work
  double* dX[2]{};
  double* dWork = nullptr;  // chol: TRSM in place; eigen: R = Z^T X
  double* dQ = nullptr;     // eigen: self-product operand
  double *dGYL = nullptr, *dGR = nullptr;
  double *dB[2]{}, *dV[2]{};
  double *dSE[2]{}, *dP[2]{};  // compact outputs (allocated on first use)
  unsigned char* dU8 = nullptr;  // unpacked 2-bit genotypes (FP64 path)
  double* dXw = nullptr;         // byte genotypes widened to FP64 (FP64 path)
  DevStatus* dst = nullptr;
  DevStatus* hst = nullptr;
  int* hst_wait = nullptr;  // pinned copy of the split plan's wait error word
  OzakiPlan* oz = nullptr;  // split-precision state (eigen / chol)
  unsigned long long wait_ns = 0;  // limit of one tcgen05 pipeline wait (0: the 2 s default)
  double tune_err = -1.0;          // probe-block beta error of the tuned slice count (-1: not tuned)
  std::vector<double> hh, hs;
  int trait_sel = -1;
  bool problem_set = false;
  std::string err;
  // per-kernel-class timing with CUDA events on the launching stream
  struct PEv {
    cudaEvent_t a, b;
    int cls;
  };
  bool prof = false;
  std::vector<PEv> pev_live, pev_pool;
  PEv pending[FGLSGPU_PROF_CLASSES]{};
  double prof_ms[FGLSGPU_PROF_CLASSES] = {0};
  long long prof_cnt[FGLSGPU_PROF_CLASSES] = {0};
  // adjoint state (eigen, FP64): allocated by fglsgpu_adjoint_reset
  double *aWc = nullptr, *aAYLc = nullptr, *aAYLs = nullptr, *atopc = nullptr, *atops = nullptr, *areml = nullptr;
  double *aGYLc = nullptr, *aGYLs = nullptr, *aGRc = nullptr, *aGRs = nullptr, *acontrib = nullptr, *ag = nullptr;
  double *agR = nullptr, *aacc = nullptr, *aU = nullptr, *aV2 = nullptr;
  bool adj_ready = false;
};

namespace {

thread_local std::string tl_err;

int fail(fglsgpu_engine* e, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (e) e->err = buf;
  tl_err = buf;
  return code;
}

int cuda_fail(fglsgpu_engine* e, cudaError_t c, const char* what) {
  return fail(e, c == cudaErrorMemoryAllocation ? FGLSGPU_ENOMEM : FGLSGPU_ECUDA, "%s: %s (%s)", what,
              cudaGetErrorString(c), cudaGetErrorName(c));
}

#define ENG_TRY(e, expr, what)                           \
  do {                                                   \
    cudaError_t _c = (expr);                             \
    if (_c != cudaSuccess) return cuda_fail(e, _c, what); \
  } while (0)

template <class T>
cudaError_t dalloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) return cudaSuccess;
  return cudaMalloc((void**)p, sizeof(T) * count);
}

// Reads the device status word after a sync; maps failures to messages that
// follow the reference's error texts (src/fgls_chol.c:266-271, :309-314, :418-434).
int check_status(fglsgpu_engine* e, const char* stage) {
  ENG_TRY(e, cudaMemcpyAsync(e->hst, e->dst, sizeof(DevStatus), cudaMemcpyDeviceToHost, e->comp), "status copy");
  *e->hst_wait = 0;
  if (e->oz)
    ENG_TRY(e, cudaMemcpyAsync(e->hst_wait, ozaki_error_word(e->oz), sizeof(int), cudaMemcpyDeviceToHost, e->comp),
            "status copy");
  ENG_TRY(e, cudaStreamSynchronize(e->comp), stage);
  const DevStatus s = *e->hst;
  const int wsite = *e->hst_wait;
  if (wsite) {
    // the tcgen05 kernels of the split path gave up on a pipeline wait: their
    // outputs since the last check are invalid; clear the word so that the
    // next launches run normally
    ENG_TRY(e, cudaMemsetAsync(ozaki_error_word(e->oz), 0, sizeof(int), e->comp), "status reset");
    ENG_TRY(e, cudaStreamSynchronize(e->comp), "status reset");
    return fail(e, FGLSGPU_ETIMEOUT, "device wait expired in %s (tensor-core kernel wait site %d)", stage, wsite);
  }
  if (s.code == FGLSGPU_OK) return FGLSGPU_OK;
  if (s.code == FGLSGPU_ENOTSPD) {
    if (!strcmp(stage, "potrf(M)"))
      return fail(e, FGLSGPU_ENOTSPD, "dpotrf(M) failed (info: %d)", s.info);
    if (s.info < 0) return fail(e, FGLSGPU_ENOTSPD, "dpotrf(scoreV) failed (info: -1) - trait: %lld", s.idx);
    return fail(e, FGLSGPU_ENOTSPD, "dpotrf(V) failed (info: %d) - i: %lld", s.info, s.idx);
  }
  if (s.code == FGLSGPU_EINVAL)
    return fail(e, FGLSGPU_EINVAL, "missing genotype (2-bit code 01) at SNP %lld, individual %d", s.idx, s.info);
  if (s.code == FGLSGPU_ETIMEOUT)
    return fail(e, FGLSGPU_ETIMEOUT, "device wait expired in %s (site %d, item %lld)", stage, s.info, s.idx);
  return fail(e, s.code, "device status %d in %s (info %d, item %lld)", s.code, stage, s.info, s.idx);
}

int reset_status(fglsgpu_engine* e) {
  ENG_TRY(e, cudaMemsetAsync(e->dst, 0, sizeof(DevStatus), e->comp), "status reset");
  return FGLSGPU_OK;
}

void free_all(fglsgpu_engine* e) {
  void* ptrs[] = {e->dPhi, e->dL,   e->dZ,    e->dW,    e->dXL,   e->dY,    e->dh,    e->dsig, e->dWY,
                  e->dZtXL, e->dZtY, e->ddinv, e->dAYL, e->dtop, e->deigwork, e->dX[0], e->dX[1], e->dWork,
                  e->dQ,   e->dGYL, e->dGR,  e->dB[0], e->dB[1], e->dV[0], e->dV[1], e->dU8, e->dst,
                  e->aWc, e->aAYLc, e->aAYLs, e->atopc, e->atops, e->areml, e->aGYLc, e->aGYLs, e->aGRc,
                  e->aGRs, e->acontrib, e->ag, e->agR, e->aacc, e->aU, e->aV2, e->dSE[0], e->dSE[1], e->dP[0],
                  e->dP[1], e->dXw};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (e->hst) cudaFreeHost(e->hst);
  if (e->hst_wait) cudaFreeHost(e->hst_wait);
  for (auto* v : {&e->pev_live, &e->pev_pool})
    for (auto& ev : *v) {
      cudaEventDestroy(ev.a);
      cudaEventDestroy(ev.b);
    }
  if (e->oz) ozaki_destroy(e->oz);
  for (int k = 0; k < 2; k++) {
    if (e->evH[k]) cudaEventDestroy(e->evH[k]);
    if (e->evC[k]) cudaEventDestroy(e->evC[k]);
    if (e->evD[k]) cudaEventDestroy(e->evD[k]);
  }
  if (e->comp) cudaStreamDestroy(e->comp);
  if (e->h2d) cudaStreamDestroy(e->h2d);
  if (e->d2h) cudaStreamDestroy(e->d2h);
}

bool split(const fglsgpu_engine* e) { return e->cfg.precision == FGLSGPU_PREC_SPLIT; }

// Brackets the kernels launched in its scope with two events on stream s
// when profiling is on; resolved by fglsgpu_profile_read.
struct Prof {
  fglsgpu_engine* e;
  cudaStream_t s;
  fglsgpu_engine::PEv ev{};
  bool on;
  static fglsgpu_engine::PEv take(fglsgpu_engine* e, int cls) {
    fglsgpu_engine::PEv ev{};
    if (e->pev_pool.empty()) {
      cudaEventCreate(&ev.a);
      cudaEventCreate(&ev.b);
    } else {
      ev = e->pev_pool.back();
      e->pev_pool.pop_back();
    }
    ev.cls = cls;
    return ev;
  }
  Prof(fglsgpu_engine* e_, int cls, cudaStream_t s_) : e(e_), s(s_), on(e_->prof) {
    if (!on) return;
    ev = take(e, cls);
    cudaEventRecord(ev.a, s);
  }
  ~Prof() {
    if (!on) return;
    cudaEventRecord(ev.b, s);
    e->pev_live.push_back(ev);
  }
};

// Stage hook of the split path: brackets each stage on the stream it runs on.
void stage_hook(void* ctx, int cls, int begin, cudaStream_t st) {
  fglsgpu_engine* e = (fglsgpu_engine*)ctx;
  if (!e->prof) return;
  if (begin) {
    e->pending[cls] = Prof::take(e, cls);
    cudaEventRecord(e->pending[cls].a, st);
  } else {
    cudaEventRecord(e->pending[cls].b, st);
    e->pev_live.push_back(e->pending[cls]);
  }
}

// Genotype formats of a block in device memory: FP64, bytes (n values per
// column) or 2-bit packed (ceil(n/4) bytes per column, PLINK .bed body).
enum { GENO_F64 = 0, GENO_U8 = 1, GENO_PACKED = 2 };

long long geno_bytes_per_col(int fmt, int n) {
  return fmt == GENO_F64 ? 8LL * n : fmt == GENO_U8 ? (long long)n : (long long)(n + 3) / 4;
}

// Compute one block already in device memory (n x x*wXR genotypes in format
// `fmt` at dX) into dB/dV with the given trait strides, on e->comp.
int compute_block(fglsgpu_engine* e, const void* dX, int fmt, int x, double* dB, double* dV, long long bstr,
                  long long vstr, long long snp_base) {
  const fglsgpu_config& c = e->cfg;
  const int n = c.n, wXL = c.wXL, wXR = c.wXR, p = e->p;
  const int t = c.variant == FGLSGPU_VARIANT_EIGEN ? c.t : 1;
  const long long cols = (long long)x * wXR;
  cudaStream_t s = e->comp;
  if (c.variant == FGLSGPU_VARIANT_CHOL && e->trait_sel < 0)
    return fail(e, FGLSGPU_ESTATE, "fglsgpu_select_trait must precede run_block (chol)");
  const double* dXin = fmt == GENO_F64 ? (const double*)dX : nullptr;
  const unsigned char* dXu8 = fmt == GENO_U8 ? (const unsigned char*)dX : nullptr;
  if (split(e)) {
    GenoBlock gb;
    gb.f64 = dXin;
    gb.u8 = dXu8;
    gb.packed = fmt == GENO_PACKED ? (const unsigned char*)dX : nullptr;
    gb.st = e->dst;
    gb.snp_base = snp_base;
    ENG_TRY(e, ozaki_block(e->oz, s, gb, x, e->dGR, stage_hook, e), "split block");
    long long ld = 0;
    const double* gyl = ozaki_gram_rows(e->oz, &ld);
    Prof pr(e, FGLSGPU_PROF_SOLVE, s);
    ENG_TRY(e, snp_solve(s, p, x, t, wXL, e->dtop, gyl, ld, 1, e->dGR, cols * wXR, dB, bstr, dV, vstr, e->dst,
                         snp_base),
            "solve");
    return FGLSGPU_OK;
  }
  if (fmt == GENO_PACKED) {
    Prof pr(e, FGLSGPU_PROF_GENOTYPES, s);
    if (!e->dU8) ENG_TRY(e, dalloc(&e->dU8, (size_t)c.x_b * c.wXR * c.n), "genotype bytes");
    ENG_TRY(e, unpack_2bit(s, (const unsigned char*)dX, n, cols, wXR, e->dU8, e->dst, snp_base), "unpack genotypes");
    dXu8 = e->dU8;
  }
  if (dXu8) {
    Prof pr(e, FGLSGPU_PROF_GENOTYPES, s);
    if (!e->dXw) ENG_TRY(e, dalloc(&e->dXw, (size_t)c.x_b * c.wXR * c.n), "widened genotypes");
    ENG_TRY(e, u8_to_f64(s, dXu8, e->dXw, (long long)cols * n), "widen genotypes");
    dXin = e->dXw;
  }
  if (c.variant == FGLSGPU_VARIANT_CHOL) {
    {
      Prof pr(e, FGLSGPU_PROF_TRSM, s);
      ENG_TRY(e, cudaMemcpyAsync(e->dWork, dXin, sizeof(double) * n * cols, cudaMemcpyDeviceToDevice, s),
              "block copy");
      ENG_TRY(e, dtrsm_llnn(s, n, (int)cols, e->dL, n, e->dWork, n), "TRSM");
    }
    Prof pr(e, FGLSGPU_PROF_GRAM, s);
    ENG_TRY(e, gram_skinny(s, n, x, wXL, wXR, e->dWork, n, e->dWY, e->dGYL, e->dGR), "gram");
  } else {
    {
      Prof pr(e, FGLSGPU_PROF_FP64_GEMM, s);
      ENG_TRY(e, dgemm(s, true, false, n, (int)cols, n, 1.0, e->dZ, n, dXin, n, 0.0, e->dWork, n), "Z^T XR");
    }
    Prof pr(e, FGLSGPU_PROF_GRAM, s);
    ENG_TRY(e, dgemm(s, true, false, (int)cols, t * (1 + wXL), n, 1.0, e->dWork, n, e->dAYL, n, 0.0, e->dGYL,
                     cols),
            "gram YL");
    const long long qcols = cols * wXR;
    ENG_TRY(e, quad_products(s, n, x, wXR, e->dWork, n, e->dQ, n), "quad");
    ENG_TRY(e, dgemm(s, true, false, (int)qcols, t, n, 1.0, e->dQ, n, e->ddinv, n, 0.0, e->dGR, qcols),
            "gram R");
  }
  Prof pr(e, FGLSGPU_PROF_SOLVE, s);
  ENG_TRY(e, snp_solve(s, p, x, t, wXL, e->dtop, e->dGYL, 1, cols, e->dGR, cols * wXR, dB, bstr, dV, vstr, e->dst,
                       snp_base),
          "solve");
  return FGLSGPU_OK;
}

int out_traits(const fglsgpu_engine* e) { return e->cfg.variant == FGLSGPU_VARIANT_EIGEN ? e->cfg.t : 1; }

// Hard calls of a probe block: SNP i with allele frequency f_i in
// [0.05, 0.5) and genotype Binomial(2, f_i), both from an integer hash of
// (SNP, individual) (fixed, so the choice is reproducible).
__device__ __forceinline__ unsigned probe_hash(unsigned h) {
  h ^= h >> 16;
  h *= 0x7feb352du;
  h ^= h >> 15;
  h *= 0x846ca68bu;
  h ^= h >> 16;
  return h;
}
__global__ void probe_genotypes_kernel(int n, int x, double* __restrict__ out) {
  const int i = blockIdx.x;
  const unsigned fi = 50 + probe_hash(0x9e3779b9u * (unsigned)(i + 1)) % 450;  // per mille
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const unsigned h1 = probe_hash((unsigned)i * 2654435761u ^ (unsigned)(2 * k + 1));
    const unsigned h2 = probe_hash((unsigned)i * 2246822519u ^ (unsigned)(2 * k + 2));
    out[(long long)i * n + k] = (double)((h1 % 1000 < fi) + (h2 % 1000 < fi));
  }
}

// Slice autotuning (cfg.slices == 0): the split operand holds 9 five-bit
// digit slices; a probe block of 256 SNPs runs through the all-FP64 path and
// through the split path with the first 6, 7, 8 and 9 slices, and the
// smallest count whose beta (normwise per trait and SNP) is within
// TUNE_TOL / 8 of the FP64 result is kept.  Then, with that slice count, the
// tensor-core quadratic Gram's base-32 digits a side (eigen, t >= 33) are
// chosen the same way from 8..11.  Called after every build of the split
// operands (they depend on the trait's weights or factor).
constexpr double TUNE_TOL = 1e-10;
constexpr int TUNE_SNPS = 256, TUNE_MIN_SLICES = 6, TUNE_MIN_QDIGITS = 8;

int tune_slices(fglsgpu_engine* e) {
  fglsgpu_config& c = e->cfg;
  if (!split(e) || !e->oz || c.slices != 0) return FGLSGPU_OK;
  cudaStream_t s = e->comp;
  const int n = c.n, p = e->p, nt = out_traits(e), xp = std::min(TUNE_SNPS, c.x_b);
  int built = 0;
  ozaki_slices(e->oz, &built);
  double *dX = nullptr, *dBr = nullptr, *dVr = nullptr, *dBs = nullptr, *dVs = nullptr, *dW = nullptr, *dQ = nullptr;
  cudaError_t r = cudaSuccess;
  auto chk = [&](cudaError_t x) {
    if (r == cudaSuccess) r = x;
  };
  chk(dalloc(&dX, (size_t)n * xp));
  chk(dalloc(&dBr, (size_t)nt * xp * p));
  chk(dalloc(&dVr, (size_t)nt * xp * p * p));
  chk(dalloc(&dBs, (size_t)nt * xp * p));
  chk(dalloc(&dVs, (size_t)nt * xp * p * p));
  if (c.variant == FGLSGPU_VARIANT_EIGEN) {
    chk(dalloc(&dW, (size_t)n * xp));
    chk(dalloc(&dQ, (size_t)n * xp));
  }
  auto release = [&]() {
    for (double* q : {dX, dBr, dVr, dBs, dVs, dW, dQ})
      if (q) cudaFree(q);
  };
  if (r != cudaSuccess) {
    release();
    return cuda_fail(e, r, "slice probe buffers");
  }
  probe_genotypes_kernel<<<xp, 256, 0, s>>>(n, xp, dX);
  note_launch();
  int rc = reset_status(e);
  // the FP64 reference on probe-sized work buffers
  double* keepW = e->dWork;
  double* keepQ = e->dQ;
  if (c.variant == FGLSGPU_VARIANT_EIGEN) {
    e->dWork = dW;
    e->dQ = dQ;
  }
  c.precision = FGLSGPU_PREC_FP64;
  if (!rc) rc = compute_block(e, dX, GENO_F64, xp, dBr, dVr, (long long)xp * p, (long long)xp * p * p, 0);
  c.precision = FGLSGPU_PREC_SPLIT;
  e->dWork = keepW;
  e->dQ = keepQ;
  std::vector<double> Br((size_t)nt * xp * p), Bs(Br.size());
  if (!rc && cudaMemcpyAsync(Br.data(), dBr, sizeof(double) * Br.size(), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    rc = fail(e, FGLSGPU_ECUDA, "slice probe copy");
  // the probe block through the split path as configured: worst beta error
  auto probe = [&](double* worst) -> int {
    int q_rc = compute_block(e, dX, GENO_F64, xp, dBs, dVs, (long long)xp * p, (long long)xp * p * p, 0);
    if (q_rc) return q_rc;
    if (cudaMemcpyAsync(Bs.data(), dBs, sizeof(double) * Bs.size(), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return fail(e, FGLSGPU_ECUDA, "slice probe copy");
    double w = 0.0;
    for (size_t q = 0; q < Br.size(); q += p) {
      double d2 = 0.0, r2 = 0.0;
      for (int k = 0; k < p; k++) {
        const double d = Bs[q + k] - Br[q + k];
        d2 += d * d;
        r2 += Br[q + k] * Br[q + k];
      }
      const double rel = r2 > 0.0 ? std::sqrt(d2 / r2) : std::sqrt(d2);
      w = (rel > w || rel != rel) ? rel : w;
    }
    *worst = w;
    return FGLSGPU_OK;
  };
  const int qbuilt = ozaki_quad_digits(e->oz);  // 0: no tensor-core quadratic Gram
  int chosen = built;
  double err = -1.0;
  for (int S = std::min(TUNE_MIN_SLICES, built); S <= built && !rc; S++) {
    ENG_TRY(e, ozaki_set_run_slices(e->oz, s, S), "slice probe");
    double worst = 0.0;
    rc = probe(&worst);
    if (rc) break;
    err = worst;
    if (worst <= TUNE_TOL / 8) {
      chosen = S;
      break;
    }
  }
  int qchosen = qbuilt;
  if (!rc && qbuilt > 0) {
    ENG_TRY(e, ozaki_set_run_slices(e->oz, s, chosen), "slice choice");
    for (int k = std::min(TUNE_MIN_QDIGITS, qbuilt); k < qbuilt && !rc; k++) {
      ozaki_set_quad_digits(e->oz, k);
      double worst = 0.0;
      rc = probe(&worst);
      if (rc) break;
      if (worst <= TUNE_TOL / 8) {
        qchosen = k;
        err = worst;
        break;
      }
    }
    ozaki_set_quad_digits(e->oz, qchosen);
  }
  release();
  if (!rc) rc = check_status(e, "slice probe");
  if (rc) return rc;
  ENG_TRY(e, ozaki_set_run_slices(e->oz, s, chosen), "slice choice");
  ENG_TRY(e, cudaStreamSynchronize(s), "slice choice");
  e->tune_err = err;
  return FGLSGPU_OK;
}

}  // namespace

extern "C" {

int fglsgpu_version(void) { return 10000; }

const char* fglsgpu_last_error(const fglsgpu_engine* e) { return e ? e->err.c_str() : tl_err.c_str(); }

long long fglsgpu_launch_count(const fglsgpu_engine*) { return g_launches.load(); }

void* fglsgpu_stream(fglsgpu_engine* e) { return e ? (void*)e->comp : nullptr; }

int fglsgpu_create(const fglsgpu_config* cfg, fglsgpu_engine** out) {
  if (!cfg || !out) return fail(nullptr, FGLSGPU_EINVAL, "null argument");
  *out = nullptr;
  const fglsgpu_config c = *cfg;
  if (c.n <= 0 || c.wXL <= 0 || c.wXR <= 0 || c.t <= 0 || c.x_b <= 0)
    return fail(nullptr, FGLSGPU_EINVAL, "invalid dimensions n=%d wXL=%d wXR=%d t=%d x_b=%d", c.n, c.wXL, c.wXR,
                c.t, c.x_b);
  if (c.wXL + c.wXR > FGLS_MAX_P || c.wXL + c.wXR < 2)
    return fail(nullptr, FGLSGPU_EINVAL, "p = wXL + wXR = %d outside [2, %d]", c.wXL + c.wXR, FGLS_MAX_P);
  if (c.wXR > FGLS_MAX_WXR) return fail(nullptr, FGLSGPU_EINVAL, "wXR = %d > %d", c.wXR, FGLS_MAX_WXR);
  if (c.n <= c.wXL) return fail(nullptr, FGLSGPU_EINVAL, "n = %d must exceed wXL = %d", c.n, c.wXL);
  if (c.variant != FGLSGPU_VARIANT_CHOL && c.variant != FGLSGPU_VARIANT_EIGEN)
    return fail(nullptr, FGLSGPU_EINVAL, "unknown variant %d", c.variant);
  if (c.precision != FGLSGPU_PREC_FP64 && c.precision != FGLSGPU_PREC_SPLIT)
    return fail(nullptr, FGLSGPU_EINVAL, "unknown precision %d", c.precision);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
    cudaGetLastError();
    return fail(nullptr, FGLSGPU_ENODEV, "no CUDA device available");
  }
  if (c.device < 0 || c.device >= ndev) return fail(nullptr, FGLSGPU_EINVAL, "device %d of %d", c.device, ndev);
  cudaError_t ce = cudaSetDevice(c.device);
  if (ce != cudaSuccess) return cuda_fail(nullptr, ce, "cudaSetDevice");
  fglsgpu_engine* e = new fglsgpu_engine();
  e->cfg = c;
  e->p = c.wXL + c.wXR;
  e->topw = c.wXL + c.wXL * c.wXL + 1;
  const long long n = c.n, t = c.t, xb = c.x_b, wXL = c.wXL, wXR = c.wXR, p = e->p;
  const int nt = c.variant == FGLSGPU_VARIANT_EIGEN ? c.t : 1;
  cudaError_t r = cudaSuccess;
  auto chk = [&](cudaError_t x) {
    if (r == cudaSuccess) r = x;
  };
  chk(cudaStreamCreateWithFlags(&e->comp, cudaStreamNonBlocking));
  chk(cudaStreamCreateWithFlags(&e->h2d, cudaStreamNonBlocking));
  chk(cudaStreamCreateWithFlags(&e->d2h, cudaStreamNonBlocking));
  for (int k = 0; k < 2; k++) {
    chk(cudaEventCreateWithFlags(&e->evH[k], cudaEventDisableTiming));
    chk(cudaEventCreateWithFlags(&e->evC[k], cudaEventDisableTiming));
    chk(cudaEventCreateWithFlags(&e->evD[k], cudaEventDisableTiming));
  }
  chk(dalloc(&e->dPhi, n * n));
  chk(dalloc(&e->dXL, n * wXL));
  chk(dalloc(&e->dY, n * t));
  chk(dalloc(&e->dh, t));
  chk(dalloc(&e->dsig, t));
  chk(dalloc(&e->dtop, t * e->topw));
  chk(dalloc(&e->dst, 1));
  chk(cudaMallocHost((void**)&e->hst, sizeof(DevStatus)));
  chk(cudaMallocHost((void**)&e->hst_wait, sizeof(int)));
  for (int k = 0; k < 2; k++) {
    chk(dalloc(&e->dX[k], n * xb * wXR));
    chk(dalloc(&e->dB[k], (long long)nt * xb * p));
    chk(dalloc(&e->dV[k], (long long)nt * xb * p * p));
  }
  chk(dalloc(&e->dGYL, xb * wXR * nt * (1 + wXL)));
  chk(dalloc(&e->dGR, xb * wXR * wXR * nt));
  if (c.variant == FGLSGPU_VARIANT_CHOL) {
    chk(dalloc(&e->dL, n * n));
    chk(dalloc(&e->dWY, n * (1 + wXL)));
    chk(dalloc(&e->dWork, n * xb * wXR));
  } else {
    chk(dalloc(&e->dL, n * n));  // eigensolver scratch
    chk(dalloc(&e->dZ, n * n));
    chk(dalloc(&e->dW, n));
    chk(dalloc(&e->dZtXL, n * wXL));
    chk(dalloc(&e->dZtY, n * t));
    chk(dalloc(&e->ddinv, n * t));
    chk(dalloc(&e->dAYL, n * t * (1 + wXL)));
    chk(cudaMalloc(&e->deigwork, eig_workspace_bytes(c.n)));
    if (c.precision == FGLSGPU_PREC_FP64) {
      chk(dalloc(&e->dWork, n * xb * wXR));
      chk(dalloc(&e->dQ, n * xb * wXR * wXR));
    }
  }
  if (r == cudaSuccess) r = cudaMemsetAsync(e->dst, 0, sizeof(DevStatus), e->comp);
  if (r == cudaSuccess) r = cudaStreamSynchronize(e->comp);
  if (r != cudaSuccess) {
    int code = cuda_fail(e, r, "engine allocation");
    tl_err = e->err;
    free_all(e);
    delete e;
    return code;
  }
  *out = e;
  return FGLSGPU_OK;
}

int fglsgpu_destroy(fglsgpu_engine* e) {
  if (!e) return FGLSGPU_OK;
  cudaSetDevice(e->cfg.device);
  if (e->comp) cudaStreamSynchronize(e->comp);
  free_all(e);
  delete e;
  return FGLSGPU_OK;
}

int fglsgpu_set_problem(fglsgpu_engine* e, const double* Phi, const double* XL, const double* Y, const double* h,
                        const double* sigma) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!Phi || !XL || !Y || !h || !sigma) return fail(e, FGLSGPU_EINVAL, "null input pointer");
  const fglsgpu_config& c = e->cfg;
  const long long n = c.n, t = c.t;
  ENG_TRY(e, cudaSetDevice(c.device), "cudaSetDevice");
  for (int j = 0; j < c.t; j++)
    if (!(h[j] >= 0.0 && h[j] <= 1.0) || !(sigma[j] > 0.0))
      return fail(e, FGLSGPU_EINVAL, "trait %d: need 0 <= h <= 1 and sigma > 0 (h=%g sigma=%g)", j, h[j], sigma[j]);
  e->hh.assign(h, h + c.t);
  e->hs.assign(sigma, sigma + c.t);
  cudaStream_t s = e->comp;
  ENG_TRY(e, cudaMemcpyAsync(e->dPhi, Phi, sizeof(double) * n * n, cudaMemcpyHostToDevice, s), "upload Phi");
  ENG_TRY(e, cudaMemcpyAsync(e->dXL, XL, sizeof(double) * n * c.wXL, cudaMemcpyHostToDevice, s), "upload XL");
  ENG_TRY(e, cudaMemcpyAsync(e->dY, Y, sizeof(double) * n * t, cudaMemcpyHostToDevice, s), "upload Y");
  ENG_TRY(e, cudaMemcpyAsync(e->dh, h, sizeof(double) * t, cudaMemcpyHostToDevice, s), "upload h");
  ENG_TRY(e, cudaMemcpyAsync(e->dsig, sigma, sizeof(double) * t, cudaMemcpyHostToDevice, s), "upload sigma");
  int rc = reset_status(e);
  if (rc) return rc;
  e->trait_sel = -1;
  e->problem_set = false;
  if (c.variant == FGLSGPU_VARIANT_EIGEN) {
    int qfail = 0;
    ENG_TRY(e, dsyev_device(s, c.n, e->dPhi, n, e->dL, e->dZ, e->dW, e->deigwork, &qfail, nullptr),
            "eigendecomposition");
    if (qfail) return fail(e, FGLSGPU_ENOCONV, "dsyevr failed (info: 1): QL iteration did not converge");
    ENG_TRY(e, dgemm(s, true, false, c.n, c.wXL, c.n, 1.0, e->dZ, n, e->dXL, n, 0.0, e->dZtXL, n), "Z^T XL");
    ENG_TRY(e, dgemm(s, true, false, c.n, c.t, c.n, 1.0, e->dZ, n, e->dY, n, 0.0, e->dZtY, n), "Z^T Y");
    ENG_TRY(e, eigen_traits(s, c.n, c.t, c.wXL, e->dW, e->dh, e->dsig, e->dZtXL, e->dZtY, e->ddinv, e->dAYL,
                            e->dtop, e->dst),
            "trait weights");
    rc = check_status(e, "eigen setup");
    if (rc) return rc;
    if (split(e)) {
      if (!e->oz) {
        ENG_TRY(e, ozaki_create(&e->oz, c.n, c.t, c.wXL, c.wXR, c.x_b, c.slices, /*eigen=*/1), "split plan");
        ozaki_set_wait_limit(e->oz, e->wait_ns);
      }
      ENG_TRY(e, ozaki_set_eigen(e->oz, s, e->dZ, e->dAYL, e->ddinv), "split operands");
      ENG_TRY(e, cudaStreamSynchronize(s), "split operands");
      rc = tune_slices(e);
      if (rc) return rc;
    }
  }
  ENG_TRY(e, cudaStreamSynchronize(s), "set_problem");
  e->problem_set = true;
  return FGLSGPU_OK;
}

int fglsgpu_select_trait(fglsgpu_engine* e, int j) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!e->problem_set) return fail(e, FGLSGPU_ESTATE, "set_problem must precede select_trait");
  const fglsgpu_config& c = e->cfg;
  if (c.variant == FGLSGPU_VARIANT_EIGEN) return FGLSGPU_OK;
  if (j < 0 || j >= c.t) return fail(e, FGLSGPU_EINVAL, "trait %d outside [0, %d)", j, c.t);
  ENG_TRY(e, cudaSetDevice(c.device), "cudaSetDevice");
  const long long n = c.n;
  cudaStream_t s = e->comp;
  int rc = reset_status(e);
  if (rc) return rc;
  const double alpha = e->hh[j] * e->hs[j];          // src/fgls_chol.c:253
  const double beta = (1.0 - e->hh[j]) * e->hs[j];   // src/fgls_chol.c:254
  ENG_TRY(e, build_shifted(s, c.n, e->dPhi, n, alpha, beta, e->dL, n), "build M");
  ENG_TRY(e, dpotrf_lower(s, c.n, e->dL, n, e->dst), "potrf");
  rc = check_status(e, "potrf(M)");
  if (rc) return rc;
  ENG_TRY(e, cudaMemcpyAsync(e->dWY, e->dY + (long long)j * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, s),
          "copy y");
  ENG_TRY(e, cudaMemcpyAsync(e->dWY + n, e->dXL, sizeof(double) * n * c.wXL, cudaMemcpyDeviceToDevice, s),
          "copy XL");
  ENG_TRY(e, dtrsm_llnn(s, c.n, 1 + c.wXL, e->dL, n, e->dWY, n), "whiten y, XL");
  ENG_TRY(e, null_model_chol(s, c.n, c.wXL, e->dWY, e->dtop, e->dst, 0), "null model");
  rc = check_status(e, "null model");
  if (rc) return rc;
  if (split(e)) {
    if (!e->oz) ENG_TRY(e, ozaki_create(&e->oz, c.n, 1, c.wXL, c.wXR, c.x_b, c.slices, /*eigen=*/0), "split plan");
    ozaki_set_wait_limit(e->oz, e->wait_ns);
    ENG_TRY(e, ozaki_set_chol(e->oz, s, e->dL, e->dWY), "split operands");
    ENG_TRY(e, cudaStreamSynchronize(s), "split operands");
    e->trait_sel = j;
    rc = tune_slices(e);
    if (rc) {
      e->trait_sel = -1;
      return rc;
    }
  }
  e->trait_sel = j;
  return FGLSGPU_OK;
}

int fglsgpu_run_block_device(fglsgpu_engine* e, const double* dXR, int x_inc, double* dB, double* dV,
                             long long bstr, long long vstr) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!e->problem_set) return fail(e, FGLSGPU_ESTATE, "set_problem must precede run_block");
  if (x_inc <= 0 || x_inc > e->cfg.x_b) return fail(e, FGLSGPU_EINVAL, "x_inc=%d outside [1, %d]", x_inc, e->cfg.x_b);
  if (!dXR || !dB || !dV) return fail(e, FGLSGPU_EINVAL, "null block pointer");
  ENG_TRY(e, cudaSetDevice(e->cfg.device), "cudaSetDevice");
  // Device failures accumulate in the status word until fglsgpu_sync.
  return compute_block(e, dXR, GENO_F64, x_inc, dB, dV, bstr, vstr, 0);
}

int fglsgpu_run_block_device_u8(fglsgpu_engine* e, const unsigned char* dXR, int x_inc, double* dB, double* dV,
                                long long bstr, long long vstr) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!e->problem_set) return fail(e, FGLSGPU_ESTATE, "set_problem must precede run_block");
  if (x_inc <= 0 || x_inc > e->cfg.x_b) return fail(e, FGLSGPU_EINVAL, "x_inc=%d outside [1, %d]", x_inc, e->cfg.x_b);
  ENG_TRY(e, cudaSetDevice(e->cfg.device), "cudaSetDevice");
  if (!dXR || !dB || !dV) return fail(e, FGLSGPU_EINVAL, "null block pointer");
  return compute_block(e, dXR, GENO_U8, x_inc, dB, dV, bstr, vstr, 0);
}

int fglsgpu_run_block_device_packed(fglsgpu_engine* e, const unsigned char* dXR2, int x_inc, double* dB, double* dV,
                                    long long bstr, long long vstr) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!e->problem_set) return fail(e, FGLSGPU_ESTATE, "set_problem must precede run_block");
  if (x_inc <= 0 || x_inc > e->cfg.x_b) return fail(e, FGLSGPU_EINVAL, "x_inc=%d outside [1, %d]", x_inc, e->cfg.x_b);
  if (!dXR2 || !dB || !dV) return fail(e, FGLSGPU_EINVAL, "null block pointer");
  ENG_TRY(e, cudaSetDevice(e->cfg.device), "cudaSetDevice");
  return compute_block(e, dXR2, GENO_PACKED, x_inc, dB, dV, bstr, vstr, 0);
}

int fglsgpu_sync(fglsgpu_engine* e) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  ENG_TRY(e, cudaSetDevice(e->cfg.device), "cudaSetDevice");
  const int rc = check_status(e, "block");
  const int rr = reset_status(e);
  return rc ? rc : rr;
}

int fglsgpu_run_block(fglsgpu_engine* e, const double* XR, int x_inc, double* B, double* V, long long bstr,
                      long long vstr) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!e->problem_set) return fail(e, FGLSGPU_ESTATE, "set_problem must precede run_block");
  if (x_inc <= 0 || x_inc > e->cfg.x_b) return fail(e, FGLSGPU_EINVAL, "x_inc=%d outside [1, %d]", x_inc, e->cfg.x_b);
  if (!XR || !B || !V) return fail(e, FGLSGPU_EINVAL, "null block pointer");
  ENG_TRY(e, cudaSetDevice(e->cfg.device), "cudaSetDevice");
  const fglsgpu_config& c = e->cfg;
  const int p = e->p;
  int rc = reset_status(e);
  if (rc) return rc;
  cudaStream_t s = e->comp;
  ENG_TRY(e, cudaMemcpyAsync(e->dX[0], XR, sizeof(double) * c.n * (size_t)x_inc * c.wXR, cudaMemcpyHostToDevice, s),
          "XR upload");
  const long long db = (long long)x_inc * p, dv = (long long)x_inc * p * p;
  rc = compute_block(e, e->dX[0], GENO_F64, x_inc, e->dB[0], e->dV[0], db, dv, 0);
  if (rc) return rc;
  const int nt = out_traits(e);
  ENG_TRY(e, cudaMemcpy2DAsync(B, sizeof(double) * bstr, e->dB[0], sizeof(double) * db, sizeof(double) * db, nt,
                               cudaMemcpyDeviceToHost, s),
          "B download");
  ENG_TRY(e, cudaMemcpy2DAsync(V, sizeof(double) * vstr, e->dV[0], sizeof(double) * dv, sizeof(double) * dv, nt,
                               cudaMemcpyDeviceToHost, s),
          "V download");
  return check_status(e, "block");
}

// Whole-job host API: m SNPs from a host array in the reference layout,
// results into host arrays in the B.out / V.out layout of the active
// traits (eigen: trait j at j*m*p; chol: the selected trait at 0).  Blocks
// of x_b SNPs flow through two device slots: H2D on one stream, compute on
// another, D2H on a third, so copies of block b+1 and b-1 overlap block b.
}  // extern "C"

namespace {

// Whole-job pipeline over host XR (format `fmt`): full (V) or compact (SE,
// P) outputs.
int run_snps_impl(fglsgpu_engine* e, const void* XR, int fmt, long long m, double* B, double* V, double* SE,
                  double* P) {
  const bool compact = V == nullptr;
  const fglsgpu_config& c = e->cfg;
  if (c.variant == FGLSGPU_VARIANT_CHOL && e->trait_sel < 0)
    return fail(e, FGLSGPU_ESTATE, "fglsgpu_select_trait must precede run_snps (chol)");
  ENG_TRY(e, cudaSetDevice(c.device), "cudaSetDevice");
  // On an early error return, copies of neighbouring blocks may still be in
  // flight on the three streams, reading XR or writing B/V/SE/P: wait for
  // all of them (their status is ignored; the first error is reported) so
  // that no copy touches the caller's arrays after this call returns.
  struct DrainOnExit {
    fglsgpu_engine* e;
    bool armed = true;
    ~DrainOnExit() {
      if (!armed) return;
      cudaStreamSynchronize(e->h2d);
      cudaStreamSynchronize(e->comp);
      cudaStreamSynchronize(e->d2h);
      cudaGetLastError();
    }
  } drain{e};
  int rc = reset_status(e);
  if (rc) return rc;
  const int p = e->p, nt = out_traits(e);
  const long long colb = geno_bytes_per_col(fmt, c.n) * c.wXR;  // genotype bytes per SNP
  const unsigned char* xr = (const unsigned char*)XR;
  // Blocks of x_b SNPs, the first two of x_b/4 and x_b/2: the first upload
  // is the only one no compute hides, so it is kept short.
  long long ib = 0;
  for (long long b = 0; ib < m; b++) {
    const int k = (int)(b & 1);
    const int want = b == 0 ? std::max(256, c.x_b / 4) : b == 1 ? std::max(256, c.x_b / 2) : c.x_b;
    const int x = (int)std::min<long long>(std::min(want, c.x_b), m - ib);
    // slot k's input is free once block b-2's compute finished
    ENG_TRY(e, cudaStreamWaitEvent(e->h2d, e->evC[k], 0), "wait");
    ENG_TRY(e, cudaMemcpyAsync(e->dX[k], xr + ib * colb, (size_t)colb * x, cudaMemcpyHostToDevice, e->h2d),
            "XR upload");
    ENG_TRY(e, cudaEventRecord(e->evH[k], e->h2d), "event");
    ENG_TRY(e, cudaStreamWaitEvent(e->comp, e->evH[k], 0), "wait");
    ENG_TRY(e, cudaStreamWaitEvent(e->comp, e->evD[k], 0), "wait");  // outputs of block b-2 downloaded
    const long long db = (long long)x * p, dv = (long long)x * p * p;
    rc = compute_block(e, e->dX[k], fmt, x, e->dB[k], e->dV[k], db, dv, ib);
    if (rc) return rc;
    if (compact)
      ENG_TRY(e, snp_compact(e->comp, x, nt, p, e->dB[k], db, e->dV[k], dv, e->dSE[k], e->dP[k], db), "compact");
    ENG_TRY(e, cudaEventRecord(e->evC[k], e->comp), "event");
    ENG_TRY(e, cudaStreamWaitEvent(e->d2h, e->evC[k], 0), "wait");
    ENG_TRY(e, cudaMemcpy2DAsync(B + ib * p, sizeof(double) * m * p, e->dB[k], sizeof(double) * db,
                                 sizeof(double) * db, nt, cudaMemcpyDeviceToHost, e->d2h),
            "B download");
    if (!compact) {
      ENG_TRY(e, cudaMemcpy2DAsync(V + ib * p * p, sizeof(double) * m * p * p, e->dV[k], sizeof(double) * dv,
                                   sizeof(double) * dv, nt, cudaMemcpyDeviceToHost, e->d2h),
              "V download");
    } else {
      ENG_TRY(e, cudaMemcpy2DAsync(SE + ib * p, sizeof(double) * m * p, e->dSE[k], sizeof(double) * db,
                                   sizeof(double) * db, nt, cudaMemcpyDeviceToHost, e->d2h),
              "SE download");
      ENG_TRY(e, cudaMemcpy2DAsync(P + ib * p, sizeof(double) * m * p, e->dP[k], sizeof(double) * db,
                                   sizeof(double) * db, nt, cudaMemcpyDeviceToHost, e->d2h),
              "P download");
    }
    ENG_TRY(e, cudaEventRecord(e->evD[k], e->d2h), "event");
    ib += x;
  }
  ENG_TRY(e, cudaStreamSynchronize(e->d2h), "run_snps");
  ENG_TRY(e, cudaStreamSynchronize(e->h2d), "run_snps");
  drain.armed = false;
  return check_status(e, "block");
}

}  // namespace

extern "C" {

int fglsgpu_run_snps(fglsgpu_engine* e, const double* XR, long long m, double* B, double* V) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!e->problem_set) return fail(e, FGLSGPU_ESTATE, "set_problem must precede run_snps");
  if (m <= 0 || !XR || !B || !V) return fail(e, FGLSGPU_EINVAL, "invalid run_snps arguments");
  return run_snps_impl(e, XR, GENO_F64, m, B, V, nullptr, nullptr);
}

int fglsgpu_run_snps_u8(fglsgpu_engine* e, const unsigned char* XR, long long m, double* B, double* V) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!e->problem_set) return fail(e, FGLSGPU_ESTATE, "set_problem must precede run_snps");
  if (m <= 0 || !XR || !B || !V) return fail(e, FGLSGPU_EINVAL, "invalid run_snps_u8 arguments");
  return run_snps_impl(e, XR, GENO_U8, m, B, V, nullptr, nullptr);
}

int fglsgpu_run_snps_packed(fglsgpu_engine* e, const unsigned char* XR2, long long m, double* B, double* V) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!e->problem_set) return fail(e, FGLSGPU_ESTATE, "set_problem must precede run_snps");
  if (m <= 0 || !XR2 || !B || !V) return fail(e, FGLSGPU_EINVAL, "invalid run_snps_packed arguments");
  return run_snps_impl(e, XR2, GENO_PACKED, m, B, V, nullptr, nullptr);
}

int fglsgpu_run_snps_compact(fglsgpu_engine* e, const double* XR, long long m, double* B, double* SE, double* P) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!e->problem_set) return fail(e, FGLSGPU_ESTATE, "set_problem must precede run_snps");
  if (m <= 0 || !XR || !B || !SE || !P) return fail(e, FGLSGPU_EINVAL, "invalid run_snps_compact arguments");
  ENG_TRY(e, cudaSetDevice(e->cfg.device), "cudaSetDevice");
  const size_t per = (size_t)out_traits(e) * e->cfg.x_b * e->p;
  for (int k = 0; k < 2; k++) {
    if (!e->dSE[k]) ENG_TRY(e, dalloc(&e->dSE[k], per), "compact buffers");
    if (!e->dP[k]) ENG_TRY(e, dalloc(&e->dP[k], per), "compact buffers");
  }
  return run_snps_impl(e, XR, GENO_F64, m, B, nullptr, SE, P);
}

int fglsgpu_set_precision(fglsgpu_engine* e, int precision) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (precision != FGLSGPU_PREC_FP64 && precision != FGLSGPU_PREC_SPLIT)
    return fail(e, FGLSGPU_EINVAL, "unknown precision %d", precision);
  fglsgpu_config& c = e->cfg;
  if (precision == c.precision) return FGLSGPU_OK;
  ENG_TRY(e, cudaSetDevice(c.device), "cudaSetDevice");
  ENG_TRY(e, cudaStreamSynchronize(e->comp), "set_precision");
  const long long n = c.n, xb = c.x_b, wXR = c.wXR;
  if (precision == FGLSGPU_PREC_FP64 && c.variant == FGLSGPU_VARIANT_EIGEN) {
    if (!e->dWork) ENG_TRY(e, dalloc(&e->dWork, n * xb * wXR), "FP64 buffers");
    if (!e->dQ) ENG_TRY(e, dalloc(&e->dQ, n * xb * wXR * wXR), "FP64 buffers");
  }
  c.precision = precision;
  if (precision == FGLSGPU_PREC_SPLIT && e->problem_set && c.variant == FGLSGPU_VARIANT_EIGEN) {
    if (!e->oz) ENG_TRY(e, ozaki_create(&e->oz, c.n, c.t, c.wXL, c.wXR, c.x_b, c.slices, 1), "split plan");
    ozaki_set_wait_limit(e->oz, e->wait_ns);
    ENG_TRY(e, ozaki_set_eigen(e->oz, e->comp, e->dZ, e->dAYL, e->ddinv), "split operands");
    ENG_TRY(e, cudaStreamSynchronize(e->comp), "split operands");
    const int rc = tune_slices(e);
    if (rc) return rc;
  }
  if (c.variant == FGLSGPU_VARIANT_CHOL) e->trait_sel = -1;  // re-select: the operands differ per path
  return FGLSGPU_OK;
}

int fglsgpu_quad_digits(fglsgpu_engine* e, int* digits) {
  if (!e || !digits) return fail(e, FGLSGPU_EINVAL, "null argument");
  *digits = e->oz ? ozaki_quad_digits(e->oz) : 0;
  return FGLSGPU_OK;
}

int fglsgpu_split_params(fglsgpu_engine* e, int* slices, double* probe_err) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (slices) *slices = e->oz ? ozaki_slices(e->oz, nullptr) : 0;
  if (probe_err) *probe_err = e->tune_err;
  return FGLSGPU_OK;
}

int fglsgpu_set_wait_limit(fglsgpu_engine* e, long long ns) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (ns < 0) return fail(e, FGLSGPU_EINVAL, "wait limit %lld < 0", ns);
  e->wait_ns = (unsigned long long)ns;
  if (e->oz) ozaki_set_wait_limit(e->oz, e->wait_ns);
  return FGLSGPU_OK;
}

int fglsgpu_pvalues_device(fglsgpu_engine* e, const double* dB, const double* dV, int x_inc, long long b_trait_stride,
                           long long v_trait_stride, double* dP, long long p_trait_stride) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!dB || !dV || !dP || x_inc <= 0) return fail(e, FGLSGPU_EINVAL, "invalid p-value arguments");
  ENG_TRY(e, cudaSetDevice(e->cfg.device), "cudaSetDevice");
  const int nt = e->cfg.variant == FGLSGPU_VARIANT_EIGEN ? e->cfg.t : 1;
  ENG_TRY(e, snp_pvalues(e->comp, x_inc, nt, e->p, e->cfg.wXL, dB, b_trait_stride, dV, v_trait_stride, dP,
                         p_trait_stride),
          "p-values");
  return FGLSGPU_OK;
}

// ---------------------------------------------------------------- adjoint
int fglsgpu_adjoint_reset(fglsgpu_engine* e) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  const fglsgpu_config& c = e->cfg;
  if (c.variant != FGLSGPU_VARIANT_EIGEN || c.wXR != 1)
    return fail(e, FGLSGPU_EINVAL, "the adjoint is defined for the eigen variant with wXR = 1");
  if (!e->problem_set) return fail(e, FGLSGPU_ESTATE, "set_problem must precede the adjoint");
  ENG_TRY(e, cudaSetDevice(c.device), "cudaSetDevice");
  const long long n = c.n, t = c.t, xb = c.x_b, wXL = c.wXL, p = e->p;
  if (!e->dWork) ENG_TRY(e, dalloc(&e->dWork, n * xb), "adjoint buffers");
  if (!e->dQ) ENG_TRY(e, dalloc(&e->dQ, n * xb), "adjoint buffers");
  if (!e->adj_ready) {
    cudaError_t r = cudaSuccess;
    auto chk = [&](cudaError_t x) {
      if (r == cudaSuccess) r = x;
    };
    chk(dalloc(&e->aWc, n * 2 * t));
    chk(dalloc(&e->aAYLc, n * t * (1 + wXL)));
    chk(dalloc(&e->aAYLs, n * t * (1 + wXL)));
    chk(dalloc(&e->atopc, t * (wXL + wXL * wXL)));
    chk(dalloc(&e->atops, t * (wXL + wXL * wXL)));
    chk(dalloc(&e->areml, 2 * t));
    chk(dalloc(&e->aGYLc, xb * t * (1 + wXL)));
    chk(dalloc(&e->aGYLs, xb * t * (1 + wXL)));
    chk(dalloc(&e->aGRc, xb * t));
    chk(dalloc(&e->aGRs, xb * t));
    chk(dalloc(&e->acontrib, 2 * t * xb));
    chk(dalloc(&e->ag, t * xb * p));
    chk(dalloc(&e->agR, xb * t));
    chk(dalloc(&e->aacc, 2 * t + t * wXL));
    chk(dalloc(&e->aU, n * t));
    chk(dalloc(&e->aV2, n * t));
    if (r != cudaSuccess) return cuda_fail(e, r, "adjoint buffers");
    e->adj_ready = true;
  }
  cudaStream_t s = e->comp;
  ENG_TRY(e, cudaMemsetAsync(e->aacc, 0, sizeof(double) * (2 * t + t * wXL), s), "adjoint reset");
  ENG_TRY(e, cudaMemsetAsync(e->aU, 0, sizeof(double) * n * t, s), "adjoint reset");
  ENG_TRY(e, adjoint_traits(s, c.n, c.t, c.wXL, e->dW, e->dh, e->dsig, e->dZtXL, e->dZtY, e->ddinv, e->aWc,
                            e->aAYLc, e->aAYLs, e->atopc, e->atops, e->areml),
          "adjoint weights");
  ENG_TRY(e, cudaStreamSynchronize(s), "adjoint reset");
  return FGLSGPU_OK;
}

int fglsgpu_adjoint_block_device(fglsgpu_engine* e, const double* dXR, int x, const double* dBbar, long long bstr) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!e->adj_ready) return fail(e, FGLSGPU_ESTATE, "fglsgpu_adjoint_reset must precede adjoint blocks");
  const fglsgpu_config& c = e->cfg;
  if (x <= 0 || x > c.x_b || !dXR || !dBbar) return fail(e, FGLSGPU_EINVAL, "invalid adjoint block");
  ENG_TRY(e, cudaSetDevice(c.device), "cudaSetDevice");
  const int n = c.n, t = c.t, wXL = c.wXL, p = e->p, nq = t * (1 + wXL);
  cudaStream_t s = e->comp;
  // recompute R = Z^T X and the d-, c- and s-weighted Gram blocks (never stored per SNP)
  ENG_TRY(e, dgemm(s, true, false, n, x, n, 1.0, e->dZ, n, dXR, n, 0.0, e->dWork, n), "Z^T XR");
  ENG_TRY(e, quad_products(s, n, x, 1, e->dWork, n, e->dQ, n), "quad");
  ENG_TRY(e, dgemm(s, true, false, x, nq, n, 1.0, e->dWork, n, e->dAYL, n, 0.0, e->dGYL, x), "gram");
  ENG_TRY(e, dgemm(s, true, false, x, t, n, 1.0, e->dQ, n, e->ddinv, n, 0.0, e->dGR, x), "gram");
  ENG_TRY(e, dgemm(s, true, false, x, nq, n, 1.0, e->dWork, n, e->aAYLc, n, 0.0, e->aGYLc, x), "gram c");
  ENG_TRY(e, dgemm(s, true, false, x, t, n, 1.0, e->dQ, n, e->aWc, n, 0.0, e->aGRc, x), "gram c");
  ENG_TRY(e, dgemm(s, true, false, x, nq, n, 1.0, e->dWork, n, e->aAYLs, n, 0.0, e->aGYLs, x), "gram s");
  ENG_TRY(e, dgemm(s, true, false, x, t, n, 1.0, e->dQ, n, e->aWc + (long long)n * t, n, 0.0, e->aGRs, x),
          "gram s");
  ENG_TRY(e, adjoint_snps(s, p, x, t, wXL, e->dtop, e->dGYL, e->dGR, e->atopc, e->aGYLc, e->aGRc, e->atops,
                          e->aGYLs, e->aGRs, dBbar, bstr, e->acontrib, e->ag, e->dst),
          "adjoint solve");
  ENG_TRY(e, adjoint_reduce(s, x, t, p, wXL, e->acontrib, e->ag, e->aacc, e->agR), "adjoint reduce");
  // U += R gR  (the SNP part of sum_i V_i g_i, accumulated over blocks)
  ENG_TRY(e, dgemm(s, false, false, n, t, x, 1.0, e->dWork, n, e->agR, x, 1.0, e->aU, n), "dy accumulate");
  return FGLSGPU_OK;
}

int fglsgpu_adjoint_read(fglsgpu_engine* e, double* dh, double* dsigma, double* dY) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!e->adj_ready) return fail(e, FGLSGPU_ESTATE, "no adjoint accumulated");
  const fglsgpu_config& c = e->cfg;
  ENG_TRY(e, cudaSetDevice(c.device), "cudaSetDevice");
  const int n = c.n, t = c.t;
  cudaStream_t s = e->comp;
  int rc = check_status(e, "adjoint");
  if (rc) return rc;
  if (dY) {
    ENG_TRY(e, adjoint_ybar(s, n, t, c.wXL, e->ddinv, e->dZtXL, e->aacc, e->aU, e->aV2), "dy");
    // dY = Z V2 (original basis), through dQ as scratch (n x t <= n x x_b when t <= x_b)
    double* out = e->dQ;
    if ((long long)t > (long long)c.x_b) return fail(e, FGLSGPU_EINVAL, "dy needs t <= x_b");
    ENG_TRY(e, dgemm(s, false, false, n, t, n, 1.0, e->dZ, n, e->aV2, n, 0.0, out, n), "dy");
    ENG_TRY(e, cudaMemcpyAsync(dY, out, sizeof(double) * (size_t)n * t, cudaMemcpyDeviceToHost, s), "dy");
  }
  std::vector<double> acc(2 * t);
  ENG_TRY(e, cudaMemcpyAsync(acc.data(), e->aacc, sizeof(double) * 2 * t, cudaMemcpyDeviceToHost, s), "dh");
  ENG_TRY(e, cudaStreamSynchronize(s), "adjoint read");
  for (int j = 0; j < t; j++) {
    if (dh) dh[j] = acc[j];
    if (dsigma) dsigma[j] = acc[t + j];
  }
  return FGLSGPU_OK;
}

int fglsgpu_reml(fglsgpu_engine* e, double* loglik, double* dloglik_dh) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!e->adj_ready) return fail(e, FGLSGPU_ESTATE, "fglsgpu_adjoint_reset computes the REML terms first");
  const int t = e->cfg.t;
  ENG_TRY(e, cudaSetDevice(e->cfg.device), "cudaSetDevice");
  std::vector<double> r(2 * t);
  ENG_TRY(e, cudaMemcpy(r.data(), e->areml, sizeof(double) * 2 * t, cudaMemcpyDeviceToHost), "reml");
  for (int j = 0; j < t; j++) {
    if (loglik) loglik[j] = r[j];
    if (dloglik_dh) dloglik_dh[j] = r[t + j];
  }
  return FGLSGPU_OK;
}

int fglsgpu_reml_fit(fglsgpu_engine* e, double h_lo, double h_hi, int grid, double* h, double* sigma,
                     double* loglik, double* dloglik_dh) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!e->problem_set) return fail(e, FGLSGPU_ESTATE, "set_problem must precede reml_fit");
  const fglsgpu_config& c = e->cfg;
  if (c.variant != FGLSGPU_VARIANT_EIGEN) return fail(e, FGLSGPU_EINVAL, "reml_fit needs the eigen variant");
  if (grid == 0) grid = 64;
  if (!(h_lo >= 0.0 && h_lo < h_hi && h_hi <= 1.0))
    return fail(e, FGLSGPU_EINVAL, "need 0 <= h_lo < h_hi <= 1 (h_lo=%g h_hi=%g)", h_lo, h_hi);
  if (grid < 2 || grid > FGLS_REML_MAX_GRID) return fail(e, FGLSGPU_EINVAL, "grid=%d outside [2, %d]", grid, FGLS_REML_MAX_GRID);
  if (c.n <= c.wXL) return fail(e, FGLSGPU_EINVAL, "n=%d must exceed wXL=%d", c.n, c.wXL);
  ENG_TRY(e, cudaSetDevice(c.device), "cudaSetDevice");
  const int t = c.t;
  int rc = reset_status(e);
  if (rc) return rc;
  double* dout = nullptr;
  ENG_TRY(e, dalloc(&dout, 4 * (size_t)t), "reml_fit output");
  std::vector<double> r(4 * (size_t)t);
  cudaError_t ce = reml_fit(e->comp, c.n, t, c.wXL, e->dW, e->dZtXL, e->dZtY, h_lo, h_hi, grid, dout, e->dst);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(r.data(), dout, sizeof(double) * 4 * t, cudaMemcpyDeviceToHost, e->comp);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(e->comp);
  cudaFree(dout);
  if (ce != cudaSuccess) return cuda_fail(e, ce, "reml_fit");
  ENG_TRY(e, cudaMemcpy(e->hst, e->dst, sizeof(DevStatus), cudaMemcpyDeviceToHost), "status copy");
  const DevStatus st = *e->hst;
  if (st.code != FGLSGPU_OK) {
    reset_status(e);
    return fail(e, st.code, "reml_fit: trait %lld: the covariate Gram is not positive definite or "
                "1 + h (w - 1) <= 0 inside [%g, %g]", st.idx, h_lo, h_hi);
  }
  for (int j = 0; j < t; j++) {
    if (h) h[j] = r[j];
    if (sigma) sigma[j] = r[t + j];
    if (loglik) loglik[j] = r[2 * t + j];
    if (dloglik_dh) dloglik_dh[j] = r[3 * t + j];
  }
  return FGLSGPU_OK;
}

int fglsgpu_set_hsigma(fglsgpu_engine* e, const double* h, const double* sigma) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (!e->problem_set) return fail(e, FGLSGPU_ESTATE, "set_problem must precede set_hsigma");
  if (!h || !sigma) return fail(e, FGLSGPU_EINVAL, "null input pointer");
  const fglsgpu_config& c = e->cfg;
  for (int j = 0; j < c.t; j++)
    if (!(h[j] >= 0.0 && h[j] <= 1.0) || !(sigma[j] > 0.0))
      return fail(e, FGLSGPU_EINVAL, "trait %d: need 0 <= h <= 1 and sigma > 0 (h=%g sigma=%g)", j, h[j], sigma[j]);
  ENG_TRY(e, cudaSetDevice(c.device), "cudaSetDevice");
  cudaStream_t s = e->comp;
  ENG_TRY(e, cudaStreamSynchronize(s), "set_hsigma");
  e->hh.assign(h, h + c.t);
  e->hs.assign(sigma, sigma + c.t);
  e->adj_ready = false;
  ENG_TRY(e, cudaMemcpyAsync(e->dh, h, sizeof(double) * c.t, cudaMemcpyHostToDevice, s), "upload h");
  ENG_TRY(e, cudaMemcpyAsync(e->dsig, sigma, sizeof(double) * c.t, cudaMemcpyHostToDevice, s), "upload sigma");
  if (c.variant != FGLSGPU_VARIANT_EIGEN) {
    e->trait_sel = -1;  // the next select_trait builds and factors M_j with the new values
    ENG_TRY(e, cudaStreamSynchronize(s), "set_hsigma");
    return FGLSGPU_OK;
  }
  int rc = reset_status(e);
  if (rc) return rc;
  e->problem_set = false;
  ENG_TRY(e, eigen_traits(s, c.n, c.t, c.wXL, e->dW, e->dh, e->dsig, e->dZtXL, e->dZtY, e->ddinv, e->dAYL,
                          e->dtop, e->dst),
          "trait weights");
  rc = check_status(e, "eigen setup");
  if (rc) return rc;
  if (split(e)) {
    if (!e->oz) ENG_TRY(e, ozaki_create(&e->oz, c.n, c.t, c.wXL, c.wXR, c.x_b, c.slices, 1), "split plan");
    ozaki_set_wait_limit(e->oz, e->wait_ns);
    ENG_TRY(e, ozaki_set_eigen(e->oz, s, e->dZ, e->dAYL, e->ddinv), "split operands");
    ENG_TRY(e, cudaStreamSynchronize(s), "split operands");
    rc = tune_slices(e);
    if (rc) return rc;
  }
  ENG_TRY(e, cudaStreamSynchronize(s), "set_hsigma");
  e->problem_set = true;
  return FGLSGPU_OK;
}

int fglsgpu_profile(fglsgpu_engine* e, int enable) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  ENG_TRY(e, cudaSetDevice(e->cfg.device), "cudaSetDevice");
  ENG_TRY(e, cudaStreamSynchronize(e->comp), "profile");
  for (auto& ev : e->pev_live) e->pev_pool.push_back(ev);
  e->pev_live.clear();
  for (int k = 0; k < FGLSGPU_PROF_CLASSES; k++) {
    e->prof_ms[k] = 0.0;
    e->prof_cnt[k] = 0;
  }
  e->prof = enable != 0;
  return FGLSGPU_OK;
}

int fglsgpu_profile_read(fglsgpu_engine* e, double* ms, long long* count) {
  if (!e || !ms || !count) return fail(e, FGLSGPU_EINVAL, "null argument");
  ENG_TRY(e, cudaSetDevice(e->cfg.device), "cudaSetDevice");
  for (auto& ev : e->pev_live) {
    ENG_TRY(e, cudaEventSynchronize(ev.b), "profile event");
    float t = 0.f;
    ENG_TRY(e, cudaEventElapsedTime(&t, ev.a, ev.b), "profile event");
    e->prof_ms[ev.cls] += t;
    e->prof_cnt[ev.cls] += 1;
    e->pev_pool.push_back(ev);
  }
  e->pev_live.clear();
  for (int k = 0; k < FGLSGPU_PROF_CLASSES; k++) {
    ms[k] = e->prof_ms[k];
    count[k] = e->prof_cnt[k];
  }
  return FGLSGPU_OK;
}

int fglsgpu_get_res_sigma(fglsgpu_engine* e, double* out) {
  if (!e || !out) return fail(e, FGLSGPU_EINVAL, "null argument");
  if (!e->problem_set) return fail(e, FGLSGPU_ESTATE, "set_problem first");
  ENG_TRY(e, cudaSetDevice(e->cfg.device), "cudaSetDevice");
  const int nt = out_traits(e);
  for (int j = 0; j < nt; j++)
    ENG_TRY(e, cudaMemcpy(out + j, e->dtop + (long long)j * e->topw + e->topw - 1, sizeof(double),
                          cudaMemcpyDeviceToHost),
            "res_sigma");
  return FGLSGPU_OK;
}

int fglsgpu_get_eigen(fglsgpu_engine* e, double* W, double* Z) {
  if (!e) return fail(nullptr, FGLSGPU_EINVAL, "null engine");
  if (e->cfg.variant != FGLSGPU_VARIANT_EIGEN || !e->problem_set) return fail(e, FGLSGPU_ESTATE, "no eigendecomposition");
  ENG_TRY(e, cudaSetDevice(e->cfg.device), "cudaSetDevice");
  const long long n = e->cfg.n;
  if (W) ENG_TRY(e, cudaMemcpy(W, e->dW, sizeof(double) * n, cudaMemcpyDeviceToHost), "W");
  if (Z) ENG_TRY(e, cudaMemcpy(Z, e->dZ, sizeof(double) * n * n, cudaMemcpyDeviceToHost), "Z");
  return FGLSGPU_OK;
}

}  // extern "C"
