// Batched uneven cohorts: many independent chol-variant FGLS problems (each
// with its own n, p, Phi, XL, traits) advanced together, one SNP block of
// every cohort per step.
//
// Per (cohort, trait) problem, once (FP64): M = s (h Phi + (1 - h) I)
// (src/fgls_chol.c:251-262), L = chol(M), the null model of
// [y~ | XL~] = L^-1 [y | XL] (src/fgls_chol.c:273-325), L^-1 by trailing
// panel TRSMs, and the split operand [L^-1 ; (L^-T [y~ | XL~])^T] cut into
// FP8 (E4M3) five-bit digit slices, resident in HBM for the whole job.
//
// Per step (one launch each, whatever the number of cohorts):
//   1. grouped_genotypes: every cohort's block -> its E4M3 operand
//   2. ozaki_grouped_gemm_kernel: one persistent launch (a CTA per SM) over
//      the tiles of all problems, listed longest first and taken from a
//      launch-wide counter -> X~ = L^-1 X, summed as R^2 over 32-row groups
//      in the last pass (X~ itself is not written), and the Gram rows
//      x~'y~, x~'XL~
//   3. unit_gram_grouped: x~'x~ per (problem, SNP), the group sums added in
//      double-FP32
//   4. snp_solve_grouped<p>: per distinct p, the p x p solves of all problems
// The per-step inputs (genotype pointer, SNP count, output pointers of each
// cohort) are one small table copied from pinned host memory at the start of
// the step, so the whole step is captured once as a CUDA graph and replayed
// (a ring of NSLOT graphs, one per pinned table).
//
// Autotuning at creation (fglsgpu_batch_config x_b = 0 and/or slices = 0):
//   slices: the smallest S in 5..9 whose beta on a probe block (hashed
//           genotypes) is within tol/8 of the FP64 path (TRSM, skinny Gram,
//           solve) for every problem;
//   x_b:    the candidate SNP block (1024 .. 8192) with the highest measured
//           tests/s on one step;
//   tile:   at that block, the faster of the grouped GEMM's two tile shapes
//           (256 x 256 over CTA pairs with 2-SM MMAs, 128 x 256 on one SM).
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <string>
#include <vector>

#include "fgls_batch.cuh"
#include "fgls_common.cuh"
#include "fgls_kernels.cuh"
#include "fgls_ozaki.cuh"
#include "fgls_selfgram.cuh"

using namespace fgls;

namespace {

constexpr int S_BUILT = 9;     // FP8 five-bit digit slices cut at setup; fewer may be used
constexpr int S_MIN_TUNE = 5;  // smallest slice count the autotuner tries
constexpr int PROBE = 256;     // SNPs of the autotuning probe block
constexpr int XB_MAX = 8192;   // largest autotuned SNP block
// Pinned step tables (and step graphs) in the ring: the host fills table k
// once the step that last used it has finished, so it may run NSLOT - 1
// steps ahead of the device and a host-side stall of that length costs no
// device time.
constexpr int NSLOT = 8;

struct Cohort {
  int n = 0, wXL = 0, p = 0, t = 0;
  int Kpad = 0, Ncap = 0;
  uint8_t* G = nullptr;           // E4M3 genotype operand (Ncap x Kpad)
  unsigned char* probe = nullptr; // PROBE x n hashed genotypes
};

struct Problem {
  int c = 0, j = 0;
  int M = 0, Mpad = 0;
  uint8_t* A = nullptr;        // S_BUILT x Mpad x Kpad E4M3 digit slices
  double* scale_built = nullptr;  // row scales of the S_BUILT-slice cut
  double* scale = nullptr;     // row scales for the slices in use
  double* top = nullptr;       // null model (wXL + wXL^2 + 1)
  double* C = nullptr;         // Mpad x Ncap split GEMM output
  float2* Q = nullptr;         // Mpad/32 x Ncap sums of R^2 over 32-row groups (ld Ncap)
  double* GR = nullptr;        // Ncap
  double* ref = nullptr;       // PROBE x p FP64-path beta on the probe block
};

}  // namespace

struct fglsgpu_batch {
  fglsgpu_batch_config cfg{};
  std::vector<Cohort> co;
  std::vector<Problem> pr;
  int x_b = 0, S = 0, ncap = 0;
  bool pair_tiles = true;  // grouped GEMM tile shape: 256 x 256 over CTA pairs, else 128 x 256
  cudaStream_t s = nullptr;
  DevStatus* dst = nullptr;
  DevStatus* hst = nullptr;
  int* derr = nullptr;
  GenoCohort* dgeno = nullptr;
  UnitGramProblem* dunit = nullptr;
  SolveProblem* dsolve = nullptr;
  int* dplist = nullptr;
  int pcount[FGLS_MAX_P + 1] = {0}, poff[FGLS_MAX_P + 1] = {0};
  // per-step table: StepCohort[C] followed by int x[C]
  size_t step_bytes = 0;
  void* hstep[NSLOT] = {};
  void* dstep = nullptr;
  cudaEvent_t slot_done[NSLOT] = {};
  int slot = 0;
  GroupedGemm* gg = nullptr;
  cudaGraphExec_t gexec[NSLOT] = {};
  long long graph_launches = 0;  // kernels per replayed step
  double tune_err = -1.0;
  std::vector<double> tune_rates;
  std::string err;
  // per-stage timing (steps then run without the graph): events around the
  // genotype, split GEMM, quadratic Gram and solve stages
  bool prof = false;
  std::vector<cudaEvent_t> pev;  // 5 per profiled step
  double prof_ms[4] = {0, 0, 0, 0};
  long long prof_steps = 0;

  StepCohort* dsc() const { return (StepCohort*)dstep; }
  int* dcols() const { return (int*)((char*)dstep + sizeof(StepCohort) * co.size()); }
};

namespace {

thread_local std::string tl_err;

int bfail(fglsgpu_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  tl_err = buf;
  return code;
}

#define B_TRY(b, expr, what)                                                                                  \
  do {                                                                                                        \
    cudaError_t _c = (expr);                                                                                  \
    if (_c != cudaSuccess)                                                                                    \
      return bfail(b, _c == cudaErrorMemoryAllocation ? FGLSGPU_ENOMEM : FGLSGPU_ECUDA, "%s: %s (%s)", what, \
                   cudaGetErrorString(_c), cudaGetErrorName(_c));                                             \
  } while (0)

template <class T>
cudaError_t dalloc(T** p, size_t count) {
  *p = nullptr;
  return cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(count, 1));
}

// genotype (0/1/2) of the probe block: a fixed integer hash of (cohort, SNP, individual)
__global__ void probe_genotypes_kernel(int c, int n, int x, unsigned char* out, double* out64) {
  const long long total = (long long)x * n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    unsigned int h = (unsigned int)(e * 2654435761u) ^ (unsigned int)(c * 40503u + 12345u);
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    const unsigned char g = (unsigned char)(h % 3u);
    if (out) out[e] = g;
    if (out64) out64[e] = (double)g;
  }
}

int check_status(fglsgpu_batch* b, const char* stage) {
  B_TRY(b, cudaMemcpyAsync(b->hst, b->dst, sizeof(DevStatus), cudaMemcpyDeviceToHost, b->s), "status copy");
  int herr = 0;
  B_TRY(b, cudaMemcpyAsync(&herr, b->derr, sizeof(int), cudaMemcpyDeviceToHost, b->s), "status copy");
  B_TRY(b, cudaStreamSynchronize(b->s), stage);
  const DevStatus st = *b->hst;
  B_TRY(b, cudaMemsetAsync(b->dst, 0, sizeof(DevStatus), b->s), "status reset");
  B_TRY(b, cudaMemsetAsync(b->derr, 0, sizeof(int), b->s), "status reset");
  if (herr) return bfail(b, FGLSGPU_ETIMEOUT, "device wait expired in %s (site %d)", stage, herr);
  if (st.code == FGLSGPU_OK) return FGLSGPU_OK;
  if (st.code == FGLSGPU_ENOTSPD && (st.info >> 8) > 0)
    return bfail(b, FGLSGPU_ENOTSPD, "dpotrf(V) failed (info: %d) - cohort %d, i: %lld", st.info & 255,
                 (st.info >> 8) - 1, st.idx);
  return bfail(b, st.code, "device status %d in %s (info %d, item %lld)", st.code, stage, st.info, st.idx);
}

void free_batch(fglsgpu_batch* b) {
  for (auto& c : b->co) {
    if (c.G) cudaFree(c.G);
    if (c.probe) cudaFree(c.probe);
  }
  for (auto& q : b->pr) {
    void* ptrs[] = {q.A, q.scale_built, q.scale, q.top, q.C, q.Q, q.GR, q.ref};
    for (void* v : ptrs)
      if (v) cudaFree(v);
  }
  void* ptrs[] = {b->dst, b->derr, b->dgeno, b->dunit, b->dsolve, b->dplist, b->dstep};
  for (void* v : ptrs)
    if (v) cudaFree(v);
  for (int k = 0; k < NSLOT; k++) {
    if (b->hstep[k]) cudaFreeHost(b->hstep[k]);
    if (b->slot_done[k]) cudaEventDestroy(b->slot_done[k]);
    if (b->gexec[k]) cudaGraphExecDestroy(b->gexec[k]);
  }
  if (b->hst) cudaFreeHost(b->hst);
  for (cudaEvent_t e : b->pev) cudaEventDestroy(e);
  if (b->gg) grouped_gemm_destroy(b->gg);
  if (b->s) cudaStreamDestroy(b->s);
}

// (Re)builds the grouped GEMM for S slices and x_b columns, and the row
// scales for S.
int configure(fglsgpu_batch* b, int S, int x_b) {
  std::vector<GroupedGemmDesc> d(b->pr.size());
  for (size_t k = 0; k < b->pr.size(); k++) {
    Problem& q = b->pr[k];
    const Cohort& c = b->co[q.c];
    B_TRY(b, split_rescale_rows(b->s, q.Mpad, q.scale_built, S_BUILT, S, q.scale), "row scales");
    d[k] = GroupedGemmDesc{q.A, S, S_BUILT, q.M, q.Mpad, c.Kpad, c.n, c.n, q.scale, c.G, c.Ncap, q.C, q.Q,
                           b->ncap, q.c};
  }
  B_TRY(b, cudaStreamSynchronize(b->s), "row scales");
  if (b->gg) grouped_gemm_destroy(b->gg);
  b->gg = nullptr;
  for (int k = 0; k < NSLOT; k++)
    if (b->gexec[k]) {
      cudaGraphExecDestroy(b->gexec[k]);
      b->gexec[k] = nullptr;
    }
  B_TRY(b, grouped_gemm_create(&b->gg, d.data(), (int)d.size(), x_b, b->derr, b->pair_tiles), "grouped GEMM plan");
  b->S = S;
  b->x_b = x_b;
  return FGLSGPU_OK;
}

// The kernels of one step, reading the per-step table at b->dstep; ev (5
// events or null) brackets the stages.
cudaError_t enqueue_step(fglsgpu_batch* b, cudaStream_t s, const void* host_table, cudaEvent_t* ev = nullptr) {
  auto mark = [&](int k) { return ev ? cudaEventRecord(ev[k], s) : cudaSuccess; };
  FGLS_CUDA_TRY(cudaMemcpyAsync(b->dstep, host_table, b->step_bytes, cudaMemcpyHostToDevice, s));
  FGLS_CUDA_TRY(mark(0));
  FGLS_CUDA_TRY(grouped_genotypes(s, b->dgeno, b->dsc(), (int)b->co.size(), b->cfg.genotypes_u8 != 0));
  FGLS_CUDA_TRY(mark(1));
  FGLS_CUDA_TRY(grouped_gemm_run(b->gg, s, b->dcols()));
  FGLS_CUDA_TRY(mark(2));
  FGLS_CUDA_TRY(unit_gram_grouped(s, b->dunit, (int)b->pr.size(), b->dsc(), b->x_b));
  FGLS_CUDA_TRY(mark(3));
  for (int p = 2; p <= FGLS_MAX_P; p++)
    if (b->pcount[p])
      FGLS_CUDA_TRY(snp_solve_grouped(s, p, b->dsolve, b->dplist + b->poff[p], b->pcount[p], b->x_b, b->dsc(), b->dst));
  FGLS_CUDA_TRY(mark(4));
  return cudaGetLastError();
}

int capture_graphs(fglsgpu_batch* b) {
  for (int k = 0; k < NSLOT; k++) {
    cudaGraph_t g = nullptr;
    const long long l0 = g_launches.load();
    B_TRY(b, cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal), "graph capture");
    const cudaError_t e1 = enqueue_step(b, b->s, b->hstep[k]);
    const cudaError_t e2 = cudaStreamEndCapture(b->s, &g);
    if (e1 != cudaSuccess || e2 != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      return bfail(b, FGLSGPU_ECUDA, "graph capture: %s", cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
    }
    b->graph_launches = g_launches.load() - l0;
    g_launches.fetch_sub(b->graph_launches);  // counted when replayed
    const cudaError_t e3 = cudaGraphInstantiate(&b->gexec[k], g, 0);
    cudaGraphDestroy(g);
    B_TRY(b, e3, "graph instantiate");
  }
  return FGLSGPU_OK;
}

// Fills the next pinned table and runs one step on b->s.
int launch_step(fglsgpu_batch* b, const void* const* dX, const int* x, double* const* dB, double* const* dV,
                const long long* base) {
  const int k = b->slot;
  B_TRY(b, cudaEventSynchronize(b->slot_done[k]), "step slot");
  const int C = (int)b->co.size();
  StepCohort* sc = (StepCohort*)b->hstep[k];
  int* cols = (int*)((char*)b->hstep[k] + sizeof(StepCohort) * C);
  for (int c = 0; c < C; c++) {
    sc[c] = StepCohort{dX[c], dB[c], dV[c], base ? base[c] : 0, x[c], 0};
    cols[c] = x[c];
  }
  if (b->prof) {
    const size_t k0 = b->pev.size();
    b->pev.resize(k0 + 5);
    for (size_t e = k0; e < k0 + 5; e++) B_TRY(b, cudaEventCreate(&b->pev[e]), "profile events");
    B_TRY(b, enqueue_step(b, b->s, b->hstep[k], &b->pev[k0]), "step");
  } else if (b->cfg.use_graph) {
    if (!b->gexec[0]) {
      const int rc = capture_graphs(b);
      if (rc) return rc;
    }
    B_TRY(b, cudaGraphLaunch(b->gexec[k], b->s), "graph launch");
    g_launches.fetch_add(b->graph_launches);
  } else {
    B_TRY(b, enqueue_step(b, b->s, b->hstep[k]), "step");
  }
  B_TRY(b, cudaEventRecord(b->slot_done[k], b->s), "step slot");
  b->slot = (b->slot + 1) % NSLOT;
  return FGLSGPU_OK;
}

int validate_args(fglsgpu_batch* b, const int* x, const void* const* dX, double* const* dB, double* const* dV) {
  if (!x || !dX || !dB || !dV) return bfail(b, FGLSGPU_EINVAL, "null step argument");
  for (size_t c = 0; c < b->co.size(); c++) {
    if (x[c] < 0 || x[c] > b->x_b) return bfail(b, FGLSGPU_EINVAL, "cohort %zu: x=%d outside [0, %d]", c, x[c], b->x_b);
    if (x[c] > 0 && (!dX[c] || !dB[c] || !dV[c])) return bfail(b, FGLSGPU_EINVAL, "cohort %zu: null pointer", c);
  }
  return FGLSGPU_OK;
}

// The probe block through the split path at S slices: max over problems and
// tests of |beta - beta_fp64| / |beta_fp64| (2-norms).
int probe_error(fglsgpu_batch* b, int S, double* out) {
  int rc = configure(b, S, PROBE);
  if (rc) return rc;
  const int C = (int)b->co.size();
  std::vector<const void*> X(C);
  std::vector<int> x(C, PROBE);
  std::vector<double*> B(C), V(C);
  std::vector<double> hB;
  for (int c = 0; c < C; c++) {
    X[c] = b->co[c].probe;
    B_TRY(b, dalloc(&B[c], (size_t)b->co[c].t * PROBE * b->co[c].p), "probe buffers");
    B_TRY(b, dalloc(&V[c], (size_t)b->co[c].t * PROBE * b->co[c].p * b->co[c].p), "probe buffers");
  }
  const int save_graph = b->cfg.use_graph, save_u8 = b->cfg.genotypes_u8;
  b->cfg.use_graph = 0;
  b->cfg.genotypes_u8 = 1;
  rc = launch_step(b, X.data(), x.data(), B.data(), V.data(), nullptr);
  b->cfg.use_graph = save_graph;
  b->cfg.genotypes_u8 = save_u8;
  if (!rc) rc = check_status(b, "autotune probe");
  double worst = 0.0;
  for (size_t k = 0; k < b->pr.size() && !rc; k++) {
    const Problem& q = b->pr[k];
    const int p = b->co[q.c].p;
    std::vector<double> got((size_t)PROBE * p), ref((size_t)PROBE * p);
    if (cudaMemcpy(got.data(), B[q.c] + (size_t)q.j * PROBE * p, sizeof(double) * got.size(),
                   cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(ref.data(), q.ref, sizeof(double) * ref.size(), cudaMemcpyDeviceToHost) != cudaSuccess) {
      rc = bfail(b, FGLSGPU_ECUDA, "probe readback");
      break;
    }
    for (int i = 0; i < PROBE; i++) {
      double num = 0.0, den = 0.0;
      for (int a = 0; a < p; a++) {
        const double d = got[(size_t)i * p + a] - ref[(size_t)i * p + a];
        num += d * d;
        den += ref[(size_t)i * p + a] * ref[(size_t)i * p + a];
      }
      const double e = den > 0.0 ? std::sqrt(num / den) : std::sqrt(num);
      if (!(e <= worst)) worst = std::isnan(e) ? INFINITY : std::max(worst, e);
    }
  }
  for (int c = 0; c < C; c++) {
    cudaFree(B[c]);
    cudaFree(V[c]);
  }
  *out = worst;
  return rc;
}

// Tests/s of one step at x_b columns (u8 genotypes replicated from the probe).
int time_step(fglsgpu_batch* b, int x_b, double* rate) {
  int rc = configure(b, b->S, x_b);
  if (rc) return rc;
  const int C = (int)b->co.size();
  std::vector<const void*> X(C);
  std::vector<unsigned char*> Xo(C, nullptr);
  std::vector<int> x(C, x_b);
  std::vector<double*> B(C, nullptr), V(C, nullptr);
  double tests = 0.0;
  for (int c = 0; c < C && !rc; c++) {
    const Cohort& co = b->co[c];
    if (cudaMalloc(&Xo[c], (size_t)x_b * co.n) != cudaSuccess ||
        dalloc(&B[c], (size_t)co.t * x_b * co.p) != cudaSuccess ||
        dalloc(&V[c], (size_t)co.t * x_b * co.p * co.p) != cudaSuccess) {
      rc = bfail(b, FGLSGPU_ENOMEM, "autotune buffers");
      break;
    }
    for (int r = 0; r < x_b; r += PROBE)
      cudaMemcpyAsync(Xo[c] + (size_t)r * co.n, co.probe, (size_t)std::min(PROBE, x_b - r) * co.n,
                      cudaMemcpyDeviceToDevice, b->s);
    X[c] = Xo[c];
    tests += (double)x_b * co.t;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (!rc) {
    const int save_u8 = b->cfg.genotypes_u8;
    b->cfg.genotypes_u8 = 1;
    const int save_graph = b->cfg.use_graph;
    b->cfg.use_graph = 0;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    rc = launch_step(b, X.data(), x.data(), B.data(), V.data(), nullptr);  // warm
    if (!rc) cudaEventRecord(e0, b->s);
    for (int r = 0; r < 2 && !rc; r++) rc = launch_step(b, X.data(), x.data(), B.data(), V.data(), nullptr);
    if (!rc) cudaEventRecord(e1, b->s);
    if (!rc) rc = check_status(b, "autotune timing");
    float ms = 0.0f;
    if (!rc) cudaEventElapsedTime(&ms, e0, e1);
    *rate = ms > 0.0f ? 2.0 * tests / (ms / 1e3) : 0.0;
    b->cfg.genotypes_u8 = save_u8;
    b->cfg.use_graph = save_graph;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamSynchronize(b->s);
  for (int c = 0; c < C; c++) {
    if (Xo[c]) cudaFree(Xo[c]);
    if (B[c]) cudaFree(B[c]);
    if (V[c]) cudaFree(V[c]);
  }
  return rc;
}

// One (cohort, trait) problem: FP64 factorisation, null model, split operand,
// FP64-path beta on the probe block.  Scratch: L, Linv, LinvT (n x n), WY,
// U (n x (1+wXL)), X64 / GYL / GR64 / Bp / Vp for the probe.
struct Scratch {
  double *L = nullptr, *Linv = nullptr, *LinvT = nullptr, *WY = nullptr, *U = nullptr;
  double *X64 = nullptr, *GYL = nullptr, *GR64 = nullptr, *Vp = nullptr;
  DevStatus* st = nullptr;
  cudaStream_t s = nullptr;
  cudaError_t alloc(int nmax, int wmax) {
    const size_t nn = (size_t)nmax * nmax;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    for (double** v : {&L, &Linv, &LinvT})
      if (e == cudaSuccess) e = dalloc(v, nn);
    if (e == cudaSuccess) e = dalloc(&WY, (size_t)nmax * (1 + wmax));
    if (e == cudaSuccess) e = dalloc(&U, (size_t)nmax * (1 + wmax));
    if (e == cudaSuccess) e = dalloc(&X64, (size_t)nmax * PROBE);
    if (e == cudaSuccess) e = dalloc(&GYL, (size_t)PROBE * (1 + wmax));
    if (e == cudaSuccess) e = dalloc(&GR64, (size_t)PROBE);
    if (e == cudaSuccess) e = dalloc(&Vp, (size_t)PROBE * FGLS_MAX_P * FGLS_MAX_P);
    if (e == cudaSuccess) e = dalloc(&st, 1);
    if (e == cudaSuccess) e = cudaMemset(st, 0, sizeof(DevStatus));
    return e;
  }
  void release() {
    void* ptrs[] = {L, Linv, LinvT, WY, U, X64, GYL, GR64, Vp, st};
    for (void* v : ptrs)
      if (v) cudaFree(v);
    if (s) cudaStreamDestroy(s);
  }
};

// Cohort inputs shared by its traits' setup streams.
struct CohortInputs {
  double *Phi = nullptr, *XL = nullptr, *Y = nullptr;
};

// Enqueues the whole one-off setup of problem q on w.s (no host waits): M,
// potrf, whitening, null model, split operand, FP64-path probe betas.  Data
// failures land in w.st and are read after the cohort.
cudaError_t setup_problem(fglsgpu_batch* b, Scratch& w, const CohortInputs& ci, Problem& q,
                          const fglsgpu_cohort& in) {
  const Cohort& c = b->co[q.c];
  const int n = c.n, wXL = c.wXL, p = c.p;
  cudaStream_t s = w.s;
  const double h = in.h[q.j], sg = in.sigma[q.j];
  probe_genotypes_kernel<<<256, 256, 0, s>>>(q.c, n, PROBE, q.j == 0 ? b->co[q.c].probe : nullptr, w.X64);
  FGLS_CUDA_TRY(build_shifted(s, n, ci.Phi, n, h * sg, (1.0 - h) * sg, w.L, n));
  FGLS_CUDA_TRY(dpotrf_lower(s, n, w.L, n, w.st));
  FGLS_CUDA_TRY(cudaMemcpyAsync(w.WY, ci.Y + (size_t)q.j * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  FGLS_CUDA_TRY(cudaMemcpyAsync(w.WY + n, ci.XL, sizeof(double) * n * wXL, cudaMemcpyDeviceToDevice, s));
  FGLS_CUDA_TRY(dtrsm_llnn(s, n, 1 + wXL, w.L, n, w.WY, n));
  FGLS_CUDA_TRY(null_model_chol(s, n, wXL, w.WY, q.top, w.st, 0));
  FGLS_CUDA_TRY(split_chol_operand(s, n, wXL, w.L, w.WY, S_BUILT, q.Mpad, c.Kpad, q.A, q.scale_built, w.Linv, w.LinvT,
                                   w.U));
  // FP64 path on the probe block (the reference's chol per-block loop)
  FGLS_CUDA_TRY(dtrsm_llnn(s, n, PROBE, w.L, n, w.X64, n));
  FGLS_CUDA_TRY(gram_skinny(s, n, PROBE, wXL, 1, w.X64, n, w.WY, w.GYL, w.GR64));
  FGLS_CUDA_TRY(snp_solve(s, p, PROBE, 1, wXL, q.top, w.GYL, 1, PROBE, w.GR64, PROBE, q.ref, 0, w.Vp, 0, w.st, 0));
  return cudaGetLastError();
}

}  // namespace

extern "C" {

const char* fglsgpu_batch_last_error(const fglsgpu_batch* b) { return b ? b->err.c_str() : tl_err.c_str(); }

int fglsgpu_batch_create(const fglsgpu_cohort* cohorts, int count, const fglsgpu_batch_config* cfg,
                         fglsgpu_batch** out) {
  if (!cohorts || !cfg || !out || count <= 0) return bfail(nullptr, FGLSGPU_EINVAL, "invalid batch arguments");
  *out = nullptr;
  if (cfg->x_b < 0 || cfg->x_b > 65536 || cfg->slices < 0 || cfg->slices > S_BUILT ||
      (cfg->tile_rows != 0 && cfg->tile_rows != 128 && cfg->tile_rows != 256))
    return bfail(nullptr, FGLSGPU_EINVAL, "invalid batch config x_b=%d slices=%d tile_rows=%d", cfg->x_b,
                 cfg->slices, cfg->tile_rows);
  for (int c = 0; c < count; c++) {
    const fglsgpu_cohort& k = cohorts[c];
    if (k.n < 2 || k.n > 16368 || k.wXL < 1 || k.wXL + 1 > FGLS_MAX_P || k.t < 1 || !k.Phi || !k.XL || !k.Y || !k.h ||
        !k.sigma)
      return bfail(nullptr, FGLSGPU_EINVAL, "cohort %d: invalid (n=%d wXL=%d t=%d; n <= 16368, wXL+1 <= %d)", c, k.n,
                   k.wXL, k.t, FGLS_MAX_P);
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return bfail(nullptr, FGLSGPU_ENODEV, "no CUDA device");
  if (cudaSetDevice(cfg->device) != cudaSuccess) return bfail(nullptr, FGLSGPU_ENODEV, "cudaSetDevice failed");
  fglsgpu_batch* b = new fglsgpu_batch();
  b->cfg = *cfg;
  b->pair_tiles = cfg->tile_rows != 128;  // given, or the default before autotuning
  if (b->cfg.tol <= 0.0) b->cfg.tol = 1e-10;
  const int xb_alloc = cfg->x_b > 0 ? cfg->x_b : XB_MAX;
  auto bail = [&](int rc) {
    free_batch(b);
    delete b;
    return rc;
  };
  int rc = 0;
  // FGLS_BATCH_TIMING=1 prints the wall time of the setup phases to stderr
  const bool timing = getenv("FGLS_BATCH_TIMING") && atoi(getenv("FGLS_BATCH_TIMING")) != 0;
  auto now = [] { return std::chrono::steady_clock::now(); };
  auto secs = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point z) {
    return std::chrono::duration<double>(z - a).count();
  };
  const auto t_start = now();
#define B_CHECK(expr, what)                                                                                  \
  do {                                                                                                       \
    cudaError_t _c = (expr);                                                                                 \
    if (_c != cudaSuccess)                                                                                   \
      return bail(bfail(nullptr, _c == cudaErrorMemoryAllocation ? FGLSGPU_ENOMEM : FGLSGPU_ECUDA, "%s: %s", \
                        what, cudaGetErrorString(_c)));                                                      \
  } while (0)
  B_CHECK(cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking), "stream");
  B_CHECK(dalloc(&b->dst, 1), "status");
  B_CHECK(dalloc(&b->derr, 1), "status");
  B_CHECK(cudaMemset(b->dst, 0, sizeof(DevStatus)), "status");
  B_CHECK(cudaMemset(b->derr, 0, sizeof(int)), "status");
  B_CHECK(cudaMallocHost(&b->hst, sizeof(DevStatus)), "status");
  for (int k = 0; k < NSLOT; k++)
    B_CHECK(cudaEventCreateWithFlags(&b->slot_done[k], cudaEventDisableTiming), "events");
  b->ncap = split_cols_padded(std::max(xb_alloc, PROBE));
  int nmax = 0, wmax = 0;
  b->co.resize(count);
  for (int c = 0; c < count; c++) {
    Cohort& k = b->co[c];
    k.n = cohorts[c].n;
    k.wXL = cohorts[c].wXL;
    k.p = k.wXL + 1;
    k.t = cohorts[c].t;
    k.Kpad = split_k_padded(k.n);
    k.Ncap = b->ncap;
    nmax = std::max(nmax, k.n);
    wmax = std::max(wmax, k.wXL);
    B_CHECK(dalloc(&k.G, (size_t)k.Ncap * k.Kpad), "genotype operand");
    B_CHECK(cudaMemset(k.G, 0, (size_t)k.Ncap * k.Kpad), "genotype operand");
    B_CHECK(dalloc(&k.probe, (size_t)PROBE * k.n), "probe block");
    for (int j = 0; j < k.t; j++) {
      Problem q;
      q.c = c;
      q.j = j;
      q.M = k.n + 1 + k.wXL;
      q.Mpad = split_rows_padded(q.M);
      b->pr.push_back(q);
    }
  }
  for (auto& q : b->pr) {
    const Cohort& k = b->co[q.c];
    B_CHECK(dalloc(&q.A, (size_t)S_BUILT * q.Mpad * k.Kpad), "split operand");
    B_CHECK(cudaMemset(q.A, 0, (size_t)S_BUILT * q.Mpad * k.Kpad), "split operand");
    B_CHECK(dalloc(&q.scale_built, q.Mpad), "row scales");
    B_CHECK(cudaMemset(q.scale_built, 0, sizeof(double) * q.Mpad), "row scales");
    B_CHECK(dalloc(&q.scale, q.Mpad), "row scales");
    B_CHECK(dalloc(&q.top, k.wXL + k.wXL * k.wXL + 1), "null model");
    B_CHECK(dalloc(&q.C, (size_t)q.Mpad * b->ncap), "split GEMM output");
    B_CHECK(dalloc(&q.Q, (size_t)(q.Mpad / 32) * b->ncap), "split GEMM group sums");
    B_CHECK(dalloc(&q.GR, b->ncap), "Gram");
    B_CHECK(dalloc(&q.ref, (size_t)PROBE * k.p), "probe reference");
  }
  // the memsets above ran on the legacy default stream, which does not order
  // against the batch's non-blocking streams: finish them first
  B_CHECK(cudaDeviceSynchronize(), "operand initialisation");
  // one-off FP64 setup of every problem: the traits of a cohort run
  // concurrently on NS streams, each with its own scratch and status word
  {
    constexpr int NS = 4;
    Scratch w[NS];
    CohortInputs ci;
    auto release = [&]() {
      for (auto& x : w) x.release();
      for (double* v : {ci.Phi, ci.XL, ci.Y})
        if (v) cudaFree(v);
    };
    auto fail_scratch = [&](cudaError_t e, const char* what) {
      release();
      return bail(bfail(nullptr, e == cudaErrorMemoryAllocation ? FGLSGPU_ENOMEM : FGLSGPU_ECUDA, "%s: %s", what,
                        cudaGetErrorString(e)));
    };
    int tmax = 1;
    size_t ymax = 0;
    for (int c = 0; c < count; c++) {
      tmax = std::max(tmax, cohorts[c].t);
      ymax = std::max(ymax, (size_t)cohorts[c].n * cohorts[c].t);
    }
    const int ns = std::min(NS, tmax);
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < ns && e == cudaSuccess; k++) e = w[k].alloc(nmax, wmax);
    if (e == cudaSuccess) e = dalloc(&ci.Phi, (size_t)nmax * nmax);
    if (e == cudaSuccess) e = dalloc(&ci.XL, (size_t)nmax * wmax);
    if (e == cudaSuccess) e = dalloc(&ci.Y, ymax);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();  // the scratch status words' memsets
    if (e != cudaSuccess) return fail_scratch(e, "setup scratch");
    cudaEvent_t up = nullptr;
    if ((e = cudaEventCreateWithFlags(&up, cudaEventDisableTiming)) != cudaSuccess)
      return fail_scratch(e, "setup events");
    size_t k = 0;
    for (int c = 0; c < count && e == cudaSuccess; c++) {
      const fglsgpu_cohort& in = cohorts[c];
      const int n = in.n;
      e = cudaMemcpyAsync(ci.Phi, in.Phi, sizeof(double) * n * n, cudaMemcpyHostToDevice, b->s);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(ci.XL, in.XL, sizeof(double) * n * in.wXL, cudaMemcpyHostToDevice, b->s);
      if (e == cudaSuccess) e = cudaMemcpyAsync(ci.Y, in.Y, sizeof(double) * n * in.t, cudaMemcpyHostToDevice, b->s);
      if (e == cudaSuccess) e = cudaEventRecord(up, b->s);
      const size_t k0 = k;
      for (; e == cudaSuccess && k < b->pr.size() && b->pr[k].c == c; k++) {
        Scratch& x = w[(k - k0) % ns];
        e = cudaStreamWaitEvent(x.s, up, 0);
        if (e == cudaSuccess) e = setup_problem(b, x, ci, b->pr[k], in);
      }
      // the next cohort's upload overwrites the inputs: wait for all traits,
      // then read the status words
      for (int q = 0; q < ns && e == cudaSuccess; q++) e = cudaStreamSynchronize(w[q].s);
      for (int q = 0; q < ns && e == cudaSuccess; q++) {
        DevStatus hs{};
        e = cudaMemcpy(&hs, w[q].st, sizeof(DevStatus), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && hs.code != FGLSGPU_OK) {
          cudaEventDestroy(up);
          release();
          return bail(bfail(nullptr, hs.code == FGLSGPU_ENOTSPD ? FGLSGPU_ENOTSPD : hs.code,
                            "cohort %d: a trait's M or null model is not positive definite (info %d, item %lld)",
                            c, hs.info, hs.idx));
        }
      }
    }
    cudaEventDestroy(up);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->s);
    if (e != cudaSuccess) return fail_scratch(e, "setup");
    release();
  }
  // device tables
  {
    const int C = count, P = (int)b->pr.size();
    std::vector<GenoCohort> geno(C);
    for (int c = 0; c < C; c++) geno[c] = GenoCohort{b->co[c].G, b->co[c].n, b->co[c].Kpad};
    std::vector<UnitGramProblem> unit(P);
    std::vector<SolveProblem> solve(P);
    std::vector<int> plist;
    for (int p = 2; p <= FGLS_MAX_P; p++) {
      b->poff[p] = (int)plist.size();
      for (int k = 0; k < P; k++)
        if (b->co[b->pr[k].c].p == p) plist.push_back(k);
      b->pcount[p] = (int)plist.size() - b->poff[p];
    }
    for (int k = 0; k < P; k++) {
      const Problem& q = b->pr[k];
      const Cohort& c = b->co[q.c];
      unit[k] = UnitGramProblem{q.Q, b->ncap, q.GR, c.n, q.c};
      solve[k] = SolveProblem{q.top, q.C + c.n, q.Mpad, q.GR, q.c, q.j};
    }
    B_CHECK(dalloc(&b->dgeno, C), "tables");
    B_CHECK(dalloc(&b->dunit, P), "tables");
    B_CHECK(dalloc(&b->dsolve, P), "tables");
    B_CHECK(dalloc(&b->dplist, plist.size()), "tables");
    B_CHECK(cudaMemcpy(b->dgeno, geno.data(), sizeof(GenoCohort) * C, cudaMemcpyHostToDevice), "tables");
    B_CHECK(cudaMemcpy(b->dunit, unit.data(), sizeof(UnitGramProblem) * P, cudaMemcpyHostToDevice), "tables");
    B_CHECK(cudaMemcpy(b->dsolve, solve.data(), sizeof(SolveProblem) * P, cudaMemcpyHostToDevice), "tables");
    B_CHECK(cudaMemcpy(b->dplist, plist.data(), sizeof(int) * plist.size(), cudaMemcpyHostToDevice), "tables");
    b->step_bytes = (sizeof(StepCohort) + sizeof(int)) * C;
    B_CHECK(cudaMalloc(&b->dstep, b->step_bytes), "step table");
    for (int k = 0; k < NSLOT; k++) {
      B_CHECK(cudaMallocHost(&b->hstep[k], b->step_bytes), "step table");
      memset(b->hstep[k], 0, b->step_bytes);
      B_CHECK(cudaEventRecord(b->slot_done[k], b->s), "events");
    }
  }
  // autotuning
  const auto t_setup = now();
  int S = cfg->slices;
  if (S == 0) {
    S = S_BUILT;
    for (int cand = S_MIN_TUNE; cand <= S_BUILT; cand++) {
      double e = 0.0;
      rc = probe_error(b, cand, &e);
      if (rc) {
        tl_err = b->err;
        return bail(rc);
      }
      if (e <= b->cfg.tol / 8.0) {
        S = cand;
        b->tune_err = e;
        break;
      }
      b->tune_err = e;
    }
  }
  b->S = S;
  const auto t_probe = now();
  int xb = cfg->x_b;
  if (xb == 0) {
    double best = -1.0;
    for (int cand = 1024; cand <= XB_MAX; cand *= 2) {
      double r = 0.0;
      rc = time_step(b, cand, &r);
      if (rc) {
        tl_err = b->err;
        return bail(rc);
      }
      b->tune_rates.push_back(r);
      if (r > best) {
        best = r;
        xb = cand;
      }
    }
    if (cfg->tile_rows == 0) {
      // the other tile shape at the chosen block
      b->pair_tiles = false;
      double r1 = 0.0;
      rc = time_step(b, xb, &r1);
      if (rc) {
        tl_err = b->err;
        return bail(rc);
      }
      b->tune_rates.push_back(r1);
      b->pair_tiles = r1 <= best;
    }
  }
  rc = configure(b, S, xb);
  if (rc) {
    tl_err = b->err;
    return bail(rc);
  }
  if (timing) {
    cudaDeviceSynchronize();
    const auto t_end = now();
    fprintf(stderr, "[fgls batch] factorisations + operands %.2f s, slice probe %.2f s, block timing %.2f s\n",
            secs(t_start, t_setup), secs(t_setup, t_probe), secs(t_probe, t_end));
  }
#undef B_CHECK
  *out = b;
  return FGLSGPU_OK;
}

int fglsgpu_batch_destroy(fglsgpu_batch* b) {
  if (!b) return FGLSGPU_OK;
  cudaSetDevice(b->cfg.device);
  if (b->s) cudaStreamSynchronize(b->s);
  free_batch(b);
  delete b;
  return FGLSGPU_OK;
}

int fglsgpu_batch_tile(const fglsgpu_batch* b, int* rows, int* cols) {
  if (!b) return bfail(nullptr, FGLSGPU_EINVAL, "null batch");
  if (rows) *rows = grouped_gemm_tile_rows(b->gg);
  if (cols) *cols = 256;
  return FGLSGPU_OK;
}

int fglsgpu_batch_params(const fglsgpu_batch* b, int* x_b, int* slices, double* probe_err) {
  if (!b) return bfail(nullptr, FGLSGPU_EINVAL, "null batch");
  if (x_b) *x_b = b->x_b;
  if (slices) *slices = b->S;
  if (probe_err) *probe_err = b->tune_err;
  return FGLSGPU_OK;
}

int fglsgpu_batch_step(fglsgpu_batch* b, const void* const* dX, const int* x, double* const* dB, double* const* dV,
                       const long long* snp_base) {
  if (!b) return bfail(nullptr, FGLSGPU_EINVAL, "null batch");
  int rc = validate_args(b, x, dX, dB, dV);
  if (rc) return rc;
  B_TRY(b, cudaSetDevice(b->cfg.device), "cudaSetDevice");
  return launch_step(b, dX, x, dB, dV, snp_base);
}

int fglsgpu_batch_sync(fglsgpu_batch* b) {
  if (!b) return bfail(nullptr, FGLSGPU_EINVAL, "null batch");
  B_TRY(b, cudaSetDevice(b->cfg.device), "cudaSetDevice");
  return check_status(b, "batch step");
}

void* fglsgpu_batch_stream(fglsgpu_batch* b) { return b ? (void*)b->s : nullptr; }

int fglsgpu_batch_profile(fglsgpu_batch* b, int enable) {
  if (!b) return bfail(nullptr, FGLSGPU_EINVAL, "null batch");
  b->prof = enable != 0;
  return FGLSGPU_OK;
}

int fglsgpu_batch_profile_read(fglsgpu_batch* b, double* ms, long long* steps) {
  if (!b || !ms) return bfail(b, FGLSGPU_EINVAL, "null argument");
  B_TRY(b, cudaStreamSynchronize(b->s), "profile read");
  for (size_t k = 0; k + 5 <= b->pev.size(); k += 5) {
    for (int c = 0; c < 4; c++) {
      float t = 0.0f;
      B_TRY(b, cudaEventElapsedTime(&t, b->pev[k + c], b->pev[k + c + 1]), "profile read");
      b->prof_ms[c] += t;
    }
    b->prof_steps++;
  }
  for (cudaEvent_t e : b->pev) cudaEventDestroy(e);
  b->pev.clear();
  for (int c = 0; c < 4; c++) ms[c] = b->prof_ms[c];
  if (steps) *steps = b->prof_steps;
  for (int c = 0; c < 4; c++) b->prof_ms[c] = 0.0;
  b->prof_steps = 0;
  return FGLSGPU_OK;
}

}  // extern "C"
