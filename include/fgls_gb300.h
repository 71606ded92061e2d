/*
 * fgls_gb300.h -- C ABI of the GB300-native FGLS association engine.
 *
 * Two layers:
 *
 * 1. Drop-in entry points with the reference's exact 17-argument C
 *    signatures.  They are file-path based like the reference (the callee
 *    opens, reads, allocates and frees everything and writes B/V), read the
 *    reference's on-disk layout, and on failure print "[Error]: ..." and
 *    exit(EXIT_FAILURE) as the reference's error_msg(..., 1) does
 *    (src/common.c:11-17).
 *
 * 2. The engine API (fglsgpu_*): plain C types and host or device pointers,
 *    status codes instead of exit(), one GPU.  The drop-in entry points are
 *    written on top of it.
 *
 * Layouts (all FP64, column-major, as in the reference files):
 *   Phi n x n (lower triangle used), XL n x wXL, Y t x n (trait j at j*n),
 *   XR block: x SNPs x wXR columns x n (SNP i column c at (i*wXR+c)*n),
 *   B: per trait x*p doubles (SNP i at i*p, order [XL coefs, XR coefs]),
 *   V: per trait x*p*p doubles (SNP i block at i*p*p, column-major p x p):
 *      lower = res_sigma * S^-1, diagonal = standard errors, strict upper 0.
 */
#ifndef FGLS_GB300_H
#define FGLS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define FGLSGPU_OK 0
#define FGLSGPU_EINVAL 1   /* invalid argument or dimensions                */
#define FGLSGPU_ENOTSPD 2  /* M_j, the covariate Gram or a per-SNP S_i is not positive definite */
#define FGLSGPU_ECUDA 3    /* CUDA runtime error (message in last_error)    */
#define FGLSGPU_EIO 4      /* open/read/write failure or short read         */
#define FGLSGPU_ENOMEM 5   /* device or pinned host allocation failed       */
#define FGLSGPU_ETIMEOUT 6 /* a bounded device-side wait expired            */
#define FGLSGPU_ENOCONV 7  /* the eigensolver did not converge              */
#define FGLSGPU_ENODEV 8   /* no usable CUDA device                         */
#define FGLSGPU_ESTATE 9   /* call out of order (e.g. run before set_problem) */

/* ------------------------------------------------- drop-in entry points */

/* Replaces fgls_chol, src/fgls_chol.h:4-10 (defined src/fgls_chol.c:29).
 * y_b is ignored (the reference forces it to 1, src/fgls_chol.c:97,102-103);
 * num_threads sizes the host I/O threads only. */
int fgls_chol(int n, int p, int m, int t, int wXL, int wXR, int x_b, int y_b, int num_threads,
              char *Phi_path, char *h2_path, char *sigma2_path, char *XL_path, char *XR_path,
              char *Y_path, char *B_path, char *V_path);

/* Replaces fgls_eigen, src/fgls_eigen.h:68-74 (defined src/fgls_eigen.c:38).
 * Writes no <path>.tmp files: the rotations Z^T XL, Z^T XR, Z^T Y stay on
 * the device.  Uses the split-precision tensor-core path when the
 * environment variable FGLS_PRECISION=split is set, FP64 otherwise. */
int fgls_eigen(int n, int p, int m, int t, int wXL, int wXR, int x_b, int y_b, int num_threads,
               char *Phi_path, char *h2_path, char *sigma2_path, char *XL_path, char *XR_path,
               char *Y_path, char *B_path, char *V_path);

/* Replaces fgls_chol_gpu, src/fgls_chol_gpu.h:4-10 (defined
 * src/fgls_chol_gpu.c:97).  Same computation as fgls_chol on one GPU; unlike
 * the reference it accepts t > 1 (src/fgls_chol_gpu.c:169-174). */
int fgls_chol_gpu(int n, int p, int m, int t, int wXL, int wXR, int x_b, int y_b,
                  int num_threads, char *Phi_path, char *h2_path, char *sigma2_path,
                  char *XL_path, char *XR_path, char *Y_path, char *B_path, char *V_path);

/* ------------------------------------------------------------ engine API */

typedef struct fglsgpu_engine fglsgpu_engine;

#define FGLSGPU_VARIANT_CHOL 0  /* per-trait Cholesky whitening (fgls_chol)  */
#define FGLSGPU_VARIANT_EIGEN 1 /* eigenbasis of Phi, all traits per block (fgls_eigen) */

#define FGLSGPU_PREC_FP64 0     /* all-FP64 arithmetic                       */
#define FGLSGPU_PREC_SPLIT 1    /* bulk GEMMs as 5-bit digit slices (FP8 E4M3) on
                                   tcgen05 tensor cores, exact FP32 accumulation,
                                   integer / FP64 recombination               */

typedef struct {
  int n;         /* individuals                                  */
  int wXL;       /* covariate columns (intercept included)       */
  int wXR;       /* columns per SNP                              */
  int t;         /* traits                                       */
  int x_b;       /* maximum SNPs per block                       */
  int variant;   /* FGLSGPU_VARIANT_*                            */
  int precision; /* FGLSGPU_PREC_*                               */
  int slices;    /* split precision: 5-bit digit slices of the FP64 operand, 1..9;
                    0 = autotune: the operand is cut into 9 slices (about 45
                    bits) and a 256-SNP probe block picks the smallest count
                    in 6..9 whose beta is within 1e-10 / 8 of the FP64 path.
                    The split path takes n <= 16368 (exact FP32 accumulation
                    of a slice pair); larger n fails with FGLSGPU_ECUDA. */
  int device;    /* CUDA device ordinal                          */
  int reserved;
} fglsgpu_config;

/* Creates an engine on cfg->device and allocates its device buffers. */
int fglsgpu_create(const fglsgpu_config *cfg, fglsgpu_engine **out);
int fglsgpu_destroy(fglsgpu_engine *e);

/* Uploads the in-core operands (host pointers, reference layouts; only the
 * first t entries of h and sigma are read) and runs the one-off setup:
 * eigen: FP64 eigendecomposition of Phi on the device, Z^T XL, Z^T Y and the
 * per-trait null-model residual variances (src/fgls_eigen.c:686-854,998-1195);
 * chol: nothing beyond the upload (the per-trait work is select_trait). */
int fglsgpu_set_problem(fglsgpu_engine *e, const double *Phi, const double *XL, const double *Y,
                        const double *h, const double *sigma);

/* chol only: factor M_j = sigma_j (h_j Phi + (1 - h_j) I) and compute trait
 * j's null model (src/fgls_chol.c:251-325).  Subsequent blocks produce
 * trait j's results.  Ignored (returns OK) for the eigen variant. */
int fglsgpu_select_trait(fglsgpu_engine *e, int j);

/* Processes one SNP block given as a HOST pointer (x_inc <= x_b SNPs,
 * reference layout, genotypes as FP64).  Host->device copy, compute and
 * device->host copy of the results run on the engine's streams; the call
 * returns when B and V are in host memory.  Results for trait j (eigen: all
 * traits; chol: the selected trait, written as trait 0) go to
 * B + j*b_trait_stride and V + j*v_trait_stride. */
int fglsgpu_run_block(fglsgpu_engine *e, const double *XR, int x_inc, double *B, double *V,
                      long long b_trait_stride, long long v_trait_stride);

/* Whole job over m SNPs given as one HOST array in the reference XR layout;
 * results to host arrays in the B.out / V.out layout (trait j of the active
 * traits at B + j*m*p and V + j*m*p*p; chol: the selected trait only).  Blocks
 * of x_b SNPs are pipelined: upload of block b+1 and download of block b-1
 * overlap the compute of block b (replaces the reference's aio double
 * buffering, src/fgls_chol.c:327-487). */
int fglsgpu_run_snps(fglsgpu_engine *e, const double *XR, long long m, double *B, double *V);

/* As fglsgpu_run_snps with the genotypes as bytes (hard calls 0/1/2, the XR
 * layout with one byte per individual): 8x fewer bytes over the host link.
 * No counterpart in the reference (it reads FP64 only, src/fgls_chol.c:333-337). */
int fglsgpu_run_snps_u8(fglsgpu_engine *e, const unsigned char *XR, long long m, double *B, double *V);

/* As fglsgpu_run_snps with the genotypes packed 2 bits per individual, the
 * body of a SNP-major PLINK .bed file (the layout fglsgpu_run_block_device_packed
 * describes: ceil(n/4) bytes per column, codes 00 -> 2, 10 -> 1, 11 -> 0,
 * 01 missing -> FGLSGPU_EINVAL naming the SNP and individual): 32x fewer
 * bytes over the host link than FP64.  No counterpart in the reference. */
int fglsgpu_run_snps_packed(fglsgpu_engine *e, const unsigned char *XR2, long long m, double *B, double *V);

/* As fglsgpu_run_snps with a compact output: instead of V (p*p doubles per
 * test) the standard errors SE and the two-sided normal p-values P of all p
 * coefficients, both in the B layout (trait j, SNP i, coefficient k at
 * (j*m + i)*p + k).  8x less output than B + V at p = 4.  No counterpart in
 * the reference (it writes B and V only, src/fgls_chol.c:464-474). */
int fglsgpu_run_snps_compact(fglsgpu_engine *e, const double *XR, long long m, double *B, double *SE,
                             double *P);

/* Same with DEVICE pointers (XR, B, V already in HBM); asynchronous with
 * respect to the host: call fglsgpu_sync before reading B/V.  The engine
 * computes on its own non-blocking stream (fglsgpu_stream), which does not
 * wait for work queued on other streams, the legacy default stream
 * included: the input must be complete when the call is made (synchronize
 * the stream that produced it, or make the engine's stream wait on an event
 * recorded after it).  The same holds for every fglsgpu_*_device call and
 * for fglsgpu_batch_step. */
int fglsgpu_run_block_device(fglsgpu_engine *e, const double *dXR, int x_inc, double *dB,
                             double *dV, long long b_trait_stride, long long v_trait_stride);

/* As run_block_device with genotypes as bytes (hard calls 0/1/2, same
 * layout as XR); 8x fewer bytes to move than FP64. */
int fglsgpu_run_block_device_u8(fglsgpu_engine *e, const unsigned char *dXR, int x_inc,
                                double *dB, double *dV, long long b_trait_stride,
                                long long v_trait_stride);

/* As run_block_device_u8 with genotypes packed 2 bits per individual, the
 * body of a SNP-major PLINK .bed file: each of the x_inc*wXR columns holds
 * ceil(n/4) bytes, individual k in bits 2(k%4)..2(k%4)+1 of byte k/4, codes
 * 00 -> 2, 10 -> 1, 11 -> 0 copies of the first allele.  Code 01 (missing)
 * is reported by fglsgpu_sync as FGLSGPU_EINVAL.  32x fewer bytes than FP64.
 * No counterpart in the reference (it reads FP64 only, src/fgls_chol.c:333-337). */
int fglsgpu_run_block_device_packed(fglsgpu_engine *e, const unsigned char *dXR2, int x_inc,
                                    double *dB, double *dV, long long b_trait_stride,
                                    long long v_trait_stride);

/* Waits for the engine's device work and reports device-side failures
 * (non-SPD per-SNP systems, expired waits). */
int fglsgpu_sync(fglsgpu_engine *e);

/* Per-trait null-model residual variance (t values; chol: selected trait). */
int fglsgpu_get_res_sigma(fglsgpu_engine *e, double *out);

/* The eigenvalues (n, ascending) and eigenvectors (n x n column-major) of
 * Phi computed by set_problem (eigen variant); either pointer may be NULL. */
int fglsgpu_get_eigen(fglsgpu_engine *e, double *W, double *Z);

/* Two-sided normal p-values p = erfc(|beta_k / SE_k| / sqrt 2) of the SNP
 * coefficients (k = wXL .. p-1) of a block's results (device pointers in
 * the B/V layouts above); P holds x_inc * wXR values per trait at
 * P + j*p_trait_stride.  Runs on the engine stream.  No counterpart in the
 * reference (it emits beta and V only). */
int fglsgpu_pvalues_device(fglsgpu_engine *e, const double *dB, const double *dV, int x_inc,
                           long long b_trait_stride, long long v_trait_stride, double *dP,
                           long long p_trait_stride);

/* ---- adjoint of fgls_eigen (FP64, wXR = 1) and the null-model REML ----
 * No counterpart in the reference (it computes no derivatives).  With a
 * cotangent Bbar for the betas (same layout as B), the vector-Jacobian
 * products sum_ij Bbar_ij . dbeta_ij/dh_j, .../dsigma_j and .../dY are
 * accumulated over blocks: reset, one call per block (device pointers, the
 * block's genotypes and its Bbar slice with the given trait stride), read
 * (host outputs; dY is n x t in the Y.in orientation, any pointer may be
 * NULL).  Gram blocks are recomputed per block, never stored per SNP. */
int fglsgpu_adjoint_reset(fglsgpu_engine *e);
int fglsgpu_adjoint_block_device(fglsgpu_engine *e, const double *dXR, int x_inc, const double *dBbar,
                                 long long bbar_trait_stride);
int fglsgpu_adjoint_read(fglsgpu_engine *e, double *dh, double *dsigma, double *dY);
/* Null-model REML log-likelihood per trait (sigma given, constants dropped)
 *   l(h) = -1/2 [ log det M + log det(XL^T M^-1 XL) + r^T M^-1 r ]
 * and dl/dh_j; valid after fglsgpu_adjoint_reset. */
int fglsgpu_reml(fglsgpu_engine *e, double *loglik, double *dloglik_dh);

/* ---- variance-component estimation (eigen variant, FP64) ----
 * No counterpart in the reference, which reads h and sigma from the H.in and
 * Sig.in files (src/fgls_chol.c:139-145).  Fits, per trait, the null model
 * y ~ N(XL b, sigma (h Phi + (1-h) I)) by REML with sigma profiled out
 * (sigma_hat = y^T P y / (n - wXL)) and h maximised over [h_lo, h_hi]
 * (0 <= h_lo < h_hi <= 1) on a grid of `grid` points (2..256; 0 = 64) whose
 * gradient sign changes are refined to roots.  Outputs (host, t each, any may
 * be NULL): h, sigma, the profiled REML log-likelihood (constants dropped;
 * equal to fglsgpu_reml's value at that h and sigma) and its h-gradient there
 * (about 0 unless the maximum is on an endpoint).  Needs set_problem; does not
 * change the engine's h and sigma. */
int fglsgpu_reml_fit(fglsgpu_engine *e, double h_lo, double h_hi, int grid, double *h, double *sigma,
                     double *loglik, double *dloglik_dh);

/* Replaces every trait's h and sigma (host arrays of t) without redoing the
 * eigendecomposition (eigen) or Phi upload (chol: the next select_trait
 * refactors M_j).  Same checks as set_problem.  Invalidates the adjoint
 * state (call fglsgpu_adjoint_reset again). */
int fglsgpu_set_hsigma(fglsgpu_engine *e, const double *h, const double *sigma);

/* Switches a live engine between FGLSGPU_PREC_FP64 and FGLSGPU_PREC_SPLIT
 * without redoing set_problem (eigen keeps its eigendecomposition; chol
 * needs select_trait again). */
int fglsgpu_set_precision(fglsgpu_engine *e, int precision);

/* The slice count the split path runs with (0 before the split operands
 * exist) and, when it was autotuned (cfg.slices == 0), the probe block's
 * largest normwise beta difference from the FP64 path at that count (-1
 * otherwise).  No counterpart in the reference. */
int fglsgpu_split_params(fglsgpu_engine *e, int *slices, double *probe_err);

/* Base-32 digits a side that the split eigen path's tensor-core quadratic
 * Gram uses (t >= 33; 0 when that path is off).  With cfg.slices == 0 the
 * probe block also chooses them, the smallest count in 8..11 whose beta stays
 * within 1e-10 / 8 of the FP64 path (after the slice choice); else 11.  No
 * reference counterpart (the reference has no split path). */
int fglsgpu_quad_digits(fglsgpu_engine *e, int *digits);

/* Limit of one pipeline wait (on an mbarrier: a TMA copy landing, an MMA
 * finishing, an epilogue draining TMEM) inside the split path's tcgen05
 * kernels, in nanoseconds; 0 restores the default of 2 s.  A wait that
 * runs out makes the kernel set an error word, let its own copies and MMAs
 * finish, free its TMEM and return; the next fglsgpu_sync (or the status
 * check of a host-API call) reports FGLSGPU_ETIMEOUT, clears the word and
 * the engine runs normally again.  No counterpart in the reference (its
 * only device work is cuBLAS, src/fgls_chol_gpu.c:550). */
int fglsgpu_set_wait_limit(fglsgpu_engine *e, long long ns);

/* Per-kernel-class device time, measured with CUDA events recorded on the
 * engine's compute stream around each class of launches. */
#define FGLSGPU_PROF_GENOTYPES 0  /* genotype widening / E4M3 operand build     */
#define FGLSGPU_PROF_SPLIT_GEMM 1 /* tcgen05 split-precision GEMM               */
#define FGLSGPU_PROF_SELFGRAM 2   /* quadratic Gram terms (all variants)        */
#define FGLSGPU_PROF_SOLVE 3      /* batched p x p solves + B/V emission        */
#define FGLSGPU_PROF_FP64_GEMM 4  /* FP64 path: Z^T XR                          */
#define FGLSGPU_PROF_TRSM 5       /* FP64 path: L^-1 XR                         */
#define FGLSGPU_PROF_GRAM 6       /* FP64 path: Gram terms                      */
#define FGLSGPU_PROF_CLASSES 8
/* Turns timing on (enable != 0) or off and zeroes the accumulators. */
int fglsgpu_profile(fglsgpu_engine *e, int enable);
/* Milliseconds and number of timed sections per class (FGLSGPU_PROF_CLASSES
 * entries each); waits for the recorded events. */
int fglsgpu_profile_read(fglsgpu_engine *e, double *ms, long long *count);

/* The CUDA stream the engine computes on (a cudaStream_t). */
void *fglsgpu_stream(fglsgpu_engine *e);

/* Number of the engine's own kernel launches since creation. */
long long fglsgpu_launch_count(const fglsgpu_engine *e);

/* Message describing the last failure on e (or on the calling thread when e
 * is NULL). */
const char *fglsgpu_last_error(const fglsgpu_engine *e);

/* Library version, major*10000 + minor*100 + patch. */
int fglsgpu_version(void);

/* Diagnostic: runs the split-precision tensor-core GEMM used by
 * FGLSGPU_PREC_SPLIT on caller data.  C = A * X^T with A M x K (row-major
 * FP64, cut into `slices` 5-bit digit slices, 1..9), X K x N (column-major, integer
 * genotypes 0..2) and C M x N column-major, all host pointers; K <= 16368.
 * No counterpart in the reference (its GEMMs are FP64 BLAS calls). */
int fglsgpu_selftest_split_gemm(int M, int K, int N, int slices, const double *A, const double *X,
                                double *C);

/* The same split-precision GEMM for callers that may not allocate device
 * memory (code running under a framework that owns the device through its
 * own memory pool, or that must keep the device's footprint fixed).  All
 * pointers are DEVICE pointers owned by the caller: A (M x K, row-major
 * FP64), X (K x N, column-major genotypes), C (M x N, column-major FP64 out).
 * The kernel's scratch lives in a fixed 5.8 MB array inside the library
 * (held by every GPU that loads it): M <= 256, K <= 2048, N <= 512,
 * slices <= 9, else FGLSGPU_EINVAL.  Runs on `stream` (a cudaStream_t, NULL
 * for the default stream), reads the kernel's error word back and returns
 * after the stream has finished (it synchronizes the stream).  Calls share the
 * array: calls that overlap on the GPU race; serialise them.  The first call
 * on a device sets up the array's address and should come before any stream
 * capture.  No counterpart in the reference. */
int fglsgpu_split_gemm_noalloc(int M, int K, int N, int slices, const double *A, const double *X,
                               double *C, void *stream);

/* ---------------------------------------------------- batched cohorts ----
 * Many independent chol-variant problems of uneven size (cohort c: n_c
 * individuals, wXL_c covariates, t_c traits, wXR = 1) advanced together, one
 * SNP block of every cohort per step: all cohorts' split GEMM tiles in one
 * launch, the quadratic Gram terms and the p x p solves grouped likewise, the
 * step replayed from a captured CUDA graph.  Per (cohort, trait) the FP64
 * Cholesky of M_j, the null model and L_j^-1 are computed once at creation
 * and the split operand stays resident in HBM.  The reference handles one
 * problem per process (fgls_chol, src/fgls_chol.c:29); it has no batched
 * counterpart.  Autotuning: x_b = 0 picks the SNP block (1024..8192) by
 * measured tests/s, slices = 0 the smallest slice count whose probe-block
 * beta is within tol/8 of the FP64 path for every problem. */
typedef struct fglsgpu_batch fglsgpu_batch;

typedef struct {
  int n, wXL, t;       /* individuals, covariate columns, traits           */
  const double *Phi;   /* host, n x n column-major (Phi.in layout)         */
  const double *XL;    /* host, n x wXL column-major                       */
  const double *Y;     /* host, t traits of n values (Y.in layout)         */
  const double *h;     /* host, t heritabilities                           */
  const double *sigma; /* host, t variance scales                          */
} fglsgpu_cohort;

typedef struct {
  int x_b;          /* SNPs per cohort per step (0: autotune)             */
  int slices;       /* FP8 five-bit digit slices 1..9 (0: autotune over   */
                    /* 5..9); cohorts need n <= 16368                     */
  int device;       /* CUDA device ordinal                                */
  int use_graph;    /* 1: replay each step from a captured CUDA graph     */
  int genotypes_u8; /* 1: genotype blocks are bytes, 0: FP64              */
  int tile_rows;    /* grouped GEMM tile rows: 256 (CTA pairs), 128 (one  */
                    /* SM); 0: autotuned with x_b = 0, else 256            */
  double tol;       /* autotune target for beta vs FP64 (0: 1e-10)        */
} fglsgpu_batch_config;

int fglsgpu_batch_create(const fglsgpu_cohort *cohorts, int count, const fglsgpu_batch_config *cfg,
                         fglsgpu_batch **out);
int fglsgpu_batch_destroy(fglsgpu_batch *b);
/* The tuned (or given) SNP block and slice count, and the probe error of
 * the slice choice (-1 when slices were given). */
int fglsgpu_batch_params(const fglsgpu_batch *b, int *x_b, int *slices, double *probe_err);

/* The grouped split GEMM's output tile: 256 x 256 (two SMs per tile,
 * tcgen05.mma.cta_group::2) or 128 x 256 (one SM).  With x_b = 0 the
 * autotuner times both at its chosen block and keeps the faster; else 256. */
int fglsgpu_batch_tile(const fglsgpu_batch *b, int *rows, int *cols);
/* One step (asynchronous; fglsgpu_batch_sync reports device failures).  Per
 * cohort c: dX[c] = device genotype block of x[c] <= x_b SNPs (SNP i at
 * dX[c] + i*n_c, bytes or doubles per the config; x[c] = 0 skips the
 * cohort), results to device dB[c] (trait j of SNP i at (j*x[c] + i)*p_c)
 * and dV[c] ((j*x[c] + i)*p_c*p_c, the V.out block layout); snp_base may be
 * NULL (first SNP index per cohort, for error reports). */
int fglsgpu_batch_step(fglsgpu_batch *b, const void *const *dX, const int *x, double *const *dB,
                       double *const *dV, const long long *snp_base);
int fglsgpu_batch_sync(fglsgpu_batch *b);
void *fglsgpu_batch_stream(fglsgpu_batch *b);
/* Per-stage timing: while enabled, steps run without the graph and CUDA
 * events bracket the stages; read returns (and clears) the summed ms of
 * [genotypes, split GEMM, quadratic Gram, solves] and the step count. */
int fglsgpu_batch_profile(fglsgpu_batch *b, int enable);
int fglsgpu_batch_profile_read(fglsgpu_batch *b, double *ms, long long *steps);
const char *fglsgpu_batch_last_error(const fglsgpu_batch *b);

#ifdef __cplusplus
}
#endif
#endif /* FGLS_GB300_H */
