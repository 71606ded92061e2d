// File-based drop-in entry points with the reference's signatures:
// fgls_chol (src/fgls_chol.c:29), fgls_eigen (src/fgls_eigen.c:38) and
// fgls_chol_gpu (src/fgls_chol_gpu.c:97).  Written only against the public
// engine API of fgls_gb300.h.
//
// The reference's POSIX-aio double buffering (src/io.c:35-98,
// src/fgls_chol.c:327-487) becomes a two-slot pinned host ring:
//   reader thread:  pread(XR block b+1) -> pinned slot
//   h2d stream:     slot -> HBM          (overlaps compute of block b)
//   compute stream: engine block b
//   d2h stream:     B/V of block b -> pinned slot
//   main thread:    pwrite(B/V of block b-1) at the reference's offsets
//                   (j*m + ib)*p and (j*m + ib)*p*p doubles (src/fgls_chol.c:464-474).
// For chol with t > 1 the XR stream is cached in HBM during the first trait
// when it fits (the reference re-reads the file for every trait).
//
// Block-granular resume (opt-in, FGLS_RESUME=1): every finished block is
// appended to the journal <B_path>.done after its B/V bytes are on disk
// (fdatasync), with a header of the run's dimensions.  A later run with the
// same arguments and FGLS_RESUME=1 keeps the output files, skips the
// journaled blocks and computes the rest; results are identical to an
// uninterrupted run because every block lands at its deterministic offset
// (src/fgls_chol.c:467,474).  FGLS_STOP_AFTER=k (host-side interruption for
// tests) exits with status 3 after k newly journaled blocks.
//
// Genotype file formats (FGLS_XR_FORMAT, opt-in; the reference reads FP64
// only, src/fgls_chol.c:333-337):
//   f64 (default)  the reference's XR.in: m*wXR columns of n doubles;
//   u8             the same layout with one byte (0/1/2) per individual;
//   bed            a SNP-major PLINK .bed file: the magic bytes 6c 1b 01, then
//                  m*wXR columns of ceil(n/4) bytes, 2 bits per individual
//                  (00 -> 2, 10 -> 1, 11 -> 0 copies of the first allele,
//                  01 missing: an error naming the SNP and the individual).
// Only the bytes of the chosen format cross the host link (8x or 32x fewer
// than FP64); the device widens them per block.
//
// Errors print "[Error]: <msg>" and exit(EXIT_FAILURE) like the reference's
// error_msg(msg, 1) (src/common.c:11-17).  Unlike the reference's sync_read,
// which prints and continues on a short read (src/io.c:13-16), a short read
// of any input is an error here.
#include <cuda_runtime.h>
#include <errno.h>
#include <fcntl.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "fgls_gb300.h"

namespace {

[[noreturn]] void die(const std::string& msg) {
  fprintf(stderr, "[Error]: %s\n", msg.c_str());
  exit(EXIT_FAILURE);
}

void cuda_check(cudaError_t c, const char* what) {
  if (c != cudaSuccess) die(std::string(what) + ": " + cudaGetErrorString(c));
}

void eng_check(fglsgpu_engine* e, int rc) {
  if (rc != FGLSGPU_OK) die(fglsgpu_last_error(e));
}

// Reads exactly `bytes` at `off` (loops over partial reads); false on EOF/error.
bool pread_full(int fd, void* buf, size_t bytes, off_t off) {
  char* p = (char*)buf;
  while (bytes > 0) {
    ssize_t r = pread(fd, p, bytes, off);
    if (r < 0 && errno == EINTR) continue;
    if (r <= 0) return false;
    p += r;
    bytes -= (size_t)r;
    off += r;
  }
  return true;
}

bool pwrite_full(int fd, const void* buf, size_t bytes, off_t off) {
  const char* p = (const char*)buf;
  while (bytes > 0) {
    ssize_t r = pwrite(fd, p, bytes, off);
    if (r < 0 && errno == EINTR) continue;
    if (r <= 0) return false;
    p += r;
    bytes -= (size_t)r;
    off += r;
  }
  return true;
}

void read_file(const char* path, double* buf, size_t count, const char* what) {
  int fd = open(path, O_RDONLY);
  if (fd < 0) die(std::string("cannot open ") + what + " file " + path + ": " + strerror(errno));
  if (!pread_full(fd, buf, sizeof(double) * count, 0)) {
    close(fd);
    die(std::string("short read of ") + what + " file " + path + " (" + std::to_string(count) + " doubles expected)");
  }
  close(fd);
}

struct Item {
  int trait;       // chol: trait of this pass; eigen: -1 (all traits)
  long long ib;    // first SNP
  int x;           // SNPs in the block
  bool read;       // from disk (else from the HBM cache)
};

enum { XR_F64 = 0, XR_U8 = 1, XR_BED = 2 };

int xr_format() {
  const char* f = getenv("FGLS_XR_FORMAT");
  if (!f || !*f || !strcmp(f, "f64")) return XR_F64;
  if (!strcmp(f, "u8")) return XR_U8;
  if (!strcmp(f, "bed")) return XR_BED;
  die(std::string("FGLS_XR_FORMAT=") + f + ": expected f64, u8 or bed");
}

// First missing call (2-bit code 01) of a .bed body region of `cols`
// columns starting at column c0: (column, individual), or (-1, -1).
std::pair<long long, int> find_missing_bed(int fd, off_t data_off, int n, long long c0, long long cols) {
  const long long bpc = (n + 3) / 4;
  std::vector<unsigned char> col((size_t)bpc);
  for (long long c = c0; c < c0 + cols; c++) {
    if (!pread_full(fd, col.data(), (size_t)bpc, data_off + (off_t)(c * bpc))) break;
    for (int k = 0; k < n; k++)
      if (((col[k >> 2] >> (2 * (k & 3))) & 3) == 1) return {c, k};
  }
  return {-1, -1};
}

struct Slot {
  unsigned char* hX = nullptr;  // genotype bytes of one block (format of the XR file)
  double *hB = nullptr, *hV = nullptr;
  unsigned char* dX = nullptr;
  double *dB = nullptr, *dV = nullptr;
  cudaEvent_t evH{}, evC{}, evD{};
  std::thread reader;
  bool read_ok = true;
  int item = -1;
};

int run_variant(int variant, int n, int p, int m, int t, int wXL, int wXR, int x_b, int num_threads,
                const char* Phi_path, const char* h_path, const char* s_path, const char* XL_path,
                const char* XR_path, const char* Y_path, const char* B_path, const char* V_path) {
  (void)num_threads;
  if (n <= 0 || m <= 0 || t <= 0 || wXL <= 0 || wXR <= 0 || x_b <= 0)
    die("invalid dimensions (n, m, t, wXL, wXR and x_b must be positive)");
  if (p != wXL + wXR) die("p must equal wXL + wXR");
  x_b = std::min(x_b, m);
  fglsgpu_config cfg{};
  cfg.n = n;
  cfg.wXL = wXL;
  cfg.wXR = wXR;
  cfg.t = t;
  cfg.x_b = x_b;
  cfg.variant = variant;
  const char* prec = getenv("FGLS_PRECISION");
  cfg.precision = (prec && !strcmp(prec, "split")) ? FGLSGPU_PREC_SPLIT : FGLSGPU_PREC_FP64;
  const char* sl = getenv("FGLS_SLICES");
  cfg.slices = sl ? atoi(sl) : 0;
  const char* dev = getenv("FGLS_DEVICE");
  cfg.device = dev ? atoi(dev) : 0;

  std::vector<double> Phi((size_t)n * n), h(t), sg(t), XL((size_t)n * wXL), Y((size_t)n * t);
  read_file(Phi_path, Phi.data(), Phi.size(), "Phi");
  read_file(h_path, h.data(), t, "h");
  read_file(s_path, sg.data(), t, "sigma");
  read_file(XL_path, XL.data(), XL.size(), "XL");
  read_file(Y_path, Y.data(), Y.size(), "Y");

  fglsgpu_engine* e = nullptr;
  if (fglsgpu_create(&cfg, &e) != FGLSGPU_OK) die(fglsgpu_last_error(nullptr));
  eng_check(e, fglsgpu_set_problem(e, Phi.data(), XL.data(), Y.data(), h.data(), sg.data()));
  Phi.clear();
  Phi.shrink_to_fit();

  int xr_fd = open(XR_path, O_RDONLY);
  if (xr_fd < 0) die(std::string("cannot open XR file ") + XR_path + ": " + strerror(errno));
  const int fmt = xr_format();
  off_t xr_off = 0;  // first genotype byte of the file
  if (fmt == XR_BED) {
    unsigned char magic[3] = {0, 0, 0};
    if (!pread_full(xr_fd, magic, 3, 0) || magic[0] != 0x6c || magic[1] != 0x1b || magic[2] != 0x01)
      die(std::string("XR file ") + XR_path + " is not a SNP-major PLINK .bed (magic bytes 6c 1b 01)");
    xr_off = 3;
  }
  // resume journal: header line, then one "<trait> <first SNP>" line per finished block
  const char* rs = getenv("FGLS_RESUME");
  const bool resume = rs && atoi(rs) != 0;
  const char* sa = getenv("FGLS_STOP_AFTER");
  const long long stop_after = sa ? atoll(sa) : -1;
  const std::string jpath = std::string(B_path) + ".done";
  char header[256];
  snprintf(header, sizeof header, "fgls-journal v1 variant=%d n=%d p=%d m=%d t=%d wXL=%d wXR=%d x_b=%d", variant, n, p,
           m, t, wXL, wXR, x_b);
  std::vector<std::pair<int, long long>> done;
  bool have_journal = false;
  if (resume) {
    FILE* jf = fopen(jpath.c_str(), "r");
    if (jf) {
      char line[512];
      if (!fgets(line, sizeof line, jf) || strncmp(line, header, strlen(header)) != 0) {
        fclose(jf);
        die("resume journal " + jpath + " was written for different arguments");
      }
      int tr;
      long long ib;
      while (fscanf(jf, "%d %lld", &tr, &ib) == 2) done.push_back({tr, ib});
      fclose(jf);
      have_journal = true;
    }
  }
  const int oflags = O_WRONLY | O_CREAT | (have_journal ? 0 : O_TRUNC);
  int b_fd = open(B_path, oflags, 0644);
  int v_fd = open(V_path, oflags, 0644);
  if (b_fd < 0 || v_fd < 0) die("cannot open the output files");
  FILE* journal = nullptr;
  if (resume) {
    journal = fopen(jpath.c_str(), have_journal ? "a" : "w");
    if (!journal) die("cannot open the resume journal " + jpath);
    if (!have_journal) {
      fprintf(journal, "%s\n", header);
      fflush(journal);
    }
  }

  const int nt = variant == FGLSGPU_VARIANT_EIGEN ? t : 1;
  const long long bpc = fmt == XR_F64 ? 8LL * n : fmt == XR_U8 ? (long long)n : (long long)(n + 3) / 4;
  const long long colb = bpc * wXR;  // genotype bytes per SNP
  cudaStream_t comp = (cudaStream_t)fglsgpu_stream(e);
  cudaStream_t h2d, d2h;
  cuda_check(cudaStreamCreateWithFlags(&h2d, cudaStreamNonBlocking), "stream");
  cuda_check(cudaStreamCreateWithFlags(&d2h, cudaStreamNonBlocking), "stream");

  // Keep XR resident in HBM across chol traits when it fits.
  unsigned char* dXall = nullptr;
  if (variant == FGLSGPU_VARIANT_CHOL && t > 1 && done.empty()) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    const size_t need = (size_t)colb * m;
    if (need + ((size_t)4 << 30) < fr) {
      if (cudaMalloc((void**)&dXall, need) != cudaSuccess) {
        cudaGetLastError();
        dXall = nullptr;
      }
    }
  }

  Slot sl2[2];
  for (Slot& s : sl2) {
    cuda_check(cudaMallocHost((void**)&s.hX, (size_t)colb * x_b), "pinned XR slot");
    cuda_check(cudaMallocHost((void**)&s.hB, sizeof(double) * nt * x_b * p), "pinned B slot");
    cuda_check(cudaMallocHost((void**)&s.hV, sizeof(double) * nt * x_b * p * p), "pinned V slot");
    cuda_check(cudaMalloc((void**)&s.dX, (size_t)colb * x_b), "XR slot");
    cuda_check(cudaMalloc((void**)&s.dB, sizeof(double) * nt * x_b * p), "B slot");
    cuda_check(cudaMalloc((void**)&s.dV, sizeof(double) * nt * x_b * p * p), "V slot");
    cuda_check(cudaEventCreateWithFlags(&s.evH, cudaEventDisableTiming), "event");
    cuda_check(cudaEventCreateWithFlags(&s.evC, cudaEventDisableTiming), "event");
    cuda_check(cudaEventCreateWithFlags(&s.evD, cudaEventDisableTiming), "event");
  }

  std::vector<Item> items;
  const int passes = variant == FGLSGPU_VARIANT_EIGEN ? 1 : t;
  long long skipped = 0;
  for (int j = 0; j < passes; j++)
    for (long long ib = 0; ib < m; ib += x_b) {
      const int tr = variant == FGLSGPU_VARIANT_EIGEN ? -1 : j;
      if (std::find(done.begin(), done.end(), std::make_pair(tr, ib)) != done.end()) {
        skipped++;
        continue;
      }
      items.push_back({tr, ib, (int)std::min<long long>(x_b, m - ib), !(dXall && j > 0)});
    }
  if (resume && skipped)
    fprintf(stderr, "[resume] %lld of %lld blocks already done\n", skipped, skipped + (long long)items.size());
  long long journaled = 0;

  auto start_read = [&](int i) {
    Slot& s = sl2[i & 1];
    const Item& it = items[i];
    s.read_ok = true;
    if (!it.read) return;
    s.reader = std::thread([&s, xr_fd, xr_off, colb, it]() {
      s.read_ok = pread_full(xr_fd, s.hX, (size_t)colb * it.x, xr_off + (off_t)(colb * it.ib));
    });
  };
  auto write_out = [&](int i) {
    Slot& s = sl2[i & 1];
    const Item& it = items[i];
    cuda_check(cudaEventSynchronize(s.evD), "download");
    for (int q = 0; q < nt; q++) {
      const int j = variant == FGLSGPU_VARIANT_EIGEN ? q : it.trait;
      const off_t ob = (off_t)sizeof(double) * ((off_t)j * m * p + (off_t)it.ib * p);
      const off_t ov = (off_t)sizeof(double) * ((off_t)j * m * p * p + (off_t)it.ib * p * p);
      if (!pwrite_full(b_fd, s.hB + (size_t)q * it.x * p, sizeof(double) * it.x * p, ob) ||
          !pwrite_full(v_fd, s.hV + (size_t)q * it.x * p * p, sizeof(double) * it.x * p * p, ov))
        die(std::string("write to ") + B_path + " / " + V_path + " failed: " + strerror(errno));
    }
    if (journal) {
      if (fdatasync(b_fd) != 0 || fdatasync(v_fd) != 0)
        die(std::string("flushing ") + B_path + " / " + V_path + " failed: " + strerror(errno));
      fprintf(journal, "%d %lld\n", it.trait, it.ib);
      if (fflush(journal) != 0 || fdatasync(fileno(journal)) != 0) die("writing the resume journal failed");
      if (stop_after >= 0 && ++journaled >= stop_after) {
        fprintf(stderr, "[resume] stopping after %lld blocks (FGLS_STOP_AFTER)\n", journaled);
        cudaDeviceSynchronize();  // leave between blocks, with no work in flight
        exit(3);
      }
    }
  };

  // Device failures are read at trait ends (chol) and at the end; a missing
  // call in a .bed file is reported with its SNP and individual, found by
  // scanning the file on the host (the device only knows the block).
  auto sync_check = [&](fglsgpu_engine* eng) {
    const int rc = fglsgpu_sync(eng);
    if (rc == FGLSGPU_OK) return;
    if (rc == FGLSGPU_EINVAL && fmt == XR_BED) {
      const auto miss = find_missing_bed(xr_fd, xr_off, n, 0, (long long)m * wXR);
      if (miss.first >= 0)
        die(std::string("missing genotype (2-bit code 01) in ") + XR_path + " at SNP " +
            std::to_string(miss.first / wXR) + ", individual " + std::to_string(miss.second));
    }
    die(fglsgpu_last_error(eng));
  };
  if (!items.empty()) start_read(0);
  int cur_trait = -1;
  for (size_t i = 0; i < items.size(); i++) {
    Slot& s = sl2[i & 1];
    Slot& o = sl2[(i + 1) & 1];
    const Item& it = items[i];
    if (variant == FGLSGPU_VARIANT_CHOL && it.trait != cur_trait) {
      if (cur_trait >= 0) sync_check(e);  // report device failures of the finished trait
      eng_check(e, fglsgpu_select_trait(e, it.trait));
      cur_trait = it.trait;
    }
    const unsigned char* src;
    if (it.read) {
      s.reader.join();
      if (!s.read_ok)
        die(std::string("short read of XR file ") + XR_path + " at SNP " + std::to_string(it.ib));
      unsigned char* dst = dXall ? dXall + it.ib * colb : s.dX;
      cuda_check(cudaStreamWaitEvent(h2d, s.evC, 0), "wait");
      cuda_check(cudaMemcpyAsync(dst, s.hX, (size_t)colb * it.x, cudaMemcpyHostToDevice, h2d), "XR upload");
      cuda_check(cudaEventRecord(s.evH, h2d), "event");
      cuda_check(cudaStreamWaitEvent(comp, s.evH, 0), "wait");
      src = dst;
    } else {
      src = dXall + it.ib * colb;
    }
    cuda_check(cudaStreamWaitEvent(comp, s.evD, 0), "wait");
    const long long bs = (long long)it.x * p, vs = (long long)it.x * p * p;
    if (fmt == XR_F64)
      eng_check(e, fglsgpu_run_block_device(e, (const double*)src, it.x, s.dB, s.dV, bs, vs));
    else if (fmt == XR_U8)
      eng_check(e, fglsgpu_run_block_device_u8(e, src, it.x, s.dB, s.dV, bs, vs));
    else
      eng_check(e, fglsgpu_run_block_device_packed(e, src, it.x, s.dB, s.dV, bs, vs));
    cuda_check(cudaEventRecord(s.evC, comp), "event");
    cuda_check(cudaStreamWaitEvent(d2h, s.evC, 0), "wait");
    cuda_check(cudaMemcpyAsync(s.hB, s.dB, sizeof(double) * nt * it.x * p, cudaMemcpyDeviceToHost, d2h), "B download");
    cuda_check(cudaMemcpyAsync(s.hV, s.dV, sizeof(double) * nt * it.x * p * p, cudaMemcpyDeviceToHost, d2h),
               "V download");
    cuda_check(cudaEventRecord(s.evD, d2h), "event");
    if (i + 1 < items.size()) {
      cuda_check(cudaEventSynchronize(o.evH), "upload");  // o.hX no longer read by block i-1's upload
      start_read((int)i + 1);
    }
    if (i >= 1) write_out((int)i - 1);
  }
  if (!items.empty()) write_out((int)items.size() - 1);
  sync_check(e);

  for (Slot& s : sl2) {
    if (s.reader.joinable()) s.reader.join();
    cudaFreeHost(s.hX);
    cudaFreeHost(s.hB);
    cudaFreeHost(s.hV);
    cudaFree(s.dX);
    cudaFree(s.dB);
    cudaFree(s.dV);
    cudaEventDestroy(s.evH);
    cudaEventDestroy(s.evC);
    cudaEventDestroy(s.evD);
  }
  if (dXall) cudaFree(dXall);
  cudaStreamDestroy(h2d);
  cudaStreamDestroy(d2h);
  close(xr_fd);
  if (journal) fclose(journal);
  if (close(b_fd) != 0 || close(v_fd) != 0) die("closing the output files failed");
  fglsgpu_destroy(e);
  return 0;
}

}  // namespace

extern "C" {

int fgls_chol(int n, int p, int m, int t, int wXL, int wXR, int x_b, int y_b, int num_threads, char* Phi_path,
              char* h2_path, char* sigma2_path, char* XL_path, char* XR_path, char* Y_path, char* B_path,
              char* V_path) {
  if (y_b != 1) fprintf(stderr, "[Warning] y_b not used (set to 1)\n");  // src/fgls_chol.c:102-103
  return run_variant(FGLSGPU_VARIANT_CHOL, n, p, m, t, wXL, wXR, x_b, num_threads, Phi_path, h2_path, sigma2_path,
                     XL_path, XR_path, Y_path, B_path, V_path);
}

int fgls_chol_gpu(int n, int p, int m, int t, int wXL, int wXR, int x_b, int y_b, int num_threads, char* Phi_path,
                  char* h2_path, char* sigma2_path, char* XL_path, char* XR_path, char* Y_path, char* B_path,
                  char* V_path) {
  return fgls_chol(n, p, m, t, wXL, wXR, x_b, y_b, num_threads, Phi_path, h2_path, sigma2_path, XL_path, XR_path,
                   Y_path, B_path, V_path);
}

int fgls_eigen(int n, int p, int m, int t, int wXL, int wXR, int x_b, int y_b, int num_threads, char* Phi_path,
               char* h2_path, char* sigma2_path, char* XL_path, char* XR_path, char* Y_path, char* B_path,
               char* V_path) {
  (void)y_b;  // traits are the GEMM N dimension: all t traits of a block in one pass
  return run_variant(FGLSGPU_VARIANT_EIGEN, n, p, m, t, wXL, wXR, x_b, num_threads, Phi_path, h2_path,
                     sigma2_path, XL_path, XR_path, Y_path, B_path, V_path);
}

}  // extern "C"
