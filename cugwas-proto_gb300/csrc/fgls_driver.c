/*
 * Command-line driver with the reference's interface (src/driver.c:15-100):
 *
 *   fgls-driver <variant> <data_set_directory> <#repetitions>
 *   stdin: n p m t wXL x_b y_b threads
 *
 * variant 'e' -> fgls_eigen, 'g' -> fgls_chol_gpu, anything else -> fgls_chol.
 * Reads <dir>/{Phi,H,Sig,XL,XR,Y}.in, writes <dir>/{B,V}.out, and prints the
 * mean wall-clock milliseconds per repetition.  wXR = p - wXL.
 */
#define _POSIX_C_SOURCE 200809L
#include <stdio.h>
#include <stdlib.h>
#include <time.h>

#include "fgls_gb300.h"

#define PATHLEN 4096

int main(int argc, char *argv[]) {
  if (argc != 4) {
    fprintf(stderr, "Usage: %s <variant - [c|e|g]> <data_set_directory> <#repetitions>\n", argv[0]);
    fprintf(stderr, "\tnote: data_set_directory must contain files:\n");
    fprintf(stderr, "- Phi.in\n- H.in\n- Sig.in\n- XL.in\n- XR.in\n- Y.in\n");
    return EXIT_FAILURE;
  }
  const char var = argv[1][0];
  const char *dir = argv[2];
  const int nrep = atoi(argv[3]);
  int n, p, m, t, wXL, x_b, y_b, threads;
  if (scanf("%d %d %d %d %d %d %d %d", &n, &p, &m, &t, &wXL, &x_b, &y_b, &threads) != 8) {
    fprintf(stderr, "[Error]: expected 'n p m t wXL x_b y_b threads' on stdin\n");
    return EXIT_FAILURE;
  }
  const int wXR = p - wXL;
  char Phi[PATHLEN], H[PATHLEN], Sig[PATHLEN], XL[PATHLEN], XR[PATHLEN], Y[PATHLEN], B[PATHLEN], V[PATHLEN];
  snprintf(Phi, PATHLEN, "%s/Phi.in", dir);
  snprintf(H, PATHLEN, "%s/H.in", dir);
  snprintf(Sig, PATHLEN, "%s/Sig.in", dir);
  snprintf(XL, PATHLEN, "%s/XL.in", dir);
  snprintf(XR, PATHLEN, "%s/XR.in", dir);
  snprintf(Y, PATHLEN, "%s/Y.in", dir);
  snprintf(B, PATHLEN, "%s/B.out", dir);
  snprintf(V, PATHLEN, "%s/V.out", dir);
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (int i = 0; i < nrep; i++) {
    if (var == 'e')
      fgls_eigen(n, p, m, t, wXL, wXR, x_b, y_b, threads, Phi, H, Sig, XL, XR, Y, B, V);
    else if (var == 'g')
      fgls_chol_gpu(n, p, m, t, wXL, wXR, x_b, y_b, threads, Phi, H, Sig, XL, XR, Y, B, V);
    else
      fgls_chol(n, p, m, t, wXL, wXR, x_b, y_b, threads, Phi, H, Sig, XL, XR, Y, B, V);
  }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  const double ms = (t1.tv_sec - t0.tv_sec) * 1e3 + (t1.tv_nsec - t0.tv_nsec) * 1e-6;
  printf("%ld\n", nrep > 0 ? (long)(ms / nrep) : 0L);
  return 0;
}
