/* A C caller of the reference's API (the pattern of tests/simple_test.c and
 * tests/check_trafo.c of the reference), built against include/pnfft.h and
 * libpnfft_gb300.so: pnfft_init_guru, pnfft_init_nodes, the reference's input
 * generators, pnfft_trafo and pnfft_adj.  It writes x, f_hat, f = trafo(f_hat)
 * and adj(f) as raw doubles into the directory argv[1] (x.bin, fhat.bin,
 * f.bin, adj.bin) for the test to check against the oracle; argv[2] = "fp32"
 * selects the FP32-mixed form.  Exit status 0 on success. */
#include <stdio.h>
#include <string.h>

#include <pnfft.h>

static int dump(const char *dir, const char *name, const void *p, size_t bytes) {
  char path[1024];
  snprintf(path, sizeof path, "%s/%s", dir, name);
  FILE *fp = fopen(path, "wb");
  if (!fp) return 1;
  size_t w = fwrite(p, 1, bytes, fp);
  fclose(fp);
  return w != bytes;
}

int main(int argc, char **argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s outdir [fp32]\n", argv[0]);
    return 2;
  }
  const int fp32 = argc > 2 && strcmp(argv[2], "fp32") == 0;
  ptrdiff_t N[3] = {16, 16, 16}, n[3] = {32, 32, 32}, M = 3000;
  double x_max[3] = {0.5, 0.5, 0.5};
  ptrdiff_t lN[3], lNs[3];
  double lo[3], up[3];
  pnfft_init();
  pnfft_local_size_guru(3, N, n, x_max, 4, MPI_COMM_WORLD, PNFFT_TRANSPOSED_NONE, lN, lNs, lo, up);
  unsigned flags = PNFFT_MALLOC_F_HAT | PNFFT_WINDOW_KAISER_BESSEL | (fp32 ? PNFFT_GB300_FP32 : 0);
  pnfft_plan p = pnfft_init_guru(3, N, n, x_max, 4, flags, PFFT_ESTIMATE, MPI_COMM_WORLD);
  pnfft_nodes nd = pnfft_init_nodes(M, PNFFT_MALLOC_X | PNFFT_MALLOC_F);
  if (!p || !nd) return 3;
  const ptrdiff_t S = lN[0] * lN[1] * lN[2];
  pnfft_init_f_hat_3d(N, lN, lNs, PNFFT_TRANSPOSED_NONE, pnfft_get_f_hat(p));
  pnfft_init_x_3d(lo, up, M, pnfft_get_x(nd));
  int rc = dump(argv[1], "x.bin", pnfft_get_x(nd), sizeof(double) * 3 * (size_t)M);
  rc |= dump(argv[1], "fhat.bin", pnfft_get_f_hat(p), sizeof(double) * 2 * (size_t)S);
  pnfft_gb300_clear_error();
  pnfft_trafo(p, nd, PNFFT_COMPUTE_F);
  if (pnfft_gb300_last_error()[0]) return 4;
  rc |= dump(argv[1], "f.bin", pnfft_get_f(nd), sizeof(double) * 2 * (size_t)M);
  pnfft_adj(p, nd, PNFFT_COMPUTE_F);
  if (pnfft_gb300_last_error()[0]) return 5;
  rc |= dump(argv[1], "adj.bin", pnfft_get_f_hat(p), sizeof(double) * 2 * (size_t)S);
  pnfft_free_nodes(nd, PNFFT_FREE_X | PNFFT_FREE_F);
  pnfft_finalize(p, PNFFT_FREE_F_HAT);
  pnfft_cleanup();
  return rc ? 6 : 0;
}
