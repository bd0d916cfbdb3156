/* Plain C client of include/sus2g.h (the binding a C host, or a cgo / FFI stub, would use):
 * loads a .sus2 model through the library's host code, prints its dimensions, cutoff and
 * parameter count, round-trips the parameter vector, and checks that a missing file is reported
 * through the error code and sus2g_last_error().  Needs no GPU.
 *
 * Usage: model_info MODEL.sus2
 * Prints: INFO <dims0> ... <dims15> <cutoff> <param count> <sum of |params|> and exits 0. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "sus2g.h"

int main(int argc, char** argv) {
  if (argc != 2) {
    fprintf(stderr, "usage: model_info MODEL.sus2\n");
    return 2;
  }
  if (sus2g_abi_version() != 100) return 3;
  sus2g_model bad = NULL;
  if (sus2g_model_load("/nonexistent/model.sus2", &bad) == 0 || bad != NULL) return 4;
  if (sus2g_last_error()[0] == '\0') return 5;

  sus2g_model m = NULL;
  if (sus2g_model_load(argv[1], &m)) {
    fprintf(stderr, "%s\n", sus2g_last_error());
    return 1;
  }
  int dims[16];
  double cutoff = 0;
  int n = 0;
  if (sus2g_model_dims(m, dims) || sus2g_model_cutoff(m, &cutoff) || sus2g_model_param_count(m, &n)) return 6;
  double* p = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  if (!p || sus2g_model_get_params(m, p, n) || sus2g_model_set_params(m, p, n)) return 7;
  double sum = 0;
  for (int i = 0; i < n; ++i) sum += fabs(p[i]);
  printf("INFO");
  for (int i = 0; i < 16; ++i) printf(" %d", dims[i]);
  printf(" %.17g %d %.17g\n", cutoff, n, sum);
  free(p);
  sus2g_model_free(m);
  return 0;
}
