/*
 * uvatrmm.x -- the reference's command line on one GB300.
 *
 *   uvatrmm.x <MatrixDimension> <reg|balanced> <boxes|trapezoid>
 *
 * Same arguments, output and exit codes as the reference program
 * (UVaTRMM/src/mm_triangular.c:7-436, usage text
 * UVaTRMM/src/mm_triangular_common.c:1206-1225):
 *   - inputs: the reference's deterministic data, A lower triangular
 *     (UVaTRMM/src/mm_triangular_common.c:1782-1805), generated on the device;
 *   - C = tril(A) * B on the GPU through uvatrmm_product; the mapping picks
 *     the tile schedule and the shape picks the diagonal-tile geometry;
 *   - stdout "\nTotal t: %lf\nTotal mpis: %d\nMult t: %lf\n" then
 *     "\nNorm: %.3lf\n", and norm_ff.txt holding the norm
 *     (UVaTRMM/src/mm_triangular.c:426, UVaTRMM/src/mm_triangular_common.c:2986-2988).
 *     "Total mpis" reports 1: one process drives one GPU.
 *   - bad arguments print the usage on stderr and exit with the reference's
 *     code for INVALID_ARGS (UVaTRMM/include/error.h:20-38, exit value + 2).
 * The shapes full / triang / triang_2buff / triang_2type / trapezoid_bilateral
 * that the reference also parses are rejected here as unknown (they are
 * broken or unreachable in the reference).
 */
#define _POSIX_C_SOURCE 200809L
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "uvatrmm.h"

enum { EXIT_INVALID_ARGS = 1 + 2, EXIT_RUNTIME = 16 + 2 };

static void usage(const char *prog, const char *msg) {
  fprintf(stderr, "\nError: %s\n", msg);
  fprintf(stderr, "\nUsage: %s <num_rows> <map_func> <comm_shape>\n\n", prog);
  fprintf(stderr, "Map functions:\n");
  fprintf(stderr, "\treg\tRegular with remainder in the last proc.\n");
  fprintf(stderr, "\tbalanced\tBalanced according to the total number of non-zero elements\n");
  fprintf(stderr, "\n");
  fprintf(stderr, "Communication shapes:\n");
  fprintf(stderr, "\tboxes\tMinimal rectangular shapes, bounding boxes including the triangle\n");
  fprintf(stderr, "\ttrapezoid\tExact comm. One indexed type with the trapezoid (rectangle + triangle\n");
  fprintf(stderr, "\n");
  exit(EXIT_INVALID_ARGS);
}

static double now(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + ts.tv_nsec * 1e-9;
}

static void die(const char *what) {
  fprintf(stderr, "uvatrmm.x: %s: %s\n", what, uvatrmm_last_error());
  exit(EXIT_RUNTIME);
}

int main(int argc, char **argv) {
  if (argc != 4) usage(argv[0], "Number of arguments");
  long long n = atoll(argv[1]);
  int schedule, shape;
  if (!strcmp(argv[2], "reg")) schedule = UVATRMM_SCHED_REG;
  else if (!strcmp(argv[2], "balanced")) schedule = UVATRMM_SCHED_BALANCED;
  else usage(argv[0], "Unknown name of mapping function");
  if (!strcmp(argv[3], "boxes")) shape = UVATRMM_SHAPE_BOXES;
  else if (!strcmp(argv[3], "trapezoid")) shape = UVATRMM_SHAPE_TRAPEZOID;
  else usage(argv[0], "Unknown name of communication shape");
  if (n < 1) usage(argv[0], "Number of rows should be equal or greater than number of processors");

  uvatrmm_handle_t h;
  if (uvatrmm_create(&h) != UVATRMM_OK) die("handle");
  size_t bytes = (size_t)n * (size_t)n * sizeof(double);
  void *dA, *dB, *dC;
  if (uvatrmm_device_alloc(bytes, &dA) || uvatrmm_device_alloc(bytes, &dB) || uvatrmm_device_alloc(bytes, &dC))
    die("device allocation");
  if (uvatrmm_gen_consecutive(h, n, 1, (double *)dA) || uvatrmm_gen_consecutive(h, n, 0, (double *)dB))
    die("input generation");
  if (uvatrmm_sync(h)) die("input generation");

  double t0 = now(), mult = 0.0;
  if (uvatrmm_product(h, n, schedule, shape, (const double *)dA, (const double *)dB, (double *)dC, &mult))
    die("product");
  double total = now() - t0;
  printf("\nTotal t: %lf\nTotal mpis: %d\nMult t: %lf\n", total, 1, mult);

  double norm = 0.0;
  if (uvatrmm_inf_norm(h, n, n, (const double *)dC, n, &norm)) die("norm");
  FILE *f = fopen("norm_ff.txt", "w+");
  printf("\nNorm: %.3lf\n", norm);
  if (f) {
    fprintf(f, "%.3lf", norm);
    fclose(f);
  }
  uvatrmm_device_free(dA);
  uvatrmm_device_free(dB);
  uvatrmm_device_free(dC);
  uvatrmm_destroy(h);
  return 0;
}
