/*
 * Golden-vector harness around the reference's own C functions.
 *
 * Test infrastructure only.  oracle/build_ref.sh compiles this file together
 * with the reference's UVaTRMM/src/mm_mapping.c and
 * UVaTRMM/src/mm_triangular_common.c (unmodified, from the reference tree)
 * and the single-rank shims in oracle/shim/, into oracle/_ref/ref_harness.
 * tests/golden/make_golden.py runs it to write the committed fixtures.
 *
 *   ref_harness maps <n> <P> <reg|balanced>
 *       one line per block index p:  p begin size  (UVaTRMM/src/mm_mapping.c:27-67
 *       map_regular, :319-366 map_balanced); where the reference aborts, the
 *       process exits with the reference's code after the lines already printed
 *   ref_harness gen <n> <row_begin> <rows> <col_begin> <cols> <triangular>
 *       the block produced by mat_consecutive_values, row-major, %.17g
 *       (UVaTRMM/src/mm_triangular_common.c:1782-1805, built with -DMININUMS=1)
 *   ref_harness result <rows> <cols> <rb> <nrows> <cb> <ncols> <rank> <procs>
 *       writes ./tests/outputs/output_golden.<rows>.<procs>.<rank>.dat with the
 *       reference's print_output_results_generic
 *       (UVaTRMM/src/mm_triangular_common.c:2134-2163) for a fixed block
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "mm_triangular.h"

int main(int argc, char **argv) {
  if (argc >= 5 && !strcmp(argv[1], "maps")) {
    unsigned long n = strtoul(argv[2], 0, 10);
    unsigned int P = (unsigned int)strtoul(argv[3], 0, 10);
    int balanced = !strcmp(argv[4], "balanced");
    for (unsigned int p = 0; p < P; p++) {
      Range r = balanced ? map_balanced(n, P, p, 0) : map_regular(n, P, p, 0);
      printf("%u %lu %lu\n", p, r.begin, r.size);
      fflush(stdout);
    }
    return 0;
  }
  if (argc >= 8 && !strcmp(argv[1], "gen")) {
    int n = atoi(argv[2]);
    Range rows = {strtoul(argv[3], 0, 10), strtoul(argv[4], 0, 10)};
    Range cols = {strtoul(argv[5], 0, 10), strtoul(argv[6], 0, 10)};
    int tri = atoi(argv[7]);
    double *m = calloc(rows.size * cols.size + 1, sizeof(double));
    mat_consecutive_values(rows, cols, m, tri, n);
    for (unsigned long i = 0; i < rows.size * cols.size; i++) printf("%.17g\n", m[i]);
    free(m);
    return 0;
  }
  if (argc >= 10 && !strcmp(argv[1], "result")) {
    /* Block entries are 0.25*k + 1/3 for k = 0, 1, ... in row-major order. */
    int rows = atoi(argv[2]), cols = atoi(argv[3]);
    Range lr = {strtoul(argv[4], 0, 10), strtoul(argv[5], 0, 10)};
    Range lc = {strtoul(argv[6], 0, 10), strtoul(argv[7], 0, 10)};
    int rank = atoi(argv[8]), procs = atoi(argv[9]);
    double *m = calloc(lr.size * lc.size + 1, sizeof(double));
    for (unsigned long i = 0; i < lr.size * lc.size; i++) m[i] = 0.25 * (double)i + 1.0 / 3.0;
    print_output_results_generic(rows, cols, lr, lc, rank, m, procs, "golden");
    free(m);
    return 0;
  }
  fprintf(stderr, "usage: %s maps <n> <P> <reg|balanced> | gen <n> <rb> <rows> <cb> <cols> <tri> |"
          " result <rows> <cols> <rb> <nrows> <cb> <ncols> <rank> <procs>\n", argv[0]);
  return 2;
}
