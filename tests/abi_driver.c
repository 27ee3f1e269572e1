/* Drives libcelllist_cuda.so through its C ABI from plain C (the way a C, Fortran or Julia `ccall`
 * client would), on cases with known answers:
 *   a simple cubic lattice of 10^3 points with spacing 1 and cutoff 1 (inclusive, src/internals/self.jl:153)
 *   - periodic box of side 10: every point has 6 neighbours at distance 1 -> 3000 pairs, sum d2 = 3000;
 *   - non-periodic: 3 x 10 x 10 x 9 = 2700 pairs;
 *   - a NaN coordinate: CLM_ERR_NAN (src/internals/CellOperations.jl:6-21).
 * Test infrastructure: compiled and run by tests/test_abi.py.  Exit status 0 on success. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "celllistmap_gb300.h"

static int fail(const char* what, clm_handle h, int st) {
  char buf[256] = {0};
  if (h) clm_last_error(h, buf, sizeof(buf));
  fprintf(stderr, "abi driver: %s failed (status %d) %s\n", what, st, buf);
  return 1;
}

static int lattice_case(int kind, int64_t want_pairs) {
  const int64_t n = 1000;
  double* x = (double*)malloc(sizeof(double) * 3 * (size_t)n);
  int64_t k = 0;
  for (int a = 0; a < 10; a++)
    for (int b = 0; b < 10; b++)
      for (int c = 0; c < 10; c++) {
        x[3 * k + 0] = a;
        x[3 * k + 1] = b;
        x[3 * k + 2] = c;
        k++;
      }
  double M[9] = {0};
  if (kind != CLM_NONPERIODIC) M[0] = M[4] = M[8] = 10.0;
  clm_handle h = NULL;
  int st = clm_create(CLM_F64, 3, 1, &h);
  if (st) return fail("clm_create", NULL, st);
  if ((st = clm_set_box(h, M, kind, 1.0, 1))) return fail("clm_set_box", h, st);
  if ((st = clm_set_positions(h, 0, x, n, 0))) return fail("clm_set_positions", h, st);
  clm_op_params p;
  clm_outputs o;
  memset(&p, 0, sizeof(p));
  memset(&o, 0, sizeof(o));
  if ((st = clm_run(h, CLM_OP_COUNT, &p, &o))) return fail("clm_run(COUNT)", h, st);
  if (o.count != want_pairs) {
    fprintf(stderr, "abi driver: %lld pairs, expected %lld\n", (long long)o.count, (long long)want_pairs);
    return 1;
  }
  memset(&o, 0, sizeof(o));
  if ((st = clm_run(h, CLM_OP_SUM_D2, &p, &o))) return fail("clm_run(SUM_D2)", h, st);
  if (o.scalar != (double)want_pairs) {
    fprintf(stderr, "abi driver: sum d2 = %.17g, expected %lld\n", o.scalar, (long long)want_pairs);
    return 1;
  }
  memset(&o, 0, sizeof(o));
  if ((st = clm_run(h, CLM_OP_NL, &p, &o))) return fail("clm_run(NL)", h, st);
  int64_t m = 0;
  if ((st = clm_nl_count(h, &m))) return fail("clm_nl_count", h, st);
  if (m != want_pairs) {
    fprintf(stderr, "abi driver: list of %lld pairs, expected %lld\n", (long long)m, (long long)want_pairs);
    return 1;
  }
  int64_t* pi = (int64_t*)malloc(sizeof(int64_t) * (size_t)m);
  int64_t* pj = (int64_t*)malloc(sizeof(int64_t) * (size_t)m);
  double* pd = (double*)malloc(sizeof(double) * (size_t)m);
  if ((st = clm_nl_fetch(h, pi, pj, pd, m, 1, 0))) return fail("clm_nl_fetch", h, st);
  for (int64_t q = 0; q < m; q++) {
    if (pd[q] != 1.0 || pi[q] < 1 || pi[q] > n || pj[q] < 1 || pj[q] > n || pi[q] == pj[q]) {
      fprintf(stderr, "abi driver: bad pair (%lld, %lld, %.17g)\n", (long long)pi[q], (long long)pj[q], pd[q]);
      return 1;
    }
  }
  /* a NaN coordinate is reported, not computed */
  x[3 * 17 + 1] = NAN;
  if ((st = clm_set_positions(h, 0, x, n, 0))) return fail("clm_set_positions(NaN)", h, st);
  st = clm_run(h, CLM_OP_COUNT, &p, &o);
  if (st != CLM_ERR_NAN) {
    fprintf(stderr, "abi driver: NaN coordinates gave status %d, expected %d\n", st, (int)CLM_ERR_NAN);
    return 1;
  }
  free(pi);
  free(pj);
  free(pd);
  free(x);
  if ((st = clm_destroy(h))) return fail("clm_destroy", NULL, st);
  return 0;
}

int main(void) {
  if (lattice_case(CLM_ORTHO, 3000)) return 1;
  if (lattice_case(CLM_NONPERIODIC, 2700)) return 1;
  printf("abi driver ok\n");
  return 0;
}
