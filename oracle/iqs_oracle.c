/* CPU oracle (test infrastructure only): see iqs_oracle.h. The function bodies live in
 * iqs_oracle_impl.inc and are instantiated for ComplexDP (double) and ComplexSP (float). */
#include "iqs_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define T double
#define S d
#include "iqs_oracle_impl.inc"
#undef T
#undef S

#define T float
#define S f
#include "iqs_oracle_impl.inc"
#undef T
#undef S

void or_set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

int or_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
