/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Nothing in the product library links,
 * loads or calls this file.
 *
 * C restatement of the reference's two Fortran helper files, which cannot be
 * compiled here (no Fortran compiler in the image):
 *
 *   ran_ / initran_   ran.f90:2-16 and ran.f90:19-48
 *       64-bit linear congruential generator
 *       x <- x * 2862933555777941757 + 1013904243   (wrapping int64)
 *       ran = 0.5 + x * (0.5 / (2^63 - 1))          (a double in (0,1))
 *   isort_ / isort2_ / dsort2_   sort2.f:5-37, sort2.f:39-74, sort2.f:76-108
 *       Shell sort with gap n/2, n/4, ..., 1 and an exchange inner loop,
 *       ascending in the first array; the companion array is permuted in
 *       lockstep.  The order in which equal keys end up is whatever this exact
 *       exchange sequence produces, which is why the truncation step (global
 *       selection of kept singular values) needs this very algorithm and not a
 *       generic stable sort.
 *
 * The symbol names carry the trailing underscore of the Fortran ABI so that the
 * unmodified reference C++ sources link against this file.
 */
#include <stdint.h>

static int64_t ran64_state = 0;
static const int64_t ran64_mul = INT64_C(2862933555777941757);
static const int64_t ran64_add = INT64_C(1013904243);

double ran_(void) {
  /* wrapping multiply-add in unsigned arithmetic (signed overflow is UB in C) */
  uint64_t x = (uint64_t)ran64_state * (uint64_t)ran64_mul + (uint64_t)ran64_add;
  ran64_state = (int64_t)x;
  /* irmax = 2*(2^31^2 - 1) + 1 = 2^63 - 1 ; dmu64 = 0.5 / dble(irmax) */
  const double dmu64 = 0.5 / 9223372036854775807.0;
  return 0.5 + dmu64 * (double)ran64_state;
}

/* The reference calls initran_ with a pointer to a C int (main_omp.cpp:38-40). */
void initran_(const int *w) { ran64_state = (int64_t)(*w); }

/* the generator's state, for tests that continue the stream across calls */
int64_t or_ran_state(void) { return ran64_state; }
void or_set_ran_state(int64_t s) { ran64_state = s; }

void isort_(const int *n, int *a) {
  int len = *n;
  for (int gap = len / 2; gap > 0; gap /= 2) {
    for (int i = gap; i < len; ++i) {
      int j = i - gap;
      while (a[j] > a[j + gap]) {
        int t = a[j]; a[j] = a[j + gap]; a[j + gap] = t;
        if (j >= gap) j -= gap; else break;
      }
    }
  }
}

void isort2_(const int *n, int *a, int *b) {
  int len = *n;
  for (int gap = len / 2; gap > 0; gap /= 2) {
    for (int i = gap; i < len; ++i) {
      int j = i - gap;
      while (a[j] > a[j + gap]) {
        int t = a[j]; a[j] = a[j + gap]; a[j + gap] = t;
        t = b[j]; b[j] = b[j + gap]; b[j + gap] = t;
        if (j >= gap) j -= gap; else break;
      }
    }
  }
}

void dsort2_(const int *n, double *a, int *b) {
  int len = *n;
  for (int gap = len / 2; gap > 0; gap /= 2) {
    for (int i = gap; i < len; ++i) {
      int j = i - gap;
      while (a[j] > a[j + gap]) {
        double t = a[j]; a[j] = a[j + gap]; a[j + gap] = t;
        int u = b[j]; b[j] = b[j + gap]; b[j + gap] = u;
        if (j >= gap) j -= gap; else break;
      }
    }
  }
}
