// Host build of the BF16 digit slicing of the split-precision products
// (slicing.cuh), for its CPU test: the same header the kernels include.
#include "../../skkr_budapest_gb300/csrc/slicing.cuh"

template <int S, int DB>
static void digits(int n, const double *x, const int *es, int *out) {
  for (int i = 0; i < n; i++) slice_digits<S, DB>(x[i], es[i], out + (long long)i * S);
}
template <int S, int DB>
static void words(const double *re, const double *im, int es, int wshift, uint32_t *wr, uint32_t *wi) {
  double r[4], m[4];
  for (int e = 0; e < 4; e++) {
    r[e] = re[e];
    m[e] = im[e];
  }
  uint32_t a[S][2], b[S][2];
  slice4<S, DB>(r, m, es, wshift, a, b);
  for (int p = 0; p < S; p++)
    for (int h = 0; h < 2; h++) {
      wr[2 * p + h] = a[p][h];
      wi[2 * p + h] = b[p][h];
    }
}

#define SLC_CASES(X) X(3, 8) X(4, 8) X(5, 8) X(6, 8) X(7, 8) X(3, 7) X(5, 7) X(7, 7) X(8, 7)

extern "C" int slice_digits_eval(int S, int DB, int n, const double *x, const int *es, int *out) {
#define X(s, d) \
  if (S == s && DB == d) return digits<s, d>(n, x, es, out), 0;
  SLC_CASES(X)
#undef X
  return -1;
}

extern "C" int slice4_eval(int S, int DB, const double *re, const double *im, int es, int wshift, uint32_t *wr,
                           uint32_t *wi) {
#define X(s, d) \
  if (S == s && DB == d) return words<s, d>(re, im, es, wshift, wr, wi), 0;
  SLC_CASES(X)
#undef X
  return -1;
}

extern "C" long long fix_round_eval(double x, int E) { return fix_round(x, E); }
