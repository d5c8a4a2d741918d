// Host build of the device Kambe lattice sums, for their CPU test: the same
// header the device code includes, compiled by g++.
#include "../../skkr_budapest_gb300/csrc/kambe_dev.cuh"

extern "C" void kambe_eval(double er, double ei, double kx, double ky, double sx, double sy, double sz, int lmax2,
                           const double *gvec, int ng, const double *rvec, int nr, double area, double factor,
                           double gcut, double rcut, double *out) {
  fcplx d[(SKKR_KAMBE_L2 + 1) * (SKKR_KAMBE_L2 + 1)];
  kambe_dlm(fc(er, ei), kx, ky, sx, sy, sz, lmax2, gvec, ng, rvec, nr, area, factor, gcut, rcut, d);
  for (int i = 0; i < (lmax2 + 1) * (lmax2 + 1); i++) {
    out[2 * i] = d[i].re;
    out[2 * i + 1] = d[i].im;
  }
}

extern "C" void kambe_alm_eval(double er, double ei, double kx, double ky, double sx, double sy, double sz,
                               int lmax, const double *gvec, int ng, const double *rvec, int nr, double area,
                               double gcut, double rcut, const double *coef, double *out) {
  fcplx d[(SKKR_KAMBE_L2 + 1) * (SKKR_KAMBE_L2 + 1)], g[256];
  kambe_dlm(fc(er, ei), kx, ky, sx, sy, sz, 2 * lmax, gvec, ng, rvec, nr, area, 1.0, gcut, rcut, d);
  kambe_alm(d, lmax, coef, g);
  for (int i = 0; i < (lmax + 1) * (lmax + 1) * (lmax + 1) * (lmax + 1); i++) {
    out[2 * i] = g[i].re;
    out[2 * i + 1] = g[i].im;
  }
}

extern "C" void slab_assemble_eval(int nk, int nl, int lm, const double *alm, const int *pmap, int nsep,
                                   const double *kxy, const double *pos, const double *alpha, int nal, double *G,
                                   double *A) {
  const long long tot = (long long)nk * nl * lm * nl * lm;
  for (long long e = 0; e < tot; e++) kambe_slab_elem(e, nl, lm, alm, pmap, nsep, kxy, pos, alpha, nal, G, A);
}

extern "C" void slab_cache_eval(int nk, int nl, int lm, int centre, int jmax, const int *blk, int nbk, const double *X,
                                double *Gc) {
  const long long tot = (long long)nk * (2 * jmax + 1) * lm * lm;
  for (long long e = 0; e < tot; e++) kambe_slab_cache_elem(e, nl, lm, centre, jmax, blk, nbk, X, Gc);
}

extern "C" void slab_extract_eval(int nk, int nl, int lm, int centre, int jmax, const double *X, double *out) {
  const long long tot = (long long)nk * (2 * jmax + 1) * lm * lm;
  for (long long e = 0; e < tot; e++) kambe_slab_extract_elem(e, nl, lm, centre, jmax, X, out);
}

extern "C" void directg_eval(double er, double ei, double kx, double ky, double sx, double sy, double sz, int lmax,
                             const double *gvec, int ng, double area, double *out) {
  fcplx g[256];
  directg_alm(fc(er, ei), kx, ky, sx, sy, sz, lmax, gvec, ng, area, g);
  for (int i = 0; i < (lmax + 1) * (lmax + 1) * (lmax + 1) * (lmax + 1); i++) {
    out[2 * i] = g[i].re;
    out[2 * i + 1] = g[i].im;
  }
}
