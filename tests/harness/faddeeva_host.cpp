// Host build of the device Faddeeva function, for its CPU test: the same
// header the device code includes, compiled by g++.
#include "../../skkr_budapest_gb300/csrc/faddeeva.cuh"

extern "C" void faddeeva_eval(int n, const double *zr, const double *zi, double *wr, double *wi) {
  for (int k = 0; k < n; k++) {
    const fcplx w = faddeeva(fc(zr[k], zi[k]));
    wr[k] = w.re;
    wi[k] = w.im;
  }
}
