// The Faddeeva function w(z) = exp(-z^2) erfc(-iz) for host and device
// code, by Weideman's rational approximation (J.A.C. Weideman, "Computation
// of the complex error function", SIAM J. Numer. Anal. 31 (1994) 1497-1518)
// with N = 40 terms:
//   w(z) = 2 p(Z) / (L - iz)^2 + 1 / (sqrt(pi) (L - iz)),  Z = (L + iz) / (L - iz),
//   p(Z) = sum_{n<N} a_n Z^(N-1-n),  L = (N / sqrt 2)^(1/2),
// for Im z >= 0, and w(z) = 2 exp(-z^2) - w(-z) below the real axis.  The
// coefficients are the 2N-point discrete Fourier coefficients of
// exp(-t^2) (L^2 + t^2), t = L tan(theta / 2), as the paper constructs them;
// against scipy.special.wofz the relative error is below 2e-14 for
// 0.01 <= |z| <= 100 in the upper half plane.  This is the erfc of the Kambe
// sums (the cerf of the reference's main/cerf.f, which evaluates the same
// function by series and continued fractions).
#pragma once
#include <math.h>

#if !defined(__CUDACC__)
#define SKKR_HD
#else
#define SKKR_HD __host__ __device__
#endif

struct fcplx {
  double re, im;
};

SKKR_HD inline fcplx fc(double r, double i) { return fcplx{r, i}; }
SKKR_HD inline fcplx fadd(fcplx a, fcplx b) { return fc(a.re + b.re, a.im + b.im); }
SKKR_HD inline fcplx fsub(fcplx a, fcplx b) { return fc(a.re - b.re, a.im - b.im); }
SKKR_HD inline fcplx fmulc(fcplx a, fcplx b) { return fc(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
// a / b by Smith's scaling
SKKR_HD inline fcplx fdivc(fcplx a, fcplx b) {
  if (fabs(b.re) >= fabs(b.im)) {
    const double r = b.im / b.re, d = b.re + b.im * r;
    return fc((a.re + a.im * r) / d, (a.im - a.re * r) / d);
  }
  const double r = b.re / b.im, d = b.re * r + b.im;
  return fc((a.re * r + a.im) / d, (a.im * r - a.re) / d);
}
SKKR_HD inline fcplx fexpc(fcplx z) {
  const double e = exp(z.re);
  return fc(e * cos(z.im), e * sin(z.im));
}

#define SKKR_WEIDEMAN_N 40
#define SKKR_WEIDEMAN_L 5.31829589694498850e+00

SKKR_HD inline fcplx faddeeva_upper(fcplx z) {
  const double a[SKKR_WEIDEMAN_N] = {
    -1.73569809987918647e-15, 1.20167491075928095e-15, 1.15191702207494847e-14,
    -5.23171636632440398e-15, -7.07108802215940845e-14, 1.37782240476640457e-14,
    4.53414489094346555e-13, 1.20333095291956798e-13, -2.90771851041427015e-12,
    -2.72777356258302445e-12, 1.77141856738671790e-11, 3.47274209389070152e-11,
    -9.05513886095832302e-11, -3.56323504036026841e-10, 2.10859907312510581e-10,
    3.01778042555156406e-09, 3.24974658294507890e-09, -1.83156168342968342e-08,
    -6.35177348301541098e-08, 1.41986423729534295e-08, 5.91213695302905726e-07,
    1.48356611331720142e-06, -1.06601389841627292e-06, -1.80074471447234073e-05,
    -5.59130926423487940e-05, -3.93936314548380510e-05, 4.39807015986967025e-04,
    2.70540563307372899e-03, 1.00481862427835352e-02, 2.92029164712418812e-02,
    7.18236177907432827e-02, 1.55042638024795038e-01, 2.99894379961500590e-01,
    5.26652898827708604e-01, 8.47217457659381501e-01, 1.25638156757651331e+00,
    1.72538308481797786e+00, 2.20151379487831189e+00, 2.61605415276185971e+00,
    2.89962450938970484e+00,
  };
  const fcplx iz = fc(-z.im, z.re);
  const fcplx lm = fsub(fc(SKKR_WEIDEMAN_L, 0.0), iz);   // L - iz
  const fcplx Z = fdivc(fadd(fc(SKKR_WEIDEMAN_L, 0.0), iz), lm);
  fcplx p = fc(a[0], 0.0);
  for (int n = 1; n < SKKR_WEIDEMAN_N; n++) p = fadd(fmulc(p, Z), fc(a[n], 0.0));
  const fcplx lm2 = fmulc(lm, lm);
  const fcplx t1 = fdivc(fc(2.0 * p.re, 2.0 * p.im), lm2);
  const fcplx t2 = fdivc(fc(0.56418958354775628695, 0.0), lm);   // 1 / sqrt(pi)
  return fadd(t1, t2);
}

SKKR_HD inline fcplx faddeeva(fcplx z) {
  if (z.im >= 0.0) return faddeeva_upper(z);
  const fcplx mz = fc(-z.re, -z.im);
  const fcplx z2 = fmulc(z, z);
  const fcplx e = fexpc(fc(-z2.re, -z2.im));
  const fcplx w = faddeeva_upper(mz);
  return fc(2.0 * e.re - w.re, 2.0 * e.im - w.im);
}
