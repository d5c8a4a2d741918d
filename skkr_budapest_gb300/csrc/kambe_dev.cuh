// Kambe's Ewald split of the 2D lattice sums of outgoing spherical waves,
// for host and device code: D_L(k, s), L = (l, m) up to l = lmax2, for one
// k point and one layer-pair separation s, in the form the reference
// evaluates per k (main/kamstr.f:72-355):
//   reciprocal part over g (incgamma.f, delkam.f; formula 35 for s_z != 0,
//   formula 50 for s = 0), real-space part over R (ilkam.f, complex Y_lm of
//   ylmc.f; formula 47), and the s = 0 correction (formula 55);
// in-plane pairs (s != 0, s_z = 0) are moved to s_z = 1.1e-4 as kamstr.f
// does.  The caller passes superset lists of g and R; terms with
// |g + k| > gcut or an in-plane |R + s| > rcut are skipped, so the same lists
// serve every k point and separation.  Index of (l, m): l(l+1) + m.
#pragma once
#include "faddeeva.cuh"

#define SKKR_KAMBE_L2 6   // lmax2 = 2 lmax, lmax <= 3

SKKR_HD inline fcplx fscal(double s, fcplx a) { return fc(s * a.re, s * a.im); }
SKKR_HD inline fcplx fneg(fcplx a) { return fc(-a.re, -a.im); }
SKKR_HD inline fcplx fconj(fcplx a) { return fc(a.re, -a.im); }
// principal square root
SKKR_HD inline fcplx fsqrtc(fcplx z) {
  const double r = hypot(z.re, z.im);
  if (r == 0.0) return fc(0.0, 0.0);
  if (z.re >= 0.0) {
    const double t = sqrt(0.5 * (r + z.re));
    return fc(t, z.im / (2.0 * t));
  }
  const double t = sqrt(0.5 * (r - z.re));
  return fc(fabs(z.im) / (2.0 * t), copysign(t, z.im));
}
// z^n, n of either sign
SKKR_HD inline fcplx fpowi(fcplx z, int n) {
  fcplx r = fc(1.0, 0.0);
  for (int i = 0; i < (n < 0 ? -n : n); i++) r = fmulc(r, z);
  return n < 0 ? fdivc(fc(1.0, 0.0), r) : r;
}
SKKR_HD inline fcplx fipow(int n) {  // i^n
  const int q = ((n % 4) + 4) % 4;
  return q == 0 ? fc(1, 0) : q == 1 ? fc(0, 1) : q == 2 ? fc(-1, 0) : fc(0, -1);
}

// Gamma(1/2 - i, z), i = 0..n (incgamma.f)
SKKR_HD inline void kambe_incgamma(int n, fcplx z, fcplx *gam) {
  const fcplx ex = fexpc(fneg(z));
  const fcplx sz = fsqrtc(z);
  const fcplx a = fc(-sz.im, sz.re);  // i sqrt(z)
  fcplx s = fscal(1.7724538509055160273, fmulc(ex, faddeeva(a)));
  gam[0] = s;
  double b = -0.5;
  fcplx zb = sz;
  for (int i = 1; i <= n; i++) {
    zb = fdivc(zb, z);
    s = fscal(1.0 / b, fsub(s, fmulc(zb, ex)));
    gam[i] = s;
    b -= 1.0;
  }
}

// real-space integrals delta(0..l) at distance t (ilkam.f)
SKKR_HD inline void kambe_ilkam(int l, fcplx alpha, double t, fcplx kappa, fcplx *delta) {
  const fcplx z = fscal(t, kappa);
  const fcplx sx = fsqrtc(alpha);
  fcplx b = fdivc(fc(2.0, 0.0), z);
  const double dc = 0.88622692545275801365;  // sqrt(pi) / 2
  const fcplx a = fdivc(fscal(0.5, z), sx);
  const fcplx ex = fexpc(fsub(alpha, fmulc(a, a)));
  const fcplx ia = fc(-a.im, a.re);
  const fcplx wp = faddeeva(fadd(sx, ia)), wm = faddeeva(fsub(ia, sx));
  const fcplx c = fscal(dc, ex);
  fcplx dl = fmulc(fmulc(fadd(wp, wm), c), b);
  const fcplx dd = fmulc(fsub(wp, wm), c);
  fcplx delm1 = fc(dd.im, -dd.re);  // / i
  delta[0] = dl;
  b = fmulc(b, b);
  fcplx cx = sx;
  double d = 0.5;
  for (int i = 1; i <= l; i++) {
    cx = fdivc(cx, alpha);
    const fcplx del2 = fmulc(fadd(fsub(fscal(d, dl), delm1), fmulc(cx, ex)), b);
    delta[i] = del2;
    delm1 = dl;
    dl = del2;
    d += 1.0;
  }
}

// delta(0..n) of the out-of-plane reciprocal term (delkam.f), n >= 1
SKKR_HD inline void kambe_delkam(int n, fcplx x, fcplx zz, fcplx *delta) {
  const fcplx z = fsqrtc(zz);
  const fcplx sx = fsqrtc(x);
  const double dc = 0.88622692545275801365;
  fcplx b = fdivc(fc(2.0, 0.0), z);
  const fcplx a = fdivc(fscal(0.5, z), sx);
  const fcplx ex = fexpc(fsub(fmulc(a, a), x));
  const fcplx isx = fc(-sx.im, sx.re);
  const fcplx wm = faddeeva(fsub(isx, a)), wp = faddeeva(fadd(a, isx));
  const fcplx c = fscal(dc, ex);
  delta[0] = fmulc(fadd(wm, wp), c);
  const fcplx t = fmulc(fmulc(fsub(wm, wp), c), b);
  delta[1] = fc(-t.im, t.re);  // * i
  fcplx fcx = sx;
  b = fmulc(b, b);
  double d = 0.5;
  for (int i = 0; i < n - 1; i++) {
    fcx = fdivc(fcx, x);
    delta[i + 2] = fmulc(b, fadd(fsub(fneg(fscal(d, delta[i + 1])), delta[i]), fmulc(ex, fcx)));
    d += 1.0;
  }
}

SKKR_HD inline double kambe_fac(int n) {
  double f = 1.0;
  for (int i = 2; i <= n; i++) f *= (double)i;
  return f;
}

// complex Y_lm(v), Condon-Shortley phase, l <= lmax2 (ylmc.f: the power
// series of d^m P_l / dx^m from the recursion of the Legendre coefficients)
SKKR_HD inline void kambe_ylm(double x, double y, double z, int lmax2, fcplx *out) {
  double a[SKKR_KAMBE_L2 + 1][SKKR_KAMBE_L2 + 1];
  for (int l = 0; l <= SKKR_KAMBE_L2; l++)
    for (int n = 0; n <= SKKR_KAMBE_L2; n++) a[l][n] = 0.0;
  a[0][0] = 1.0;
  if (SKKR_KAMBE_L2 >= 1) a[1][1] = 1.0;
  if (SKKR_KAMBE_L2 >= 2) {
    a[2][0] = -0.5;
    a[2][2] = 1.5;
  }
  for (int l = 3; l <= lmax2; l++) {
    const double fa1 = (2.0 * l - 1.0) / l, fa2 = -(l - 1.0) / l;
    a[l][0] = fa2 * a[l - 2][0];
    for (int n = 1; n < l - 1; n++) a[l][n] = fa1 * a[l - 1][n - 1] + fa2 * a[l - 2][n];
    a[l][l - 1] = fa1 * a[l - 1][l - 2];
    a[l][l] = fa1 * a[l - 1][l - 1];
  }
  const double r = sqrt(x * x + y * y + z * z);
  double cth = 0.0;
  fcplx ephi = fc(1.0, 0.0);
  if (r >= 1e-16) {
    cth = z / r;
    const double d = sqrt(x * x + y * y);
    if (d >= 1e-6) ephi = fc(x / d, y / d);
  }
  const double px = sqrt(fmax(1.0 - cth * cth, 0.0)) + 1e-30;
  for (int l = 0; l <= lmax2; l++)
    for (int m = -l; m <= l; m++) {
      const int mb = m < 0 ? -m : m;
      // t = sum_k a(l, k + mb) (k + mb)! / k! cth^k
      double t = 0.0, p = 1.0;
      for (int k = 0; k <= l - mb; k++) {
        t += a[l][k + mb] * (kambe_fac(k + mb) / kambe_fac(k)) * p;
        p *= cth;
      }
      const double nrm = sqrt((2.0 * l + 1.0) * kambe_fac(l - mb) / (12.566370614359172954 * kambe_fac(l + mb)));
      const fcplx cf = fscal(nrm, fipow(m + mb));
      out[l * (l + 1) + m] = fmulc(fscal(pow(px, mb) * t, cf), fpowi(ephi, m));
    }
}

// Per-(k, s) constants of the sums (kamstr.f:72-140): kappa, the prefactors
// of the two parts, the Ewald alpha, the flm normalisation, the in-plane
// shift of in-plane pairs, and (sz kappa)^l of the out-of-plane form.
struct KambeSetup {
  fcplx e, kappa, cs1, cs2, alpha, w, xrot;
  double kx, ky, sx, sy, sz, s;
  int lmax2;
  bool f35;
  double flm[(SKKR_KAMBE_L2 + 1) * (SKKR_KAMBE_L2 + 1)];
  fcplx cs[SKKR_KAMBE_L2 + 1];
};

SKKR_HD inline void kambe_setup(fcplx e, double kx, double ky, double sx, double sy, double sz, int lmax2,
                                double area, double factor, KambeSetup &K) {
  K.e = e;
  K.kx = kx;
  K.ky = ky;
  K.lmax2 = lmax2;
  K.kappa = fsqrtc(e);
  K.cs1 = fdivc(fc(-1.0 / area, 0.0), K.kappa);
  K.cs2 = fscal(-0.28209479177387814347, K.kappa);  // -kappa / (2 sqrt(pi))
  K.alpha = fscal(factor * area / 12.566370614359172954, e);
  K.w = fdivc(fscal(2.0, K.alpha), e);
  for (int l = 0; l <= lmax2; l++)
    for (int m = 0; m <= l; m++) {
      const double v = pow(2.0, -l) * sqrt((2.0 * l + 1.0) * kambe_fac(l + m) * kambe_fac(l - m));
      K.flm[l * (l + 1) + m] = v;
      K.flm[l * (l + 1) - m] = v;
    }
  double s = sqrt(sx * sx + sy * sy + sz * sz);
  const double ctol = 1e-4;
  K.s = s;  // before the in-plane shift: s < ctol selects formula 55
  if (s > ctol && fabs(sz) < ctol) {
    sz = 1.1 * ctol;
    s = sqrt(sx * sx + sy * sy + sz * sz);
  }
  K.sx = sx;
  K.sy = sy;
  K.sz = sz;
  K.f35 = s > ctol && fabs(sz) > ctol;
  K.cs[0] = fc(1.0, 0.0);
  for (int l = 1; l <= lmax2; l++) K.cs[l] = fmulc(K.cs[l - 1], fscal(sz, K.kappa));
  K.xrot = fexpc(fc(0.0, -3.14159265358979323846));  // exp(-i pi) of kamstr.f
}

// formula 55 (s = 0): d003 = -kappa (e^alpha c - i) / (2 sqrt(pi)),
// c = i (e^-alpha - w(sqrt alpha)) - 1 / (sqrt(pi) sqrt(alpha))
SKKR_HD inline void kambe_self_term(const KambeSetup &K, fcplx *out) {
  if (K.s >= 1e-4) return;
  const fcplx a = fsqrtc(K.alpha);
  const fcplx t = fsub(fexpc(fneg(K.alpha)), faddeeva(a));
  const fcplx c = fsub(fc(-t.im, t.re), fdivc(fc(0.56418958354775628695, 0.0), a));
  const fcplx u = fsub(fmulc(fexpc(K.alpha), c), fc(0.0, 1.0));
  out[0] = fadd(out[0], fscal(-0.28209479177387814347, fmulc(K.kappa, u)));
}

// the reciprocal-space term of one g (formula 35 out of plane, 50 in plane)
SKKR_HD inline void kambe_gterm(const KambeSetup &K, double gx, double gy, double gcut, fcplx *out) {
  const int lmax2 = K.lmax2;
  const double gkx = gx + K.kx, gky = gy + K.ky;
  const double km2 = gkx * gkx + gky * gky, km = sqrt(km2);
  if (km > gcut) return;
  fcplx gam[SKKR_KAMBE_L2 + 1], dl[SKKR_KAMBE_L2 + 2], cp[SKKR_KAMBE_L2 + 1], cm[SKKR_KAMBE_L2 + 1];
  const fcplx e = K.e, kappa = K.kappa;
  const fcplx kp = fsqrtc(fsub(e, fc(km2, 0.0)));
  const fcplx ex2 = km > 1e-10 ? fc(gkx / km, gky / km) : fc(1.0, 0.0);
  const fcplx xc = fscal(0.5, fmulc(fmulc(K.xrot, fsub(e, fc(km * km, 0.0))), K.w));
  kambe_incgamma(lmax2, xc, gam);
  const fcplx rp = fdivc(kp, kappa), rm = fdivc(fc(km, 0.0), kappa);
  for (int l = 0; l <= lmax2; l++) {
    cp[l] = fpowi(rp, 2 * l - 1);
    cm[l] = fpowi(rm, l);
  }
  if (K.f35) {
    const double sz = K.sz;
    kambe_delkam(lmax2, xc, fmulc(fscal(sz, kp), fscal(sz, kp)), dl);
    const fcplx ex1 = fmulc(fexpc(fc(0.0, gkx * K.sx + gky * K.sy)), K.cs1);
    for (int l = 0; l <= lmax2; l++)
      for (int m = -l; m <= l; m++) {
        const int mm = m < 0 ? -m : m, ipar = (l - mm) % 2;
        const fcplx ex = fmulc(fpowi(ex2, -m), ex1);
        fcplx csum = fc(0.0, 0.0);
        for (int n = 0; n <= l - mm; n++) {
          fcplx b = fc(0.0, 0.0);
          const int kmax = 2 * n < l - mm ? 2 * n : l - mm;
          for (int k = n + (n + ipar) % 2; k <= kmax; k += 2) {
            const int i = 2 * n - k, j = l - k;
            const fcplx cc = fscal(1.0 / (kambe_fac(i) * kambe_fac(k - n)), fmulc(K.cs[i], cm[j]));
            b = fadd(b, fscal(1.0 / (kambe_fac((l - mm - k) / 2) * kambe_fac((l + mm - k) / 2)), cc));
          }
          csum = fadd(csum, fmulc(fmulc(cp[n], dl[n]), b));
        }
        const int lm = l * (l + 1) + m;
        out[lm] = fadd(out[lm], fmulc(fscal(K.flm[lm], fmulc(ex, csum)), fipow(1 - m)));
      }
  } else {
    for (int l = 0; l <= lmax2; l++)
      for (int m = -l; m <= l; m++) {
        const int mm = m < 0 ? -m : m;
        if ((l - mm) % 2) continue;
        const fcplx ex = fmulc(fpowi(ex2, -m), K.cs1);
        fcplx csum = fc(0.0, 0.0);
        for (int n = 0; n <= (l - mm) / 2; n++) {
          const fcplx t = fmulc(fmulc(cp[n], cm[l - 2 * n]), gam[n]);
          csum = fadd(csum, fscal(1.0 / (kambe_fac(n) * kambe_fac((l - mm - 2 * n) / 2) *
                                         kambe_fac((l + mm - 2 * n) / 2)), t));
        }
        const int lm = l * (l + 1) + m;
        out[lm] = fadd(out[lm], fmulc(fscal(K.flm[lm], fmulc(ex, csum)), fipow(1 - m)));
      }
  }
}

// the real-space term of one R (formula 47)
SKKR_HD inline void kambe_rterm(const KambeSetup &K, double rx, double ry, double rcut, fcplx *out) {
  const int lmax2 = K.lmax2;
  const double vx = rx + K.sx, vy = ry + K.sy, vz = K.sz;
  const double rs = sqrt(vx * vx + vy * vy + vz * vz);
  if (rs < 1e-5 || sqrt(vx * vx + vy * vy) > rcut) return;
  fcplx ylm[(SKKR_KAMBE_L2 + 1) * (SKKR_KAMBE_L2 + 1)], intil[SKKR_KAMBE_L2 + 1];
  const fcplx ex1 = fexpc(fc(0.0, -(rx * K.kx + ry * K.ky)));
  kambe_ylm(vx, vy, vz, lmax2, ylm);
  kambe_ilkam(lmax2, K.alpha, rs, K.kappa, intil);
  const fcplx a = fscal(-0.5 * rs, K.kappa);
  fcplx b = fdivc(fmulc(ex1, K.cs2), a);
  for (int l = 0; l <= lmax2; l++) {
    b = fmulc(b, a);
    const fcplx c = fmulc(intil[l], b);
    for (int m = -l; m <= l; m++) {
      const int lm = l * (l + 1) + m;
      out[lm] = fadd(out[lm], fmulc(c, fconj(ylm[lm])));
    }
  }
}

// D_L(k, s) into out[(lmax2+1)^2] (kamstr.f dlm1 + dlm2): the self term,
// then the g terms and the R terms in list order
SKKR_HD inline void kambe_dlm(fcplx e, double kx, double ky, double sx, double sy, double sz, int lmax2,
                              const double *gvec, int ng, const double *rvec, int nr, double area,
                              double factor, double gcut, double rcut, fcplx *out) {
  const int lmmx = (lmax2 + 1) * (lmax2 + 1);
  KambeSetup K;
  kambe_setup(e, kx, ky, sx, sy, sz, lmax2, area, factor, K);
  for (int i = 0; i < lmmx; i++) out[i] = fc(0.0, 0.0);
  kambe_self_term(K, out);
  for (int ig = 0; ig < ng; ig++) kambe_gterm(K, gvec[2 * ig], gvec[2 * ig + 1], gcut, out);
  for (int ir = 0; ir < nr; ir++) kambe_rterm(K, rvec[2 * ir], rvec[2 * ir + 1], rcut, out);
}

// alm(k, s)[L][L'] = sum_L'' coef[L][L'][L''] D_L''(k, s), the layer-pair
// structure constants kamstr.f forms from its lattice sums (in this library's
// harmonics: coef = 4 pi <Y_L Y*_L' Y_L''> i^(l'-l-l'') with D taken at
// (l'', -m'') and signed (-1)^(l''+m''), prepared by the host).  coef is
// [lmmax][lmmax][lmmx2] complex (re, im interleaved); out [lmmax][lmmax].
SKKR_HD inline void kambe_alm(const fcplx *d, int lmax, const double *coef, fcplx *out) {
  const int lm = (lmax + 1) * (lmax + 1), lm2 = (2 * lmax + 1) * (2 * lmax + 1);
  for (int a = 0; a < lm; a++)
    for (int b = 0; b < lm; b++) {
      fcplx s = fc(0.0, 0.0);
      const double *c = coef + 2 * ((long long)(a * lm + b) * lm2);
      for (int q = 0; q < lm2; q++) s = fadd(s, fmulc(fc(c[2 * q], c[2 * q + 1]), d[q]));
      out[a * lm + b] = s;
    }
}

// ---------------------------------------------------------------------------
// The plane-wave form of the same layer-pair blocks, which gstore.f uses for
// layers far apart (|s_z| |b|_min >= 5; main/directg.f:2-151):
//   alm(k, s)[L][L'] = -i (8 pi^2 / A) sum_g e^{i (k+g).s_par + i K_z |s_z|} / K_z
//                      Yl_L(g) Yr_L'(g),   K_z = sqrt(kappa^2 - |k+g|^2),
// the harmonics taken at the complex direction (K_z, |k+g|, phi) / kappa
// (sphrm.f).  s_z > 0 gives directg's gp block of s, s_z < 0 its gm block of
// -s; they differ in which of Y_lm and Y_l,-m carries the sign (-1)^l and
// which the sign (-1)^m.
#define SKKR_DG_LM 16  // (lmax + 1)^2 for lmax <= 3

// Y_lm of the complex angles (cos, sin, e^{i phi}), l <= lmax, index
// l(l+1)+m: the m = l and m = l - 1 forms, then the recurrence in l (sphrm.f)
SKKR_HD inline void directg_sphrm(fcplx ct, fcplx st, fcplx cf, int lmax, fcplx *yo) {
  fcplx y[SKKR_DG_LM + 1];  // 1-based, as the recurrences index it
  for (int i = 0; i <= SKKR_DG_LM; i++) y[i] = fc(0.0, 0.0);
  const double pi = 3.14159265358979323846;
  y[1] = fc(sqrt(0.25 / pi), 0.0);
  double a = 1.0, b = 1.0, asg = 1.0;
  fcplx sf = fc(1.0, 0.0), sa = fc(1.0, 0.0);
  int lp = 1;
  for (int l = 1; l <= lmax; l++) {
    const double fl = l;
    a = 0.5 * a * fl * (2.0 * fl - 1.0);
    b = fl * b;
    asg = -asg;
    const int lm = lp + 1;
    lp = lp + l + l + 1;
    sf = fmulc(sf, cf);
    fcplx fac = fscal(sqrt((2.0 * fl + 1.0) * a / (4.0 * pi * b * b)), sa);
    y[lm] = fdivc(fmulc(fac, st), sf);
    y[lp] = fscal(asg, fmulc(fmulc(fac, st), sf));
    fac = fscal(sqrt(2.0 * fl), fmulc(fac, ct));
    y[lm + 1] = fdivc(fmulc(fac, cf), sf);
    y[lp - 1] = fscal(-asg, fdivc(fmulc(fac, sf), cf));
    sa = fmulc(sa, st);
  }
  for (int m = 2; m <= lmax; m++) {
    const int mm = m + m - 4;
    const double fm = m - 2;
    double aa = sqrt(1.0 / (fm + fm + 3.0));
    int ln = m * m - 1, lm = ln - m - m + 2;
    for (int l = m; l <= lmax; l++) {
      const double fl = l;
      const double bb = sqrt((fl + fm) * (fl - fm) / ((fl + fl + 1.0) * (fl + fl - 1.0)));
      const int lq = ln + l + l;
      y[lq] = fscal(1.0 / bb, fsub(fmulc(ct, y[ln]), fscal(aa, y[lm])));
      y[lq - mm] = fscal(1.0 / bb, fsub(fmulc(ct, y[ln - mm]), fscal(aa, y[lm - mm])));
      aa = bb;
      lm = ln;
      ln = lq;
    }
  }
  for (int i = 0; i < (lmax + 1) * (lmax + 1); i++) yo[i] = y[i + 1];
}

// the g term of the plane-wave form: its scalar factor and the left / right
// harmonic vectors (yl over L, yr over L'); f1 = 8 pi^2 / A
SKKR_HD inline void directg_gterm(fcplx kappa2, fcplx kappa, double kx, double ky, double sx, double sy, double sz,
                                  int lmax, double gx, double gy, double f1, fcplx *fac, fcplx *yl, fcplx *yr) {
  const double gkx = gx + kx, gky = gy + ky, gk2 = gkx * gkx + gky * gky, gk = sqrt(gk2);
  const fcplx gkz = fsqrtc(fsub(kappa2, fc(gk2, 0.0)));
  const fcplx phi = gk > 1e-6 ? fc(gkx / gk, gky / gk) : fc(1.0, 0.0);
  fcplx y[SKKR_DG_LM];
  directg_sphrm(fdivc(gkz, kappa), fdivc(fc(gk, 0.0), kappa), phi, lmax, y);
  const double az = fabs(sz);
  // e^{i (gkx sx + gky sy + K_z |s_z|)}
  const fcplx ph = fexpc(fc(-gkz.im * az, gkx * sx + gky * sy + gkz.re * az));
  *fac = fdivc(fmulc(fc(0.0, -f1), ph), gkz);
  for (int l = 0; l <= lmax; l++)
    for (int m = -l; m <= l; m++) {
      const int L = l * (l + 1) + m, Ln = l * (l + 1) - m;
      const fcplx il = fipow(l);
      const double sl = (l & 1) ? -1.0 : 1.0, sm = (m & 1) ? -1.0 : 1.0;
      if (sz > 0.0) {
        yr[L] = fscal(sl, fmulc(il, y[L]));
        yl[L] = fscal(sm, fmulc(il, y[Ln]));
      } else {
        yr[L] = fscal(sm, fmulc(il, y[L]));
        yl[L] = fscal(sl, fmulc(il, y[Ln]));
      }
    }
}

// the whole block, one thread (host check of the device kernel's terms):
// out [lm][lm], g terms summed in list order
SKKR_HD inline void directg_alm(fcplx e, double kx, double ky, double sx, double sy, double sz, int lmax,
                                const double *gvec, int ng, double area, fcplx *out) {
  const int lm = (lmax + 1) * (lmax + 1);
  const fcplx kappa = fsqrtc(e);
  const double f1 = 8.0 * 3.14159265358979323846 * 3.14159265358979323846 / area;
  for (int i = 0; i < lm * lm; i++) out[i] = fc(0.0, 0.0);
  for (int ig = 0; ig < ng; ig++) {
    fcplx fac, yl[SKKR_DG_LM], yr[SKKR_DG_LM];
    directg_gterm(e, kappa, kx, ky, sx, sy, sz, lmax, gvec[2 * ig], gvec[2 * ig + 1], f1, &fac, yl, yr);
    for (int a = 0; a < lm; a++) {
      const fcplx fa = fmulc(fac, yl[a]);
      for (int b = 0; b < lm; b++) out[a * lm + b] = fadd(out[a * lm + b], fmulc(fa, yr[b]));
    }
  }
}

// element e of the slab matrices of one batch (column-major N x N per k,
// N = nl lm): G[(a,L),(b,L')] = e^{ik.(pos_b - pos_a)} alm_ab[L][L'],
// A = 1 - alpha[a][l(L)] G; alm, alpha, G, A complex (re, im interleaved)
SKKR_HD inline void kambe_slab_elem(long long e, int nl, int lm, const double *alm, const int *pmap, int nsep,
                                    const double *kxy, const double *pos, const double *alpha, int nal, double *G,
                                    double *A) {
  const int N = nl * lm;
  const long long NN = (long long)N * N;
  const int k = (int)(e / NN);
  const long long rem = e - (long long)k * NN;
  const int col = (int)(rem / N), row = (int)(rem - (long long)col * N);
  const int a = row / lm, L = row - a * lm, b = col / lm, Lp = col - b * lm;
  int l = 0;
  while ((l + 1) * (l + 1) <= L) l++;
  // the pair's lattice sums: alm[k][pmap[a][b]] (its separation among nsep)
  const long long iv = (((long long)k * nsep + pmap[a * nl + b]) * lm + L) * lm + Lp;
  const double ph = kxy[2 * k] * (pos[3 * b] - pos[3 * a]) + kxy[2 * k + 1] * (pos[3 * b + 1] - pos[3 * a + 1]);
  const fcplx g = fmulc(fc(alm[2 * iv], alm[2 * iv + 1]), fc(cos(ph), sin(ph)));
  const fcplx al = fc(alpha[2 * (a * nal + l)], alpha[2 * (a * nal + l) + 1]);
  fcplx m = fneg(fmulc(al, g));
  if (row == col) m.re += 1.0;
  G[2 * e] = g.re;
  G[2 * e + 1] = g.im;
  A[2 * e] = m.re;
  A[2 * e + 1] = m.im;
}

// element e (k, j, L', L) of the structure-constant cache: block blk[j] of
// k, column-major lm x lm, = X[k][(centre, L), (centre + j - jmax, L')];
// offsets with blk[j] < 0 are not written
SKKR_HD inline void kambe_slab_cache_elem(long long e, int nl, int lm, int centre, int jmax, const int *blk, int nbk,
                                          const double *X, double *Gc) {
  const int N = nl * lm, nj = 2 * jmax + 1;
  const int L = (int)(e % lm), Lp = (int)((e / lm) % lm), j = (int)((e / ((long long)lm * lm)) % nj);
  const int k = (int)(e / ((long long)lm * lm * nj));
  const int b = blk[j];
  if (b < 0) return;
  const int row = centre * lm + L, col = (centre + j - jmax) * lm + Lp;
  const long long ix = (long long)k * N * N + row + (long long)col * N;
  const long long o = ((long long)k * nbk + b) * lm * lm + L + (long long)Lp * lm;
  Gc[2 * o] = X[2 * ix];
  Gc[2 * o + 1] = X[2 * ix + 1];
}

// element e of out[k][j][L][L'] = X[k][(centre, L), (centre + j - jmax, L')]
SKKR_HD inline void kambe_slab_extract_elem(long long e, int nl, int lm, int centre, int jmax, const double *X,
                                            double *out) {
  const int N = nl * lm, nj = 2 * jmax + 1;
  const int Lp = (int)(e % lm), L = (int)((e / lm) % lm), j = (int)((e / ((long long)lm * lm)) % nj);
  const int k = (int)(e / ((long long)lm * lm * nj));
  const int row = centre * lm + L, col = (centre + j - jmax) * lm + Lp;
  const long long ix = (long long)k * N * N + row + (long long)col * N;
  out[2 * e] = X[2 * ix];
  out[2 * e + 1] = X[2 * ix + 1];
}

