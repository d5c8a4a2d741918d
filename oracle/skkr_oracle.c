/*
 * skkr_oracle.c -- CPU FP64 restatement of the reference's 2D-BZ tau path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker): tests/, __graft_entry__.smoke()
 * and bench.py's CPU baseline leg may load it; the product never does.
 *
 * Each function names the reference routine it restates (paths relative to
 * the laszloffy/skkr_budapest tree).  Loop order, pivoting and accumulation
 * order follow the Fortran so that rounding behaves the same way; the only
 * deliberate differences are: errors are returned as status codes instead of
 * `stop`, and all k points are cached (the reference caches the first
 * mkpar1 and recomputes the rest, which gives identical values).
 *
 * Parity unpinned at the tau / coherent-t level: the reference has no tests
 * and no golden vectors for this path, and no Fortran compiler exists here or
 * on the GPU machine.  The generators are pinned against the reference's
 * sample/02-layer-scf run log (tests/golden/sample02_contour.json).
 *
 * Compiled with -fcx-fortran-rules so complex * and / follow gfortran's
 * semantics (no C99 Annex-G NaN recovery).
 */
#include "skkr_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IX(i, j, ld) ((size_t)(i) + (size_t)(j) * (size_t)(ld))

static void czero(zc *a, size_t n) { memset(a, 0, n * sizeof(zc)); }

/* ===================================================================== *
 * main/gjinv.f:2-59  Gauss-Jordan inversion, pivot searched along row i  *
 * (column pivoting), columns swapped back at the end.                    *
 * ===================================================================== */
void orc_gjinv(zc *a, int n, int nmax, zc *detl) {
  const zc cpi = 3.1415926535897932 * I;
  int *ind = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  zc q;
  *detl = 0.0;
  for (int i = 0; i < n; i++) {
    int k = i;
    double amaxi = cabs(a[IX(i, i, nmax)]);
    for (int j = i + 1; j < n; j++) {
      double atest = cabs(a[IX(i, j, nmax)]);
      if (atest <= amaxi) continue;
      k = j;
      amaxi = atest;
    }
    ind[i] = k;
    if (k != i) {
      *detl -= cpi;
      for (int j = 0; j < n; j++) {
        q = a[IX(j, i, nmax)];
        a[IX(j, i, nmax)] = a[IX(j, k, nmax)];
        a[IX(j, k, nmax)] = q;
      }
    }
    q = a[IX(i, i, nmax)];
    *detl += clog(q);
    q = 1.0 / q;
    a[IX(i, i, nmax)] = 1.0;
    for (int j = 0; j < n; j++) a[IX(j, i, nmax)] *= q;
    for (int j = 0; j < n; j++) {
      if (j == i) continue;
      q = a[IX(i, j, nmax)];
      a[IX(i, j, nmax)] = 0.0;
      for (int kk = 0; kk < n; kk++) a[IX(kk, j, nmax)] -= a[IX(kk, i, nmax)] * q;
    }
  }
  for (int i = n - 1; i >= 0; i--) {
    int j = ind[i];
    if (i == j) continue;
    for (int kk = 0; kk < n; kk++) {
      q = a[IX(i, kk, nmax)];
      a[IX(i, kk, nmax)] = a[IX(j, kk, nmax)];
      a[IX(j, kk, nmax)] = q;
    }
  }
  free(ind);
}

/* main/matops.f doubmt2: c = a*b, a n1 x n2, b n2 x n3 */
void orc_doubmt2(const zc *a, const zc *b, zc *c, int n1, int n2, int n3, int ld) {
  for (int i = 0; i < n1; i++)
    for (int k = 0; k < n3; k++) {
      zc sum = 0.0;
      for (int j = 0; j < n2; j++) sum += b[IX(j, k, ld)] * a[IX(i, j, ld)];
      c[IX(i, k, ld)] = sum;
    }
}

/* main/matops.f tripmt: b = u * b * ust (scratch c, as the reference) */
void orc_tripmt(const zc *u, zc *b, const zc *ust, int ndi1, int ndi2, int ld) {
  zc *c = (zc *)malloc(sizeof(zc) * (size_t)ndi1 * (size_t)ndi2 + 16);
  for (int i = 0; i < ndi1; i++)
    for (int j = 0; j < ndi2; j++) {
      zc x = 0.0;
      for (int k = 0; k < ndi1; k++) x += b[IX(k, j, ld)] * u[IX(i, k, ld)];
      c[IX(i, j, ndi1)] = x;
    }
  for (int i = 0; i < ndi1; i++)
    for (int j = 0; j < ndi2; j++) {
      zc x = 0.0;
      for (int k = 0; k < ndi2; k++) x += ust[IX(k, j, ld)] * c[IX(i, k, ndi1)];
      b[IX(i, j, ld)] = x;
    }
  free(c);
}

/* main/matops.f tripmt2: b1 = u * b * v (u ndi1 x ndi2, b ndi2 x ndi3, v ndi3 x ndi4) */
void orc_tripmt2(const zc *u, const zc *b, const zc *v, zc *b1, int ndi1,
                 int ndi2, int ndi3, int ndi4, int ld, int ldb1) {
  zc *c = (zc *)malloc(sizeof(zc) * (size_t)ndi1 * (size_t)ndi3 + 16);
  for (int i = 0; i < ndi1; i++)
    for (int j = 0; j < ndi3; j++) {
      zc x = 0.0;
      for (int k = 0; k < ndi2; k++) x += b[IX(k, j, ld)] * u[IX(i, k, ld)];
      c[IX(i, j, ndi1)] = x;
    }
  for (int i = 0; i < ndi1; i++)
    for (int j = 0; j < ndi4; j++) {
      zc x = 0.0;
      for (int k = 0; k < ndi3; k++) x += v[IX(k, j, ld)] * c[IX(i, k, ndi1)];
      b1[IX(i, j, ldb1)] = x;
    }
  free(c);
}

/* main/matops.f compmat: 1 if ||x-y||_F < tol ||x||_F */
int orc_compmat(const zc *x, const zc *y, int n, int ld, double tol) {
  if (tol <= 0.0) tol = 1.0e-12;
  double xn = 0.0, dn = 0.0;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      zc xx = x[IX(i, j, ld)], dx = x[IX(i, j, ld)] - y[IX(i, j, ld)];
      xn += creal(xx) * creal(xx) + cimag(xx) * cimag(xx);
      dn += creal(dx) * creal(dx) + cimag(dx) * cimag(dx);
    }
  return sqrt(dn) < tol * sqrt(xn) ? 1 : 0;
}

/* ===================================================================== *
 * main/clebsch.f:2-76  lm -> (kappa,mu) Clebsch-Gordan rectangular maps  *
 * (1-based indices in ind1/ind2, as the reference)                       *
 * ===================================================================== */
void orc_clebsch(double u1[72], double u2[72], int ind1[72], int ind2[72]) {
  for (int i = 0; i < 72; i++) { u1[i] = 0; u2[i] = 0; ind1[i] = 0; ind2[i] = 0; }
  int inr = 0;
  for (int l = 0; l <= 5; l++) {
    double twolp1 = (double)(2 * l + 1);
    for (int m = -l; m <= l; m++) {
      inr++;
      int kap = l, ir;
      if (kap != 0) {
        ir = 2 * kap * kap + kap + m;           /* j=l-1/2, ms=-1/2 */
        u1[ir - 1] = sqrt((l + m) / twolp1);
        ind1[ir - 1] = inr;
        ir = 2 * kap * kap + kap + m + 1;       /* ms=+1/2 */
        u2[ir - 1] = -sqrt((l - m) / twolp1);
        ind2[ir - 1] = inr;
      }
      kap = -l - 1;                             /* j=l+1/2 */
      ir = 2 * kap * kap + kap + m;
      u1[ir - 1] = sqrt((l - m + 1) / twolp1);
      ind1[ir - 1] = inr;
      ir = 2 * kap * kap + kap + m + 1;
      u2[ir - 1] = sqrt((l + m + 1) / twolp1);
      ind2[ir - 1] = inr;
    }
  }
  for (int ir = 0; ir < 72; ir++) {
    if (ind1[ir] == 0) ind1[ir] = 1;
    if (ind2[ir] == 0) ind2[ir] = 1;
  }
}

/* main/relmtrx.f:2-45  b = U1 (c a) U1^T + U2 (c a) U2^T in (kappa,mu) */
static double cg_u1[72], cg_u2[72];
static int cg_ind1[72], cg_ind2[72], cg_init = 0;
static void cg_table_init(void) {
  if (!cg_init) { orc_clebsch(cg_u1, cg_u2, cg_ind1, cg_ind2); cg_init = 1; }
}

void orc_relmtrx(const zc *a, int lda, zc *b, int ldb, zc fac, int lmax) {
  const double *u1 = cg_u1, *u2 = cg_u2;
  const int *ind1 = cg_ind1, *ind2 = cg_ind2;
  cg_table_init();
  int lmmax = (lmax + 1) * (lmax + 1), kmymax = 2 * lmmax;
  zc a1[36 * 36];
  memset(a1, 0, sizeof(a1));
  for (int i = 0; i < lmmax; i++)
    for (int j = 0; j < lmmax; j++) a1[IX(i, j, 36)] = fac * a[IX(i, j, lda)];
  for (int i = 0; i < kmymax; i++) {
    int i1 = ind1[i] - 1, i2 = ind2[i] - 1;
    for (int j = 0; j < kmymax; j++) {
      int j1 = ind1[j] - 1, j2 = ind2[j] - 1;
      b[IX(i, j, ldb)] = u1[i] * a1[IX(i1, j1, 36)] * u1[j] + u2[i] * a1[IX(i2, j2, 36)] * u2[j];
    }
  }
}

/* ===================================================================== *
 * main/packer.f:6-100  M00, M0-1 (m10), M01 = -G blocks of one PL        *
 * g2d(.,.,j,i) is looked up through the block map.                      *
 * ===================================================================== */
static const zc *g2d_block(const orc_g2dmap *map, const zc *blocks, int slot, int i, int j) {
  if (j < -map->jmax || j > map->jmax || i < 1 || i > map->mi) return NULL;
  int nj = 2 * map->jmax + 1;
  int b = map->blkmap[((size_t)slot * map->mi + (i - 1)) * nj + (j + map->jmax)];
  if (b < 0) return NULL;
  return blocks + (size_t)b * map->lmmax * map->lmmax;
}

static void put_block(zc *m, int mdim, int kki, int kkj, int lkmax, const zc *g,
                      const orc_g2dmap *map, int irel, zc fac) {
  zc rg[72 * 72];
  const int lmmax = map->lmmax, lmax = map->lmax;
  if (g == NULL) {
    for (int k1 = 0; k1 < lkmax; k1++)
      for (int k2 = 0; k2 < lkmax; k2++) m[IX(k1 + kki, k2 + kkj, mdim)] = 0.0;
    return;
  }
  if (irel == 2) {
    /* g2d_pack.f: blockdiag(G_e, G_h), then relmtrx.f with fac (e) / fach (h) */
    const int km = lkmax / 2;
    const zc *gh = g + (size_t)map->nblk * lmmax * lmmax;
    for (int k1 = 0; k1 < lkmax; k1++)
      for (int k2 = 0; k2 < lkmax; k2++) m[IX(k1 + kki, k2 + kkj, mdim)] = 0.0;
    orc_relmtrx(g, lmmax, rg, 72, fac, lmax);
    for (int k1 = 0; k1 < km; k1++)
      for (int k2 = 0; k2 < km; k2++) m[IX(k1 + kki, k2 + kkj, mdim)] = -rg[IX(k1, k2, 72)];
    orc_relmtrx(gh, lmmax, rg, 72, map->fach, lmax);
    for (int k1 = 0; k1 < km; k1++)
      for (int k2 = 0; k2 < km; k2++) m[IX(k1 + km + kki, k2 + km + kkj, mdim)] = -rg[IX(k1, k2, 72)];
  } else if (irel == 1) {
    orc_relmtrx(g, lmmax, rg, 72, fac, lmax);
    for (int k1 = 0; k1 < lkmax; k1++)
      for (int k2 = 0; k2 < lkmax; k2++) m[IX(k1 + kki, k2 + kkj, mdim)] = -rg[IX(k1, k2, 72)];
  } else {
    for (int k1 = 0; k1 < lkmax; k1++)
      for (int k2 = 0; k2 < lkmax; k2++) m[IX(k1 + kki, k2 + kkj, mdim)] = -g[IX(k1, k2, lmmax)];
  }
}

void orc_packer(int ni, int nim, int nip, const orc_g2dmap *map, int slot,
                const zc *blocks, zc *m00, zc *m10, zc *m01, int lkmax,
                int mdim, int irel, zc fac) {
  czero(m01, (size_t)mdim * mdim);
  czero(m10, (size_t)mdim * mdim);
  for (int i = 1; i <= ni; i++) {
    int jmin, jmax;
    if (ni <= nim) jmin = -nim;
    else jmin = -(ni < nim + i - 1 ? ni : nim + i - 1);
    if (ni <= nip) jmax = nip;
    else jmax = (ni < nip + ni - i ? ni : nip + ni - i);
    int kki = (i - 1) * lkmax;
    for (int j = jmin; j <= -i; j++) {           /* M0-1 */
      int jp = nim + i + j;
      put_block(m10, mdim, kki, (jp - 1) * lkmax, lkmax, g2d_block(map, blocks, slot, i, j),
                map, irel, fac);
    }
    for (int j = 1 - i; j <= ni - i; j++) {      /* M00 */
      int jp = j + i;
      put_block(m00, mdim, kki, (jp - 1) * lkmax, lkmax, g2d_block(map, blocks, slot, i, j),
                map, irel, fac);
    }
    for (int j = ni - i + 1; j <= jmax; j++) {   /* M01 */
      int jp = j + i - ni;
      put_block(m01, mdim, kki, (jp - 1) * lkmax, lkmax, g2d_block(map, blocks, slot, i, j),
                map, irel, fac);
    }
  }
}

/* ===================================================================== *
 * main/surfgf.f:2-108  decimation for f(x) = ml (m0 - x)^-1 mr           *
 * ===================================================================== */
int orc_surfgfd(const zc *ml, const zc *m0, const zc *mmr, zc *x, int kdim,
                int mdim, int itermax, double errmax, int *iters) {
  const double errmin = 1.0e10;
  size_t sz = (size_t)mdim * mdim;
  zc *alfa = calloc(sz, sizeof(zc)), *beta = calloc(sz, sizeof(zc)), *eps = calloc(sz, sizeof(zc));
  zc *y1 = calloc(sz, sizeof(zc)), *y2 = calloc(sz, sizeof(zc)), *y3 = calloc(sz, sizeof(zc)),
     *y4 = calloc(sz, sizeof(zc));
  zc detl;
  int status = 0;
  czero(x, sz);
  for (int i = 0; i < kdim; i++)
    for (int j = 0; j < kdim; j++) {
      eps[IX(i, j, mdim)] = m0[IX(i, j, mdim)];
      alfa[IX(i, j, mdim)] = -ml[IX(i, j, mdim)];
      beta[IX(i, j, mdim)] = -mmr[IX(i, j, mdim)];
      x[IX(i, j, mdim)] = m0[IX(i, j, mdim)];
    }
  int iter = 1;
  for (;;) {
    for (int i = 0; i < kdim; i++)
      for (int j = 0; j < kdim; j++) y1[IX(i, j, mdim)] = eps[IX(i, j, mdim)];
    orc_gjinv(y1, kdim, mdim, &detl);
    for (int i = 0; i < kdim; i++)
      for (int j = 0; j < kdim; j++) {
        y2[IX(i, j, mdim)] = y1[IX(i, j, mdim)];
        y3[IX(i, j, mdim)] = y1[IX(i, j, mdim)];
        y4[IX(i, j, mdim)] = y1[IX(i, j, mdim)];
      }
    orc_tripmt(alfa, y1, alfa, kdim, kdim, mdim);
    orc_tripmt(beta, y2, beta, kdim, kdim, mdim);
    orc_tripmt(alfa, y3, beta, kdim, kdim, mdim);
    orc_tripmt(beta, y4, alfa, kdim, kdim, mdim);
    double sum = 0.0;
    for (int i = 0; i < kdim; i++)
      for (int j = 0; j < kdim; j++) {
        alfa[IX(i, j, mdim)] = y1[IX(i, j, mdim)];
        beta[IX(i, j, mdim)] = y2[IX(i, j, mdim)];
        eps[IX(i, j, mdim)] = eps[IX(i, j, mdim)] - y3[IX(i, j, mdim)] - y4[IX(i, j, mdim)];
        x[IX(i, j, mdim)] = x[IX(i, j, mdim)] - y3[IX(i, j, mdim)];
        double xre = creal(alfa[IX(i, j, mdim)]), xim = cimag(alfa[IX(i, j, mdim)]);
        sum = sum + xre * xre + xim * xim;
      }
    double err = sqrt(sum);
    if (err < errmax || iter > itermax) break;
    if (err > errmin) { status = 2; break; }
    iter++;
  }
  if (status == 0 && iter > itermax) status = 1;
  if (iters) *iters = iter;
  orc_gjinv(x, kdim, mdim, &detl);
  free(alfa); free(beta); free(eps); free(y1); free(y2); free(y3); free(y4);
  return status;
}

/* main/dugo.f:9-120, bulk branch (the reference only calls dugo with
 * bulk=.true., rsp-scf/cpacoord_ksave.f:261-305).  slot_bulk is the lead's
 * own slot (0 for L, nprc+1 for R), slot_int the adjacent interface slot. */
int orc_dugo(int side, const int *ninprc, int nprc, const orc_g2dmap *map,
             const zc *blocks, int slot_bulk, int slot_int, const zc *tminvb,
             int lkmaxp, zc *xy, int mdimp, int lkmax, int irel, zc fac,
             int itermax, double errmax, int *iters) {
  (void)nprc;
  int mdim = mdimp;
  size_t sz = (size_t)mdim * mdim;
  zc *m00 = calloc(sz, sizeof(zc)), *m01 = calloc(sz, sizeof(zc)), *m10 = calloc(sz, sizeof(zc));
  zc *mt = calloc(sz, sizeof(zc)), *xys = calloc(sz, sizeof(zc));
  int ncpl = ninprc[1], ncpli = ncpl;
  if (side == 'L')
    orc_packer(ncpl, ncpl, ncpl, map, slot_bulk, blocks, m00, m10, mt, lkmax, mdim, irel, fac);
  else
    orc_packer(ncpl, ncpl, ncpl, map, slot_bulk, blocks, m00, mt, m01, lkmax, mdim, irel, fac);
  orc_packer(ncpl, ncpl, ncpl, map, slot_int, blocks, m00, m10, m01, lkmax, mdim, irel, fac);
  int nn = ncpl * lkmax, ni = ncpli * lkmax;
  for (int inprc = 0; inprc < ncpl; inprc++)
    for (int kmy = 0; kmy < lkmax; kmy++)
      for (int kmyp = 0; kmyp < lkmax; kmyp++) {
        int i = inprc * lkmax + kmy, j = inprc * lkmax + kmyp;
        m00[IX(i, j, mdim)] = tminvb[IX(kmy, kmyp, lkmaxp) + (size_t)inprc * lkmaxp * lkmaxp] + m00[IX(i, j, mdim)];
      }
  int st;
  if (side == 'L') {
    st = orc_surfgfd(m10, m00, m01, xys, nn, mdim, itermax, errmax, iters);
    orc_tripmt2(m10, xys, mt, xy, ni, nn, nn, ni, mdim, mdimp);
  } else {
    st = orc_surfgfd(m01, m00, m10, xys, nn, mdim, itermax, errmax, iters);
    orc_tripmt2(m01, xys, mt, xy, ni, nn, nn, ni, mdim, mdimp);
  }
  free(m00); free(m01); free(m10); free(mt); free(xys);
  return st;
}

/* ===================================================================== *
 * main/tau2d.f:2-152  Godfrin block-tridiagonal PL-diagonal tau          *
 * ===================================================================== */
void orc_tau2d(int irel, double wgeff, int bulkgeo, const int *ninprc,
               int nprc, const orc_g2dmap *map, const zc *blocks,
               const zc *tminv, int lkmaxp, int lkmax, const zc *x,
               const zc *y, int mdimp, zc *tau, zc fac) {
  int mdim = mdimp;
  size_t sz = (size_t)mdim * mdim;
  zc *xx = calloc(sz * nprc, sizeof(zc)), *yy = calloc(sz * nprc, sizeof(zc));
  zc *tau00 = calloc(sz * nprc, sizeof(zc));
  zc *m00 = calloc(sz, sizeof(zc)), *m01 = calloc(sz, sizeof(zc)), *m10 = calloc(sz, sizeof(zc));
  zc *help = calloc(sz, sizeof(zc));
  zc detl;
  int ndim = lkmax * ninprc[1];
  for (int i = 0; i < ndim; i++)
    for (int j = 0; j < ndim; j++) yy[IX(i, j, mdim)] = y[IX(i, j, mdimp)];
  ndim = lkmax * ninprc[nprc];
  for (int i = 0; i < ndim; i++)
    for (int j = 0; j < ndim; j++) xx[IX(i, j, mdim) + sz * (nprc - 1)] = x[IX(i, j, mdimp)];

  int ilay = 0;
  for (int ipl = 1; ipl <= nprc; ipl++) {
    int slot = bulkgeo ? 1 : ipl;
    ndim = lkmax * ninprc[ipl];
    orc_packer(ninprc[ipl], ninprc[ipl - 1], ninprc[ipl + 1], map, slot, blocks, m00, m10, m01,
               lkmax, mdim, irel, fac);
    for (int li = 0; li < ninprc[ipl]; li++) {
      for (int k1 = 0; k1 < lkmax; k1++)
        for (int k2 = 0; k2 < lkmax; k2++) {
          int kk1 = li * lkmax + k1, kk2 = li * lkmax + k2;
          m00[IX(kk1, kk2, mdim)] = tminv[IX(k1, k2, lkmaxp) + (size_t)ilay * lkmaxp * lkmaxp] + m00[IX(kk1, kk2, mdim)];
        }
      ilay++;
    }
    zc *t00 = tau00 + sz * (ipl - 1), *yyp = yy + sz * (ipl - 1);
    for (int i = 0; i < ndim; i++)
      for (int j = 0; j < ndim; j++) t00[IX(i, j, mdim)] = m00[IX(i, j, mdim)];
    if (ipl > 1) {
      int ndim0 = lkmax * ninprc[ipl - 1];
      orc_doubmt2(m10, yyp, help, ndim, ndim0, ndim, mdim);
      for (int i = 0; i < ndim; i++)
        for (int j = 0; j < ndim; j++) yyp[IX(i, j, mdim)] = help[IX(i, j, mdim)];
    }
    if (ipl < nprc) {
      int ndim1 = lkmax * ninprc[ipl + 1];
      for (int i = 0; i < ndim; i++)
        for (int j = 0; j < ndim; j++) m00[IX(i, j, mdim)] -= yyp[IX(i, j, mdim)];
      orc_gjinv(m00, ndim, mdim, &detl);
      orc_doubmt2(m00, m01, yy + sz * ipl, ndim, ndim, ndim1, mdim);
    }
  }
  for (int ipl = nprc; ipl >= 1; ipl--) {
    int slot = bulkgeo ? 1 : ipl;
    ndim = lkmax * ninprc[ipl];
    orc_packer(ninprc[ipl], ninprc[ipl - 1], ninprc[ipl + 1], map, slot, blocks, m00, m10, m01,
               lkmax, mdim, irel, fac);
    zc *xxp = xx + sz * (ipl - 1);
    if (ipl < nprc) {
      int ndim1 = lkmax * ninprc[ipl + 1];
      orc_doubmt2(m01, xxp, m00, ndim, ndim1, ndim, mdim);
      for (int i = 0; i < ndim; i++)
        for (int j = 0; j < ndim; j++) xxp[IX(i, j, mdim)] = m00[IX(i, j, mdim)];
    }
    if (ipl > 1) {
      int ndim0 = lkmax * ninprc[ipl - 1];
      zc *t00 = tau00 + sz * (ipl - 1);
      for (int i = 0; i < ndim; i++)
        for (int j = 0; j < ndim; j++) m00[IX(i, j, mdim)] = t00[IX(i, j, mdim)] - xxp[IX(i, j, mdim)];
      orc_gjinv(m00, ndim, mdim, &detl);
      orc_doubmt2(m00, m10, xx + sz * (ipl - 2), ndim, ndim, ndim0, mdim);
    }
  }
  ilay = 0;
  for (int ipl = 1; ipl <= nprc; ipl++) {
    ndim = lkmax * ninprc[ipl];
    zc *t00 = tau00 + sz * (ipl - 1), *xxp = xx + sz * (ipl - 1), *yyp = yy + sz * (ipl - 1);
    for (int i = 0; i < ndim; i++)
      for (int j = 0; j < ndim; j++)
        t00[IX(i, j, mdim)] = t00[IX(i, j, mdim)] - xxp[IX(i, j, mdim)] - yyp[IX(i, j, mdim)];
    orc_gjinv(t00, ndim, mdim, &detl);
    int il0 = 0;
    for (int inprc = 0; inprc < ninprc[ipl]; inprc++) {
      zc *tl = tau + (size_t)ilay * lkmaxp * lkmaxp;
      for (int l = 0; l < lkmax; l++)
        for (int lp = 0; lp < lkmax; lp++) tl[IX(l, lp, lkmaxp)] = wgeff * t00[IX(il0 + l, il0 + lp, mdim)];
      il0 += lkmax;
      ilay++;
    }
  }
  free(xx); free(yy); free(tau00); free(m00); free(m01); free(m10); free(help);
}

/* ===================================================================== *
 * skkr_dbogo_bsf/clu/tau2d_god.f:2-270  full Godfrin tau: every layer    *
 * pair of the interface.  The forward and backward sweeps are tau2d.f's; *
 * dd(p) = -(m00 - yy(p))^-1 m01 and cc(p) = -(tau00(p) - xx(p))^-1 m10   *
 * are kept, and the PL-diagonal tau(p,p) is carried down the slab by      *
 * tau(q,p) = cc(q) tau(q-1,p) (q > p) and up by tau(q,p) = dd(q)          *
 * tau(q+1,p) (q < p).  tauij[(a*nintfc + b)*ld*ld] = wgeff tau_{a,b}     *
 * (row layer a, column layer b).                                          *
 * ===================================================================== */
void orc_tau2dgod(int irel, double wgeff, int bulkgeo, const int *ninprc,
                  int nprc, const orc_g2dmap *map, const zc *blocks,
                  const zc *tminv, int lkmaxp, int lkmax, const zc *x,
                  const zc *y, int mdimp, zc *tauij, int nintfc, zc fac) {
  int mdim = mdimp;
  size_t sz = (size_t)mdim * mdim, lsz = (size_t)lkmaxp * lkmaxp;
  zc *xx = calloc(sz * nprc, sizeof(zc)), *yy = calloc(sz * nprc, sizeof(zc));
  zc *tau00 = calloc(sz * nprc, sizeof(zc));
  zc *cc = calloc(sz * nprc, sizeof(zc)), *dd = calloc(sz * nprc, sizeof(zc));
  zc *m00 = calloc(sz, sizeof(zc)), *m01 = calloc(sz, sizeof(zc)), *m10 = calloc(sz, sizeof(zc));
  zc *help = calloc(sz, sizeof(zc)), *help1 = calloc(sz, sizeof(zc));
  int *nnprc = calloc(nprc, sizeof(int));
  zc detl;
  for (int ipl = 0, acc = 0; ipl < nprc; ipl++) {
    nnprc[ipl] = acc;
    acc += ninprc[ipl + 1];
  }
  int ndim = lkmax * ninprc[1];
  for (int i = 0; i < ndim; i++)
    for (int j = 0; j < ndim; j++) yy[IX(i, j, mdim)] = y[IX(i, j, mdimp)];
  ndim = lkmax * ninprc[nprc];
  for (int i = 0; i < ndim; i++)
    for (int j = 0; j < ndim; j++) xx[IX(i, j, mdim) + sz * (nprc - 1)] = x[IX(i, j, mdimp)];

  int ilay = 0;
  for (int ipl = 1; ipl <= nprc; ipl++) {
    int slot = bulkgeo ? 1 : ipl;
    ndim = lkmax * ninprc[ipl];
    orc_packer(ninprc[ipl], ninprc[ipl - 1], ninprc[ipl + 1], map, slot, blocks, m00, m10, m01,
               lkmax, mdim, irel, fac);
    for (int li = 0; li < ninprc[ipl]; li++) {
      for (int k1 = 0; k1 < lkmax; k1++)
        for (int k2 = 0; k2 < lkmax; k2++) {
          int kk1 = li * lkmax + k1, kk2 = li * lkmax + k2;
          m00[IX(kk1, kk2, mdim)] = tminv[IX(k1, k2, lkmaxp) + (size_t)ilay * lsz] + m00[IX(kk1, kk2, mdim)];
        }
      ilay++;
    }
    zc *t00 = tau00 + sz * (ipl - 1), *yyp = yy + sz * (ipl - 1);
    for (int i = 0; i < ndim; i++)
      for (int j = 0; j < ndim; j++) t00[IX(i, j, mdim)] = m00[IX(i, j, mdim)];
    if (ipl > 1) {
      int ndim0 = lkmax * ninprc[ipl - 1];
      orc_doubmt2(m10, yyp, help, ndim, ndim0, ndim, mdim);
      for (int i = 0; i < ndim; i++)
        for (int j = 0; j < ndim; j++) yyp[IX(i, j, mdim)] = help[IX(i, j, mdim)];
    }
    if (ipl < nprc) {
      int ndim1 = lkmax * ninprc[ipl + 1];
      for (int i = 0; i < ndim; i++)
        for (int j = 0; j < ndim; j++) m00[IX(i, j, mdim)] -= yyp[IX(i, j, mdim)];
      orc_gjinv(m00, ndim, mdim, &detl);
      orc_doubmt2(m00, m01, yy + sz * ipl, ndim, ndim, ndim1, mdim);
      zc *ddp = dd + sz * (ipl - 1), *yn = yy + sz * ipl;   /* dd = -yy(ipl+1), tau2d_god.f:85-90 */
      for (int i = 0; i < ndim1; i++)
        for (int j = 0; j < ndim; j++) ddp[IX(j, i, mdim)] = -yn[IX(j, i, mdim)];
    }
  }
  for (int ipl = nprc; ipl >= 1; ipl--) {
    int slot = bulkgeo ? 1 : ipl;
    ndim = lkmax * ninprc[ipl];
    orc_packer(ninprc[ipl], ninprc[ipl - 1], ninprc[ipl + 1], map, slot, blocks, m00, m10, m01,
               lkmax, mdim, irel, fac);
    zc *xxp = xx + sz * (ipl - 1);
    if (ipl < nprc) {
      int ndim1 = lkmax * ninprc[ipl + 1];
      orc_doubmt2(m01, xxp, m00, ndim, ndim1, ndim, mdim);
      for (int i = 0; i < ndim; i++)
        for (int j = 0; j < ndim; j++) xxp[IX(i, j, mdim)] = m00[IX(i, j, mdim)];
    }
    if (ipl > 1) {
      int ndim0 = lkmax * ninprc[ipl - 1];
      zc *t00 = tau00 + sz * (ipl - 1);
      for (int i = 0; i < ndim; i++)
        for (int j = 0; j < ndim; j++) m00[IX(i, j, mdim)] = t00[IX(i, j, mdim)] - xxp[IX(i, j, mdim)];
      orc_gjinv(m00, ndim, mdim, &detl);
      orc_doubmt2(m00, m10, xx + sz * (ipl - 2), ndim, ndim, ndim0, mdim);
      zc *ccp = cc + sz * (ipl - 1), *xn = xx + sz * (ipl - 2);  /* cc = -xx(ipl-1), :108-113 */
      for (int i = 0; i < ndim0; i++)
        for (int j = 0; j < ndim; j++) ccp[IX(j, i, mdim)] = -xn[IX(j, i, mdim)];
    }
  }
  for (int ip = 0; ip < nprc; ip++) {
    ndim = lkmax * ninprc[ip + 1];
    zc *t00 = tau00 + sz * ip, *xxp = xx + sz * ip, *yyp = yy + sz * ip;
    for (int i = 0; i < ndim; i++)
      for (int j = 0; j < ndim; j++)
        t00[IX(i, j, mdim)] = t00[IX(i, j, mdim)] - xxp[IX(i, j, mdim)] - yyp[IX(i, j, mdim)];
    orc_gjinv(t00, ndim, mdim, &detl);
    /* PL block (q, ip) -> layer blocks (nnprc[q] + a, nnprc[ip] + b) */
#define PUT_BLOCK(Q, HB)                                                                          \
    for (int a = 0; a < ninprc[(Q) + 1]; a++)                                                     \
      for (int b = 0; b < ninprc[ip + 1]; b++) {                                                  \
        zc *tl = tauij + ((size_t)(nnprc[Q] + a) * nintfc + (nnprc[ip] + b)) * lsz;               \
        for (int r = 0; r < lkmax; r++)                                                           \
          for (int c2 = 0; c2 < lkmax; c2++)                                                      \
            tl[IX(r, c2, lkmaxp)] = wgeff * (HB)[IX(a * lkmax + r, b * lkmax + c2, mdim)];        \
      }
    PUT_BLOCK(ip, t00)
    for (int i = 0; i < ndim; i++)
      for (int j = 0; j < ndim; j++) help[IX(i, j, mdim)] = t00[IX(i, j, mdim)];
    for (int q = ip + 1; q < nprc; q++) {     /* down: tau(q,ip) = cc(q) tau(q-1,ip) */
      int jdim = lkmax * ninprc[q + 1], jdim0 = lkmax * ninprc[q];
      orc_doubmt2(cc + sz * q, help, help1, jdim, jdim0, ndim, mdim);
      for (int i = 0; i < jdim; i++)
        for (int j = 0; j < ndim; j++) help[IX(i, j, mdim)] = help1[IX(i, j, mdim)];
      PUT_BLOCK(q, help)
    }
    for (int i = 0; i < ndim; i++)
      for (int j = 0; j < ndim; j++) help[IX(i, j, mdim)] = t00[IX(i, j, mdim)];
    for (int q = ip - 1; q >= 0; q--) {       /* up: tau(q,ip) = dd(q) tau(q+1,ip) */
      int jdim = lkmax * ninprc[q + 1], jdim1 = lkmax * ninprc[q + 2];
      orc_doubmt2(dd + sz * q, help, help1, jdim, jdim1, ndim, mdim);
      for (int i = 0; i < jdim; i++)
        for (int j = 0; j < ndim; j++) help[IX(i, j, mdim)] = help1[IX(i, j, mdim)];
      PUT_BLOCK(q, help)
    }
#undef PUT_BLOCK
  }
  free(xx); free(yy); free(tau00); free(cc); free(dd); free(m00); free(m01); free(m10);
  free(help); free(help1); free(nnprc);
}

/* ===================================================================== *
 * rsp-scf/fullcpa.f:2-155  ATA start, Ginatempo-Staunton CPA update      *
 * ===================================================================== */
void orc_tata(double conc, int n, int ld, zc *mc, const zc *ma, const zc *mb) {
  double cca = conc, ccb = 1.0 - cca;
  zc det;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) mc[IX(i, j, ld)] = cca * mb[IX(i, j, ld)] + ccb * ma[IX(i, j, ld)];
  orc_gjinv(mc, n, ld, &det);
  orc_tripmt(mb, mc, ma, n, n, ld);
}

void orc_cpasol(double conc, zc *mc, const zc *ma, const zc *mb,
                const zc *tauc, zc *taua, zc *taub, int n, int ld,
                double *error1, double *error2, double *error3) {
  size_t sz = (size_t)ld * ld;
  zc *h = calloc(sz, sizeof(zc)), *da = calloc(sz, sizeof(zc)), *db = calloc(sz, sizeof(zc));
  zc *xc = calloc(sz, sizeof(zc)), *xa = calloc(sz, sizeof(zc)), *xb = calloc(sz, sizeof(zc));
  zc det;
  double cca = conc, ccb = 1.0 - cca;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      da[IX(i, j, ld)] = mc[IX(i, j, ld)] - ma[IX(i, j, ld)];
      db[IX(i, j, ld)] = mc[IX(i, j, ld)] - mb[IX(i, j, ld)];
      xa[IX(i, j, ld)] = da[IX(i, j, ld)];
      xb[IX(i, j, ld)] = db[IX(i, j, ld)];
    }
  orc_gjinv(xa, n, ld, &det);
  orc_gjinv(xb, n, ld, &det);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      xa[IX(i, j, ld)] -= tauc[IX(i, j, ld)];
      xb[IX(i, j, ld)] -= tauc[IX(i, j, ld)];
    }
  orc_gjinv(xa, n, ld, &det);
  orc_gjinv(xb, n, ld, &det);
  *error1 = 0.0;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      xc[IX(i, j, ld)] = cca * xa[IX(i, j, ld)] + ccb * xb[IX(i, j, ld)];
      double d = cabs(xc[IX(i, j, ld)]);
      if (d > *error1) *error1 = d;
    }
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) h[IX(i, j, ld)] = xc[IX(i, j, ld)];
  orc_gjinv(h, n, ld, &det);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) h[IX(i, j, ld)] += tauc[IX(i, j, ld)];
  orc_gjinv(h, n, ld, &det);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) mc[IX(i, j, ld)] -= h[IX(i, j, ld)];
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) xc[IX(i, j, ld)] = tauc[IX(i, j, ld)];
  orc_tripmt(da, xc, db, n, n, ld);
  *error2 = 0.0;
  double d1 = 0.0, d2 = 0.0;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      xc[IX(i, j, ld)] = xc[IX(i, j, ld)] - cca * da[IX(i, j, ld)] - ccb * db[IX(i, j, ld)];
      double d = cabs(xc[IX(i, j, ld)]);
      if (d > *error2) *error2 = d;
      d1 = d1 + creal(h[IX(i, j, ld)] * conj(h[IX(i, j, ld)]));
      d2 = d2 + creal(mc[IX(i, j, ld)] * conj(mc[IX(i, j, ld)]));
    }
  *error3 = sqrt(d1 / d2);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      taua[IX(i, j, ld)] = xa[IX(i, j, ld)];
      taub[IX(i, j, ld)] = xb[IX(i, j, ld)];
    }
  orc_tripmt(tauc, taua, tauc, n, n, ld);
  orc_tripmt(tauc, taub, tauc, n, n, ld);
  for (int i = 0; i < n; i++)
    for (int j = 0; j < n; j++) {
      taua[IX(i, j, ld)] += tauc[IX(i, j, ld)];
      taub[IX(i, j, ld)] += tauc[IX(i, j, ld)];
    }
  free(h); free(da); free(db); free(xc); free(xa); free(xb);
}

void orc_cpacor(const double *conc, zc *mc, const zc *ma, const zc *mb,
                const zc *tauc, zc *taua, zc *taub, int n, int ld, int nintfc,
                int *itcpa, int itcpam, double cpatol, int *cpacon,
                int *concpa, double *error) {
  const double tiny = 1.0e-6, tol = 1.0e-10;
  size_t sz = (size_t)ld * ld;
  *error = 0.0;
  for (int li = 0; li < nintfc; li++) {
    int cpalay = (1.0 - conc[li]) > tiny;
    int ica = orc_compmat(ma + sz * li, mc + sz * li, n, ld, tol);
    int icb = orc_compmat(mb + sz * li, mc + sz * li, n, ld, tol);
    if (!cpalay || ica + icb >= 1) {
      for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
          taua[sz * li + IX(i, j, ld)] = tauc[sz * li + IX(i, j, ld)];
          taub[sz * li + IX(i, j, ld)] = tauc[sz * li + IX(i, j, ld)];
        }
      continue;
    }
    double e1, e2, e3;
    orc_cpasol(conc[li], mc + sz * li, ma + sz * li, mb + sz * li, tauc + sz * li,
               taua + sz * li, taub + sz * li, n, ld, &e1, &e2, &e3);
    if (e3 >= *error) *error = e3;
  }
  if (*error <= cpatol) *concpa = 0;
  if (*itcpa >= itcpam) *cpacon = 0;
  (*itcpa)++;
}

/* cluster/rsp-lay/phystau2.f:2-60 and skkr_dbogo_bsf/clu/phystau2.f:2-75:
 * the block tau_ij between layers i and j, screened -> physical:
 *   tau := (1 + alpha1 tinv1) tau (1 + tinv2 alpha2)  [- (alpha1 + alpha1 tinv1 alpha2) if idiag],
 * alpha1 / tinv1 those of layer i (rows), alpha2 / tinv2 of layer j (columns).
 * The same l index tables as rsp-scf/phystau.f:2-61 (irel=1, ldex over
 * kappa-mu), nrsp-scf/phystau.f (irel=0, l over lm).  alpha[l], l = 0..lmax. */
void orc_phystau2(zc *tau, const zc *tinv1, const zc *alpha1, const zc *tinv2,
                  const zc *alpha2, int lmax, int irel, int ld, int idiag) {
  int lmmax = (lmax + 1) * (lmax + 1);
  int nd = irel == 2 ? 4 * lmmax : irel ? 2 * lmmax : lmmax;
  size_t sz = (size_t)ld * ld;
  zc *lmat = calloc(sz, sizeof(zc)), *rmat = calloc(sz, sizeof(zc)), *cmat = calloc(sz, sizeof(zc));
  int *ldex = malloc(sizeof(int) * nd);
  if (irel) {
    /* ldex table of rsp-scf/phystau.f: 2,6,10,14,18 entries per l; BdG
       (skkr_dbogo_bsf cpacoord_ksave.f:497): the hole half uses alpha_h,
       stored after alpha_e as alpha[lmax+1+l] */
    int kmymax = 2 * lmmax, k = 0;
    for (int l = 0; k < kmymax; l++) {
      int cnt = (l == 0) ? 2 : 4 * l + 2;
      for (int c = 0; c < cnt && k < kmymax; c++) ldex[k++] = l;
    }
    for (int q = kmymax; q < nd; q++) ldex[q] = ldex[q - kmymax] + lmax + 1;
  } else {
    for (int l = 0, k = 0; l <= lmax; l++)
      for (int m = -l; m <= l; m++) ldex[k++] = l;
  }
  for (int a = 0; a < nd; a++) {
    zc al = alpha1[ldex[a]];
    for (int b = 0; b < nd; b++) {
      zc alp = alpha2[ldex[b]];
      lmat[IX(a, b, ld)] = al * tinv1[IX(a, b, ld)];
      rmat[IX(a, b, ld)] = tinv2[IX(a, b, ld)] * alp;
      cmat[IX(a, b, ld)] = al * tinv1[IX(a, b, ld)] * alp;
    }
    lmat[IX(a, a, ld)] = 1.0 + lmat[IX(a, a, ld)];
    rmat[IX(a, a, ld)] = 1.0 + rmat[IX(a, a, ld)];
    cmat[IX(a, a, ld)] = al + cmat[IX(a, a, ld)];
  }
  orc_tripmt(lmat, tau, rmat, nd, nd, ld);
  if (idiag == 1)
    for (int a = 0; a < nd; a++)
      for (int b = 0; b < nd; b++) tau[IX(a, b, ld)] -= cmat[IX(a, b, ld)];
  free(lmat); free(rmat); free(cmat); free(ldex);
}

/* rsp-scf/phystau.f:2-61, nrsp-scf/phystau.f: one screening set on both sides */
void orc_phystau(zc *tau, const zc *tinv1, const zc *tinv2, const zc *alpha,
                 int lmax, int irel, int ld, int idiag) {
  orc_phystau2(tau, tinv1, alpha, tinv2, alpha, lmax, irel, ld, idiag);
}

/* ===================================================================== *
 * rsp-scf/sorttmat.f:2-205  rotate t^-1 by each g, find equivalent g     *
 * (ieqg etc. returned 1-based, as the reference)                         *
 * ===================================================================== */
void orc_sorttmat(int lkmax, int ld, int nintfc, int nl, int nr, int ngeff,
                  const zc *rg, const zc *lg, const zc *tminvl,
                  const zc *tminvr, const zc *tminv, zc *ttmpl, zc *ttmpr,
                  zc *ttmp, int *ieqgl, int *ieqgr, int *ieqg, int *igordl,
                  int *igordr) {
  const double tol = 1.0e-8;
  size_t sz = (size_t)ld * ld;
  for (int ig = 0; ig < ngeff; ig++) {
    for (int li = 0; li < nl; li++) {
      zc *t = ttmpl + sz * ((size_t)ig * nl + li);
      memcpy(t, tminvl + sz * li, sz * sizeof(zc));
      orc_tripmt(rg + sz * ig, t, lg + sz * ig, lkmax, lkmax, ld);
    }
    for (int li = 0; li < nr; li++) {
      zc *t = ttmpr + sz * ((size_t)ig * nr + li);
      memcpy(t, tminvr + sz * li, sz * sizeof(zc));
      orc_tripmt(rg + sz * ig, t, lg + sz * ig, lkmax, lkmax, ld);
    }
    for (int li = 0; li < nintfc; li++) {
      zc *t = ttmp + sz * ((size_t)ig * nintfc + li);
      memcpy(t, tminv + sz * li, sz * sizeof(zc));
      orc_tripmt(rg + sz * ig, t, lg + sz * ig, lkmax, lkmax, ld);
    }
  }
#define TL(ig, li) (ttmpl + sz * ((size_t)(ig) * nl + (li)))
#define TR(ig, li) (ttmpr + sz * ((size_t)(ig) * nr + (li)))
#define TI(ig, li) (ttmp + sz * ((size_t)(ig) * nintfc + (li)))
  ieqg[0] = 1;
  for (int ig = 1; ig < ngeff; ig++) {
    int found = -1;
    for (int iig = 0; iig < ig && found < 0; iig++) {
      int ok = 1;
      for (int li = 0; li < nl && ok; li++) ok = orc_compmat(TL(iig, li), TL(ig, li), lkmax, ld, tol);
      for (int li = 0; li < nr && ok; li++) ok = orc_compmat(TR(iig, li), TR(ig, li), lkmax, ld, tol);
      for (int li = 0; li < nintfc && ok; li++) ok = orc_compmat(TI(iig, li), TI(ig, li), lkmax, ld, tol);
      if (ok) found = iig;
    }
    ieqg[ig] = found < 0 ? ig + 1 : found + 1;
  }
  ieqgl[0] = 1; igordl[0] = 1;
  for (int ig = 1; ig < ngeff; ig++) {
    int found = -1;
    for (int iig = 0; iig < ig && found < 0; iig++) {
      int ok = 1;
      for (int li = 0; li < nl && ok; li++) ok = orc_compmat(TL(iig, li), TL(ig, li), lkmax, ld, tol);
      if (ok) found = iig;
    }
    if (found < 0) {
      ieqgl[ig] = ig + 1;
      igordl[ig] = igordl[ieqgl[ig - 1] - 1] + 1;
    } else ieqgl[ig] = found + 1;
  }
  ieqgr[0] = 1; igordr[0] = 1;
  for (int ig = 1; ig < ngeff; ig++) {
    int found = -1;
    for (int iig = 0; iig < ig && found < 0; iig++) {
      int ok = 1;
      for (int li = 0; li < nr && ok; li++) ok = orc_compmat(TR(iig, li), TR(ig, li), lkmax, ld, tol);
      if (ok) found = iig;
    }
    if (found < 0) {
      ieqgr[ig] = ig + 1;
      igordr[ig] = igordr[ieqgr[ig - 1] - 1] + 1;
    } else ieqgr[ig] = found + 1;
  }
#undef TL
#undef TR
#undef TI
}

/* G_scr(k) blocks from the real-space screened table (no reference
 * counterpart: the reference builds G(k) by Kambe Ewald sums, main/gstore.f).
 * blocks[b] = sum_{r in block b} exp(+i k.R_r) G(R_r). */
void orc_gk_from_rtable(int nblk, const int *rstart, const double *rvec,
                        const zc *gR, int lmmax, double kx, double ky, zc *blocks) {
  size_t bs = (size_t)lmmax * lmmax;
  for (int b = 0; b < nblk; b++) {
    zc *out = blocks + bs * b;
    czero(out, bs);
    for (int r = rstart[b]; r < rstart[b + 1]; r++) {
      double ph = kx * rvec[2 * r] + ky * rvec[2 * r + 1];
      zc e = cos(ph) + sin(ph) * I;
      const zc *g = gR + bs * r;
      for (size_t q = 0; q < bs; q++) out[q] += e * g[q];
    }
  }
}

static orc_reduce_fn g_red_fn = NULL;
static void *g_red_user = NULL;
void orc_set_reduce(orc_reduce_fn fn, void *user) {
  g_red_fn = fn;
  g_red_user = user;
}

/* ===================================================================== *
 * rsp-scf/cpacoord_ksave.f:139-419  CPA loop around the k loop           *
 * ===================================================================== */
int orc_cpacoord(const orc_problem *p, const double *conc, const zc *tminvl,
                 const zc *tminvr, zc *tminv, const zc *tminva,
                 const zc *tminvb, zc *tauc, zc *taua, zc *taub, int ld,
                 orc_result *res, int nthreads) {
  const int nprc = p->nprc, lkmax = p->lkmax, ngeff = p->ngeff, nk = p->nk;
  const int nl = p->ninprc[0], nr = p->ninprc[nprc + 1], nintfc = p->nintfc;
  int mdim = 0;
  for (int i = 0; i <= nprc + 1; i++)
    if (p->ninprc[i] * lkmax > mdim) mdim = p->ninprc[i] * lkmax;
  const size_t sz = (size_t)ld * ld, msz = (size_t)mdim * mdim;
  const size_t bsz = (size_t)p->map->lmmax * p->map->lmmax;
  if (nthreads < 1) nthreads = 1;
  cg_table_init(); /* before the threaded k loop */

  zc *ttmpl = calloc(sz * nl * ngeff, sizeof(zc)), *ttmpr = calloc(sz * nr * ngeff, sizeof(zc));
  zc *ttmp = calloc(sz * nintfc * ngeff, sizeof(zc));
  int *ieqg = malloc(sizeof(int) * ngeff), *ieqgl = malloc(sizeof(int) * ngeff),
      *ieqgr = malloc(sizeof(int) * ngeff), *igordl = malloc(sizeof(int) * ngeff),
      *igordr = malloc(sizeof(int) * ngeff);
  const int nbk = p->irel == 2 ? 2 * p->nblk : p->nblk; /* blocks per k */
  zc *gcache = calloc(bsz * nbk * (size_t)nk, sizeof(zc));
  zc *ysave = calloc(msz * ngeff * (size_t)nk, sizeof(zc));
  zc *xsave = calloc(msz * ngeff * (size_t)nk, sizeof(zc));
  zc *taupart = calloc(sz * nintfc * (size_t)nthreads, sizeof(zc));
  int *stat_thr = calloc(nthreads, sizeof(int)), *maxit_thr = calloc(nthreads, sizeof(int));
  int64_t *totit_thr = calloc(nthreads, sizeof(int64_t));

  int itcpa = 1, concpa = 1, cpacon = 1, status = 0;
  double cpaerr = 0.0;
  for (;;) {
    orc_sorttmat(lkmax, ld, nintfc, nl, nr, ngeff, p->rg, p->lg, tminvl, tminvr, tminv, ttmpl,
                 ttmpr, ttmp, ieqgl, ieqgr, ieqg, igordl, igordr);
    czero(taupart, sz * nintfc * (size_t)nthreads);
    const int first = (itcpa == 1);
#pragma omp parallel num_threads(nthreads)
    {
      int tid = 0;
#ifdef _OPENMP
      tid = omp_get_thread_num();
#endif
      zc *xx = calloc(msz, sizeof(zc)), *yy = calloc(msz, sizeof(zc));
      zc *tau1 = calloc(sz * nintfc * ngeff, sizeof(zc)), *tau2 = calloc(sz, sizeof(zc));
      zc *mytau = taupart + sz * nintfc * tid;
      /* round-robin k split, as modulo(ik-1,nprocs)==myrank */
      for (int ik = tid; ik < nk; ik += nthreads) {
        zc *blocks = gcache + bsz * nbk * (size_t)ik;
        if (first) {
          orc_gk_from_rtable(p->nblk, p->rstart, p->rvec, p->gR, p->map->lmmax, p->xk[2 * ik],
                             p->xk[2 * ik + 1], blocks);
          if (p->irel == 2) /* hole table: same R vectors, entries after the electron ones */
            orc_gk_from_rtable(p->nblk, p->rstart, p->rvec, p->gR + bsz * p->rstart[p->nblk],
                               p->map->lmmax, p->xk[2 * ik], p->xk[2 * ik + 1], blocks + bsz * p->nblk);
        }
        for (int ig = 0; ig < ngeff; ig++) {
          int ige = ieqg[ig] - 1, igel = ieqgl[ig] - 1, iger = ieqgr[ig] - 1;
          zc *ys = ysave + msz * ((size_t)ik * ngeff + (igordl[igel] - 1));
          zc *xs = xsave + msz * ((size_t)ik * ngeff + (igordr[iger] - 1));
          if (igel == ig && first) {
            int it = 0;
            int st = orc_dugo('L', p->ninprc, nprc, p->map, blocks, 0, 1, ttmpl + sz * (size_t)igel * nl,
                              ld, yy, mdim, lkmax, p->irel, p->fac, p->itermaxl, p->errmax, &it);
            if (st && !stat_thr[tid]) stat_thr[tid] = st;
            if (it > maxit_thr[tid]) maxit_thr[tid] = it;
            totit_thr[tid] += it;
            memcpy(ys, yy, msz * sizeof(zc));
          } else memcpy(yy, ys, msz * sizeof(zc));
          if (iger == ig && first) {
            int it = 0;
            int st = orc_dugo('R', p->ninprc, nprc, p->map, blocks, nprc + 1, 1,
                              ttmpr + sz * (size_t)iger * nr, ld, xx, mdim, lkmax, p->irel, p->fac,
                              p->itermaxr, p->errmax, &it);
            if (st && !stat_thr[tid]) stat_thr[tid] = st;
            if (it > maxit_thr[tid]) maxit_thr[tid] = it;
            totit_thr[tid] += it;
            memcpy(xs, xx, msz * sizeof(zc));
          } else memcpy(xx, xs, msz * sizeof(zc));
          if (ige == ig) {
            double wgeff = p->wk[ik] / ngeff;
            orc_tau2d(p->irel, wgeff, p->bulkgeo, p->ninprc, nprc, p->map, blocks,
                      ttmp + sz * (size_t)ig * nintfc, ld, lkmax, xx, yy, mdim,
                      tau1 + sz * (size_t)ig * nintfc, p->fac);
          }
          for (int li = 0; li < nintfc; li++) {
            memcpy(tau2, tau1 + sz * ((size_t)ige * nintfc + li), sz * sizeof(zc));
            orc_tripmt(p->lg + sz * ig, tau2, p->rg + sz * ig, lkmax, lkmax, ld);
            zc *t = mytau + sz * li;
            for (int i = 0; i < lkmax; i++)
              for (int j = 0; j < lkmax; j++) t[IX(i, j, ld)] += tau2[IX(i, j, ld)];
          }
        }
      }
      free(xx); free(yy); free(tau1); free(tau2);
    }
    /* the allreduce: sum the per-rank partial taus in rank order */
    czero(tauc, sz * nintfc);
    for (int t = 0; t < nthreads; t++)
      for (size_t q = 0; q < sz * nintfc; q++) tauc[q] += taupart[sz * nintfc * t + q];
    for (int t = 0; t < nthreads; t++)
      if (stat_thr[t] && !status) status = stat_thr[t];
    if (g_red_fn) {
      /* the allreduce across ranks of a k-split energy; a failed rank sends its flag */
      const long long nz = (long long)(sz * nintfc);
      double *buf = calloc((size_t)(2 * nz + 1), sizeof(double));
      if (!status) memcpy(buf, tauc, (size_t)nz * sizeof(zc));
      buf[2 * nz] = status ? 1.0 : 0.0;
      int rrc = g_red_fn(g_red_user, buf, 2 * nz + 1);
      if (!status) {
        if (rrc != 0 || buf[2 * nz] != 0.0) status = 3;
        else memcpy(tauc, buf, (size_t)nz * sizeof(zc));
      }
      free(buf);
    }
    if (status) break;
    orc_cpacor(conc, tminv, tminva, tminvb, tauc, taua, taub, lkmax, ld, nintfc, &itcpa,
               p->itcpam, p->cpatol, &cpacon, &concpa, &cpaerr);
    if (!(concpa && cpacon)) break;
  }
  if (res) {
    res->cpa_iterations = itcpa - 1;
    res->cpa_error = cpaerr;
    res->sgf_status = status;
    res->max_dec_iters = 0;
    res->dec_iters_total = 0;
    for (int t = 0; t < nthreads; t++) {
      if (maxit_thr[t] > res->max_dec_iters) res->max_dec_iters = maxit_thr[t];
      res->dec_iters_total += totit_thr[t];
    }
  }
  free(ttmpl); free(ttmpr); free(ttmp); free(ieqg); free(ieqgl); free(ieqgr);
  free(igordl); free(igordr); free(gcache); free(ysave); free(xsave); free(taupart);
  free(stat_thr); free(maxit_thr); free(totit_thr);
  return status;
}

/* ===================================================================== *
 * skkr_dbogo_bsf/rsp-scf/cpacoord_ksave.f:638-660, 760-840  off-diagonal *
 * tau of the interface for cluster embedding: one k loop with the given   *
 * t^-1 (no CPA update), tau2dgod per class, and for each pair (R = n1 a1 *
 * + n2 a2, layers li, lj)                                                 *
 *   tau_ij += w_k/ngeff e^{+i k.g(R+b)} [L_g tau^(g)(k) R_g]_{li,lj}      *
 *   tau_ji += w_k/ngeff e^{-i k.g(R+b)} [L_g tau^(g)(k) R_g]_{lj,li}      *
 * with b = c_li - c_lj and g(v) = a0mat(g) v.  This is the reference's    *
 * e^{-i k.dcpar}, dcpar = -g(R) - g(b) + b, written for structure         *
 * constants whose Bloch phases carry the full in-plane site vectors (the *
 * real-space table form: tau_ab(k) here = e^{i k.(c_b - c_a)} tau_ab(k)  *
 * of the lattice-vector phase convention).  tauc gets the layer-diagonal *
 * k sum as orc_cpacoord forms it.  pairs[4 q] = (n1, n2, li, lj), layers  *
 * 0-based; a0mat[4 g] = (a11, a12, a21, a22); cvec[2 l] in-plane          *
 * positions of the interface layers.                                      *
 * ===================================================================== */
int orc_tauij(const orc_problem *p, const zc *tminvl, const zc *tminvr, const zc *tminv, int npair,
              const int *pairs, const double *a1, const double *a2, const double *cvec,
              const double *a0mat, zc *tau_ij, zc *tau_ji, zc *tauc, int ld, int nthreads) {
  const int nprc = p->nprc, lkmax = p->lkmax, ngeff = p->ngeff, nk = p->nk;
  const int nl = p->ninprc[0], nr = p->ninprc[nprc + 1], nintfc = p->nintfc;
  int mdim = 0;
  for (int i = 0; i <= nprc + 1; i++)
    if (p->ninprc[i] * lkmax > mdim) mdim = p->ninprc[i] * lkmax;
  const size_t sz = (size_t)ld * ld, msz = (size_t)mdim * mdim;
  const size_t bsz = (size_t)p->map->lmmax * p->map->lmmax;
  const size_t nfull = (size_t)nintfc * nintfc;
  if (nthreads < 1) nthreads = 1;
  cg_table_init();
  zc *ttmpl = calloc(sz * nl * ngeff, sizeof(zc)), *ttmpr = calloc(sz * nr * ngeff, sizeof(zc));
  zc *ttmp = calloc(sz * nintfc * ngeff, sizeof(zc));
  int *ieqg = malloc(sizeof(int) * ngeff), *ieqgl = malloc(sizeof(int) * ngeff),
      *ieqgr = malloc(sizeof(int) * ngeff), *igordl = malloc(sizeof(int) * ngeff),
      *igordr = malloc(sizeof(int) * ngeff);
  orc_sorttmat(lkmax, ld, nintfc, nl, nr, ngeff, p->rg, p->lg, tminvl, tminvr, tminv, ttmpl, ttmpr,
               ttmp, ieqgl, ieqgr, ieqg, igordl, igordr);
  const int nbk = p->irel == 2 ? 2 * p->nblk : p->nblk;
  zc *part_ij = calloc(sz * npair * (size_t)nthreads, sizeof(zc));
  zc *part_ji = calloc(sz * npair * (size_t)nthreads, sizeof(zc));
  zc *part_c = calloc(sz * nintfc * (size_t)nthreads, sizeof(zc));
  int *stat_thr = calloc(nthreads, sizeof(int));
#pragma omp parallel num_threads(nthreads)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    zc *blocks = calloc(bsz * nbk, sizeof(zc));
    zc *xx = calloc(msz * ngeff, sizeof(zc)), *yy = calloc(msz * ngeff, sizeof(zc));
    zc *tau1 = calloc(sz * nfull * ngeff, sizeof(zc)), *t2 = calloc(sz, sizeof(zc));
    zc *pij = part_ij + sz * npair * tid, *pji = part_ji + sz * npair * tid, *pc = part_c + sz * nintfc * tid;
    for (int ik = tid; ik < nk; ik += nthreads) {
      const double kx = p->xk[2 * ik], ky = p->xk[2 * ik + 1];
      orc_gk_from_rtable(p->nblk, p->rstart, p->rvec, p->gR, p->map->lmmax, kx, ky, blocks);
      if (p->irel == 2)
        orc_gk_from_rtable(p->nblk, p->rstart, p->rvec, p->gR + bsz * p->rstart[p->nblk], p->map->lmmax,
                           kx, ky, blocks + bsz * p->nblk);
      for (int ig = 0; ig < ngeff; ig++) {
        int ige = ieqg[ig] - 1, igel = ieqgl[ig] - 1, iger = ieqgr[ig] - 1;
        int it = 0, st;
        if (igel == ig) {
          st = orc_dugo('L', p->ninprc, nprc, p->map, blocks, 0, 1, ttmpl + sz * (size_t)igel * nl, ld,
                        yy + msz * igel, mdim, lkmax, p->irel, p->fac, p->itermaxl, p->errmax, &it);
          if (st && !stat_thr[tid]) stat_thr[tid] = st;
        }
        if (iger == ig) {
          st = orc_dugo('R', p->ninprc, nprc, p->map, blocks, nprc + 1, 1, ttmpr + sz * (size_t)iger * nr,
                        ld, xx + msz * iger, mdim, lkmax, p->irel, p->fac, p->itermaxr, p->errmax, &it);
          if (st && !stat_thr[tid]) stat_thr[tid] = st;
        }
        if (ige == ig)
          orc_tau2dgod(p->irel, p->wk[ik] / ngeff, p->bulkgeo, p->ninprc, nprc, p->map, blocks,
                       ttmp + sz * (size_t)ig * nintfc, ld, lkmax, xx + msz * iger, yy + msz * igel, mdim,
                       tau1 + sz * nfull * ig, nintfc, p->fac);
        const zc *tg = tau1 + sz * nfull * ige;
        for (int li = 0; li < nintfc; li++) {
          memcpy(t2, tg + sz * ((size_t)li * nintfc + li), sz * sizeof(zc));
          orc_tripmt(p->lg + sz * ig, t2, p->rg + sz * ig, lkmax, lkmax, ld);
          zc *t = pc + sz * li;
          for (int i = 0; i < lkmax; i++)
            for (int j = 0; j < lkmax; j++) t[IX(i, j, ld)] += t2[IX(i, j, ld)];
        }
        const double *am = a0mat + 4 * ig;
        for (int q = 0; q < npair; q++) {
          const int n1 = pairs[4 * q], n2 = pairs[4 * q + 1], li = pairs[4 * q + 2], lj = pairs[4 * q + 3];
          const double vx = n1 * a1[0] + n2 * a2[0] + cvec[2 * li] - cvec[2 * lj];
          const double vy = n1 * a1[1] + n2 * a2[1] + cvec[2 * li + 1] - cvec[2 * lj + 1];
          const double gx = am[0] * vx + am[1] * vy, gy = am[2] * vx + am[3] * vy;
          const double ph = kx * gx + ky * gy;
          const zc f = cos(ph) + I * sin(ph);
          memcpy(t2, tg + sz * ((size_t)li * nintfc + lj), sz * sizeof(zc));
          orc_tripmt(p->lg + sz * ig, t2, p->rg + sz * ig, lkmax, lkmax, ld);
          zc *t = pij + sz * q;
          for (int i = 0; i < lkmax; i++)
            for (int j = 0; j < lkmax; j++) t[IX(i, j, ld)] += f * t2[IX(i, j, ld)];
          memcpy(t2, tg + sz * ((size_t)lj * nintfc + li), sz * sizeof(zc));
          orc_tripmt(p->lg + sz * ig, t2, p->rg + sz * ig, lkmax, lkmax, ld);
          t = pji + sz * q;
          for (int i = 0; i < lkmax; i++)
            for (int j = 0; j < lkmax; j++) t[IX(i, j, ld)] += conj(f) * t2[IX(i, j, ld)];
        }
      }
    }
    free(blocks); free(xx); free(yy); free(tau1); free(t2);
  }
  czero(tau_ij, sz * npair);
  czero(tau_ji, sz * npair);
  czero(tauc, sz * nintfc);
  for (int t = 0; t < nthreads; t++) {
    for (size_t q = 0; q < sz * npair; q++) {
      tau_ij[q] += part_ij[sz * npair * t + q];
      tau_ji[q] += part_ji[sz * npair * t + q];
    }
    for (size_t q = 0; q < sz * nintfc; q++) tauc[q] += part_c[sz * nintfc * t + q];
  }
  int status = 0;
  for (int t = 0; t < nthreads; t++)
    if (stat_thr[t] && !status) status = stat_thr[t];
  free(ttmpl); free(ttmpr); free(ttmp); free(ieqg); free(ieqgl); free(ieqgr); free(igordl); free(igordr);
  free(part_ij); free(part_ji); free(part_c); free(stat_thr);
  return status;
}

/* ===================================================================== *
 * generators                                                            *
 * ===================================================================== */
/* main/legpol.f */
static void legpol(double x, int l, double *pl, double *plm1, double *dpl) {
  double pnm1 = 1.0, pn = x;
  for (int n = 1; n <= l - 1; n++) {
    double pnp1 = ((n + n + 1) * x * pn - n * pnm1) / (n + 1.0);
    pnm1 = pn;
    pn = pnp1;
  }
  *pl = pn;
  *plm1 = pnm1;
  *dpl = l * (x * (*pl) - (*plm1)) / (x * x - 1.0);
}

/* main/legzero.f: Gauss-Legendre nodes/weights by Newton from A&S starts */
void orc_legzero(int ng, double *xx, double *wx) {
  const double pi = 3.1415926535897932, small = 1.0e-14;
  int n = ng / 2;
  for (int i = 1; i <= n; i++) {
    double phi = (4 * i - 1) * pi / (4 * ng + 2.0);
    double x = cos(phi + 1.0 / (8.0 * ng * ng * tan(phi)));
    double pl, plm1, dpl, dx;
    int ind = 0;
    do {
      legpol(x, ng, &pl, &plm1, &dpl);
      ind++;
      if (ind > 100) break;
      dx = pl / dpl;
      x = x - dx;
    } while (fabs(dx) > small);
    double w = 2.0 * (1.0 - x * x) / (ng * ng * plm1 * plm1);
    xx[ng - i] = x;
    xx[i - 1] = -x;
    wx[ng - i] = w;
    wx[i - 1] = w;
  }
  if (2 * n != ng) {
    double pl, plm1, dpl;
    legpol(0.0, ng, &pl, &plm1, &dpl);
    xx[n] = 0.0;
    wx[n] = 2.0 / (ng * ng * plm1 * plm1);
  }
}

/* main/zmesh.f:55-83  imesh=1: semicircle, log-Gauss-Legendre in phi */
void orc_zmesh_semicircle(int nepanel, double ebottom, double etop,
                          double epsilon, zc *z, zc *ww) {
  const double eps0 = 1.0e-5, pi = 4.0 * atan(1.0);
  double x[512], w[512], eps = 0.0, y1 = 0.0, y2 = 0.0;
  if (epsilon > eps0) eps = 1.0 / epsilon;
  double r = (etop - ebottom) / 2.0, phi1 = pi, phi2 = 0.0;
  if (epsilon > eps0) {
    y1 = -log(1.0 + phi1 / eps);
    y2 = -log(1.0 + phi2 / eps);
  }
  zc z0 = ebottom + r;
  orc_legzero(nepanel, x, w);
  for (int ii = 0; ii < nepanel; ii++) {
    if (epsilon > eps0) {
      double y = 0.5 * (y2 - y1) * x[ii] + 0.5 * (y2 + y1);
      double phi = eps * (exp(-y) - 1.0);
      z[ii] = r * cexp(I * phi) + z0;
      ww[ii] = -0.5 * (y2 - y1) * eps * exp(-y) * I * (z[ii] - z0) * w[ii];
    } else {
      double phi = 0.5 * (phi2 - phi1) * x[ii] + 0.5 * (phi2 + phi1);
      z[ii] = r * cexp(I * phi) + z0;
      ww[ii] = 0.5 * (phi2 - phi1) * I * (z[ii] - z0) * w[ii];
    }
  }
}

/* main/speck2.f:2-257  minimum-IBZ point sets; k in units of 1 (then * pi/a) */
static void vecrot(double *v, double phi) {
  double c = cos(phi), s = sin(phi), x = v[0], y = v[1];
  v[0] = c * x - s * y;
  v[1] = s * x + c * y;
}

int orc_speck2(int nset, double *xk, double *yk, double *wk, int ilat,
               double alat, double beta, double delta, int cap) {
  const double pi = 3.1415926535897932;
  int n = nset, nk = 0;
  if (ilat <= 0 || ilat > 5) return -1;
#define PUSH(X, Y, W) do { if (nk >= cap) return -2; xk[nk] = (X); yk[nk] = (Y); wk[nk] = (W); nk++; } while (0)
  if (ilat == 1) {
    double del = delta < 0 ? -delta : delta;
    int m = (int)(n / sqrt(beta * beta + del * del)) + 1;
    double dk1x = 2.0 / n, dk1y = -2.0 * del / (n * beta), dk2x = 0.0, dk2y = 2.0 / (m * beta);
    double bod = beta / del, bo1md = beta / (1.0 - del), tiny = 1.0e-6 * dk2y;
    double xmax = 1.0 + (1.0 / bod + 1.0 / bo1md) / (bod + bo1md);
    for (int i = 1; i <= n; i++)
      for (int j = -m + 1; j <= m; j++) {
        double x = (i - 0.5) * dk1x + (j - 0.5) * dk2x, y = (i - 0.5) * dk1y + (j - 0.5) * dk2y;
        if (x > xmax) continue;
        double ymax1 = 1.0 / beta, ymax2 = -bo1md * (x - 1.0) + 1.0 / bo1md;
        double ymax = ymax1 < ymax2 ? ymax1 : ymax2;
        double ymin1 = -1.0 / beta, ymin2 = bod * (x - 1.0) - 1.0 / bod;
        double ymin = ymin1 > ymin2 ? ymin1 : ymin2;
        double dymax1 = ymax1 - y, dymax2 = ymax2 - y, dymin1 = y - ymin1, dymin2 = y - ymin2;
        if (!(y <= ymax && y >= ymin)) continue;
        double w;
        if (dymax1 < tiny) w = dymax2 < tiny ? 0.25 : 0.5;
        else if (dymax2 < tiny) w = dymin1 < tiny ? 0.25 : 0.5;
        else if (dymin1 < tiny) w = dymin2 < tiny ? 0.25 : 0.5;
        else if (dymin2 < tiny) w = 0.5;
        else w = 1.0;
        PUSH(x, y, w);
      }
    if (delta < 0)
      for (int ik = 0; ik < nk; ik++) yk[ik] = -yk[ik];
  }
  if (ilat == 2) {
    double dkx = 2.0 / (double)(n + 1), dky = 2.0 / (double)(n + 2) / beta, tiny = dkx * 1.0e-6;
    double x = dkx / 2.0;
    while (x <= 2.0) {
      double difx = fabs(x - 2.0), y = dky / 2.0, ymax = -x * beta + (beta + 1.0 / beta);
      while (y <= ymax) {
        double dify = fabs(y - ymax), w;
        if (difx < tiny) w = dify < tiny ? 0.25 : 0.5;
        else w = dify < tiny ? 0.5 : 1.0;
        PUSH(x, y, w);
        y = y + dky;
      }
      x = x + dkx;
    }
  }
  if (ilat == 3) {
    double dkx = 1.0 / (double)n, dky = (1.0 / beta) / (double)n, x = dkx / 2.0;
    while (x <= 1.0) {
      double y = dky / 2.0;
      while (y <= 1.0 / beta) {
        PUSH(x, y, 1.0);
        y = y + dky;
      }
      x = x + dkx;
    }
  }
  if (ilat == 4) {
    for (int i = 1; i <= n; i++) {
      double x = 0.5 * (double)(2 * i - 1) / n;
      for (int j = 1; j <= i; j++) {
        double y = 0.5 * (double)(2 * j - 1) / n;
        PUSH(x, y, i == j ? 0.5 : 1.0);
      }
    }
  }
  if (ilat == 5) {
    double dxk = 2.0 / (double)n, dyk = dxk / sqrt(3.0);
    for (int nu = 1; nu <= 2; nu++) {
      double anu3 = nu / 3.0;
      for (int i = 1; i <= n; i++)
        for (int j = i; j <= n; j++) {
          int iy = i + 2 * j + nu - 3;
          if (iy > n) continue;
          double ajm = 1.0;
          if (i == j || iy == n) ajm = 2.0;
          if (i == j && iy == n) ajm = 6.0;
          PUSH((i - 1 + anu3) * dxk, iy * dyk, 1.0 / ajm);
        }
    }
    for (int ik = 0; ik < nk; ik++) {
      double v[2] = {xk[ik], yk[ik]};
      vecrot(v, -pi / 3.0);
      xk[ik] = v[0];
      yk[ik] = v[1];
    }
  }
#undef PUSH
  double cst = pi / alat;
  for (int ik = 0; ik < nk; ik++) { xk[ik] *= cst; yk[ik] *= cst; }
  return nk;
}

/* main/kmesh2d.f:5-254 for the point groups whose IBZ equals the minimum
 * wedge (ibz.f ngeff=1: C4v on the square lattice, C2v on rectangular
 * lattices), intbz<=1, kunning=0, no extra rotation (phik=0).  Weights are
 * reassigned from the BZ-boundary test and the IBZ-boundary factors, then
 * normalised to 1 (kmesh2d.f:139-251). */
int orc_kmesh2d_ibz(int iset, int i2dlat, const char *idgroup, double a2d,
                    double beta, double delta, double *xk, double *yk,
                    double *wk, int cap) {
  const double tol = 1.0e-10;
  int nk = orc_speck2(iset, xk, yk, wk, i2dlat, a2d, beta, delta, cap);
  if (nk < 0) return nk;
  /* primkr2d.f: direct lattice, then reciprocal vectors */
  double ax[2] = {a2d, 0.0}, ay[2];
  if (i2dlat == 2) { ay[0] = 0.5 * a2d; ay[1] = 0.5 * a2d * beta; }
  else if (i2dlat == 3) { ay[0] = 0.0; ay[1] = a2d * beta; }
  else if (i2dlat == 4) { ay[0] = 0.0; ay[1] = a2d; }
  else if (i2dlat == 1) { ay[0] = a2d * delta; ay[1] = a2d * beta; }
  else { ay[0] = 0.5 * a2d; ay[1] = 0.5 * sqrt(3.0) * a2d; }
  double det = ax[0] * ay[1] - ax[1] * ay[0], tpi = 2.0 * 3.1415926535897932;
  double bx[2] = {tpi * ay[1] / det, -tpi * ay[0] / det};
  double by[2] = {-tpi * ax[1] / det, tpi * ax[0] / det};
  for (int ik = 0; ik < nk; ik++) {
    int ibound = 0;
    for (int i = -2; i <= 2; i++)
      for (int j = -2; j <= 2; j++) {
        if (i == 0 && j == 0) continue;
        double gx = i * bx[0] + j * by[0], gy = i * bx[1] + j * by[1];
        double g2o2 = 0.5 * (gx * gx + gy * gy), gk = gx * xk[ik] + gy * yk[ik];
        if (fabs(gk - g2o2) < tol) ibound++;
      }
    if (ibound == 0) wk[ik] = 1.0;
    if (ibound == 1) wk[ik] = 0.5;
    if (ibound == 2) wk[ik] = (i2dlat == 3 || i2dlat == 4) ? 0.25 : 1.0 / 3.0;
  }
  for (int ik = 0; ik < nk; ik++) {
    if (strcmp(idgroup, "C4v") == 0) {
      if (fabs(xk[ik]) < tol) wk[ik] *= fabs(yk[ik]) < tol ? 0.125 : 0.5;
      else if (fabs(xk[ik] - yk[ik]) < tol) wk[ik] *= 0.5;
    } else if (strcmp(idgroup, "C4") == 0 || strcmp(idgroup, "C2v") == 0) {
      if (fabs(xk[ik]) < tol) wk[ik] *= fabs(yk[ik]) < tol ? 0.25 : 0.5;
      else if (fabs(yk[ik]) < tol) wk[ik] *= 0.5;
    }
  }
  double wsum = 0.0;
  for (int ik = 0; ik < nk; ik++) wsum += wk[ik];
  for (int ik = 0; ik < nk; ik++) wk[ik] /= wsum;
  return nk;
}

/* main/csbf.f: spherical Bessel / Neumann / Hankel of complex argument */
void orc_csbf(int n, zc p, double r, zc *fb, zc *fn, zc *fh) {
  zc x1 = r * p, x2 = x1 * x1;
  fb[0] = csin(x1) / x1;
  fb[1] = csin(x1) / x2 - ccos(x1) / x1;
  fn[0] = -ccos(x1) / x1;
  fn[1] = -ccos(x1) / x2 - csin(x1) / x1;
  fh[0] = fb[0] + I * fn[0];
  fh[1] = fb[1] + I * fn[1];
  for (int l = 2; l <= n; l++) fb[l] = (2 * l - 1) * fb[l - 1] / x1 - fb[l - 2];
  for (int l = 2; l <= n; l++) fn[l] = (2 * l - 1) * fn[l - 1] / x1 - fn[l - 2];
  for (int l = 2; l <= n; l++) fh[l] = fb[l] + I * fn[l];
}

/* main/alphamat.f:2-96 (iscreen<=1): alpha_l = t-matrix of a square barrier
 * of height vscreen and radius rs at energy ce */
void orc_alpha_sqwell(zc ce, double vscreen, double rs, int lmax, zc *alpha) {
  zc fmb[16], fmn[16], fmh[16], fodb[16], fodn[16], fodh[16];
  zc cs = ce - vscreen, csk = csqrt(cs), ck = csqrt(ce);
  if (cimag(csk) < 0) csk = -csk;
  if (cimag(ck) < 0) ck = -ck;
  orc_csbf(lmax + 1, ck, rs, fmb, fmn, fmh);
  orc_csbf(lmax + 1, csk, rs, fodb, fodn, fodh);
  for (int l = 0; l <= lmax; l++) {
    zc tand = (ck * fmb[l + 1] * fodb[l] - csk * fmb[l] * fodb[l + 1]) /
              (ck * fmn[l + 1] * fodb[l] - csk * fmn[l] * fodb[l + 1]);
    zc react = -tand / ck;
    alpha[l] = react / (1.0 + I * ck * react);
  }
}

/* ---------------------------------------------------------------------------
 * Layer DOS from the physical site-diagonal tau (lambda = 0 moment).
 * nrsp-scf/moment.f:47-110: gf = fac*(Rreg o coeff) tau - fac*(Rirr o coeff),
 * coeff = sqrt(4 pi) Gaunt(l,0,l') = identity (main/gafill.f:14-35), so
 * gf_ii = fac (F_i tau_ii - G_i); the real-harmonic transform of moment.f:96-98
 * keeps the sum over m.  locquant.f:115-122 sums zqmom over m into zdos(l).
 * rsp-scf/moment.f keeps the (kappa,mu) diagonal (rgacoeff = identity).
 */
void orc_layer_dos(int mode, int lmax, int nlay, const zc *tau, int ld, const zc *F,
                   const zc *G, int para, zc *zmom, zc *zdos_l) {
  const int lmmax = (lmax + 1) * (lmax + 1);
  const int nd = mode ? 2 * lmmax : lmmax;
  double fac = -1.0 / (4.0 * atan(1.0));
  if (para && !mode) fac *= 2.0;
  int *lof = malloc(sizeof(int) * nd);
  if (mode) {
    /* (kappa,mu) order of main/clebsch.f: kappa = -1, 1, -2, 2, -3, ... with
       2|kappa| components each; l = kappa for kappa > 0, -kappa-1 otherwise */
    int k = 0;
    for (int a = 1; k < nd; a++) {
      for (int s = 0; s < 2 && k < nd; s++) {
        int kap = s == 0 ? -a : a;
        if (kap == 0) continue;
        int l = kap > 0 ? kap : -kap - 1;
        int cnt = 2 * (kap > 0 ? kap : -kap);
        for (int c = 0; c < cnt && k < nd; c++) lof[k++] = l;
      }
    }
  } else {
    for (int l = 0, k = 0; l <= lmax; l++)
      for (int m = -l; m <= l; m++) lof[k++] = l;
  }
  for (int li = 0; li < nlay; li++) {
    const zc *t = tau + (size_t)li * ld * ld;
    for (int l = 0; l <= lmax; l++) zdos_l[(size_t)li * (lmax + 1) + l] = 0;
    for (int i = 0; i < nd; i++) {
      size_t q = (size_t)li * nd + i;
      zc z = fac * (F[q] * t[IX(i, i, ld)] - G[q]);
      zmom[q] = z;
      zdos_l[(size_t)li * (lmax + 1) + lof[i]] += z;
    }
  }
  free(lof);
}
