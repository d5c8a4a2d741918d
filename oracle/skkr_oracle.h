/*
 * skkr_oracle.h -- CPU FP64 restatement of the screened-KKR 2D Brillouin-zone
 * integration path of laszloffy/skkr_budapest (skkr_kpar_v6).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * __graft_entry__.smoke() and the cpu_baseline / reference arm of bench.py
 * may call it, nothing in the product path may.
 *
 * Every routine follows one reference routine line by line (cited per
 * function in skkr_oracle.c), keeping the reference's column-major layout,
 * loop order and Gauss-Jordan column pivoting.  Arrays are complex*16
 * interleaved (double _Complex), column-major, with explicit leading
 * dimensions; all indices below are 0-based unless stated.
 *
 * Parity status: the reference ships no golden vectors for tau, DOS or the
 * coherent t-matrix, and no Fortran compiler exists on either machine, so at
 * that level parity is unpinned by the reference itself.  The generators
 * (zmesh energies, k-mesh sizes) are pinned against the reference's own
 * sample run log (tests/golden).
 */
#ifndef SKKR_ORACLE_H
#define SKKR_ORACLE_H
#include <complex.h>
#include <stdint.h>

typedef double _Complex zc;

#ifdef __cplusplus
extern "C" {
#endif

/* ---- dense kernels: main/gjinv.f, main/matops.f ---------------------- */
void orc_gjinv(zc *a, int n, int nmax, zc *detl);
void orc_doubmt2(const zc *a, const zc *b, zc *c, int n1, int n2, int n3, int ld);
void orc_tripmt(const zc *u, zc *b, const zc *ust, int ndi1, int ndi2, int ld);
void orc_tripmt2(const zc *u, const zc *b, const zc *v, zc *b1, int ndi1,
                 int ndi2, int ndi3, int ndi4, int ld, int ldb1);
int orc_compmat(const zc *x, const zc *y, int n, int ld, double tol);

/* ---- lm -> (kappa,mu): main/clebsch.f, main/relmtrx.f ---------------- */
void orc_clebsch(double u1[72], double u2[72], int ind1[72], int ind2[72]);
void orc_relmtrx(const zc *a, int lda, zc *b, int ldb, zc fac, int lmax);

/* ---- structure-constant block table (see skkr_oracle.c, orc_g2d_*) ---
 * g2d blocks are lmmax x lmmax (lm basis).  blkmap[(slot*mi + (i-1))*nj + (j+jmax)]
 * gives the block index (>=0) coupling layer i (1-based) of a principal layer
 * stored in `slot` to layer i+j, or -1 for a zero block.  mi = max layers per
 * principal layer, nj = 2*jmax+1. */
typedef struct {
  int lmax, lmmax;   /* lm basis size */
  int nslot;         /* principal-layer slots (0 = left bulk, 1..: interface / bulk) */
  int mi;            /* max layers per principal layer */
  int jmax;          /* max |layer offset| kept */
  const int *blkmap; /* [nslot][mi][2*jmax+1] */
  /* BdG (skkr_dbogo_bsf): the hole block of block b sits at b + nblk and is
   * mapped to (kappa,mu) with fach (main/g2d_pack.f + main/relmtrx.f) */
  int bdg, nblk;
  zc fach;
} orc_g2dmap;

/* ---- per-principal-layer packing: main/packer.f ------------------------ */
void orc_packer(int ni, int nim, int nip, const orc_g2dmap *map, int slot,
                const zc *blocks, zc *m00, zc *m10, zc *m01, int lkmax,
                int mdim, int irel, zc fac);

/* ---- decimation: main/surfgf.f, main/dugo.f -------------------------- */
/* status: 0 ok, 1 itermax exceeded, 2 diverged ("enormous error") */
int orc_surfgfd(const zc *ml, const zc *m0, const zc *mr, zc *x, int kdim,
                int mdim, int itermax, double errmax, int *iters);
int orc_dugo(int side /*'L' or 'R'*/, const int *ninprc, int nprc,
             const orc_g2dmap *map, const zc *blocks, int slot_bulk,
             int slot_int, const zc *tminvb, int lkmaxp, zc *xy, int mdimp,
             int lkmax, int irel, zc fac, int itermax, double errmax,
             int *iters);

/* ---- block-tridiagonal tau: main/tau2d.f ------------------------------ */
void orc_tau2d(int irel, double wgeff, int bulkgeo, const int *ninprc,
               int nprc, const orc_g2dmap *map, const zc *blocks,
               const zc *tminv, int lkmaxp, int lkmax, const zc *x,
               const zc *y, int mdimp, zc *tau, zc fac);

/* ---- CPA: rsp-scf/fullcpa.f; screened->physical: rsp-scf/phystau.f ----- */
void orc_tata(double conc, int n, int ld, zc *mc, const zc *ma, const zc *mb);
void orc_cpasol(double conc, zc *mc, const zc *ma, const zc *mb,
                const zc *tauc, zc *taua, zc *taub, int n, int ld,
                double *e1, double *e2, double *e3);
void orc_cpacor(const double *conc, zc *mc, const zc *ma, const zc *mb,
                const zc *tauc, zc *taua, zc *taub, int n, int ld, int nintfc,
                int *itcpa, int itcpam, double cpatol, int *cpacon,
                int *concpa, double *error);
void orc_phystau(zc *tau, const zc *tinv1, const zc *tinv2, const zc *alpha,
                 int lmax, int irel, int ld, int idiag);
/* pair blocks (cluster/rsp-lay/phystau2.f, skkr_dbogo_bsf/clu/phystau2.f):
 * alpha1 / tinv1 of the row layer, alpha2 / tinv2 of the column layer */
void orc_phystau2(zc *tau, const zc *tinv1, const zc *alpha1, const zc *tinv2,
                  const zc *alpha2, int lmax, int irel, int ld, int idiag);

/* ---- layer DOS: nrsp-scf/moment.f:47-110 + locquant.f:86-126 (lm),
 *      rsp-scf/moment.f:60-140 + locquant.f:197-232 (kappa,mu) ----------
 * zmom[li][i] = fac (F[li][i] tau_ii - G[li][i]), fac = -1/pi (x2 if para and
 * mode 0); zdos_l[li][l] = sum of zmom over the basis indices of orbital l.
 * The DOS is the imaginary part.  tau: physical tau [nlay][ld][ld]. */
void orc_layer_dos(int mode, int lmax, int nlay, const zc *tau, int ld, const zc *F,
                   const zc *G, int para, zc *zmom, zc *zdos_l);

/* ---- sorttmat: rsp-scf/sorttmat.f ------------------------------------- */
void orc_sorttmat(int lkmax, int ld, int nintfc, int nl, int nr, int ngeff,
                  const zc *rg /*R_g [ngeff][ld][ld]*/,
                  const zc *lg /*L_g [ngeff][ld][ld]*/, const zc *tminvl,
                  const zc *tminvr, const zc *tminv, zc *ttmpl, zc *ttmpr,
                  zc *ttmp, int *ieqgl, int *ieqgr, int *ieqg, int *igordl,
                  int *igordr);

/* ---- G_scr(k) = sum_R exp(i k.R) G_scr(R): the real-space table form ---- */
void orc_gk_from_rtable(int nblk, const int *rstart /*[nblk+1]*/,
                        const double *rvec /*[nR][2]*/,
                        const zc *gR /*[nR][lmmax][lmmax] col-major blocks*/,
                        int lmmax, double kx, double ky, zc *blocks);

/* ---- the CPA + k loop: rsp-scf/cpacoord_ksave.f:139-489 --------------- */
typedef struct {
  int irel;            /* 0 non-relativistic (lm), 1 relativistic (kappa,mu), 2 BdG (e + h kappa,mu) */
  int lmax, lkmax;     /* lkmax = (lmax+1)^2, 2(lmax+1)^2 or 4(lmax+1)^2 */
  int nprc;            /* interface principal layers */
  const int *ninprc;   /* [nprc+2]: layers per PL, 0 = left bulk, nprc+1 = right */
  int bulkgeo;         /* 1: every interface PL uses slot 1 */
  int nintfc;          /* interface layers = sum ninprc[1..nprc] */
  const orc_g2dmap *map;
  int nk;
  const double *xk;    /* [nk][2] */
  const double *wk;    /* [nk] */
  int ngeff;
  const zc *lg, *rg;   /* k-sum: tau += L_g tau R_g ; t rotation: R_g t L_g */
  int itermaxl, itermaxr;
  double errmax;
  int itcpam;
  double cpatol;
  zc fac;              /* relmtrx factor psq/E (1 for non-rel) */
  /* G_scr(R) table per energy */
  int nblk;
  const int *rstart;
  const double *rvec;
  const zc *gR;        /* [nR] (BdG: [2][nR], electron then hole table) */
} orc_problem;

typedef struct {
  int cpa_iterations;
  double cpa_error;
  int sgf_status;      /* first non-zero surfgfd status */
  int max_dec_iters;
  int64_t dec_iters_total;
} orc_result;

/* tminv: inout [nintfc][ld][ld] coherent screened t^-1; tminva/b [nintfc];
 * tminvl [ninprc0], tminvr [ninprc(nprc+1)]; taua/taub out (screened, k-summed,
 * after the CPA; phystau NOT applied); tauc out (last k-summed coherent tau). */
/* Host reduction for a k-split energy (cpacoord_ksave.f:189 k split with the
 * mpi_allreduce of :406): when set, orc_cpacoord calls fn(user, buf, n) once
 * per CPA iteration with buf = [tauc (2*nintfc*ld*ld doubles), failed flag],
 * and fn must replace buf by its sum over the ranks.  A rank whose
 * decimation failed sends the flag and returns its own status; the others
 * return status 3.  fn = NULL switches it off (process wide). */
typedef int (*orc_reduce_fn)(void *user, double *buf, long long n);
void orc_set_reduce(orc_reduce_fn fn, void *user);

int orc_cpacoord(const orc_problem *p, const double *conc, const zc *tminvl,
                 const zc *tminvr, zc *tminv, const zc *tminva,
                 const zc *tminvb, zc *tauc, zc *taua, zc *taub, int ld,
                 orc_result *res, int nthreads);

/* full Godfrin tau of one k (skkr_dbogo_bsf/clu/tau2d_god.f): tauij[(a*nintfc+b)]
 * = wgeff tau_{a,b}, every interface layer pair; args as orc_tau2d */
void orc_tau2dgod(int irel, double wgeff, int bulkgeo, const int *ninprc,
                  int nprc, const orc_g2dmap *map, const zc *blocks,
                  const zc *tminv, int lkmaxp, int lkmax, const zc *x,
                  const zc *y, int mdimp, zc *tauij, int nintfc, zc fac);
/* off-diagonal k sums for pairs (n1, n2, li, lj) with phases and group
 * rotations (skkr_dbogo_bsf/rsp-scf/cpacoord_ksave.f:760-840), one k loop
 * with fixed t^-1; see skkr_oracle.c */
int orc_tauij(const orc_problem *p, const zc *tminvl, const zc *tminvr, const zc *tminv, int npair,
              const int *pairs, const double *a1, const double *a2, const double *cvec,
              const double *a0mat, zc *tau_ij, zc *tau_ji, zc *tauc, int ld, int nthreads);

/* ---- generators: main/zmesh.f, main/legzero.f, main/speck2.f, main/kmesh2d.f,
 *      main/alphamat.f, main/csbf.f ----------------------------------- */
void orc_legzero(int ng, double *xx, double *wx);
void orc_zmesh_semicircle(int nepanel, double ebottom, double etop,
                          double epsilon, zc *z, zc *ww);
int orc_speck2(int nset, double *xk, double *yk, double *wk, int ilat,
               double alat, double beta, double delta, int cap);
int orc_kmesh2d_ibz(int iset, int i2dlat, const char *idgroup, double a2d,
                    double beta, double delta, double *xk, double *yk,
                    double *wk, int cap);
void orc_csbf(int n, zc p, double r, zc *fb, zc *fn, zc *fh);
void orc_alpha_sqwell(zc ce, double vscreen, double rs, int lmax, zc *alpha);

#ifdef __cplusplus
}
#endif
#endif
