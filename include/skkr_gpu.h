/*
 * skkr_gpu.h -- C ABI of the GB300 2D-Brillouin-zone tau / CPA library.
 *
 * Drop-in for the per-energy k integration and CPA loop of the screened-KKR
 * layer code laszloffy/skkr_budapest:
 *
 *   subroutine cpacoord(itscf,ie,ce,lmax,nintfc,eta,rightm,bulk,bulkgeo,wrel,
 *                       kset,xk,wk,nk,intbz,iek,conc,itcpam,cpatol,cpatest,
 *                       dmata,dmatb,dmatpa,dmatpb,tminvl,tminvr,tminv,tminva,
 *                       tminvb,taua,taub,gtaua,gtaub)
 *     skkr_kpar_v6/rsp-scf/cpacoord_ksave.f:3-9     (relativistic, kappa-mu)
 *     skkr_kpar_v6/nrsp-scf/cpacoord.f:2-6          (non-relativistic, lm)
 *
 * Plain pointers and sizes only.  Matrices are complex*16 (interleaved
 * re/im doubles, C `double _Complex`), column-major, leading dimension `ld`
 * (the Fortran kmymaxp / lmmaxp may be passed as-is).  All host buffers are
 * owned by the caller and read/written synchronously; no pointer is kept
 * after a call returns.  The library never aborts the process: every entry
 * point returns SKKR_OK or a negative error code and, where it takes one,
 * fills an skkr_status.
 *
 * Everything runs on the CUDA device current when skkr_gpu_create is called;
 * there is no CPU fallback.
 */
#ifndef SKKR_GPU_H
#define SKKR_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define SKKR_MAX_PRC 16   /* interface principal layers (param.h mprc) */
#define SKKR_MAX_G 12     /* point-group operations (param.h melem)     */

/* NONREL: lm basis (nrsp-scf); REL: (kappa,mu) (rsp-scf); BDG: electron
 * (kappa,mu) block then hole block, 4 (lmax+1)^2 per site (skkr_dbogo_bsf) */
enum skkr_mode { SKKR_NONREL = 0, SKKR_REL = 1, SKKR_BDG = 2 };
enum skkr_precision { SKKR_FP64 = 0, SKKR_MIXED = 1 };

enum skkr_error {
  SKKR_OK = 0,
  SKKR_ERR_ARG = -1,          /* bad size / pointer / layout              */
  SKKR_ERR_CUDA = -2,         /* CUDA runtime error (message via skkr_gpu_last_error) */
  SKKR_ERR_SGF_ITERMAX = -3,  /* decimation hit itermax (main/surfgf.f:98-101 `stop`) */
  SKKR_ERR_SGF_DIVERGED = -4, /* decimation error > 1e10 (main/surfgf.f:88-93)        */
  SKKR_ERR_UNSUPPORTED = -5,  /* input outside the implemented scope                  */
  SKKR_ERR_NOMEM = -6,
  SKKR_ERR_NONFINITE = -7,    /* NaN/Inf in a result                                  */
  SKKR_ERR_PEER = -8          /* another rank of a k-split energy failed, or the reduction hook did */
};

/* Sizes of one system: the runtime equivalent of param.h plus the
 * /lay2d/ and /iterpar/ COMMON blocks read by cpacoord
 * (rsp-scf/cpacoord_ksave.f:71-80). */
typedef struct {
  int mode;                       /* skkr_mode; kappa-mu block 2(lmax+1)^2 or lm (lmax+1)^2 */
  int lmax;                       /* <= 3 */
  int nprc;                       /* interface principal layers, 1..SKKR_MAX_PRC */
  int ninprc[SKKR_MAX_PRC + 2];   /* layers per PL: [0] left lead, [1..nprc], [nprc+1] right lead */
  int bulkgeo;                    /* 1: every interface PL uses structure-constant slot 1 */
  int ngeff;                      /* point-group operations summed in the k integral */
  int itermaxl, itermaxr;         /* decimation caps (/iterpar/) */
  double errmax;                  /* decimation tolerance (/iterpar/) */
  int itcpam;                     /* CPA iteration cap */
  double cpatol;                  /* CPA tolerance on error3 (rsp-scf/fullcpa.f:142) */
  int precision;                  /* skkr_precision */
  int nk_chunk;                   /* k points per device batch (0: automatic) */
  int slices;                     /* SKKR_MIXED: BF16 slices per product operand, 3..8 (0: 6).
                                     Digits are 8-bit for a product depth K <= 128 (8 slices act
                                     as 7), 7-bit above.  SKKR_BDG splits every product into its
                                     electron and hole K halves, each with its own scales */
} skkr_sizes;

/* Real-space screened structure constants of one energy, grouped in
 * lm x lm blocks: block b of G_scr(k) = sum over r in [rstart[b], rstart[b+1])
 * of exp(+i k.rvec[r]) gR[r].  blkmap[(slot*mi + i-1)*(2*jmax+1) + j+jmax]
 * is the block coupling layer i of a principal layer of structure-constant
 * slot `slot` (0 left lead, 1.. interface, nprc+1 right lead) to layer i+j,
 * or -1.  This replaces the per-k Kambe evaluation of main/gstore.f:6-283
 * (g2d(lmmaxp,lmmaxp,-minprc:minprc,minprc,0:mprc1+1)). */
typedef struct {
  int nblk;
  int nr;
  const int *rstart;          /* [nblk+1] */
  const double *rvec;         /* [nr][2] */
  const double *gR;           /* [nr] column-major (lmax+1)^2 square complex blocks */
  int nslot, mi, jmax;
  const int *blkmap;          /* [nslot][mi][2*jmax+1] */
} skkr_rtable;

typedef struct {
  int code;                   /* skkr_error of the call */
  int ik;                     /* first failing k point (0-based) or -1 */
  int cpa_iterations;         /* itcpa-1 on exit, as printed by cpacoord */
  double cpa_error;           /* last max error3 */
  int max_dec_iters;          /* largest decimation iteration count */
  long long dec_iters_total;  /* summed decimation iterations */
  long long gpu_launches;     /* kernels launched by this call */
  double max_refine_resid;    /* mixed precision: largest accepted Newton residual |I - AX|_F
                                 (before the last correction) */
  double run_ms;              /* device time of the call (CUDA events on the library stream) */
  long long inv_fallbacks;    /* mixed precision: inverses whose residual stayed above 1e-6
                                 and were redone in FP64 */
  long long k_fp64;           /* mixed precision: k points redone in FP64 (dominant contributions) */
  long long inv_refined;      /* mixed precision: inverses that took further Newton steps (residual
                                 above 1e-6 after the standard steps, below 1/2) */
  double alg_flops;           /* FP64-equivalent algorithmic work of the call in the reference's
                                 operation count, U = 8 n_PL^3 real FLOP per block operation:
                                 (9 it + 3) U per lead decimation of `it` iterations (surfgf.f,
                                 dugo.f) and (7 nprc - 6) U per tau2d item (tau2d.f) on every
                                 CPA iteration; the precision guards' FP64 redos are not counted */
  long long graph_launches;   /* CUDA graph launches of the call (the captured decimation loops) */
  long long graph_kernels;    /* kernels those graphs ran (counted on the device; included in
                                 gpu_launches, which minus these plus graph_launches gives the
                                 launch operations the host issued) */
} skkr_status;

typedef struct skkr_ctx skkr_ctx;

/* Create a context on the current CUDA device (replaces the Fortran `save`
 * arrays xsave, ysave, g2d of cpacoord_ksave.f:86). */
int skkr_gpu_create(const skkr_sizes *sizes, skkr_ctx **ctx);
int skkr_gpu_destroy(skkr_ctx *ctx);

/* Split-precision policy near the real axis, where the lead and slab
 * matrices become ill-conditioned and rounding of the products is amplified
 * by their condition number: decimation runs in FP64 when |Im E| < dec_fp64_im
 * (default 2e-4 Ry); the products use slices_near BF16 slices on the
 * exact-level tile when |Im E| < near_im (defaults 7 slices below 1e-3 Ry;
 * 3..8, 0 = off);
 * every k point whose contribution exceeds dominant_frac (default 1e-2) of
 * the norm of the k-summed tau, and ten times the mean contribution of a k
 * point (an isolated peak), is recomputed in FP64 (0 = off).  Inverses
 * whose Newton residual is above 1e-6 after the standard steps take up to
 * four further steps while it stays below 1/2; those still above 1e-6 are
 * always redone in FP64.  An energy whose decimation runs in FP64 on blocks
 * above 128 rows (the split inverse's limit) runs wholly in FP64: splitting
 * the tau2d products alone does not repay the splits and the peak redo. */
int skkr_gpu_set_mixed_policy(skkr_ctx *ctx, double dec_fp64_im, double near_im, int slices_near,
                              double dominant_frac);

/* Standard Newton steps X += X (I - A X) after the FP32 Gauss-Jordan start of
 * every split-precision inverse (1..3, default 2).  The acceptance test is
 * unchanged: the residual before the last correction must be below 1e-6 (or
 * the further steps and the FP64 redo take over), so one step suits inputs
 * whose FP32 start is already that close. */
int skkr_gpu_set_newton(skkr_ctx *ctx, int steps);

/* The FP32 start of split-precision inverses above 64 rows: blocked != 0
 * (the default) forms it by 2 x 2 blocks (two 64-row Gauss-Jordan inverses
 * with pivoting inside each block, six FP32 block products); 0 runs the
 * Gauss-Jordan of main/gjinv.f's column pivoting on the whole matrix.  The
 * Newton steps, their acceptance test and the FP64 redo are the same. */
int skkr_gpu_set_inverse_start(skkr_ctx *ctx, int blocked);

/* The B operand of every split-precision product on the default tile: on
 * != 0 (the default) the product reads B in FP64 and forms its BF16 slices in
 * shared memory, tile by tile, with the warps that later run the epilogue; 0
 * splits B into a staging buffer first and loads its tiles by TMA.  Both give
 * the same slices, hence the same result bit for bit. */
int skkr_gpu_set_fused_split(skkr_ctx *ctx, int on);

/* Autotuner of the split-precision inverse's FP32 Gauss-Jordan: each size
 * class (n <= 32, 64, 128) has 2-3 thread layouts that give the same inverse
 * bit for bit; the first batch of each (class, batch size) times them (best
 * of three runs each; a later layout must be 5 % faster to be chosen) and
 * later calls use the choice (process wide).  report (may be NULL)
 * receives the choices so far, e.g. "n<=128 >=4 waves: 64x2x8; ".
 * force > 0 makes every class use its layout force - 1 (tests); force = 0
 * with report NULL forgets the choices and tunes afresh. */
int skkr_gpu_autotune(int force, char *report, int len);

/* Decimation loop as a CUDA graph (default on): after the first iteration,
 * the remaining iterations of every k chunk run as one graph launch whose
 * WHILE node repeats the iteration body until no (k, lead) item is left,
 * with the convergence test, the iteration count and the split-precision
 * inverse's further Newton steps (IF nodes) decided on the device.  on = 0
 * runs every iteration from the host (one stream synchronisation per
 * iteration); results are identical.  While per-kernel statistics are on
 * (skkr_gpu_kernel_stats), and inside skkr_gpu_cpacoord_many (contexts driven
 * from several host threads at once), the host loop is used; callers that
 * drive contexts from their own threads concurrently should switch graphs
 * off the same way. */
int skkr_gpu_set_graphs(skkr_ctx *ctx, int on);

/* Off-diagonal tau of the interface for cluster embedding
 * (skkr_dbogo_bsf/clu/tau2d_god.f with the pair sums of
 * skkr_dbogo_bsf/rsp-scf/cpacoord_ksave.f:760-840): one k loop of the staged
 * energy with its current t^-1 (no CPA update).  For pair q,
 * pairs[4q..4q+3] = (n1, n2, li, lj) with 0-based interface layers, the
 * results are the inter-site scattering path operators
 *   tau_ij[q] = tau(layer li in cell 0, layer lj in cell n1 a1 + n2 a2)
 *             = sum_k w_k/ngeff sum_g e^{+i k.g(v)} [L_g tau^(g)(k) R_g]_{li,lj}
 *   tau_ji[q] = tau(layer lj in cell n1 a1 + n2 a2, layer li in cell 0)
 * with v = n1 a1 + n2 a2 + c_li - c_lj, a1/a2 the in-plane lattice vectors,
 * cvec[2 l] the in-plane position of interface layer l and a0mat[4 g] the
 * row-major 2x2 in-plane matrix of group element g applied to v: the
 * transpose (inverse) of the in-plane rotation whose D matrices are
 * L_g = lg[g], R_g = rg[g] (the IBZ point k stands for a0mat[g]^T k of the
 * full zone).  tau_ij / tau_ji are [npair][ld][ld] column-major; npair *
 * ngeff <= 65535; non-relativistic and relativistic modes (BdG:
 * SKKR_ERR_UNSUPPORTED).  The status carries the decimation counters. */
int skkr_gpu_tauij(skkr_ctx *ctx, int npair, const int *pairs, const double *a1, const double *a2,
                   const double *cvec, const double *a0mat, double *tau_ij, double *tau_ji, int ld,
                   skkr_status *status);

/* Host reduction for an energy whose k points are split over ranks (the
 * modulo(ik-1,nprocs) split of cpacoord_ksave.f:189 with the mpi_allreduce of
 * the k-summed tau at :406).  When set, every CPA iteration calls
 *   fn(user, buf, n)   with n = 2*nintfc*lk*lk + 1 doubles:
 *   buf[0 .. n-2]  this rank's k-summed screened tau, [nintfc][col][row] re/im,
 *   buf[n-1]       1.0 if this rank failed (decimation cap / divergence), else 0.0,
 * and fn must overwrite buf with the element-wise sum over all ranks (an
 * allreduce SUM) and return 0.  Each rank passes only its own k points and
 * their global weights; the CPA update then runs replicated on identical
 * data, so all ranks take the same number of CPA iterations.  A rank that
 * fails still calls fn (with the flag set) before it returns its own code;
 * the other ranks then return SKKR_ERR_PEER.  fn = NULL switches it off. */
typedef int (*skkr_reduce_fn)(void *user, double *buf, long long n);
int skkr_gpu_set_reduce(skkr_ctx *ctx, skkr_reduce_fn fn, void *user);

/* The same reduction on the device, for a collective library that works on
 * device memory (an NCCL allreduce): every CPA iteration the context calls
 *   fn(user, buf, n, stream)   with buf a DEVICE pointer to the n doubles laid
 *                              out as for skkr_gpu_set_reduce (k-summed tau,
 *                              then the failure flag),
 * after queueing the writes of buf on `stream` (the context's cudaStream_t).
 * fn must leave the element-wise sum over all ranks in buf, ordered on that
 * stream (for NCCL: the allreduce enqueued on it, in place), and return 0;
 * buf stays valid until the context is destroyed.  Replaces the host copies
 * of skkr_gpu_set_reduce by one device-to-device copy each way and the read
 * of the flag; when both are set this one is used.  fn = NULL switches it off. */
typedef int (*skkr_reduce_dev_fn)(void *user, double *buf, long long n, void *stream);
int skkr_gpu_set_reduce_device(skkr_ctx *ctx, skkr_reduce_dev_fn fn, void *user);

/* One energy: the CPA loop around the k loop, k-sum with point-group
 * rotation and the CPA update (cpacoord_ksave.f:139-419).
 *   ce, fac        complex energy and relmtrx factor psq/ce (1 non-rel)
 *   rt             structure-constant table of this energy
 *   nk, xk, wk     k points [nk][2] and normalised weights
 *   lg, rg         [ngeff] ld x ld: k-sum adds lg*tau*rg; t^-1 rotates as rg*t*lg
 *                  (rmatp(invg(g)), rmat(invg(g)) of the reference)
 *   conc           [nintfc] concentration of species A
 *   tminvl/tminvr  [ninprc[0]] / [ninprc[nprc+1]] lead screened t^-1
 *   tminv          [nintfc] in: starting coherent t^-1, out: converged
 *   tminva/tminvb  [nintfc] species t^-1
 *   tauc           [nintfc] out: k-summed screened coherent tau
 *   taua/taub      [nintfc] out: screened species tau (before phystau, as cpacor leaves them)
 */
int skkr_gpu_cpacoord(skkr_ctx *ctx, double ce_re, double ce_im, double fac_re,
                      double fac_im, const skkr_rtable *rt, int nk,
                      const double *xk, const double *wk, const double *lg,
                      const double *rg, const double *conc,
                      const double *tminvl, const double *tminvr,
                      double *tminv, const double *tminva,
                      const double *tminvb, double *tauc, double *taua,
                      double *taub, int ld, skkr_status *status);

/* BdG energy (skkr_dbogo_bsf/rsp-scf/cpacoord_ksave.f): as skkr_gpu_cpacoord
 * on a SKKR_BDG context, with the hole factor fach = conj(psqh)/conj(celoch)
 * (:160-169).  rt->gR holds 2 * rstart[nblk] blocks: the electron table, then
 * the hole table (main/gstore.f:208-216: conjugate-transposed and
 * lmtolmconj-transformed, screened with the hole alpha) on the same R
 * vectors; site blocks are blockdiag(relmtrx(G_e, fac), relmtrx(G_h, fach))
 * (main/g2d_pack.f, main/relmtrx.f).  lg / rg are the BdG point-group
 * matrices, e.g. blockdiag(D, D*).  The slot API does not take BdG energies. */
int skkr_gpu_cpacoord_bdg(skkr_ctx *ctx, double ce_re, double ce_im, double fac_re,
                          double fac_im, double fach_re, double fach_im, const skkr_rtable *rt,
                          int nk, const double *xk, const double *wk, const double *lg,
                          const double *rg, const double *conc, const double *tminvl,
                          const double *tminvr, double *tminv, const double *tminva,
                          const double *tminvb, double *tauc, double *taua, double *taub, int ld,
                          skkr_status *st);

/* The arguments of one skkr_gpu_cpacoord / skkr_gpu_cpacoord_bdg call
 * (fach is read for SKKR_BDG contexts only). */
typedef struct {
  double ce_re, ce_im, fac_re, fac_im, fach_re, fach_im;
  const skkr_rtable *rt;
  int nk;
  const double *xk, *wk, *lg, *rg, *conc, *tminvl, *tminvr;
  double *tminv;
  const double *tminva, *tminvb;
  double *tauc, *taua, *taub;
  int ld;
} skkr_energy_args;

/* A list of energies of one system in one call (the contour loop of
 * rsp-scf/skkr.f:389-486 around its cpacoord call at :439): energy e runs
 * args[e] as skkr_gpu_cpacoord would (SKKR_BDG contexts: as
 * skkr_gpu_cpacoord_bdg), in order on the context's stream, each with its
 * decimation graphs; st[e] (st may be NULL) receives its status.  Every
 * energy runs even after one fails; returns the first nonzero code. */
int skkr_gpu_contour(skkr_ctx *ctx, int ne, const skkr_energy_args *args, skkr_status *st);

/* Several systems in one call (e.g. interfaces of different lmax / PL size):
 * energy args[e] runs on context ctx[e] (n distinct contexts, each of its
 * own system) concurrently, each context on its own stream driven by its own
 * host thread, so that small systems fill the SMs a large one leaves idle.
 * Results and st[e] are those of the single calls; returns the first
 * nonzero code. */
int skkr_gpu_cpacoord_many(int n, skkr_ctx *const *ctx, const skkr_energy_args *args,
                           skkr_status *st);

/* Split form for callers that keep inputs resident on the device across
 * calls: stage (host -> device), run (device only), fetch (device -> host).
 * skkr_gpu_cpacoord == stage + run + fetch. */
int skkr_gpu_stage(skkr_ctx *ctx, double ce_re, double ce_im, double fac_re,
                   double fac_im, const skkr_rtable *rt, int nk,
                   const double *xk, const double *wk, const double *lg,
                   const double *rg, const double *conc,
                   const double *tminvl, const double *tminvr,
                   const double *tminv, const double *tminva,
                   const double *tminvb, int ld);
int skkr_gpu_run(skkr_ctx *ctx, skkr_status *status);
int skkr_gpu_fetch(skkr_ctx *ctx, double *tminv, double *tauc, double *taua,
                   double *taub, int ld);

/* The same split form for several energies kept resident at once: each
 * `slot` (0, 1, ...) holds one staged energy's inputs and results; the work
 * buffers of the context are shared, so slots cost only their inputs. */
int skkr_gpu_stage_slot(skkr_ctx *ctx, int slot, double ce_re, double ce_im,
                        double fac_re, double fac_im, const skkr_rtable *rt,
                        int nk, const double *xk, const double *wk,
                        const double *lg, const double *rg, const double *conc,
                        const double *tminvl, const double *tminvr,
                        const double *tminv, const double *tminva,
                        const double *tminvb, int ld);
int skkr_gpu_run_slot(skkr_ctx *ctx, int slot, skkr_status *status);
int skkr_gpu_fetch_slot(skkr_ctx *ctx, int slot, double *tminv, double *tauc,
                        double *taua, double *taub, int ld);

/* Per-kernel-class timing with CUDA events (process wide).  enable=1 resets
 * and starts; enable=0 stops and writes out[cls*4 + {launches, total ms,
 * work, FP64-equivalent algorithmic work}] (5 x 4 doubles) for cls = 0 FP64
 * complex GEMM (FLOP), 1 Gauss-Jordan inverse (8 n^3 FLOP per inverse), 2 G(k)
 * transform (bytes written), 3 other (bytes), 4 sliced complex GEMM on the
 * tensor cores (work: BF16 FLOP of every slice pair; FP64-equivalent: 8 n^2 K
 * per complex product).  The events add a gap around every launch: time
 * throughput with the statistics off. */
int skkr_gpu_kernel_stats(int enable, double *out);

/* Screened -> physical tau of one layer on the device
 * (rsp-scf/phystau.f:2-61, nrsp-scf/phystau.f): tau := (1+a t)tau(1+t a) - (a + a t a).
 * alpha[l], l = 0..lmax; SKKR_BDG: alpha_e[0..lmax] then alpha_h[0..lmax]
 * (skkr_dbogo_bsf cpacoord_ksave.f:497). */
int skkr_gpu_phystau(int mode, int lmax, double *tau, const double *tinv,
                     const double *alpha, int ld);

/* Screened -> physical tau of one off-diagonal block tau_ij on the device
 * (cluster/rsp-lay/phystau2.f:2-60, skkr_dbogo_bsf/clu/phystau2.f:2-75, in
 * the form the cpacoord of skkr_dbogo_bsf applies to tau_ij and tau_ji
 * before writing them for the cluster code, rsp-scf/cpacoord_ksave.f:976-988,
 * idiag = 0): tau := (1 + alpha1 tinv1) tau (1 + tinv2 alpha2), alpha1 /
 * tinv1 of the row layer i, alpha2 / tinv2 of the column layer j; alpha as
 * for skkr_gpu_phystau. */
int skkr_gpu_phystau2(int mode, int lmax, double *tau, const double *tinv1, const double *alpha1,
                      const double *tinv2, const double *alpha2, int ld);

/* Learned CPA warm start: a dense MLP with tanh hidden layers and a linear
 * output layer, FP64 on the device (forward, backward and AdamW are this
 * library's own kernels).  nlayer layers (1..8) of sizes dims[0..nlayer]
 * (1..4096); params packs W_0 [dims0][dims1] (row-major), b_0 [dims1],
 * W_1, b_1, ...; x [n][dims0], y [n][dims_last], row-major.  rows[r] = 1
 * puts row r in the training loss, 0 holds it out (rows NULL: all rows
 * train).  The loss is the mean squared error over the training rows and
 * all outputs. */
int skkr_gpu_mlp_forward(int nlayer, const int *dims, const double *params, int n, const double *x, double *y);
/* loss and its gradient w.r.t. params (packed like params) */
int skkr_gpu_mlp_grad(int nlayer, const int *dims, const double *params, int n, const double *x,
                      const double *y, const unsigned char *rows, double *loss, double *grad);
/* Full-batch AdamW (beta 0.9 / 0.999, eps 1e-8, decoupled weight decay) for
 * `epochs` steps from params; train_loss[ep] is the training loss before
 * step ep, params receives the final parameters.  With held-out rows and
 * eval_every > 0 the held-out loss is evaluated after the steps ep with
 * ep % eval_every == 0 and after the last one; best_params receives the
 * parameters of the lowest held-out loss and best = {that loss, the training
 * loss of its epoch}.  Without them best = {NaN, last training loss} and
 * best_params the final parameters (either may be NULL). */
int skkr_gpu_mlp_train(int nlayer, const int *dims, double *params, int n, const double *x, const double *y,
                       const unsigned char *rows, int epochs, double lr, double weight_decay, int eval_every,
                       double *train_loss, double *best, double *best_params);

/* The same network in the precision of the C4 warm-start surrogate: FP32
 * master parameters (packed like params above), whose weights the products
 * read as BF16 (round to nearest even) with FP32 activations and FP32
 * accumulation; the gradient is that of the BF16-weight network, applied to
 * the FP32 masters by AdamW (beta 0.9 / 0.999, eps 1e-8), after which the
 * BF16 copies are refreshed.  Arguments and outputs as for the FP64 forms. */
int skkr_gpu_mlp16_forward(int nlayer, const int *dims, const float *params, int n, const float *x, float *y);
int skkr_gpu_mlp16_grad(int nlayer, const int *dims, const float *params, int n, const float *x, const float *y,
                        const unsigned char *rows, float *loss, float *grad);
int skkr_gpu_mlp16_train(int nlayer, const int *dims, float *params, int n, const float *x, const float *y,
                         const unsigned char *rows, int epochs, float lr, float weight_decay, int eval_every,
                         float *train_loss, float *best, float *best_params);
/* The same network kept on the device for repeated inference (the warm start
 * of one energy runs it on a few rows): load uploads the parameters once and
 * sizes the buffers for up to maxrows rows; infer runs n <= maxrows rows on
 * the handle's own stream and returns when y is written; free releases it. */
typedef struct skkr_mlp16 skkr_mlp16;
int skkr_gpu_mlp16_load(int nlayer, const int *dims, const float *params, int maxrows, skkr_mlp16 **net);
int skkr_gpu_mlp16_infer(skkr_mlp16 *net, int n, const float *x, float *y);
int skkr_gpu_mlp16_free(skkr_mlp16 *net);

/* The reference's k-space structure constants (main/kamstr.f:20-392): the
 * Kambe lattice sums D_L(k, s) of outgoing spherical waves over a 2D lattice,
 * L = (l, m) up to l = lmax2 (0..6), index l(l+1)+m, for nitem items of one
 * energy e (k point kxy[2 item], layer-pair separation sep[3 item], a.u.).
 * gvec [ng][2] / rvec [nr][2]: reciprocal and direct lattice vectors (any
 * superset: terms with |g + k| > gcut or an in-plane |R + s| > rcut are
 * skipped); area the cell area; factor the Ewald parameter (eta of the
 * input, 1 in the reference's samples).  out [nitem][(lmax2+1)^2] complex. */
int skkr_gpu_kambe_dlm(int nitem, double e_re, double e_im, const double *kxy, const double *sep, int lmax2,
                       const double *gvec, int ng, const double *rvec, int nr, double area, double factor,
                       double gcut, double rcut, double *out);
/* The coefficients that turn those sums into the layer-pair structure
 * constants, alm[L][L'] = sum_q coef[L][L'][q] D_q (kamstr.f:355-390 in this
 * library's harmonics), for lmax 0..3: coef [lmmax][lmmax][(2 lmax+1)^2]
 * complex.  Host only: no device call. */
int skkr_gpu_kambe_coef(int lmax, double *out);
/* The layer-pair structure constants alm(k, s) [lmmax][lmmax] of nitem items
 * (kamstr.f's output; the arguments as for skkr_gpu_kambe_dlm with lmax
 * 0..3 in place of lmax2): the lattice sums and their contraction on the
 * device, one thread per item.  out [nitem][lmmax][lmmax] complex, row L. */
int skkr_gpu_kambe_alm(int nitem, double e_re, double e_im, const double *kxy, const double *sep, int lmax,
                       const double *gvec, int ng, const double *rvec, int nr, double area, double factor,
                       double gcut, double rcut, double *out);
/* The reference's screened G_scr(k) (main/gstore.f:146-282 with
 * main/scrstr.f:2-138) on the device: for each of nk k points the layer-pair
 * blocks of a slab of nl layers at pos [nl][3] (block (a, b) with the
 * in-plane phase e^{ik.(pos_b - pos_a)}, the orientation of the real-space
 * tables), G' = G (1 - alpha G)^-1 with alpha [nl][lmax+1] complex, and the
 * blocks (centre, centre + j) for j = -jmax..jmax into
 * out [nk][2 jmax + 1][lmmax][lmmax] complex.  nl (lmax+1)^2 <= 512.  The
 * lattice sums run once per distinct layer separation of the slab, one
 * thread block per (k, separation) item. */
int skkr_gpu_kambe_screened(int nk, double e_re, double e_im, const double *kxy, int nl, const double *pos,
                            const double *alpha, int lmax, const double *gvec, int ng, const double *rvec, int nr,
                            double area, double factor, double gcut, double rcut, int centre, int jmax,
                            double *out);

/* The reference's own k-space structure constants in place of the table
 * transform, for the energy staged last by skkr_gpu_stage (not the slot
 * API): per k point the Kambe lattice sums of every distinct layer
 * separation of a slab of nl layers (main/kamstr.f:20-392, gstore.f:146-282),
 * the slab screening G' = G (1 - alpha G)^-1 (main/scrstr.f:2-138,
 * main/scrinv.f:2-63; nl (lmax+1)^2 <= 512) and, as the blocks of the staged
 * table's layer offsets j, the slab blocks (centre, centre + j).  The staged
 * block map must send an offset to one block from every layer and slot (a
 * stacking of equivalent layers).  Packing, decimation, tau2d, the k-sum and
 * the CPA update are unchanged.  kf = NULL, or a new skkr_gpu_stage, returns
 * to the table transform.  Not for SKKR_BDG contexts. */
typedef struct {
  double e_re, e_im;          /* energy of the lattice sums (kappa^2; psq in the relativistic code) */
  int nl;                     /* layers of the screening slab */
  const double *pos;          /* [nl][3] layer positions (a.u.), in the table's orientation */
  const double *alpha;        /* [nl][lmax+1] complex screening constants */
  int centre;                 /* slab layer whose blocks are kept (centre +- jmax inside the slab) */
  const double *gvec;         /* [ng][2] reciprocal lattice vectors (a superset: |g + k| > gcut skipped) */
  int ng;
  const double *rvec;         /* [nr][2] direct lattice vectors (in-plane |R + s| > rcut skipped) */
  int nr;
  double area, factor;        /* 2D cell area; Ewald parameter (1 in the reference's samples) */
  double gcut, rcut;
} skkr_kambe_form;
int skkr_gpu_stage_kambe(skkr_ctx *ctx, const skkr_kambe_form *kf);

/* Layer DOS of nlay layers from their physical site-diagonal tau (replaces
 * the lambda = 0 moment of nrsp-scf/moment.f:47-110 with locquant.f:86-126,
 * and rsp-scf/moment.f:60-140 with locquant.f:197-232):
 *   zmom[li][i]   = fac (F[li][i] tau_li(i,i) - G[li][i])   per basis index,
 *   zdos_l[li][l] = sum of zmom over the indices of orbital l,
 * fac = -1/pi, doubled for para != 0 in the lm basis.  F, G are the
 * single-site radial integrals int Z^2 r^2 dr, int Z J r^2 dr per basis index
 * (complex, [nlay][nd]); tau is [nlay][ld][ld].  The DOS is Im(zmom) /
 * Im(zdos_l); the host accumulates the contour sums of locquant.f itself. */
int skkr_gpu_layer_dos(int mode, int lmax, int nlay, const double *tau, int ld, const double *F,
                       const double *G, int para, double *zmom, double *zdos_l);

/* Bloch spectral function of nlay (<= 16) interface layers at nk k points
 * (replaces skkr_dbogo_bsf/rsp-scf/bsf.f:2-437 with gf.f:1-103 at reg =
 * .true., pairing.f and moment.f at lambda = 0; the non-BdG modes keep its
 * bsfe).  All taus are physical, nd x nd column-major (nd of phystau's
 * mode): tauk [nk][nlay] the coherent tau of each k point, tauc / taua /
 * taub [nlay] the k-integrated coherent and component taus of the CPA
 * (bsf.f's tau_kint, taua_kint, taub_kint).  A layer with 1 - conc > 1e-6
 * takes the CPA form: A0 = sum_a c_a R_aa tau_a and A1 = sum_ab c_a c_b
 * R_ab D_a (tau(k) - tau_c) D~_b, D_a = tau_a tau_c^-1, D~_b = tau_c^-1 tau_b
 * (species a = A, B with weights conc, 1 - conc); other layers R_AA tau(k).
 * R are the radial overlaps of the right solution of species a with the
 * left solution of species b: F [nlay][a][b][nd] on the basis diagonal
 * (BdG: electron then hole half) and, for BdG, Feh [nlay][a][b][nde][nde]
 * (column-major, nde = nd / 2) on the electron-hole block, contracted with
 * the four pairing operators pair [4][nde][nde] (singlet, T0, T-up,
 * T-down of pairing.f).  out [nk][nlay][6] = -1/pi Im of: the electron
 * diagonal sum (bsfe), the hole diagonal sum (bsfh), tr(P_x G_eh) for the
 * four operators (bsfeh, bsfhe, bsfteh, bsfthe); zero where a mode has no
 * such part; doubled for para != 0 in the lm basis.  Feh / pair may be
 * NULL outside BdG. */
int skkr_gpu_bsf(int mode, int lmax, int nk, int nlay, const double *conc, const double *tauk,
                 const double *tauc, const double *taua, const double *taub, const double *F,
                 const double *Feh, const double *pair, int para, double *out);

/* Lower-level batched kernels, exported for tests. */
/* In-place inverses of `batch` n x n matrices, n <= 512 (main/gjinv.f:2-59, column pivoting). */
int skkr_gpu_gjinv_batch(int n, int batch, double *a, int ld);
/* Decimation of `batch` (ml, m0, mr) triples -> x = (m0 - ...)^-1 (main/surfgf.f:2-108).
 * iters[b] receives the iteration count, stat[b] 0 / SKKR_ERR_SGF_*. */
int skkr_gpu_surfgf_batch(int n, int batch, const double *ml, const double *m0,
                          const double *mr, double *x, int ld, int itermax,
                          double errmax, int *iters, int *stat);
/* Decimation exactly like skkr_gpu_surfgf_batch, for callers that are not
 * allowed to allocate device memory (a host code whose device memory belongs
 * to another layer, such as an OpenACC / CUDA Fortran data region or the
 * application's own pool, or a run with a fixed device-memory budget).
 * No counterpart in the reference.
 *   ml, m0, mr, x  DEVICE pointers owned by the caller: `batch` column-major
 *                  n x n matrices, leading dimension ld, one ld*ld block each
 *   iters, stat    host arrays [batch] or NULL;  stream: a cudaStream_t or NULL
 * It calls no cudaMalloc / cudaFree: its work space is one static device array
 * of SKKR_NOALLOC_SCRATCH_BYTES (32 MiB, held by every GPU that loads the
 * library until the process exits).  A request needing more than
 * batch * (8 * n * n * 16 + 20) + 64 > SKKR_NOALLOC_SCRATCH_BYTES bytes is
 * rejected with SKKR_ERR_NOMEM, and batch > 65535 with SKKR_ERR_ARG, before
 * anything runs.  The first call on each device looks up the array's device
 * address (cudaGetSymbolAddress); make that first call before any stream
 * capture.  After every decimation iteration the call reads the number of
 * items still iterating from the device, synchronizing `stream`, and it
 * returns after a final synchronization, with x, iters and stat written.
 * All calls share the one array: calls that overlap on the GPU (several
 * streams or host threads) race. */
#define SKKR_NOALLOC_SCRATCH_BYTES (32u << 20)
int skkr_gpu_surfgf_batch_noalloc(int n, int batch, const double *ml,
                                  const double *m0, const double *mr,
                                  double *x, int ld, int itermax,
                                  double errmax, int *iters, int *stat,
                                  void *stream);

/* c = a*b for `batch` complex n x n matrices (host arrays, ld), in FP64 or
 * split precision (`slices` 3 or 5 BF16 slices per operand on the tensor
 * cores).  Test and benchmark entry point of the products used by
 * surfgf / tau2d (main/matops.f doubmt2 / tripmt). */
int skkr_gpu_zgemm_batch(int precision, int slices, int n, int batch,
                         const double *a, const double *b, double *c, int ld);
/* In-place inverses in FP64 (main/gjinv.f) or split precision (FP32
 * Gauss-Jordan + `newton` refinement steps; n <= 128).  max_resid (may be
 * NULL) receives the largest ||I - A X||_F before the last step. */
int skkr_gpu_zinv_batch(int precision, int n, int batch, double *a, int ld,
                        int newton, double *max_resid);

/* G_scr(k) blocks of nk k points: out [nk][nblk] lm x lm column-major. */
int skkr_gpu_gk(const skkr_rtable *rt, int lmax, int nk, const double *xk, double *out);

/* tau2d (main/tau2d.f:2-152) for `batch` independent items of nprc principal
 * layers of n rows (n = layers per PL x lk), FP64, host arrays, column-major
 * n x n blocks without padding: m00, m01, m10 [batch][nprc] the packed PL
 * matrices (M00 with the layers' t^-1 blocks added; M01 couples PL p to
 * p+1, M10 to p-1), x and y [batch] the right and left surface operators.
 * tau [batch][nprc * n/lk] receives wgeff times the layer-diagonal lk x lk
 * blocks of the PL-diagonal tau.  batch * nprc <= 65535, n <= 512. */
int skkr_gpu_tau2d(int batch, int nprc, int n, int lk, double wgeff, const double *m00, const double *m01,
                   const double *m10, const double *x, const double *y, double *tau);

/* Text of the last CUDA error seen by the library in this process. */
const char *skkr_gpu_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
