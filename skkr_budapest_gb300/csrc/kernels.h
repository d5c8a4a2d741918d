// Host launch wrappers of the batched device kernels.
#pragma once
#include "common.cuh"

// G_scr(k): out[(k*nblk + b)] lm x lm blocks (column-major, ld = lmmax)
void launch_gk_ft(const zd *gR, const double *rvec, const int *rstart, int nblk, int lmmax,
                  const double *xk, int nk, zd *out, cudaStream_t st);

// packer.f jobs: one n x n matrix per (k, job)
struct PackJob {
  int slot, ni, nim, nip;
  int which;  // 0: M00, 1: M10 (M0-1), 2: M01
  int dest;   // matrix index in the per-k pool
};
cudaError_t pack_set_tables(int irel, int lmax);
void launch_pack(const zd *G, int nblk, int nbk, const int *d_blkmap, int mi, int jmax,
                 const PackJob *d_jobs, int njobs, int lk, int lmmax, int mode, zd fac, zd fach, int nk,
                 zd *pool, int nmat, int npl, int ehsplit, cudaStream_t st);

// batched complex GEMM, items (k, c) with k < nk, c < nc; act[k*nc+c]==0 skips.
// mode 0: C = A*B        1: C = C - A*B
// mode 2: y = A*B ; D -= y ; E -= y  (C unused)
// mode 3: C = D - A*B
void launch_zgemm(int mode, const MatRef &A, const MatRef &B, const MatRef &C, const MatRef &D,
                  const MatRef &E, int m, int n, int kdim, int nk, int nc, const int *act,
                  cudaStream_t st);

// in-place Gauss-Jordan inverses (gjinv.f), one CTA per item, n <= 512
void launch_zgj(const MatRef &A, int n, int nk, int nc, const int *act, cudaStream_t st);

// elementwise: out = a + s1*b + s2*d over n x n (b/d may be null)
void launch_zaxpby(const MatRef &out, const MatRef &a, const MatRef *b, double s1, const MatRef *d,
                   double s2, int n, int nk, int nc, const int *act, cudaStream_t st);
// out = in + block-diagonal t (nl layers of lk x lk, t base from tref for item);
// ehsplit: principal-layer matrices in the electron-first BdG layout
void launch_add_tblocks(const MatRef &out, const MatRef &in, const MatRef &t, int lk, int nl,
                        int n, int nk, int nc, const int *act, int ehsplit, cudaStream_t st);
// Frobenius norms of items -> out[k*nc+c]
void launch_fnorm(const MatRef &a, int n, int nk, int nc, const int *act, double *out,
                  cudaStream_t st);
// decimation state update (surfgf.f:81-96)
void launch_dec_state(const double *err, int *act, int *stat, int *iters, int nitems, int iter,
                      int itermax, double errmax, cudaStream_t st);
// the same with the iteration number on the device and the count of items
// left iterating added to *nactive; then the loop step of a captured WHILE
// node: iteration number + 1, *nactive cleared, condition set
void launch_dec_state_dev(const double *err, int *act, int *stat, int *iters, int nitems, const int *iter_p,
                          int itermax, double errmax, int *nactive, cudaStream_t st);
void launch_dec_advance(int *iter_p, int *nactive, int itermax, const int *errflag, cudaGraphConditionalHandle cond,
                        int *runs, cudaStream_t st);
// tau(k) diagonal-block extraction: out[k][c][layer] = (wk[k]*wscale) * W(layer block)
void launch_extract_tau(const MatRef &W, int lk, int nl, int layer0, const double *wk,
                        double wscale, zd *out, long long out_sk, long long out_sc, int nk,
                        int nc, int ehsplit, cudaStream_t st);
// per-k norms of k-resolved contributions tk[k][E] -> out[k]; S[e] += sign x[e]
void launch_knorm(const zd *tk, int nk, long long E, double *out, cudaStream_t st);
void launch_axpy_flat(zd *S, const zd *x, long long E, double sign, cudaStream_t st);
// deterministic k-sum (warp-shuffle): S[e] (+)= sum_k tk[k*E + e]
void launch_ksum(const zd *tk, int nk, long long E, zd *S, int accumulate, cudaStream_t st);
// sum over g of T[layer][g] -> out[layer]
void launch_gsum(const zd *T, int ng, int lk, int nl, zd *out, cudaStream_t st);
// layer-pair blocks of one PL block of the full tau, and the phased pair k sums
void launch_extract_pairs(const MatRef &W, int lk, int nl, int rowlay0, int collay0, int nintfc,
                          const double *wk, double wscale, zd *out, long long out_sk, long long out_sc,
                          int nk, int nc, int ehsplit, cudaStream_t st);
void launch_pair_sum(const zd *tauf, int nkc, int nc, int nintfc, int lk, const int *cls_of_g, int ngeff,
                     int npair, const int *pairs, const double *vecs, const double *a0mat, const double *xk,
                     zd *acc_ij, zd *acc_ji, cudaStream_t st);
// CPA helpers
void launch_layer_dos(int rel, int nd, int nl, int nlay, const zd *tau, int ld, const zd *F,
                      const zd *G, double fac, zd *zmom, zd *zdos_l, cudaStream_t st);
// Bloch spectral function sums of (k, layer) items (k_bsf_reduce)
void launch_bsf_reduce(int nd, int nde, int bdg, int nlay, int nitems, const double *conc, const int *cpa,
                       const zd *del, const zd *M, long long msec, const zd *ta, const zd *tb, const zd *F,
                       const zd *Feh, const zd *P, double fac, double *out, cudaStream_t st);
void launch_cpa_mix(const zd *X, const double *conc, const int *act, int lk, int nl, zd *xc,
                    cudaStream_t st);

// split-precision engine (kernels_mixed.cu)
struct MixedWork;
MixedWork *mixed_create();
void mixed_destroy(MixedWork *w);
int mixed_error_flag(MixedWork *w);
int *mixed_error_ptr(MixedWork *w);   // device flag set by an expired tensor-core wait
// autotuned FP32 Gauss-Jordan layouts: force layout v - 1 for every size
// class (v > 0), or tune afresh (v = 0); the layouts chosen so far
int gj_tune_force(int v);
#include <string>
std::string gj_tune_report();
// kernels run so far by the IF bodies of captured further Newton steps
// (device count since mixed_resid_reset; synchronizes st)
long long mixed_graph_kernels(MixedWork *w, cudaStream_t st);
// conditional graph nodes inside a stream capture (kernels_mixed.cu): a
// handle on the graph being captured, then an IF / WHILE node after the
// stream's current work whose body is captured on `side` until cond_end
int cond_handle(cudaStream_t st, cudaGraphConditionalHandle *h);
int cond_begin(cudaStream_t st, cudaStream_t side, cudaGraphConditionalHandle h, int type);
int cond_end(cudaStream_t side);
bool stream_capturing(cudaStream_t st);
// modes as launch_zgemm plus 4: C = I - A*B, 5: C = C + A*B; S = slices (3..7)
// Split operands live in MIXED_SLOTS staging slots per side (0: A, 1: B);
// slot 0 is the one mixed_zgemm / mixed_zgemm_k / mixed_zinv use.  Splitting
// once and multiplying several times reuses an operand's slices.
constexpr int MIXED_SLOTS = 6;
// further Newton steps (at most) for inverses left above the residual limit
constexpr int NEWTON_EXTRA = 4;
// A B operand (side 1) is recorded, not split, when products form their B
// tiles themselves (mixed_set_fused, the default), unless `reused`: an operand
// that several products read is split once into its slot instead
int mixed_split(MixedWork *w, int side, int slot, int S, const MatRef &M, int n, int K, int nk, int nc,
                const int *act, cudaStream_t st, bool reused = false);
// products of 6+ slices on 64-column tiles with 7 TMEM accumulators (levels
// 0..5 exact): rounding below FP64's, for ill-conditioned energies
void mixed_set_precise(MixedWork *w, bool on);
// the 2 x 2 block FP32 start of inverses above 64 rows (default on)
void mixed_set_blocked(MixedWork *w, bool on);
// B operands formed by the products themselves (default on)
void mixed_set_fused(MixedWork *w, bool on);
int mixed_gemm_staged(MixedWork *w, int mode, int S, int sa, int sb, const MatRef &C, const MatRef &D,
                      const MatRef &E, int n, int K, int nk, int nc, const int *act, cudaStream_t st);
// C (op) A[:, 0:K] B[0:K, :] for n x K by K x n blocks (A, B already offset
// to the K range): the operand scales cover these K columns / rows only
int mixed_zgemm_k(MixedWork *w, int mode, int S, const MatRef &A, const MatRef &B, const MatRef &C,
                  const MatRef &D, const MatRef &E, int n, int K, int nk, int nc, const int *act,
                  cudaStream_t st);
int mixed_zgemm(MixedWork *w, int mode, int S, const MatRef &A, const MatRef &B, const MatRef &C,
                const MatRef &D, const MatRef &E, int n, int nk, int nc, const int *act, cudaStream_t st);
int mixed_zinv(MixedWork *w, const MatRef &A, const MatRef &X, int n, int nk, int nc, const int *act,
               int newton, int sres, bool inplace, cudaStream_t st);
// running maximum of the accepted Newton residual norms and the count of
// inverses redone in FP64 (device scalars), and the count of inverses that
// took further Newton steps (host): reset asynchronously, read with a
// stream synchronisation
int mixed_resid_reset(MixedWork *w, cudaStream_t st);
int mixed_resid_read(MixedWork *w, double *out, long long *fallbacks, long long *refined, cudaStream_t st);

// dense tanh MLP of the learned CPA warm start (kernels_mlp.cu), FP64,
// row-major H[n][d], W[din][dout]
void mlp_launch_dense(const double *H, int n, int din, const double *W, const double *b, int dout, int act,
                      double *A, cudaStream_t st);
// rowsum, dY (may be null) and out[0] = scale * sum of squared errors over
// the rows with sel[r] == want (sel null: all rows); dY = scale * 2 (Yh - Y)
void mlp_launch_loss(const double *Yh, const double *Y, const unsigned char *sel, int want, int n, int dout,
                     double scale, double *dY, double *rowsum, double *out, cudaStream_t st);
void mlp_launch_tanh_back(const double *A, double *G, long long m, cudaStream_t st);
void mlp_launch_wgrad(const double *H, const double *dZ, int n, int din, int dout, double *g, cudaStream_t st);
void mlp_launch_hgrad(const double *dZ, const double *W, int n, int din, int dout, double *dH, cudaStream_t st);
void mlp_launch_adamw(double *p, const double *g, double *m, double *v, long long np, double lr, double wd,
                      double b1, double b2, double eps, double step_size, double bc2_sqrt, cudaStream_t st);
void mlp_launch_keep_best(const double *val, const double *train, double *best, const double *p, double *pbest,
                          long long np, cudaStream_t st);

// the warm-start network with BF16 weights and FP32 activations
// (kernels_mlp16.cu): Z = act(H W16 + b), dH = dZ W16^T, the packed W-then-b
// gradient with its row sum split into nsplit ordered ranges (part:
// [nsplit][din][dout] scratch), loss, tanh', AdamW on the FP32 masters with
// their BF16 copies refreshed
struct __nv_bfloat16;
void mlp16_dense(const float *H, int n, int din, const __nv_bfloat16 *W16, const float *b, int dout, int act, float *Z,
                 cudaStream_t st);
void mlp16_hgrad(const float *dZ, int n, int din, int dout, const __nv_bfloat16 *W16, float *dH, cudaStream_t st);
void mlp16_wgrad(const float *H, const float *dZ, int n, int din, int dout, float *g, float *part, int nsplit,
                 cudaStream_t st);
void mlp16_loss(const float *Yh, const float *Y, const unsigned char *sel, int want, int n, int dout, float scale,
                float *dY, float *rowsum, float *out, cudaStream_t st);
void mlp16_tanh_back(const float *A, float *G, long long m, cudaStream_t st);
void mlp16_adamw(float *p, const float *g, float *m, float *v, __nv_bfloat16 *p16, long long np, float lr, float wd,
                 float b1, float b2, float eps, float step_size, float bc2_sqrt, cudaStream_t st);
void mlp16_to_bf16(const float *p, __nv_bfloat16 *q, long long np, cudaStream_t st);
void mlp16_keep_best(const float *val, const float *train, float *best, const float *p, float *pbest, long long np,
                     cudaStream_t st);

// Kambe lattice sums D_L(k, s) (kernels_kambe.cu): out[item][(lmax2+1)^2] complex
void launch_kambe_dlm(int nitem, double er, double ei, const double *kxy, const double *sep, int lmax2,
                      const double *gvec, int ng, const double *rvec, int nr, double area, double factor,
                      double gcut, double rcut, double *out, cudaStream_t st);
// layer-pair blocks alm(k, s) (kernels_kambe.cu): out[item][lmmax][lmmax]
// complex, coef from skkr_gpu_kambe_coef; items with far[item % nsep] != 0
// are left to launch_directg (far may be null: every item here)
void launch_kambe_alm(int nitem, double er, double ei, const double *kxy, const double *sep, int lmax,
                      const double *gvec, int ng, const double *rvec, int nr, double area, double factor,
                      double gcut, double rcut, const double *coef, const int *far, int nsep, double *out,
                      cudaStream_t st);
// the plane-wave form (directg.f) of the blocks of the items with
// far[item % nsep] != 0, same layout
void launch_directg(int nitem, double er, double ei, const double *kxy, const double *sep, int lmax,
                    const double *gvec, int ng, double area, const int *far, int nsep, double *out,
                    cudaStream_t st);
// slab screening of the reference's k-space form (kernels_kambe.cu):
// G and A = 1 - alpha G per k from the layer-pair blocks, and the central
// layer offsets of X = G A^-1
void launch_slab_assemble(int nk, int nl, int lm, const zd *alm, const int *pmap, int nsep, const double *kxy,
                          const double *pos, const zd *alpha, int nal, zd *G, zd *A, cudaStream_t st);
void launch_slab_extract(int nk, int nl, int lm, int centre, int jmax, const zd *X, zd *out, cudaStream_t st);
// the central offsets straight into the structure-constant cache: block
// blk[j] of each k (column-major lm x lm, nbk blocks per k)
void launch_slab_cache(int nk, int nl, int lm, int centre, int jmax, const int *blk, int nbk, const zd *X, zd *Gc,
                       cudaStream_t st);
// the (k, separation) items of the lattice sums: xk[it / nsep], seps[it % nsep]
void launch_kambe_items(int nk, int nsep, const double *xk, const double *seps, double *ik, double *is,
                        cudaStream_t st);

