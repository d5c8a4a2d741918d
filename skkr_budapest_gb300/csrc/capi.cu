// C ABI and host orchestration of the 2D-BZ tau / CPA path.
//
// One context owns the device state that the reference keeps in Fortran
// `save` arrays (rsp-scf/cpacoord_ksave.f:86: xsave, ysave, g2d): the
// structure-constant blocks of every k and the surface scattering-path
// operators of every k, which the CPA iterations after the first reuse.
// All dense work runs in the batched kernels of kernels_fp64.cu (FP64 path)
// or kernels_mixed.cu (split precision); the host only sequences launches
// and reads back small control values (decimation / CPA convergence).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <thread>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/skkr_gpu.h"
#include "kernels.h"
#include "kambe_dev.cuh"

thread_local long long g_skkr_launches = 0;
thread_local long long g_skkr_if_captured = 0;
static thread_local std::string g_last_error;

#define CK(x)                                                                          \
  do {                                                                                 \
    cudaError_t e_ = (x);                                                              \
    if (e_ != cudaSuccess) {                                                           \
      g_last_error = std::string(#x) + ": " + cudaGetErrorString(e_);                 \
      return SKKR_ERR_CUDA;                                                            \
    }                                                                                  \
  } while (0)
#define CKR(x)                      \
  do {                              \
    int r_ = (x);                   \
    if (r_ != SKKR_OK) return r_;   \
  } while (0)

extern "C" const char *skkr_gpu_last_error(void) { return g_last_error.c_str(); }

std::recursive_mutex &skkr_device_mutex() {
  static std::recursive_mutex m;
  return m;
}

static int g_sync_check = -1;
// ---- per-kernel-class event timing --------------------------------------
namespace {
// shared by all host threads (contexts may run concurrently): guarded by mu;
// each thread keeps the slot of its own open begin/end pair
struct KStats {
  std::mutex mu;
  int on = 0;
  std::vector<cudaEvent_t> ev;
  size_t used = 0;
  std::vector<int> cls;
  std::vector<double> work, work2;
  std::vector<char> done;   // end event recorded
};
KStats g_ks;
thread_local long long g_active_hint = -1;
thread_local long long g_ks_open = -1;
}  // namespace

void skkr_set_active_items(long long n) { g_active_hint = n; }
long long skkr_active_items(long long all) { return g_active_hint >= 0 ? g_active_hint : all; }

void kstat_begin2(int cls, double work, double work2, cudaStream_t st) {
  if (!g_ks.on) return;
  std::lock_guard<std::mutex> lk(g_ks.mu);
  if (!g_ks.on) return;
  if (g_ks.used + 2 > g_ks.ev.size()) {
    for (int i = 0; i < 256; i++) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      g_ks.ev.push_back(e);
    }
  }
  g_ks_open = (long long)g_ks.used;
  cudaEventRecord(g_ks.ev[g_ks.used], st);
  g_ks.cls.push_back(cls);
  g_ks.work.push_back(work);
  g_ks.work2.push_back(work2);
  g_ks.done.push_back(0);
  g_ks.used += 2;
}

void kstat_begin(int cls, double work, cudaStream_t st) { kstat_begin2(cls, work, work, st); }

// per-launch events and the per-launch synchronisation check record every
// launch from the host: the decimation then runs without graphs
static bool launches_observed() { return g_ks.on || g_sync_check == 1; }

void kstat_end(cudaStream_t st) {
  if (g_ks_open < 0) return;
  std::lock_guard<std::mutex> lk(g_ks.mu);
  if (g_ks.on && (size_t)g_ks_open + 1 < g_ks.used) {
    cudaEventRecord(g_ks.ev[g_ks_open + 1], st);
    g_ks.done[g_ks_open / 2] = 1;
  }
  g_ks_open = -1;
}

// enable=1: reset and start; enable=0: stop and report out[cls*4 + {0 launches,
// 1 total ms, 2 total work, 3 total FP64-equivalent algorithmic work}] for the
// KS_NCLS classes.
extern "C" int skkr_gpu_kernel_stats(int enable, double *out) {
  std::lock_guard<std::mutex> lk(g_ks.mu);
  if (enable) {
    g_ks.on = 1;
    g_ks.used = 0;
    g_ks.cls.clear();
    g_ks.work.clear();
    g_ks.work2.clear();
    g_ks.done.clear();
    return SKKR_OK;
  }
  g_ks.on = 0;
  CK(cudaDeviceSynchronize());
  if (out)
    for (int i = 0; i < KS_NCLS * 4; i++) out[i] = 0.0;
  for (size_t i = 0; i < g_ks.cls.size() && 2 * i + 1 < g_ks.used; i++) {
    if (!g_ks.done[i]) continue;
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, g_ks.ev[2 * i], g_ks.ev[2 * i + 1]));
    if (out) {
      out[g_ks.cls[i] * 4 + 0] += 1.0;
      out[g_ks.cls[i] * 4 + 1] += ms;
      out[g_ks.cls[i] * 4 + 2] += g_ks.work[i];
      out[g_ks.cls[i] * 4 + 3] += g_ks.work2[i];
    }
  }
  return SKKR_OK;
}

static void trace_point(const char *what) {
  if (g_sync_check != 1) return;
  cudaError_t e = cudaPeekAtLastError();
  fprintf(stderr, "skkr trace: %s: %s\n", what, cudaGetErrorString(e));
}
void skkr_after_launch(const char *file, int line) {
  ++g_skkr_launches;
  if (g_sync_check < 0) {
    const char *e = getenv("SKKR_SYNC_CHECK");
    g_sync_check = (e && e[0] == '1') ? 1 : 0;
  }
  if (!g_sync_check) return;
  cudaError_t e1 = cudaGetLastError();
  cudaError_t e2 = cudaDeviceSynchronize();
  if ((e1 != cudaSuccess || e2 != cudaSuccess) && g_last_error.find("launch at") == std::string::npos) {
    g_last_error = std::string("launch at ") + file + ":" + std::to_string(line) + ": " +
                   cudaGetErrorString(e1 != cudaSuccess ? e1 : e2);
    fprintf(stderr, "skkr: %s\n", g_last_error.c_str());
  }
}

namespace {

// growable device buffer
// The library stream is non-blocking, so cudaFree does not wait for its
// queued kernels: a buffer is freed (to grow it, or on release) only after the
// device is idle.  Growth is rare; steady state never frees.
struct DBuf {
  void *p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes) {
    if (bytes <= cap) return SKKR_OK;
    std::lock_guard<std::recursive_mutex> lk(skkr_device_mutex());
    if (p) {
      cudaDeviceSynchronize();
      cudaFree(p);
    }
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
      g_last_error = std::string("cudaMalloc: ") + cudaGetErrorString(e);
      return SKKR_ERR_NOMEM;
    }
    cap = bytes;
    return SKKR_OK;
  }
  template <class T>
  T *as() const { return (T *)p; }
  void release() {
    if (p) {
      std::lock_guard<std::recursive_mutex> lk(skkr_device_mutex());
      cudaDeviceSynchronize();
      cudaFree(p);
    }
    p = nullptr;
    cap = 0;
  }
};

// The reference's screened structure constants G_scr(k) (main/gstore.f:146-282
// with main/scrstr.f:2-138, main/scrinv.f) on the device for batches of k
// points: the Kambe lattice sums once per distinct layer separation of the
// slab (kamstr.f), the slab G and 1 - alpha G through the pair map, the
// batched Gauss-Jordan inverse (N = nl (lmax+1)^2 <= 512) and the product
// X = G (1 - alpha G)^-1.  setup() takes the lattice and slab once, screen()
// runs one batch of k points whose coordinates are already on the device.
struct KambeDev {
  int lmax = 0, lm = 0, nl = 0, N = 0, nsep = 0, ng = 0, nr = 0, centre = 0, jmax = 0;
  double er = 0, ei = 0, area = 0, factor = 1, gcut = 0, rcut = 0;
  int nfar = 0;
  DBuf gvec, rvec, coef, pos, alpha, seps, pmap, far, ik, is, alm, Gs, A, X;

  void release() {
    DBuf *all[] = {&gvec, &rvec, &coef, &pos, &alpha, &seps, &pmap, &far, &ik, &is, &alm, &Gs, &A, &X};
    for (DBuf *b : all) b->release();
  }
  size_t per_k() const {
    return (size_t)nsep * lm * lm * sizeof(zd) + 3 * (size_t)N * N * sizeof(zd) + (size_t)nsep * 5 * sizeof(double);
  }
  int setup(double e_re, double e_im, int lmax_, int nl_, const double *pos_h, const double *alpha_h, int centre_,
            int jmax_, const double *gvec_h, int ng_, const double *rvec_h, int nr_, double area_, double factor_,
            double gcut_, double rcut_, cudaStream_t st);
  int screen(const double *xk, int m, cudaStream_t st);
};

}  // namespace

int KambeDev::setup(double e_re, double e_im, int lmax_, int nl_, const double *pos_h, const double *alpha_h,
                    int centre_, int jmax_, const double *gvec_h, int ng_, const double *rvec_h, int nr_, double area_,
                    double factor_, double gcut_, double rcut_, cudaStream_t st) {
  if (nl_ < 1 || !pos_h || !alpha_h || !gvec_h || !rvec_h || ng_ < 1 || nr_ < 1) return SKKR_ERR_ARG;
  if (lmax_ < 0 || lmax_ > 3 || !(area_ > 0.0) || !(factor_ > 0.0) || !(gcut_ > 0.0) || !(rcut_ > 0.0))
    return SKKR_ERR_ARG;
  if (e_re == 0.0 && e_im == 0.0) return SKKR_ERR_ARG;
  lmax = lmax_;
  lm = (lmax + 1) * (lmax + 1);
  nl = nl_;
  N = nl * lm;
  if (N > 512 || jmax_ < 0 || centre_ - jmax_ < 0 || centre_ + jmax_ >= nl) return SKKR_ERR_ARG;
  er = e_re;
  ei = e_im;
  centre = centre_;
  jmax = jmax_;
  ng = ng_;
  nr = nr_;
  area = area_;
  factor = factor_;
  gcut = gcut_;
  rcut = rcut_;
  // distinct separations pos_a - pos_b (to 1e-9 a.u.) and the pair map
  std::vector<double> sv;
  std::vector<int> pm((size_t)nl * nl);
  for (int a = 0; a < nl; a++)
    for (int b = 0; b < nl; b++) {
      double d[3];
      for (int c = 0; c < 3; c++) d[c] = pos_h[3 * a + c] - pos_h[3 * b + c];
      int f = -1;
      for (size_t q = 0; q < sv.size() / 3 && f < 0; q++)
        if (std::fabs(sv[3 * q] - d[0]) < 1e-9 && std::fabs(sv[3 * q + 1] - d[1]) < 1e-9 &&
            std::fabs(sv[3 * q + 2] - d[2]) < 1e-9)
          f = (int)q;
      if (f < 0) {
        f = (int)(sv.size() / 3);
        sv.insert(sv.end(), d, d + 3);
      }
      pm[(size_t)a * nl + b] = f;
    }
  nsep = (int)(sv.size() / 3);
  // gstore.f:158-166: pairs with |s_z| |b|_min >= 5 take the plane-wave form
  // of directg.f; |b|_min is the shortest nonzero vector of the g list
  double bmin = 0.0;
  for (int q = 0; q < ng_; q++) {
    const double b = std::hypot(gvec_h[2 * q], gvec_h[2 * q + 1]);
    if (b > 1e-9 && (bmin == 0.0 || b < bmin)) bmin = b;
  }
  std::vector<int> fr(nsep);
  nfar = 0;
  for (int q = 0; q < nsep; q++) {
    fr[q] = std::fabs(sv[3 * q + 2]) * bmin >= 5.0;
    nfar += fr[q];
  }
  const int lm2 = (2 * lmax + 1) * (2 * lmax + 1);
  std::vector<double> cf(2 * (size_t)lm * lm * lm2);
  CKR(skkr_gpu_kambe_coef(lmax, cf.data()));
  CKR(gvec.ensure(2 * (size_t)ng * sizeof(double)));
  CKR(rvec.ensure(2 * (size_t)nr * sizeof(double)));
  CKR(coef.ensure(cf.size() * sizeof(double)));
  CKR(pos.ensure(3 * (size_t)nl * sizeof(double)));
  CKR(alpha.ensure((size_t)nl * (lmax + 1) * sizeof(zd)));
  CKR(seps.ensure(sv.size() * sizeof(double)));
  CKR(pmap.ensure(pm.size() * sizeof(int)));
  CKR(far.ensure(fr.size() * sizeof(int)));
  CK(cudaMemcpyAsync(far.p, fr.data(), fr.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(gvec.p, gvec_h, 2 * (size_t)ng * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(rvec.p, rvec_h, 2 * (size_t)nr * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(coef.p, cf.data(), cf.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(pos.p, pos_h, 3 * (size_t)nl * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(alpha.p, alpha_h, (size_t)nl * (lmax + 1) * sizeof(zd), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(seps.p, sv.data(), sv.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(pmap.p, pm.data(), pm.size() * sizeof(int), cudaMemcpyHostToDevice, st));
  CK(cudaStreamSynchronize(st));  // cf, sv, pm, fr are host temporaries
  return SKKR_OK;
}

int KambeDev::screen(const double *xk, int m, cudaStream_t st) {
  const long long items = (long long)m * nsep, NN = (long long)N * N;
  CKR(ik.ensure((size_t)items * 2 * sizeof(double)));
  CKR(is.ensure((size_t)items * 3 * sizeof(double)));
  CKR(alm.ensure((size_t)items * lm * lm * sizeof(zd)));
  CKR(Gs.ensure((size_t)m * NN * sizeof(zd)));
  CKR(A.ensure((size_t)m * NN * sizeof(zd)));
  CKR(X.ensure((size_t)m * NN * sizeof(zd)));
  launch_kambe_items(m, nsep, xk, seps.as<double>(), ik.as<double>(), is.as<double>(), st);
  launch_kambe_alm((int)items, er, ei, ik.as<double>(), is.as<double>(), lmax, gvec.as<double>(), ng,
                   rvec.as<double>(), nr, area, factor, gcut, rcut, coef.as<double>(), far.as<int>(), nsep,
                   alm.as<double>(), st);
  if (nfar > 0)
    launch_directg((int)items, er, ei, ik.as<double>(), is.as<double>(), lmax, gvec.as<double>(), ng, area,
                   far.as<int>(), nsep, alm.as<double>(), st);
  launch_slab_assemble(m, nl, lm, alm.as<zd>(), pmap.as<int>(), nsep, xk, pos.as<double>(), alpha.as<zd>(), lmax + 1,
                       Gs.as<zd>(), A.as<zd>(), st);
  launch_zgj(mref(A.as<zd>(), NN, 0, N), N, m, 1, nullptr, st);
  MatRef x = mref(X.as<zd>(), NN, 0, N);
  launch_zgemm(0, mref(Gs.as<zd>(), NN, 0, N), mref(A.as<zd>(), NN, 0, N), x, x, x, N, N, N, m, 1, nullptr, st);
  return SKKR_OK;
}

struct skkr_ctx {
  skkr_sizes sz;
  int lk = 0, lmmax = 0, pl = 0, n = 0, nintfc = 0, nprc = 0, ngeff = 1;
  int dev = 0;    // CUDA device current at creation
  cudaStream_t st = nullptr;
  // staged energy
  int staged = 0;
  int nk = 0, nblk = 0, nrt = 0, nslot = 0, mi = 0, jmax = 0, maxr = 0;
  int nbk = 0;    // structure-constant blocks per k (BdG: electron then hole, 2 nblk)
  zd fac, ce;
  zd fach = {1.0, 0.0};  // BdG: relmtrx factor of the hole block
  std::vector<int> blkmap;
  std::vector<double> conc_h;
  DBuf gR, rvec, rstart, blkmap_d, xk, wk, lg, rg, conc;
  DBuf tcat;      // [nl + nr + nintfc][lk^2]: lead L, lead R, interface coherent
  DBuf tab;       // [nintfc][2][lk^2]: species A, B
  DBuf trot, trtmp;  // [ngeff][nlay][lk^2]
  DBuf pnorm;     // sorttmat / compmat norms
  // per-energy caches over all k
  DBuf G;         // [nk][nbk][lmmax^2]
  DBuf sspo;      // [nk][nsl][n^2]
  // chunk work
  DBuf pool, jobs, dec, decf, deci, tauw, tauk;
  DBuf S, T1, T2, tauc, cpa, cpan, cpaact;
  std::vector<PackJob> jobs_h;
  int nmat = 0;
  int idx00 = 0, idx10 = 0, idx01 = 0, idxmtL = 0, idxmtR = 0;
  // classes (rsp-scf/sorttmat.f)
  std::vector<int> ieqg, ieqgl, ieqgr, igordl, igordr;
  int nsl = 0;    // SSPO slots (L then R)
  int nls = 0;    // left-lead SSPO slots
  int kc = 0;     // chunk size
  // status accumulation
  int max_dec = 0;
  long long tot_dec = 0;
  int first_bad_k = -1;
  int err_code = 0;
  std::vector<struct SlotStore *> slots;
  MixedWork *mw = nullptr;   // split-precision engine (precision == SKKR_MIXED)
  int slices = 6, slices_res = 7;  // BF16 slices of products / of Newton residuals
  // split-precision policy near the real axis (skkr_gpu_set_mixed_policy)
  double dec_fp64_im = 2.0e-4;   // decimation in FP64 when |Im E| is below
  double near_im = 1.0e-3;       // products use slices_near when |Im E| is below
  int slices_near = 7;
  double dominant_frac = 1.0e-2; // k points carrying more of |sum_k tau_k| are redone in FP64
  bool force_fp64 = false;       // set while such a k point is redone
  DBuf knorm;                    // [nk] norms of the k-resolved tau contributions
  long long k_fp64 = 0;          // k points redone in FP64 in this run
  skkr_reduce_fn red_fn = nullptr;  // host allreduce of tauc for a k-split energy
  void *red_user = nullptr;
  skkr_reduce_dev_fn red_dev_fn = nullptr;  // the same on a device buffer (NCCL)
  void *red_dev_user = nullptr;
  DBuf redd;                                // [2 nz + 1] doubles handed to red_dev_fn
  std::vector<double> red_buf;
  double max_resid = 0.0;    // largest accepted Newton residual seen in this run
  long long inv_fallbacks = 0;  // inverses redone in FP64 in this run
  long long inv_refined = 0;    // inverses that took further Newton steps in this run
  double alg_units = 0.0;       // reference block operations (8 n^3 FLOP each) of this run
  bool graphs = true;           // decimation loop as a CUDA graph WHILE node (skkr_gpu_set_graphs)
  int newton = 2;               // standard Newton steps of the split-precision inverse (skkr_gpu_set_newton)
  int blocked_start = 1;        // 2 x 2 block FP32 start above 64 rows (skkr_gpu_set_inverse_start)
  int fused_b = 1;              // B operands formed inside the sliced products (skkr_gpu_set_fused_split)
  DBuf decctl;                  // [0] iteration, [1] items left, [2] half-bodies run (captured loop)
  long long graph_kernels = 0;  // kernels run inside graphs in this run
  long long graph_launches = 0; // graph launches in this run
  // the reference's k-space G_scr(k) in place of the table transform for the
  // energy staged last (skkr_gpu_stage_kambe)
  bool kambe_on = false;
  KambeDev kd;
  DBuf kblk;                    // [2 jmax + 1] cache block of each layer offset, or -1
};

// Inputs and outputs of one staged energy.  A context keeps any number of
// them resident on the device (skkr_gpu_stage_slot); run/fetch swap a slot
// into the working fields, so the per-energy work buffers are shared.
struct SlotStore {
  DBuf gR, rvec, rstart, blkmap_d, xk, wk, lg, rg, conc, tcat, tab, tauc, cpa;
  int staged = 0, nk = 0, nblk = 0, nrt = 0, nslot = 0, mi = 0, jmax = 0, maxr = 0, nbk = 0;
  zd fac = {0, 0}, ce = {0, 0}, fach = {1, 0};
  std::vector<int> blkmap;
  std::vector<double> conc_h;
};

static void swap_slot(skkr_ctx *c, SlotStore &s) {
  std::swap(c->gR, s.gR);
  std::swap(c->rvec, s.rvec);
  std::swap(c->rstart, s.rstart);
  std::swap(c->blkmap_d, s.blkmap_d);
  std::swap(c->xk, s.xk);
  std::swap(c->wk, s.wk);
  std::swap(c->lg, s.lg);
  std::swap(c->rg, s.rg);
  std::swap(c->conc, s.conc);
  std::swap(c->tcat, s.tcat);
  std::swap(c->tab, s.tab);
  std::swap(c->tauc, s.tauc);
  std::swap(c->cpa, s.cpa);
  std::swap(c->staged, s.staged);
  std::swap(c->nk, s.nk);
  std::swap(c->nblk, s.nblk);
  std::swap(c->nbk, s.nbk);
  std::swap(c->fach, s.fach);
  std::swap(c->nrt, s.nrt);
  std::swap(c->nslot, s.nslot);
  std::swap(c->mi, s.mi);
  std::swap(c->jmax, s.jmax);
  std::swap(c->maxr, s.maxr);
  std::swap(c->fac, s.fac);
  std::swap(c->ce, s.ce);
  std::swap(c->blkmap, s.blkmap);
  std::swap(c->conc_h, s.conc_h);
}

// ---------------------------------------------------------------------------
extern "C" int skkr_gpu_create(const skkr_sizes *sizes, skkr_ctx **out) {
  if (!sizes || !out) return SKKR_ERR_ARG;
  const skkr_sizes &s = *sizes;
  if (s.mode != SKKR_NONREL && s.mode != SKKR_REL && s.mode != SKKR_BDG) return SKKR_ERR_ARG;
  if (s.lmax < 0 || s.lmax > 3 || s.nprc < 1 || s.nprc > SKKR_MAX_PRC) return SKKR_ERR_ARG;
  if (s.ngeff < 1 || s.ngeff > 8) return SKKR_ERR_ARG;
  if (s.precision != SKKR_FP64 && s.precision != SKKR_MIXED) return SKKR_ERR_ARG;
  // uniform principal layers (the reference's dugo.f bulk branch sizes both
  // leads with ninprc(1); tau2d.f then needs ninprc(1)=ninprc(nprc))
  for (int i = 0; i <= s.nprc + 1; i++)
    if (s.ninprc[i] != s.ninprc[1] || s.ninprc[i] < 1) return SKKR_ERR_UNSUPPORTED;
  skkr_ctx *c = new skkr_ctx();
  c->sz = s;
  c->lmmax = (s.lmax + 1) * (s.lmax + 1);
  c->lk = s.mode == SKKR_BDG ? 4 * c->lmmax : s.mode == SKKR_REL ? 2 * c->lmmax : c->lmmax;
  c->pl = s.ninprc[1];
  c->n = c->pl * c->lk;
  c->nprc = s.nprc;
  c->nintfc = c->pl * s.nprc;
  c->ngeff = s.ngeff;
  if (s.slices != 0) {
    if (s.slices < 3 || s.slices > 8) {
      delete c;
      return SKKR_ERR_ARG;
    }
    c->slices = s.slices;
    c->slices_res = s.slices < 8 ? s.slices + 1 : 8;
  }
  if (c->n > 256) {
    delete c;
    return SKKR_ERR_UNSUPPORTED;
  }
  if (cudaGetDevice(&c->dev) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return SKKR_ERR_CUDA;
  }
  // always the full (kappa,mu) tables: contexts of different modes may be
  // alive at once and the lm packer never reads them
  cudaError_t e = pack_set_tables(1, s.lmax);
  if (e != cudaSuccess) {
    g_last_error = std::string("pack_set_tables: ") + cudaGetErrorString(e);
    cudaStreamDestroy(c->st);
    delete c;
    return SKKR_ERR_CUDA;
  }
  *out = c;
  return SKKR_OK;
}

extern "C" int skkr_gpu_destroy(skkr_ctx *c) {
  if (!c) return SKKR_OK;
  DBuf *all[] = {&c->gR, &c->rvec, &c->rstart, &c->blkmap_d, &c->xk, &c->wk, &c->lg, &c->rg,
                 &c->conc, &c->tcat, &c->tab, &c->trot, &c->trtmp, &c->pnorm, &c->G, &c->sspo,
                 &c->pool, &c->jobs, &c->dec, &c->decf, &c->deci, &c->tauw, &c->tauk, &c->S,
                 &c->T1, &c->T2, &c->tauc, &c->cpa, &c->cpan, &c->cpaact, &c->decctl, &c->knorm,
                 &c->redd};
  for (DBuf *b : all) b->release();
  c->kd.release();
  c->kblk.release();
  if (c->mw) mixed_destroy(c->mw);
  for (SlotStore *sl : c->slots) {
    DBuf *sb[] = {&sl->gR, &sl->rvec, &sl->rstart, &sl->blkmap_d, &sl->xk, &sl->wk, &sl->lg,
                  &sl->rg, &sl->conc, &sl->tcat, &sl->tab, &sl->tauc, &sl->cpa};
    for (DBuf *b : sb) b->release();
    delete sl;
  }
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return SKKR_OK;
}

// copy ld-strided column-major host matrices into packed lk x lk device blocks
static int put_mats(DBuf &dst, size_t off_elems, const double *src, int count, int lk, int ld,
                    cudaStream_t st) {
  if (count <= 0) return SKKR_OK;
  std::vector<zd> tmp((size_t)count * lk * lk);
  for (int m = 0; m < count; m++)
    for (int c = 0; c < lk; c++)
      for (int r = 0; r < lk; r++) {
        size_t s = ((size_t)m * ld * ld + r + (size_t)c * ld) * 2;
        tmp[(size_t)m * lk * lk + r + (size_t)c * lk] = zmk(src[s], src[s + 1]);
      }
  CK(cudaMemcpyAsync(dst.as<zd>() + off_elems, tmp.data(), tmp.size() * sizeof(zd),
                     cudaMemcpyHostToDevice, st));
  CK(cudaStreamSynchronize(st));
  return SKKR_OK;
}

static int get_mats(double *dst, const zd *src_dev, int count, int lk, int ld, cudaStream_t st,
                    long long src_stride = -1) {
  if (count <= 0) return SKKR_OK;
  long long sstride = src_stride < 0 ? (long long)lk * lk : src_stride;
  std::vector<zd> tmp((size_t)(count - 1) * sstride + (size_t)lk * lk);
  CK(cudaMemcpyAsync(tmp.data(), src_dev, tmp.size() * sizeof(zd), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  for (int m = 0; m < count; m++)
    for (int c = 0; c < lk; c++)
      for (int r = 0; r < lk; r++) {
        zd v = tmp[(size_t)m * sstride + r + (size_t)c * lk];
        size_t d = ((size_t)m * ld * ld + r + (size_t)c * ld) * 2;
        dst[d] = v.x;
        dst[d + 1] = v.y;
      }
  return SKKR_OK;
}

// ---------------------------------------------------------------------------
extern "C" int skkr_gpu_stage(skkr_ctx *c, double ce_re, double ce_im, double fac_re,
                              double fac_im, const skkr_rtable *rt, int nk, const double *xk,
                              const double *wk, const double *lg, const double *rg,
                              const double *conc, const double *tminvl, const double *tminvr,
                              const double *tminv, const double *tminva, const double *tminvb,
                              int ld) {
  if (!c || !rt || nk < 1 || !xk || !wk || !lg || !rg || !conc || !tminvl || !tminvr || !tminv ||
      !tminva || !tminvb)
    return SKKR_ERR_ARG;
  if (ld < c->lk) return SKKR_ERR_ARG;
  if (rt->nslot < c->nprc + 2 || rt->mi < c->pl || rt->nblk < 1 || rt->jmax < 0) return SKKR_ERR_ARG;
  const int lk = c->lk, lk2 = lk * lk, ng = c->ngeff;
  c->ce = zmk(ce_re, ce_im);
  c->fac = zmk(fac_re, fac_im);
  c->nk = nk;
  c->kambe_on = false;  // a new energy starts from its table
  c->nblk = rt->nblk;
  const bool bdg = c->sz.mode == SKKR_BDG;
  c->nbk = bdg ? 2 * rt->nblk : rt->nblk;
  c->nrt = rt->rstart[rt->nblk];
  c->nslot = rt->nslot;
  c->mi = rt->mi;
  c->jmax = rt->jmax;
  c->maxr = 0;
  for (int b = 0; b < rt->nblk; b++) c->maxr = std::max(c->maxr, rt->rstart[b + 1] - rt->rstart[b]);
  if (c->maxr > 64) return SKKR_ERR_UNSUPPORTED;
  const int nj = 2 * rt->jmax + 1;
  c->blkmap.assign(rt->blkmap, rt->blkmap + (size_t)rt->nslot * rt->mi * nj);
  for (int v : c->blkmap)
    if (v >= rt->nblk) return SKKR_ERR_ARG;
  const size_t bs = (size_t)c->lmmax * c->lmmax;
  const int ntab = bdg ? 2 : 1;  // BdG: electron table, then the hole table on the same R
  CKR(c->gR.ensure(ntab * c->nrt * bs * sizeof(zd)));
  CKR(c->rvec.ensure(ntab * c->nrt * 2 * sizeof(double)));
  CKR(c->rstart.ensure((c->nbk + 1) * sizeof(int)));
  CKR(c->blkmap_d.ensure(c->blkmap.size() * sizeof(int)));
  CKR(c->xk.ensure((size_t)nk * 2 * sizeof(double)));
  CKR(c->wk.ensure((size_t)nk * sizeof(double)));
  CKR(c->lg.ensure((size_t)ng * lk2 * sizeof(zd)));
  CKR(c->rg.ensure((size_t)ng * lk2 * sizeof(zd)));
  CKR(c->conc.ensure((size_t)c->nintfc * sizeof(double)));
  const int nlay = 2 * c->pl + c->nintfc;
  CKR(c->tcat.ensure((size_t)nlay * lk2 * sizeof(zd)));
  CKR(c->tab.ensure((size_t)c->nintfc * 2 * lk2 * sizeof(zd)));
  cudaStream_t st = c->st;
  CK(cudaMemcpyAsync(c->gR.p, rt->gR, ntab * c->nrt * bs * sizeof(zd), cudaMemcpyHostToDevice, st));
  {
    // block b >= nblk (hole) reads rows nrt + rstart[b - nblk] .. of the doubled table
    std::vector<int> rs(c->nbk + 1);
    std::vector<double> rv((size_t)ntab * c->nrt * 2);
    for (int b = 0; b <= c->nbk; b++)
      rs[b] = b <= rt->nblk ? rt->rstart[b] : c->nrt + rt->rstart[b - rt->nblk];
    for (int t = 0; t < ntab; t++)
      std::copy(rt->rvec, rt->rvec + (size_t)c->nrt * 2, rv.begin() + (size_t)t * c->nrt * 2);
    CK(cudaMemcpyAsync(c->rvec.p, rv.data(), rv.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(c->rstart.p, rs.data(), rs.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));  // rs / rv are host temporaries
  }
  CK(cudaMemcpyAsync(c->blkmap_d.p, c->blkmap.data(), c->blkmap.size() * sizeof(int),
                     cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->xk.p, xk, (size_t)nk * 2 * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->wk.p, wk, (size_t)nk * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(c->conc.p, conc, (size_t)c->nintfc * sizeof(double), cudaMemcpyHostToDevice, st));
  c->conc_h.assign(conc, conc + c->nintfc);
  CKR(put_mats(c->lg, 0, lg, ng, lk, ld, st));
  CKR(put_mats(c->rg, 0, rg, ng, lk, ld, st));
  CKR(put_mats(c->tcat, 0, tminvl, c->pl, lk, ld, st));
  CKR(put_mats(c->tcat, (size_t)c->pl * lk2, tminvr, c->pl, lk, ld, st));
  CKR(put_mats(c->tcat, (size_t)2 * c->pl * lk2, tminv, c->nintfc, lk, ld, st));
  // species: [layer][2]
  {
    std::vector<zd> tmp((size_t)c->nintfc * 2 * lk2);
    for (int l = 0; l < c->nintfc; l++)
      for (int sdx = 0; sdx < 2; sdx++) {
        const double *src = sdx == 0 ? tminva : tminvb;
        for (int cc = 0; cc < lk; cc++)
          for (int r = 0; r < lk; r++) {
            size_t s = ((size_t)l * ld * ld + r + (size_t)cc * ld) * 2;
            tmp[((size_t)l * 2 + sdx) * lk2 + r + (size_t)cc * lk] = zmk(src[s], src[s + 1]);
          }
      }
    CK(cudaMemcpyAsync(c->tab.p, tmp.data(), tmp.size() * sizeof(zd), cudaMemcpyHostToDevice, st));
  }
  CK(cudaStreamSynchronize(st));
  c->staged = 1;
  return SKKR_OK;
}

// ---------------------------------------------------------------------------
// packing plan: dedupe structure-constant slots with identical block maps
static void plan_pack(skkr_ctx *c) {
  const int nj = 2 * c->jmax + 1, rowlen = c->mi * nj;
  auto canon = [&](int slot) {
    for (int s2 = 0; s2 < slot; s2++)
      if (std::equal(c->blkmap.begin() + (size_t)s2 * rowlen, c->blkmap.begin() + (size_t)(s2 + 1) * rowlen,
                     c->blkmap.begin() + (size_t)slot * rowlen))
        return s2;
    return slot;
  };
  c->jobs_h.clear();
  auto job = [&](int slot, int which) {
    slot = canon(slot);
    for (auto &j : c->jobs_h)
      if (j.slot == slot && j.which == which) return j.dest;
    PackJob j{slot, c->pl, c->pl, c->pl, which, (int)c->jobs_h.size()};
    c->jobs_h.push_back(j);
    return j.dest;
  };
  // bulkgeo: interface PLs use slot 1 (tau2d.f:51-52)
  c->idx00 = job(1, 0);
  c->idx10 = job(1, 1);
  c->idx01 = job(1, 2);
  c->idxmtL = job(0, 2);                  // dugo.f 'L': packer(..,g2d slot 0,..,mt) -> M01
  c->idxmtR = job(c->nprc + 1, 1);        // dugo.f 'R': M10 of the right lead slot
  c->nmat = (int)c->jobs_h.size();
}

// rsp-scf/sorttmat.f on device data: rotate t^-1 by every g, compare.
__global__ void k_pair_norms(const zd *trot, int ng, int nlay, int lk2, double *out) {
  // out[(pair*nlay + layer)*2 + {0: ||x-y||^2, 1: ||x||^2}], pair over iig<ig
  const int layer = blockIdx.y, pair = blockIdx.x;
  int ig = 1, acc = 0;
  while (acc + ig <= pair) { acc += ig; ig++; }
  const int iig = pair - acc;
  const zd *x = trot + ((long long)iig * nlay + layer) * lk2;
  const zd *y = trot + ((long long)ig * nlay + layer) * lk2;
  double dn = 0, xn = 0;
  for (int e = threadIdx.x; e < lk2; e += blockDim.x) {
    zd a = x[e], b = y[e];
    xn += a.x * a.x + a.y * a.y;
    double dx = a.x - b.x, dy = a.y - b.y;
    dn += dx * dx + dy * dy;
  }
  __shared__ double s1[256], s2[256];
  s1[threadIdx.x] = dn;
  s2[threadIdx.x] = xn;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      s1[threadIdx.x] += s1[threadIdx.x + o];
      s2[threadIdx.x] += s2[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[((long long)pair * nlay + layer) * 2] = s1[0];
    out[((long long)pair * nlay + layer) * 2 + 1] = s2[0];
  }
}

static int sorttmat_dev(skkr_ctx *c) {
  const int lk = c->lk, lk2 = lk * lk, ng = c->ngeff;
  const int nl = c->pl, nr = c->pl, ni = c->nintfc, nlay = nl + nr + ni;
  cudaStream_t st = c->st;
  CKR(c->trot.ensure((size_t)ng * nlay * lk2 * sizeof(zd)));
  CKR(c->trtmp.ensure((size_t)ng * nlay * lk2 * sizeof(zd)));
  // tmp[g][layer] = R_g t ; trot[g][layer] = tmp L_g
  MatRef R = mref(c->rg.as<zd>(), 0, lk2, lk);
  MatRef Tc = mref(c->tcat.as<zd>(), lk2, 0, lk);
  MatRef Tm = mref(c->trtmp.as<zd>(), lk2, (long long)nlay * lk2, lk);
  MatRef L = mref(c->lg.as<zd>(), 0, lk2, lk);
  MatRef Tr = mref(c->trot.as<zd>(), lk2, (long long)nlay * lk2, lk);
  launch_zgemm(0, R, Tc, Tm, Tm, Tm, lk, lk, lk, nlay, ng, nullptr, st);
  launch_zgemm(0, Tm, L, Tr, Tr, Tr, lk, lk, lk, nlay, ng, nullptr, st);
  c->ieqg.assign(ng, 1);
  c->ieqgl.assign(ng, 1);
  c->ieqgr.assign(ng, 1);
  c->igordl.assign(ng, 1);
  c->igordr.assign(ng, 1);
  if (ng > 1) {
    const int npair = ng * (ng - 1) / 2;
    CKR(c->pnorm.ensure((size_t)npair * nlay * 2 * sizeof(double)));
    dim3 grid(npair, nlay);
    k_pair_norms<<<grid, 256, 0, st>>>(c->trot.as<zd>(), ng, nlay, lk2, c->pnorm.as<double>());
    SKKR_LAUNCHED();
    std::vector<double> pn((size_t)npair * nlay * 2);
    CK(cudaMemcpyAsync(pn.data(), c->pnorm.p, pn.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    const double tol = 1.0e-8;  // sorttmat.f:27
    auto eq = [&](int iig, int ig, int layer) {
      int pair = ig * (ig - 1) / 2 + iig;
      double dn = pn[((size_t)pair * nlay + layer) * 2], xn = pn[((size_t)pair * nlay + layer) * 2 + 1];
      return std::sqrt(dn) < tol * std::sqrt(xn);  // matops.f compmat
    };
    auto all_eq = [&](int iig, int ig, int l0, int l1) {
      for (int l = l0; l < l1; l++)
        if (!eq(iig, ig, l)) return false;
      return true;
    };
    for (int ig = 1; ig < ng; ig++) {
      int f = -1;
      for (int iig = 0; iig < ig && f < 0; iig++)
        if (all_eq(iig, ig, 0, nl) && all_eq(iig, ig, nl, nl + nr) && all_eq(iig, ig, nl + nr, nlay)) f = iig;
      c->ieqg[ig] = f < 0 ? ig + 1 : f + 1;
    }
    for (int ig = 1; ig < ng; ig++) {
      int f = -1;
      for (int iig = 0; iig < ig && f < 0; iig++)
        if (all_eq(iig, ig, 0, nl)) f = iig;
      if (f < 0) {
        c->ieqgl[ig] = ig + 1;
        c->igordl[ig] = c->igordl[c->ieqgl[ig - 1] - 1] + 1;
      } else c->ieqgl[ig] = f + 1;
    }
    for (int ig = 1; ig < ng; ig++) {
      int f = -1;
      for (int iig = 0; iig < ig && f < 0; iig++)
        if (all_eq(iig, ig, nl, nl + nr)) f = iig;
      if (f < 0) {
        c->ieqgr[ig] = ig + 1;
        c->igordr[ig] = c->igordr[c->ieqgr[ig - 1] - 1] + 1;
      } else c->ieqgr[ig] = f + 1;
    }
  }
  return SKKR_OK;
}

// L/R lead classes computed on the first pass: list of g with ieqgl(g)==g
static void lead_classes(const skkr_ctx *c, std::vector<int> &lg_of, std::vector<int> &rg_of) {
  lg_of.clear();
  rg_of.clear();
  for (int g = 0; g < c->ngeff; g++) {
    if (c->ieqgl[g] == g + 1) lg_of.push_back(g);
    if (c->ieqgr[g] == g + 1) rg_of.push_back(g);
  }
}

static int check_slot_quirk(const skkr_ctx *c) {
  // igordl/igordr must give distinct cache slots to distinct classes; the
  // reference's formula (sorttmat.f:167,191) can collide for non-monotone
  // class patterns, which this library refuses instead of reproducing.
  std::vector<int> seen;
  for (int g = 0; g < c->ngeff; g++)
    if (c->ieqgl[g] == g + 1) {
      int s = c->igordl[g];
      if (std::find(seen.begin(), seen.end(), s) != seen.end()) return SKKR_ERR_UNSUPPORTED;
      seen.push_back(s);
    }
  seen.clear();
  for (int g = 0; g < c->ngeff; g++)
    if (c->ieqgr[g] == g + 1) {
      int s = c->igordr[g];
      if (std::find(seen.begin(), seen.end(), s) != seen.end()) return SKKR_ERR_UNSUPPORTED;
      seen.push_back(s);
    }
  return SKKR_OK;
}

// ---------------------------------------------------------------------------
// engine: the dense operations of decimation and tau2d in FP64 or split
// precision (tcgen05 sliced products, FP32 inverse + Newton refinement)
// electron-first principal-layer layout: BdG on the split-precision path
static int ehsplit(const skkr_ctx *c) {
  return c->sz.mode == SKKR_BDG && c->sz.precision == SKKR_MIXED;
}

// slices of the products of the staged energy (more near the real axis)
static int slices_for(const skkr_ctx *c) {
  return (c->slices_near > 0 && std::fabs(c->ce.y) < c->near_im) ? c->slices_near : c->slices;
}

static MatRef offset(const MatRef &m, long long elems) {
  MatRef r = m;
  r.base += elems;
  return r;
}

static int eng_gemm(skkr_ctx *c, bool mixed, int mode, const MatRef &A, const MatRef &B, const MatRef &C,
                    const MatRef &D, const MatRef &E, int n, int nk, int nc, const int *act) {
  if (mixed && ehsplit(c)) {
    // BdG: A B = A[:, e] B[e, :] + A[:, h] B[h, :] over the electron and hole
    // K halves of the electron-first layout, each half with its own operand
    // scales (the O(delta) e-h blocks keep their full relative precision)
    const int h = n / 2;
    const MatRef A2 = offset(A, (long long)h * A.ld), B2 = offset(B, h);
    int m2;
    switch (mode) {
      case 0: m2 = 5; break;   // C = A1 B1, then C += A2 B2
      case 4: m2 = 1; break;   // C = I - A1 B1, then C -= A2 B2
      default: m2 = mode;      // 1 (C -=), 2 (D -=, E -=), 5 (C +=) are additive per half
    }
    int rc = mixed_zgemm_k(c->mw, mode, slices_for(c), A, B, C, D, E, n, h, nk, nc, act, c->st);
    if (rc) return rc;
    return mixed_zgemm_k(c->mw, m2, slices_for(c), A2, B2, C, D, E, n, h, nk, nc, act, c->st);
  }
  if (mixed) return mixed_zgemm(c->mw, mode, slices_for(c), A, B, C, D, E, n, nk, nc, act, c->st);
  launch_zgemm(mode, A, B, C, D, E, n, n, n, nk, nc, act, c->st);
  return SKKR_OK;
}

// X = A^-1 (X may be the same matrices as A when inplace)
static int eng_inv(skkr_ctx *c, bool mixed, const MatRef &A, const MatRef &X, bool inplace, int n, int nk,
                   int nc, const int *act) {
  if (mixed && n <= 128) {
    mixed_set_blocked(c->mw, c->blocked_start != 0);
    return mixed_zinv(c->mw, A, X, n, nk, nc, act, c->newton,
                      std::min(8, std::max(c->slices_res, slices_for(c) + 1)), inplace, c->st);
  }
  if (!inplace) launch_zaxpby(X, A, nullptr, 0, nullptr, 0, n, nk, nc, act, c->st);
  launch_zgj(X, n, nk, nc, act, c->st);
  return SKKR_OK;
}

static bool use_mixed(const skkr_ctx *c, bool decimation) {
  if (c->sz.precision != SKKR_MIXED || c->force_fp64) return false;
  // decimation near the real axis stays in FP64 (default: within 2e-4 Ry)
  const bool dec_fp64 = std::fabs(c->ce.y) < c->dec_fp64_im;
  if (decimation && dec_fp64) return false;
  // with the decimation in FP64 and blocks above the split inverse's 128
  // rows, only the tau2d products would be split: the splitting and the FP64
  // redo of the integrand's peaks cost more than they save (BdG n_PL = 256 at
  // Im E = 1e-4 Ry ran at 0.74 of the FP64 rate), so the energy runs in FP64
  if (dec_fp64 && c->n > 128) return false;
  return true;
}


// ---------------------------------------------------------------------------
// The decimation iterations from `first` on as one CUDA graph: a WHILE node
// (condition 1 at launch) whose body is two iterations, each followed by
// k_dec_advance (iteration number + 1, loop condition from the count of
// items left).  The body is captured on the context stream into the node's
// graph; the mixed inverse inside it adds IF nodes for its further Newton
// steps.  Kernels run inside the graph are counted from device counters.
template <class Iterate>
static int decimation_graph(skkr_ctx *c, int first, int itermax, Iterate &iterate) {
  cudaStream_t st = c->st;
  // capture, instantiation and launch never overlap a device-synchronising
  // allocation of another host thread
  std::lock_guard<std::recursive_mutex> lk(skkr_device_mutex());
  CKR(c->decctl.ensure(4 * sizeof(int)));
  int *ctl = c->decctl.as<int>();
  const int init[4] = {first, 0, 0, 0};
  CK(cudaMemcpyAsync(ctl, init, sizeof(init), cudaMemcpyHostToDevice, st));
  long long if0 = 0;
  if (c->mw) if0 = mixed_graph_kernels(c->mw, st);  // also completes the copy above
  else CK(cudaStreamSynchronize(st));
  cudaGraph_t G = nullptr;
  cudaGraphExec_t X = nullptr;
  CK(cudaGraphCreate(&G, 0));
  struct Done {
    cudaGraph_t &g;
    cudaGraphExec_t &x;
    ~Done() {
      if (x) cudaGraphExecDestroy(x);
      if (g) cudaGraphDestroy(g);
    }
  } done{G, X};
  cudaGraphConditionalHandle h;
  CK(cudaGraphConditionalHandleCreate(&h, G, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeWhile;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, G, nullptr, nullptr, 0, &p));
  cudaGraph_t body = p.conditional.phGraph_out[0];
  const long long l0 = g_skkr_launches, i0 = g_skkr_if_captured;
  CK(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  const int *errflag = c->mw ? mixed_error_ptr(c->mw) : nullptr;
  int rc = SKKR_OK;
  for (int half = 0; half < 2 && rc == SKKR_OK; half++) {
    rc = iterate(((first + half) & 1) != 0, 0, ctl, ctl + 1);
    if (rc == SKKR_OK) launch_dec_advance(ctl, ctl + 1, itermax, errflag, h, ctl + 2, st);
  }
  cudaGraph_t cap = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(st, &cap);
  // kernels captured into the body (outside the IF bodies), per half
  const long long per_half = (g_skkr_launches - l0) / 2;
  g_skkr_launches = l0;
  g_skkr_if_captured = i0;
  if (rc != SKKR_OK) return rc;
  CK(ec);
  CK(cudaGraphInstantiate(&X, G, 0));
  CK(cudaGraphLaunch(X, st));
  int halves = 0;
  CK(cudaMemcpyAsync(&halves, ctl + 2, sizeof(int), cudaMemcpyDeviceToHost, st));
  long long if1 = 0;
  if (c->mw) if1 = mixed_graph_kernels(c->mw, st);
  else CK(cudaStreamSynchronize(st));
  c->graph_launches += 1;
  c->graph_kernels += per_half * halves + (if1 - if0);
  return SKKR_OK;
}

// ---------------------------------------------------------------------------
// decimation (main/dugo.f + main/surfgf.f) for the k points [k0, k0+nkc)
// items (k, s): s < nLc left-lead classes, then right-lead classes.
static int run_decimation(skkr_ctx *c, int k0, int nkc, const std::vector<int> &lcls,
                          const std::vector<int> &rcls) {
  const int n = c->n, n2 = n * n, lk = c->lk, lk2 = lk * lk, pl = c->pl;
  const int nLc = (int)lcls.size(), nRc = (int)rcls.size(), nc = nLc + nRc;
  const int nit = nkc * nc;
  const long long MB = n2;  // elements per matrix
  CKR(c->dec.ensure((size_t)nit * 9 * MB * sizeof(zd)));
  CKR(c->decf.ensure((size_t)nit * sizeof(double)));
  CKR(c->deci.ensure((size_t)nit * 3 * sizeof(int)));
  cudaStream_t st = c->st;
  zd *W = c->dec.as<zd>();
  // buffers per item: 0 eps, 1 alfa0, 2 alfa1, 3 beta0, 4 beta1, 5 x, 6 y1, 7 P, 8 Q
  auto buf = [&](int b) { return mref(W + (long long)b * MB, (long long)nc * 9 * MB, 9 * MB, n); };
  int *act = c->deci.as<int>(), *stat = act + nit, *iters = act + 2 * nit;
  double *err = c->decf.as<double>();
  zd *poolk = c->pool.as<zd>();
  const long long psk = (long long)c->nmat * MB;
  int mapml[SKKR_MAPN], mapm0[SKKR_MAPN], mapmr[SKKR_MAPN], mapt[SKKR_MAPN], mapmt[SKKR_MAPN],
      mapsl[SKKR_MAPN];
  for (int s = 0; s < nc; s++) {
    bool L = s < nLc;
    int g = L ? lcls[s] : rcls[s - nLc];
    mapml[s] = L ? c->idx10 : c->idx01;
    mapm0[s] = c->idx00;
    mapmr[s] = L ? c->idx01 : c->idx10;
    mapmt[s] = L ? c->idxmtL : c->idxmtR;
    // rotated lead t: trot[g][layer], layers 0..pl-1 left lead, pl..2pl-1 right lead
    mapt[s] = g * 2 + (L ? 0 : 1);
    mapsl[s] = L ? (c->igordl[g] - 1) : (c->nls + c->igordr[g] - 1);
  }
  const int nlay = 2 * pl + c->nintfc;
  MatRef Pml = mref_map(poolk, psk, MB, n, mapml, nc);
  MatRef Pm0 = mref_map(poolk, psk, MB, n, mapm0, nc);
  MatRef Pmr = mref_map(poolk, psk, MB, n, mapmr, nc);
  MatRef Pmt = mref_map(poolk, psk, MB, n, mapmt, nc);
  // trot layout [g][layer][lk2]: item t base = trot + g*nlay*lk2 + side*pl*lk2
  int mapt2[SKKR_MAPN];
  for (int s = 0; s < nc; s++) mapt2[s] = (mapt[s] / 2) * nlay + (mapt[s] % 2) * pl;
  MatRef Tt = mref_map(c->trot.as<zd>(), 0, lk2, lk, mapt2, nc);
  MatRef eps = buf(0), a0 = buf(1), a1 = buf(2), b0 = buf(3), b1 = buf(4), x = buf(5), y1 = buf(6),
         P = buf(7), Q = buf(8);
  // init: eps = m0 + t ; x = eps ; alfa = -ml ; beta = -mr   (surfgf.f:37-45)
  launch_add_tblocks(eps, Pm0, Tt, lk, pl, n, nkc, nc, nullptr, ehsplit(c), st);
  launch_zaxpby(x, eps, nullptr, 0, nullptr, 0, n, nkc, nc, nullptr, st);
  // ml + (-2) ml is exactly -ml in floating point
  launch_zaxpby(a0, Pml, &Pml, -2.0, nullptr, 0, n, nkc, nc, nullptr, st);
  launch_zaxpby(b0, Pmr, &Pmr, -2.0, nullptr, 0, n, nkc, nc, nullptr, st);
  {
    std::vector<int> ones(nit, 1);
    CK(cudaMemcpyAsync(act, ones.data(), nit * sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(stat, 0, nit * sizeof(int), st));
    CK(cudaMemsetAsync(iters, 0, nit * sizeof(int), st));
  }
  const int itermax = std::max(c->sz.itermaxl, c->sz.itermaxr);
  const bool mx = use_mixed(c, true);
  // one iteration (surfgf.f:47-96); the parity picks the alfa / beta buffers
  // read and written; iter_dev: the iteration number lives on the device (the
  // captured loop), else `iter` from the host
  auto iterate = [&](bool odd, int iter, const int *iter_dev, int *nact_dev) -> int {
    MatRef &ac = odd ? a0 : a1, &an = odd ? a1 : a0;
    MatRef &bc = odd ? b0 : b1, &bn = odd ? b1 : b0;
    CKR(eng_inv(c, mx, eps, y1, false, n, nkc, nc, act));              // y1 = eps^-1
    if (mx && !ehsplit(c)) {
      // split-precision engine: each operand split once (B slots 1-3: y1,
      // alfa, beta; A slots 1-4: alfa, beta, P, Q) for the six products
      MixedWork *w = c->mw;
      const int S = slices_for(c);
      CKR(mixed_split(w, 1, 1, S, y1, n, n, nkc, nc, act, st, true));
      CKR(mixed_split(w, 0, 1, S, ac, n, n, nkc, nc, act, st));
      CKR(mixed_split(w, 0, 2, S, bc, n, n, nkc, nc, act, st));
      CKR(mixed_gemm_staged(w, 0, S, 1, 1, P, P, P, n, n, nkc, nc, act, st));        // P = alfa y1
      CKR(mixed_gemm_staged(w, 0, S, 2, 1, Q, Q, Q, n, n, nkc, nc, act, st));        // Q = beta y1
      CKR(mixed_split(w, 1, 2, S, ac, n, n, nkc, nc, act, st, true));
      CKR(mixed_split(w, 1, 3, S, bc, n, n, nkc, nc, act, st, true));
      CKR(mixed_split(w, 0, 3, S, P, n, n, nkc, nc, act, st));
      CKR(mixed_split(w, 0, 4, S, Q, n, n, nkc, nc, act, st));
      CKR(mixed_gemm_staged(w, 0, S, 3, 2, an, an, an, n, n, nkc, nc, act, st));     // alfa' = P alfa
      CKR(mixed_gemm_staged(w, 0, S, 4, 3, bn, bn, bn, n, n, nkc, nc, act, st));     // beta' = Q beta
      CKR(mixed_gemm_staged(w, 2, S, 3, 3, P, eps, x, n, n, nkc, nc, act, st));      // eps, x -= P beta
      CKR(mixed_gemm_staged(w, 1, S, 4, 2, eps, eps, eps, n, n, nkc, nc, act, st));  // eps -= Q alfa
    } else {
      CKR(eng_gemm(c, mx, 0, ac, y1, P, P, P, n, nkc, nc, act));        // P = alfa y1
      CKR(eng_gemm(c, mx, 0, bc, y1, Q, Q, Q, n, nkc, nc, act));        // Q = beta y1
      CKR(eng_gemm(c, mx, 0, P, ac, an, an, an, n, nkc, nc, act));      // alfa' = P alfa
      CKR(eng_gemm(c, mx, 0, Q, bc, bn, bn, bn, n, nkc, nc, act));      // beta' = Q beta
      CKR(eng_gemm(c, mx, 2, P, bc, P, eps, x, n, nkc, nc, act));       // y3: eps -= y3, x -= y3
      CKR(eng_gemm(c, mx, 1, Q, ac, eps, eps, eps, n, nkc, nc, act));   // eps -= y4
    }
    launch_fnorm(an, n, nkc, nc, act, err, st);
    // the two leads may carry different caps (itermaxl / itermaxr)
    if (iter_dev)
      launch_dec_state_dev(err, act, stat, iters, nit, iter_dev, itermax, c->sz.errmax, nact_dev, st);
    else
      launch_dec_state(err, act, stat, iters, nit, iter, itermax, c->sz.errmax, st);
    return SKKR_OK;
  };
  skkr_set_active_items(nit);
  // The first iteration runs eagerly (it sizes every work buffer); the rest
  // is one CUDA graph whose WHILE node repeats a body of two iterations (odd
  // and even buffers) until no item is left, with the iteration number, the
  // count of items left and the loop condition on the device: no host
  // round trip per iteration.  Observed launches (per-kernel statistics, the
  // synchronisation check) keep the host loop.
  for (int iter = 1;; iter++) {
    CKR(iterate(iter & 1, iter, nullptr, nullptr));
    long long cnt = 0;
    {
      std::vector<int> h(nit);
      CK(cudaMemcpyAsync(h.data(), act, nit * sizeof(int), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      for (int v : h) cnt += v;
      skkr_set_active_items(cnt);
    }
    if (cnt == 0 || iter > itermax + 1) break;
    if (c->graphs && !launches_observed()) {
      CKR(decimation_graph(c, iter + 1, itermax, iterate));
      break;
    }
  }
  skkr_set_active_items(-1);
  // statuses
  {
    std::vector<int> hs(nit), hi(nit);
    CK(cudaMemcpyAsync(hs.data(), stat, nit * sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hi.data(), iters, nit * sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int it = 0; it < nit; it++) {
      int kk = it / nc, s = it % nc;
      int cap = s < nLc ? c->sz.itermaxl : c->sz.itermaxr;
      int code = hs[it];
      if (code == 0 && hi[it] > cap) code = SKKR_ERR_SGF_ITERMAX;
      c->max_dec = std::max(c->max_dec, hi[it]);
      c->tot_dec += hi[it];
      if (code != 0 && c->err_code == 0) {
        c->err_code = code;
        c->first_bad_k = k0 + kk;
      }
    }
  }
  // X = x^-1 ; xy = ml X mt (tripmt2) into the SSPO cache
  CKR(eng_inv(c, mx, x, x, true, n, nkc, nc, nullptr));
  CKR(eng_gemm(c, mx, 0, Pml, x, y1, y1, y1, n, nkc, nc, nullptr));
  MatRef SS = mref_map(c->sspo.as<zd>() + (long long)k0 * c->nsl * MB, (long long)c->nsl * MB, MB, n,
                       mapsl, nc);
  CKR(eng_gemm(c, mx, 0, y1, Pmt, SS, SS, SS, n, nkc, nc, nullptr));
  return SKKR_OK;
}

// ---------------------------------------------------------------------------
// tau2d (main/tau2d.f) for k in [k0, k0+nkc), items (k, class)
static int run_tau2d(skkr_ctx *c, int k0, int nkc, const std::vector<int> &icls) {
  const int n = c->n, lk = c->lk, lk2 = lk * lk, pl = c->pl, nprc = c->nprc, ni = c->nintfc;
  const int nc = (int)icls.size();
  const long long MB = (long long)n * n;
  const int nbuf = 5 * nprc + 1;
  CKR(c->tauw.ensure((size_t)nkc * nc * nbuf * MB * sizeof(zd)));
  CKR(c->tauk.ensure((size_t)nkc * nc * ni * lk2 * sizeof(zd)));
  cudaStream_t st = c->st;
  zd *Wb = c->tauw.as<zd>();
  auto buf = [&](int b) { return mref(Wb + (long long)b * MB, (long long)nc * nbuf * MB, nbuf * MB, n); };
  // buffers: T00[p]=p, YY[p]=nprc+p, Yraw[p]=2nprc+p, XX[p]=3nprc+p, Xraw[p]=4nprc+p, W=5nprc
  auto T00 = [&](int p) { return buf(p); };
  auto YY = [&](int p) { return buf(nprc + p); };
  auto Yr = [&](int p) { return buf(2 * nprc + p); };
  auto XX = [&](int p) { return buf(3 * nprc + p); };
  auto Xr = [&](int p) { return buf(4 * nprc + p); };
  MatRef Wm = buf(5 * nprc);
  zd *poolk = c->pool.as<zd>();
  const long long psk = (long long)c->nmat * MB;
  int m00[SKKR_MAPN], m10[SKKR_MAPN], m01[SKKR_MAPN], ysl[SKKR_MAPN], xsl[SKKR_MAPN], tmap[SKKR_MAPN];
  const int nlay = 2 * pl + ni;
  for (int s = 0; s < nc; s++) {
    int g = icls[s];
    m00[s] = c->idx00;
    m10[s] = c->idx10;
    m01[s] = c->idx01;
    ysl[s] = c->igordl[c->ieqgl[g] - 1] - 1;
    xsl[s] = c->nls + c->igordr[c->ieqgr[g] - 1] - 1;
    tmap[s] = g * nlay + 2 * pl;  // interface layers of trot[g]
  }
  MatRef M00 = mref_map(poolk, psk, MB, n, m00, nc);
  MatRef M10 = mref_map(poolk, psk, MB, n, m10, nc);
  MatRef M01 = mref_map(poolk, psk, MB, n, m01, nc);
  zd *sbase = c->sspo.as<zd>() + (long long)k0 * c->nsl * MB;
  MatRef Ys = mref_map(sbase, (long long)c->nsl * MB, MB, n, ysl, nc);
  MatRef Xs = mref_map(sbase, (long long)c->nsl * MB, MB, n, xsl, nc);
  const bool mx = use_mixed(c, false);
  // split-precision engine: M10 and M01 enter every step on the same side,
  // so they are split once (A slot 1 = M10, B slot 1 = M01, A slot 3 = M01,
  // B slot 3 = M10); the per-step operands use slot 2
  const bool staged = mx && !ehsplit(c);
  MixedWork *w = c->mw;
  const int S = slices_for(c);
  auto prod = [&](int sa, const MatRef *A, int sb, const MatRef *B, const MatRef &C) -> int {
    if (A) CKR(mixed_split(w, 0, sa, S, *A, n, n, nkc, nc, nullptr, st));
    if (B) CKR(mixed_split(w, 1, sb, S, *B, n, n, nkc, nc, nullptr, st));
    return mixed_gemm_staged(w, 0, S, sa, sb, C, C, C, n, n, nkc, nc, nullptr, st);
  };
  if (staged) {
    CKR(mixed_split(w, 0, 1, S, M10, n, n, nkc, nc, nullptr, st));
    CKR(mixed_split(w, 1, 1, S, M01, n, n, nkc, nc, nullptr, st, true));
  }
  // forward (tau2d.f:53-85)
  for (int p = 0; p < nprc; p++) {
    int tm2[SKKR_MAPN];
    for (int s = 0; s < nc; s++) tm2[s] = tmap[s] + p * pl;
    MatRef Tt = mref_map(c->trot.as<zd>(), 0, lk2, lk, tm2, nc);
    launch_add_tblocks(T00(p), M00, Tt, lk, pl, n, nkc, nc, nullptr, ehsplit(c), st);
    if (p == 0) {
      launch_zaxpby(YY(0), Ys, nullptr, 0, nullptr, 0, n, nkc, nc, nullptr, st);
    } else if (staged) {
      MatRef yr = Yr(p);
      CKR(prod(1, nullptr, 2, &yr, YY(p)));                       // YY = M10 Yr
    } else {
      CKR(eng_gemm(c, mx, 0, M10, Yr(p), YY(p), YY(p), YY(p), n, nkc, nc, nullptr));
    }
    if (p < nprc - 1) {
      MatRef yy = YY(p);
      launch_zaxpby(Wm, T00(p), &yy, -1.0, nullptr, 0, n, nkc, nc, nullptr, st);
      CKR(eng_inv(c, mx, Wm, Wm, true, n, nkc, nc, nullptr));
      if (staged)
        CKR(prod(2, &Wm, 1, nullptr, Yr(p + 1)));                  // Yr(p+1) = W M01
      else
        CKR(eng_gemm(c, mx, 0, Wm, M01, Yr(p + 1), Yr(p + 1), Yr(p + 1), n, nkc, nc, nullptr));
    }
  }
  if (staged) {
    CKR(mixed_split(w, 0, 3, S, M01, n, n, nkc, nc, nullptr, st));
    CKR(mixed_split(w, 1, 3, S, M10, n, n, nkc, nc, nullptr, st, true));
  }
  // backward (tau2d.f:89-109)
  for (int p = nprc - 1; p >= 0; p--) {
    if (p == nprc - 1) {
      launch_zaxpby(XX(p), Xs, nullptr, 0, nullptr, 0, n, nkc, nc, nullptr, st);
    } else if (staged) {
      MatRef xr = Xr(p);
      CKR(prod(3, nullptr, 2, &xr, XX(p)));                       // XX = M01 Xr
    } else {
      CKR(eng_gemm(c, mx, 0, M01, Xr(p), XX(p), XX(p), XX(p), n, nkc, nc, nullptr));
    }
    if (p > 0) {
      MatRef xx = XX(p);
      launch_zaxpby(Wm, T00(p), &xx, -1.0, nullptr, 0, n, nkc, nc, nullptr, st);
      CKR(eng_inv(c, mx, Wm, Wm, true, n, nkc, nc, nullptr));
      if (staged)
        CKR(prod(2, &Wm, 3, nullptr, Xr(p - 1)));                  // Xr(p-1) = W M10
      else
        CKR(eng_gemm(c, mx, 0, Wm, M10, Xr(p - 1), Xr(p - 1), Xr(p - 1), n, nkc, nc, nullptr));
    }
  }
  // diagonal blocks (tau2d.f:114-149), weight wk/ngeff
  for (int p = 0; p < nprc; p++) {
    MatRef xx = XX(p), yy = YY(p);
    launch_zaxpby(Wm, T00(p), &xx, -1.0, &yy, -1.0, n, nkc, nc, nullptr, st);
    CKR(eng_inv(c, mx, Wm, Wm, true, n, nkc, nc, nullptr));
    launch_extract_tau(Wm, lk, pl, p * pl, c->wk.as<double>() + k0, 1.0 / c->ngeff, c->tauk.as<zd>(),
                       (long long)nc * ni * lk2, (long long)ni * lk2, nkc, nc, ehsplit(c), st);
  }
  return SKKR_OK;
}

// ---------------------------------------------------------------------------
// full Godfrin tau (skkr_dbogo_bsf/clu/tau2d_god.f) for k in [k0, k0+nkc),
// items (k, class): the sweeps of run_tau2d, then every PL block carried
// from the diagonal, tau(q,p) = cc(q) tau(q-1,p) below (cc(q) = -Xr(q-1)) and
// tau(q,p) = dd(q) tau(q+1,p) above (dd(q) = -Yr(q+1)); the signs are applied
// at the extraction into tauf[item][li][lj][lk^2] (weight wk/ngeff).
static int run_tau2d_full(skkr_ctx *c, int k0, int nkc, const std::vector<int> &icls, zd *tauf) {
  const int n = c->n, lk = c->lk, lk2 = lk * lk, pl = c->pl, nprc = c->nprc, ni = c->nintfc;
  const int nc = (int)icls.size();
  const long long MB = (long long)n * n;
  const int nbuf = 5 * nprc + 1;
  CKR(c->tauw.ensure((size_t)nkc * nc * nbuf * MB * sizeof(zd)));
  cudaStream_t st = c->st;
  zd *Wb = c->tauw.as<zd>();
  auto buf = [&](int b) { return mref(Wb + (long long)b * MB, (long long)nc * nbuf * MB, nbuf * MB, n); };
  auto T00 = [&](int p) { return buf(p); };
  auto YY = [&](int p) { return buf(nprc + p); };
  auto Yr = [&](int p) { return buf(2 * nprc + p); };
  auto XX = [&](int p) { return buf(3 * nprc + p); };
  auto Xr = [&](int p) { return buf(4 * nprc + p); };
  MatRef Wm = buf(5 * nprc);
  zd *poolk = c->pool.as<zd>();
  const long long psk = (long long)c->nmat * MB;
  int m00[SKKR_MAPN], m10[SKKR_MAPN], m01[SKKR_MAPN], ysl[SKKR_MAPN], xsl[SKKR_MAPN], tmap[SKKR_MAPN];
  const int nlay = 2 * pl + ni;
  for (int s = 0; s < nc; s++) {
    int g = icls[s];
    m00[s] = c->idx00;
    m10[s] = c->idx10;
    m01[s] = c->idx01;
    ysl[s] = c->igordl[c->ieqgl[g] - 1] - 1;
    xsl[s] = c->nls + c->igordr[c->ieqgr[g] - 1] - 1;
    tmap[s] = g * nlay + 2 * pl;
  }
  MatRef M00 = mref_map(poolk, psk, MB, n, m00, nc);
  MatRef M10 = mref_map(poolk, psk, MB, n, m10, nc);
  MatRef M01 = mref_map(poolk, psk, MB, n, m01, nc);
  zd *sbase = c->sspo.as<zd>() + (long long)k0 * c->nsl * MB;
  MatRef Ys = mref_map(sbase, (long long)c->nsl * MB, MB, n, ysl, nc);
  MatRef Xs = mref_map(sbase, (long long)c->nsl * MB, MB, n, xsl, nc);
  const bool mx = use_mixed(c, false);
  for (int p = 0; p < nprc; p++) {  // forward (tau2d_god.f:53-91)
    int tm2[SKKR_MAPN];
    for (int s = 0; s < nc; s++) tm2[s] = tmap[s] + p * pl;
    MatRef Tt = mref_map(c->trot.as<zd>(), 0, lk2, lk, tm2, nc);
    launch_add_tblocks(T00(p), M00, Tt, lk, pl, n, nkc, nc, nullptr, ehsplit(c), st);
    if (p == 0)
      launch_zaxpby(YY(0), Ys, nullptr, 0, nullptr, 0, n, nkc, nc, nullptr, st);
    else
      CKR(eng_gemm(c, mx, 0, M10, Yr(p), YY(p), YY(p), YY(p), n, nkc, nc, nullptr));
    if (p < nprc - 1) {
      MatRef yy = YY(p);
      launch_zaxpby(Wm, T00(p), &yy, -1.0, nullptr, 0, n, nkc, nc, nullptr, st);
      CKR(eng_inv(c, mx, Wm, Wm, true, n, nkc, nc, nullptr));
      CKR(eng_gemm(c, mx, 0, Wm, M01, Yr(p + 1), Yr(p + 1), Yr(p + 1), n, nkc, nc, nullptr));
    }
  }
  for (int p = nprc - 1; p >= 0; p--) {  // backward (:93-114)
    if (p == nprc - 1)
      launch_zaxpby(XX(p), Xs, nullptr, 0, nullptr, 0, n, nkc, nc, nullptr, st);
    else
      CKR(eng_gemm(c, mx, 0, M01, Xr(p), XX(p), XX(p), XX(p), n, nkc, nc, nullptr));
    if (p > 0) {
      MatRef xx = XX(p);
      launch_zaxpby(Wm, T00(p), &xx, -1.0, nullptr, 0, n, nkc, nc, nullptr, st);
      CKR(eng_inv(c, mx, Wm, Wm, true, n, nkc, nc, nullptr));
      CKR(eng_gemm(c, mx, 0, Wm, M10, Xr(p - 1), Xr(p - 1), Xr(p - 1), n, nkc, nc, nullptr));
    }
  }
  // PL-diagonal tau(p,p) in place of T00(p) (:115-119)
  for (int p = 0; p < nprc; p++) {
    MatRef t = T00(p), xx = XX(p), yy = YY(p);
    launch_zaxpby(t, t, &xx, -1.0, &yy, -1.0, n, nkc, nc, nullptr, st);
    CKR(eng_inv(c, mx, t, t, true, n, nkc, nc, nullptr));
  }
  // every PL block, carried from the diagonal (:151-205); YY(0) and XX(0)
  // serve as the two work matrices
  const double ws = 1.0 / c->ngeff;
  const long long osk = (long long)nc * ni * ni * lk2, osc = (long long)ni * ni * lk2;
  const double *wk = c->wk.as<double>() + k0;
  for (int p = 0; p < nprc; p++) {
    launch_extract_pairs(T00(p), lk, pl, p * pl, p * pl, ni, wk, ws, tauf, osk, osc, nkc, nc, ehsplit(c), st);
    MatRef cur = T00(p);
    for (int q = p + 1; q < nprc; q++) {  // below: tau(q,p) = -Xr(q-1) tau(q-1,p)
      MatRef nxt = ((q - p) & 1) ? YY(0) : XX(0);
      CKR(eng_gemm(c, mx, 0, Xr(q - 1), cur, nxt, nxt, nxt, n, nkc, nc, nullptr));
      launch_extract_pairs(nxt, lk, pl, q * pl, p * pl, ni, wk, ((q - p) & 1) ? -ws : ws, tauf, osk, osc, nkc, nc,
                           ehsplit(c), st);
      cur = nxt;
    }
    cur = T00(p);
    for (int q = p - 1; q >= 0; q--) {  // above: tau(q,p) = -Yr(q+1) tau(q+1,p)
      MatRef nxt = ((p - q) & 1) ? YY(0) : XX(0);
      CKR(eng_gemm(c, mx, 0, Yr(q + 1), cur, nxt, nxt, nxt, n, nkc, nc, nullptr));
      launch_extract_pairs(nxt, lk, pl, q * pl, p * pl, ni, wk, ((p - q) & 1) ? -ws : ws, tauf, osk, osc, nkc, nc,
                           ehsplit(c), st);
      cur = nxt;
    }
  }
  return SKKR_OK;
}

// ---------------------------------------------------------------------------
// CPA update (rsp-scf/fullcpa.f cpacor/cpasol) on the device
__global__ void k_cpa_norms(const zd *mc, const zd *tab, int lk2, double *out) {
  // out[l*4 + {0 ||ma-mc||^2, 1 ||ma||^2, 2 ||mb-mc||^2, 3 ||mb||^2}]
  const int l = blockIdx.x;
  const zd *m = mc + (long long)l * lk2, *a = tab + (long long)(2 * l) * lk2, *b = tab + (long long)(2 * l + 1) * lk2;
  double s[4] = {0, 0, 0, 0};
  for (int e = threadIdx.x; e < lk2; e += blockDim.x) {
    zd va = a[e], vb = b[e], vm = m[e];
    double dx = va.x - vm.x, dy = va.y - vm.y;
    s[0] += dx * dx + dy * dy;
    s[1] += va.x * va.x + va.y * va.y;
    dx = vb.x - vm.x;
    dy = vb.y - vm.y;
    s[2] += dx * dx + dy * dy;
    s[3] += vb.x * vb.x + vb.y * vb.y;
  }
  __shared__ double sh[4][256];
  for (int q = 0; q < 4; q++) sh[q][threadIdx.x] = s[q];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int q = 0; q < 4; q++) sh[q][threadIdx.x] += sh[q][threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x < 4) out[l * 4 + threadIdx.x] = sh[threadIdx.x][0];
}

static int cpa_step(skkr_ctx *c, int *itcpa, int *cpacon, int *concpa, double *error) {
  const int lk = c->lk, lk2 = lk * lk, ni = c->nintfc;
  cudaStream_t st = c->st;
  zd *mc = c->tcat.as<zd>() + (size_t)2 * c->pl * lk2;  // coherent t^-1 (in place)
  zd *tauc = c->tauc.as<zd>();
  // buffers: [ni][2] xa/xb, [ni][2] da/db, [ni] xc/h, [ni][2] tmp, [ni][2] tauab
  CKR(c->cpa.ensure((size_t)ni * 9 * lk2 * sizeof(zd)));
  CKR(c->cpan.ensure((size_t)ni * 6 * sizeof(double)));
  // flags: act [ni], act2 [2 ni], not-act2 [2 ni]
  CKR(c->cpaact.ensure((size_t)ni * 5 * sizeof(int)));
  zd *X = c->cpa.as<zd>(), *Dd = X + (size_t)ni * 2 * lk2, *H = Dd + (size_t)ni * 2 * lk2,
     *Tm = H + (size_t)ni * lk2, *TAB = Tm + (size_t)ni * 2 * lk2;
  double *nrm = c->cpan.as<double>();
  k_cpa_norms<<<ni, 256, 0, st>>>(mc, c->tab.as<zd>(), lk2, nrm);
  SKKR_LAUNCHED();
  std::vector<double> hn((size_t)ni * 4);
  CK(cudaMemcpyAsync(hn.data(), nrm, hn.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  const double tiny = 1.0e-6, tol = 1.0e-10;  // fullcpa.f:41
  std::vector<int> act(ni), act2(2 * ni), nact2(2 * ni);
  int nalloy = 0;
  for (int l = 0; l < ni; l++) {
    bool cpalay = (1.0 - c->conc_h[l]) > tiny;
    bool ica = std::sqrt(hn[l * 4 + 0]) < tol * std::sqrt(hn[l * 4 + 1]);
    bool icb = std::sqrt(hn[l * 4 + 2]) < tol * std::sqrt(hn[l * 4 + 3]);
    act[l] = (cpalay && !ica && !icb) ? 1 : 0;
    nalloy += act[l];
    act2[2 * l] = act2[2 * l + 1] = act[l];
    nact2[2 * l] = nact2[2 * l + 1] = !act[l];
  }
  int *dact = c->cpaact.as<int>(), *dact2 = dact + ni, *dnact2 = dact + 3 * ni;
  CK(cudaMemcpyAsync(dact, act.data(), ni * sizeof(int), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(dact2, act2.data(), 2 * ni * sizeof(int), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(dnact2, nact2.data(), 2 * ni * sizeof(int), cudaMemcpyHostToDevice, st));
  // non-alloy layers: taua = taub = tauc (fullcpa.f:45-48)
  MatRef TABm = mref(TAB, 2LL * lk2, lk2, lk);
  MatRef tauc2 = mref(tauc, lk2, 0, lk);
  launch_zaxpby(TABm, tauc2, nullptr, 0, nullptr, 0, lk, ni, 2, dnact2, st);
  *error = 0.0;
  if (nalloy > 0) {
    MatRef Xm = mref(X, 2LL * lk2, lk2, lk), Dm = mref(Dd, 2LL * lk2, lk2, lk);
    MatRef mc2 = mref(mc, lk2, 0, lk), tab2 = mref(c->tab.as<zd>(), 2LL * lk2, lk2, lk);
    (void)Dd;
    // da = mc - ma ; db = mc - mb ; xa = da ; xb = db   (cpasol.f:94-99)
    skkr_set_active_items(2LL * nalloy);
    launch_zaxpby(Dm, mc2, &tab2, -1.0, nullptr, 0, lk, ni, 2, dact2, st);
    launch_zaxpby(Xm, Dm, nullptr, 0, nullptr, 0, lk, ni, 2, dact2, st);
    launch_zgj(Xm, lk, ni, 2, dact2, st);
    launch_zaxpby(Xm, Xm, &tauc2, -1.0, nullptr, 0, lk, ni, 2, dact2, st);
    launch_zgj(Xm, lk, ni, 2, dact2, st);
    // xc = c xa + (1-c) xb ; h = (xc^-1 + tauc)^-1 ; mc -= h   (:109-124)
    MatRef Hm = mref(H, lk2, 0, lk), mc1 = mref(mc, lk2, 0, lk), tauc1 = mref(tauc, lk2, 0, lk);
    launch_cpa_mix(X, c->conc.as<double>(), dact, lk, ni, H, st);
    skkr_set_active_items(nalloy);
    launch_zgj(Hm, lk, ni, 1, dact, st);
    launch_zaxpby(Hm, Hm, &tauc1, 1.0, nullptr, 0, lk, ni, 1, dact, st);
    launch_zgj(Hm, lk, ni, 1, dact, st);
    launch_zaxpby(mc1, mc1, &Hm, -1.0, nullptr, 0, lk, ni, 1, dact, st);
    // error3 = ||h||_F / ||mc||_F (:126-142)
    CK(cudaMemsetAsync(nrm, 0, 2 * ni * sizeof(double), st));
    launch_fnorm(Hm, lk, ni, 1, dact, nrm, st);
    launch_fnorm(mc1, lk, ni, 1, dact, nrm + ni, st);
    // tau_A = tauc + tauc xa tauc ; tau_B likewise (:145-150)
    skkr_set_active_items(2LL * nalloy);
    MatRef Tmm = mref(Tm, 2LL * lk2, lk2, lk);
    launch_zgemm(0, tauc2, Xm, Tmm, Tmm, Tmm, lk, lk, lk, ni, 2, dact2, st);
    launch_zgemm(0, Tmm, tauc2, TABm, TABm, TABm, lk, lk, lk, ni, 2, dact2, st);
    launch_zaxpby(TABm, TABm, &tauc2, 1.0, nullptr, 0, lk, ni, 2, dact2, st);
    skkr_set_active_items(-1);
    std::vector<double> hn2(2 * ni);
    CK(cudaMemcpyAsync(hn2.data(), nrm, 2 * ni * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int l = 0; l < ni; l++)
      if (act[l]) {
        double e3 = hn2[l] / hn2[ni + l];
        if (e3 >= *error) *error = e3;
      }
  }
  if (*error <= c->sz.cpatol) *concpa = 0;
  if (*itcpa >= c->sz.itcpam) *cpacon = 0;
  (*itcpa)++;
  return SKKR_OK;
}

// ---------------------------------------------------------------------------
// Sum of the k-summed tau over the ranks of a k-split energy through the
// host hook (cpacoord_ksave.f:406).  `failed` ranks send the flag only.
static int reduce_tauc(skkr_ctx *c, bool failed) {
  const size_t nz = (size_t)c->nintfc * c->lk * c->lk;
  if (c->red_dev_fn) {
    // device form: tauc and the flag into one device buffer, the hook sums it
    // in place on the context stream, the sum goes back into tauc
    CKR(c->redd.ensure((2 * nz + 1) * sizeof(double)));
    double *b = c->redd.as<double>();
    if (failed) CK(cudaMemsetAsync(b, 0, 2 * nz * sizeof(double), c->st));
    else CK(cudaMemcpyAsync(b, c->tauc.p, nz * sizeof(zd), cudaMemcpyDeviceToDevice, c->st));
    const double flag = failed ? 1.0 : 0.0;
    CK(cudaMemcpyAsync(b + 2 * nz, &flag, sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));  // `flag` is a host temporary
    if (c->red_dev_fn(c->red_dev_user, b, (long long)(2 * nz + 1), (void *)c->st) != 0) {
      g_last_error = "reduction hook returned an error";
      return SKKR_ERR_PEER;
    }
    if (failed) return SKKR_OK;
    double sum_flag = 0.0;
    CK(cudaMemcpyAsync(&sum_flag, b + 2 * nz, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    if (sum_flag != 0.0) {
      g_last_error = "another rank of the k-split energy failed";
      return SKKR_ERR_PEER;
    }
    CK(cudaMemcpyAsync(c->tauc.p, b, nz * sizeof(zd), cudaMemcpyDeviceToDevice, c->st));
    return SKKR_OK;
  }
  c->red_buf.assign(2 * nz + 1, 0.0);
  if (!failed) {
    CK(cudaMemcpyAsync(c->red_buf.data(), c->tauc.p, nz * sizeof(zd), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  c->red_buf[2 * nz] = failed ? 1.0 : 0.0;
  if (c->red_fn(c->red_user, c->red_buf.data(), (long long)(2 * nz + 1)) != 0) {
    g_last_error = "reduction hook returned an error";
    return SKKR_ERR_PEER;
  }
  if (failed) return SKKR_OK;
  if (c->red_buf[2 * nz] != 0.0) {
    g_last_error = "another rank of the k-split energy failed";
    return SKKR_ERR_PEER;
  }
  CK(cudaMemcpyAsync(c->tauc.p, c->red_buf.data(), nz * sizeof(zd), cudaMemcpyHostToDevice, c->st));
  return SKKR_OK;
}

// Accuracy guard of the split-precision path: near the real axis a few k
// points sit close to an interface resonance, carry much of |sum_k tau_k| and
// see the product rounding amplified by their conditioning.  Every k whose
// contribution exceeds dominant_frac of the k-summed norm and DOMINANT_PEAK
// times the mean per-k norm is recomputed in FP64 and its contribution
// swapped in the class sums: the selected k are
// gathered into compact buffers (structure-constant blocks, cached surface
// operators, weights) that stand in for the context's, their mixed
// contribution is recomputed from the same cached state and subtracted, the
// decimation and tau2d are redone in FP64 and added, and the FP64 surface
// operators are scattered back for the later CPA iterations.
constexpr double DOMINANT_PEAK = 10.0;  // a redone k point carries this many times the mean per-k norm

static int redo_dominant_k(skkr_ctx *c, int itcpa, const std::vector<int> &lcls, const std::vector<int> &rcls,
                           const std::vector<int> &icls) {
  (void)itcpa;
  const int nk = c->nk, ni = c->nintfc, lk2 = c->lk * c->lk, ncls = (int)icls.size();
  const long long E = (long long)ncls * ni * lk2;
  const size_t bs = (size_t)c->lmmax * c->lmmax, gk = (size_t)c->nbk * bs;
  const size_t sk = (size_t)c->nsl * c->n * c->n;   // SSPO elements per k
  cudaStream_t st = c->st;
  std::vector<double> kn(nk);
  std::vector<zd> Sh((size_t)E);
  CK(cudaMemcpyAsync(kn.data(), c->knorm.p, nk * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(Sh.data(), c->S.p, (size_t)E * sizeof(zd), cudaMemcpyDeviceToHost, st));
  std::vector<double> wkh(nk);
  CK(cudaMemcpyAsync(wkh.data(), c->wk.p, nk * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  double s2 = 0.0;
  for (const zd &v : Sh) s2 += v.x * v.x + v.y * v.y;
  // an isolated peak of the integrand: above dominant_frac of the k-summed
  // norm and above DOMINANT_PEAK times the mean per-k norm (on coarse meshes
  // of smooth integrands the largest points stay within a few times the mean,
  // and their split-precision rounding is not amplified)
  double ksum = 0.0;
  for (int k = 0; k < nk; k++) ksum += kn[k];
  const double lim = std::max(c->dominant_frac * std::sqrt(s2), DOMINANT_PEAK * ksum / nk);
  std::vector<int> sel;
  for (int k = 0; k < nk; k++)
    if (kn[k] > lim) sel.push_back(k);
  if (sel.empty()) return SKKR_OK;
  DBuf Gc, Sc, Wc, T;
  struct Release {  // compact buffers are local (cudaFree waits for their last use)
    DBuf *b[4];
    ~Release() {
      for (DBuf *x : b) x->release();
    }
  } release_on_return{{&Gc, &Sc, &Wc, &T}};
  for (size_t g0 = 0; g0 < sel.size(); g0 += (size_t)c->kc) {
    const int m = (int)std::min<size_t>((size_t)c->kc, sel.size() - g0);
    CKR(Gc.ensure((size_t)m * gk * sizeof(zd)));
    CKR(Sc.ensure((size_t)m * sk * sizeof(zd)));
    CKR(Wc.ensure((size_t)m * sizeof(double)));
    CKR(T.ensure((size_t)E * sizeof(zd)));
    std::vector<double> w(m);
    for (int i = 0; i < m; i++) {
      const int k = sel[g0 + i];
      w[i] = wkh[k];
      CK(cudaMemcpyAsync(Gc.as<zd>() + (size_t)i * gk, c->G.as<zd>() + (size_t)k * gk, gk * sizeof(zd),
                         cudaMemcpyDeviceToDevice, st));
      CK(cudaMemcpyAsync(Sc.as<zd>() + (size_t)i * sk, c->sspo.as<zd>() + (size_t)k * sk, sk * sizeof(zd),
                         cudaMemcpyDeviceToDevice, st));
    }
    CK(cudaMemcpyAsync(Wc.p, w.data(), m * sizeof(double), cudaMemcpyHostToDevice, st));
    std::swap(c->G, Gc);
    std::swap(c->sspo, Sc);
    std::swap(c->wk, Wc);
    int rc = SKKR_OK;
    launch_pack(c->G.as<zd>(), c->nblk, c->nbk, c->blkmap_d.as<int>(), c->mi, c->jmax, c->jobs.as<PackJob>(),
                c->nmat, c->lk, c->lmmax, c->sz.mode, c->fac, c->fach, m, c->pool.as<zd>(), c->nmat, c->n,
                ehsplit(c), st);
    rc = run_tau2d(c, 0, m, icls);            // the mixed contributions summed above
    if (rc == SKKR_OK) {
      launch_ksum(c->tauk.as<zd>(), m, E, T.as<zd>(), 0, st);
      launch_axpy_flat(c->S.as<zd>(), T.as<zd>(), E, -1.0, st);
      c->force_fp64 = true;
      rc = run_decimation(c, 0, m, lcls, rcls);
      if (c->err_code && c->first_bad_k >= 0 && c->first_bad_k < m) c->first_bad_k = sel[g0 + c->first_bad_k];
      if (rc == SKKR_OK && !c->err_code) rc = run_tau2d(c, 0, m, icls);
      c->force_fp64 = false;
    }
    std::swap(c->G, Gc);
    std::swap(c->sspo, Sc);
    std::swap(c->wk, Wc);
    if (rc != SKKR_OK) return rc;
    if (c->err_code) return SKKR_OK;
    launch_ksum(c->tauk.as<zd>(), m, E, T.as<zd>(), 0, st);
    launch_axpy_flat(c->S.as<zd>(), T.as<zd>(), E, 1.0, st);
    for (int i = 0; i < m; i++)
      CK(cudaMemcpyAsync(c->sspo.as<zd>() + (size_t)sel[g0 + i] * sk, Sc.as<zd>() + (size_t)i * sk,
                         sk * sizeof(zd), cudaMemcpyDeviceToDevice, st));
    c->k_fp64 += m;
  }
  return SKKR_OK;
}

// Off-diagonal tau of the interface for cluster embedding
// (skkr_dbogo_bsf/rsp-scf/cpacoord_ksave.f:638-660, 760-840): one k loop of
// the staged energy with its current t^-1 -- G(k), decimation, the full
// Godfrin tau per class, the phased pair sums per group element -- then the
// group rotations L_g (.) R_g summed over g.
extern "C" int skkr_gpu_tauij(skkr_ctx *c, int npair, const int *pairs, const double *a1, const double *a2,
                              const double *cvec, const double *a0mat, double *tau_ij, double *tau_ji, int ld,
                              skkr_status *status) {
  if (!c || !c->staged || npair < 1 || (long long)npair * c->ngeff > 65535 || !pairs || !a1 || !a2 || !cvec || !a0mat || !tau_ij ||
      !tau_ji || ld < c->lk)
    return SKKR_ERR_ARG;
  // BdG energies run through skkr_gpu_cpacoord_bdg, which stages the hole factors itself
  if (c->sz.mode == SKKR_BDG) return SKKR_ERR_UNSUPPORTED;
  const int n = c->n, lk = c->lk, lk2 = lk * lk, ni = c->nintfc, nk = c->nk, ng = c->ngeff;
  for (int q = 0; q < npair; q++)
    if (pairs[4 * q + 2] < 0 || pairs[4 * q + 2] >= ni || pairs[4 * q + 3] < 0 || pairs[4 * q + 3] >= ni)
      return SKKR_ERR_ARG;
  const long long l0 = g_skkr_launches;
  const long long MB = (long long)n * n;
  const size_t bs = (size_t)c->lmmax * c->lmmax;
  cudaStream_t st = c->st;
  c->max_dec = 0;
  c->tot_dec = 0;
  c->err_code = 0;
  c->first_bad_k = -1;
  if (c->sz.precision == SKKR_MIXED && !c->mw) {
    c->mw = mixed_create();
    if (!c->mw) return SKKR_ERR_NOMEM;
  }
  if (c->mw) {
    CKR(mixed_resid_reset(c->mw, st));
    mixed_set_precise(c->mw, c->slices_near > 0 && std::fabs(c->ce.y) < c->near_im);
    mixed_set_fused(c->mw, c->fused_b != 0);
  }
  plan_pack(c);
  CKR(c->jobs.ensure(c->jobs_h.size() * sizeof(PackJob)));
  CK(cudaMemcpyAsync(c->jobs.p, c->jobs_h.data(), c->jobs_h.size() * sizeof(PackJob), cudaMemcpyHostToDevice,
                     st));
  CKR(c->G.ensure((size_t)nk * c->nbk * bs * sizeof(zd)));
  CKR(sorttmat_dev(c));
  CKR(check_slot_quirk(c));
  std::vector<int> lcls, rcls, icls;
  lead_classes(c, lcls, rcls);
  for (int g = 0; g < ng; g++)
    if (c->ieqg[g] == g + 1) icls.push_back(g);
  const int nc = (int)icls.size();
  {
    int nLs = 0, nRs = 0;
    for (int g : lcls) nLs = std::max(nLs, c->igordl[g]);
    for (int g : rcls) nRs = std::max(nRs, c->igordr[g]);
    c->nls = nLs;
    c->nsl = nLs + nRs;
  }
  // chunk: the run's per-k work plus the full tau of every class
  int kc;
  {
    const int ncmax = 2 * ng;
    double per_k = (double)MB * sizeof(zd) * (c->nmat + 9.0 * ncmax + (5.0 * c->nprc + 1) * ng) +
                   (double)nc * ni * ni * lk2 * sizeof(zd);
    if (c->sz.precision == SKKR_MIXED) {
      const double Mp = 128.0 * ((n + 127) / 128), Np = 96.0 * ((2 * n + 95) / 96), Kp = 32.0 * ((2 * n + 31) / 32);
      per_k += (double)ncmax * MIXED_SLOTS * c->slices_res * (Mp + Np) * Kp * 2.0;
    }
    kc = c->sz.nk_chunk > 0 ? c->sz.nk_chunk : (int)std::max(1.0, std::floor(32.0e9 / per_k));
    kc = std::max(1, std::min(std::min(kc, 65535 / (2 * ng)), nk));
  }
  CKR(c->pool.ensure((size_t)kc * c->nmat * MB * sizeof(zd)));
  CKR(c->sspo.ensure((size_t)nk * c->nsl * MB * sizeof(zd)));
  launch_gk_ft(c->gR.as<zd>(), c->rvec.as<double>(), c->rstart.as<int>(), c->nbk, c->lmmax, c->xk.as<double>(), nk,
               c->G.as<zd>(), st);
  // pair data: class of each g, R + c_li - c_lj, a0mat
  std::vector<int> cls(ng);
  for (int g = 0; g < ng; g++)
    cls[g] = (int)(std::find(icls.begin(), icls.end(), c->ieqg[g] - 1) - icls.begin());
  std::vector<double> vecs(2 * (size_t)npair);
  for (int q = 0; q < npair; q++) {
    const int n1 = pairs[4 * q], n2 = pairs[4 * q + 1], li = pairs[4 * q + 2], lj = pairs[4 * q + 3];
    vecs[2 * q] = n1 * a1[0] + n2 * a2[0] + cvec[2 * li] - cvec[2 * lj];
    vecs[2 * q + 1] = n1 * a1[1] + n2 * a2[1] + cvec[2 * li + 1] - cvec[2 * lj + 1];
  }
  DBuf tauf, acc, misc, rot;
  struct Release {
    DBuf *b[4];
    ~Release() {
      for (DBuf *x : b) x->release();
    }
  } release_on_return{{&tauf, &acc, &misc, &rot}};
  const size_t accn = (size_t)npair * ng * lk2;
  CKR(tauf.ensure((size_t)kc * nc * ni * ni * lk2 * sizeof(zd)));
  CKR(acc.ensure(2 * accn * sizeof(zd)));
  CKR(rot.ensure(4 * accn * sizeof(zd)));
  const size_t moff_vec = ((size_t)ng + 4 * npair) * sizeof(int);
  const size_t moff_a0 = moff_vec + 2 * (size_t)npair * sizeof(double);
  CKR(misc.ensure(moff_a0 + 4 * (size_t)ng * sizeof(double)));
  char *mb = misc.as<char>();
  CK(cudaMemcpyAsync(mb, cls.data(), ng * sizeof(int), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(mb + ng * sizeof(int), pairs, 4 * (size_t)npair * sizeof(int), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(mb + moff_vec, vecs.data(), vecs.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(mb + moff_a0, a0mat, 4 * (size_t)ng * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(acc.p, 0, 2 * accn * sizeof(zd), st));
  CK(cudaStreamSynchronize(st));  // the host vectors above are temporaries
  zd *acc_ij = acc.as<zd>(), *acc_ji = acc_ij + accn;
  for (int k0 = 0; k0 < nk; k0 += kc) {
    const int nkc = std::min(kc, nk - k0);
    launch_pack(c->G.as<zd>() + (size_t)k0 * c->nbk * bs, c->nblk, c->nbk, c->blkmap_d.as<int>(), c->mi, c->jmax,
                c->jobs.as<PackJob>(), c->nmat, lk, c->lmmax, c->sz.mode, c->fac, c->fach, nkc, c->pool.as<zd>(),
                c->nmat, n, ehsplit(c), st);
    CKR(run_decimation(c, k0, nkc, lcls, rcls));
    if (c->err_code) break;
    CKR(run_tau2d_full(c, k0, nkc, icls, tauf.as<zd>()));
    launch_pair_sum(tauf.as<zd>(), nkc, nc, ni, lk, (const int *)mb, ng, npair, (const int *)(mb + ng * sizeof(int)),
                    (const double *)(mb + moff_vec), (const double *)(mb + moff_a0), c->xk.as<double>() + 2 * k0,
                    acc_ij, acc_ji, st);
  }
  if (!c->err_code) {
    // tau_ij[q] = sum_g L_g acc[q][g] R_g, likewise tau_ji
    zd *T1 = rot.as<zd>(), *T2 = T1 + 2 * accn;
    MatRef Lm = mref(c->lg.as<zd>(), 0, lk2, lk), Rm = mref(c->rg.as<zd>(), 0, lk2, lk);
    for (int side = 0; side < 2; side++) {
      MatRef Am = mref((side ? acc_ji : acc_ij), (long long)ng * lk2, lk2, lk);
      MatRef T1m = mref(T1 + side * accn, (long long)ng * lk2, lk2, lk);
      MatRef T2m = mref(T2 + side * accn, (long long)ng * lk2, lk2, lk);
      launch_zgemm(0, Lm, Am, T1m, T1m, T1m, lk, lk, lk, npair, ng, nullptr, st);
      launch_zgemm(0, T1m, Rm, T2m, T2m, T2m, lk, lk, lk, npair, ng, nullptr, st);
      launch_gsum(T2 + side * accn, ng, lk, npair, T1 + side * accn, st);
    }
    CKR(get_mats(tau_ij, T1, npair, lk, ld, st));
    CKR(get_mats(tau_ji, T1 + accn, npair, lk, ld, st));
  }
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());
  if (status) {
    *status = skkr_status{};
    status->code = c->err_code;
    status->ik = c->first_bad_k;
    status->max_dec_iters = c->max_dec;
    status->dec_iters_total = c->tot_dec;
    status->gpu_launches = g_skkr_launches - l0;
  }
  return c->err_code;
}

extern "C" int skkr_gpu_set_mixed_policy(skkr_ctx *c, double dec_fp64_im, double near_im, int slices_near,
                                         double dominant_frac) {
  if (!c || dec_fp64_im < 0.0 || near_im < 0.0 || (slices_near != 0 && (slices_near < 3 || slices_near > 8)) ||
      dominant_frac < 0.0)
    return SKKR_ERR_ARG;
  c->dec_fp64_im = dec_fp64_im;
  c->near_im = near_im;
  c->slices_near = slices_near;
  c->dominant_frac = dominant_frac;
  return SKKR_OK;
}

extern "C" int skkr_gpu_autotune(int force, char *report, int len) {
  if (force < 0 || force > 3) return SKKR_ERR_ARG;
  if (force > 0 || (!report && force == 0)) gj_tune_force(force);
  if (report && len > 0) {
    const std::string r = gj_tune_report();
    std::snprintf(report, (size_t)len, "%s", r.c_str());
  }
  return SKKR_OK;
}

extern "C" int skkr_gpu_set_newton(skkr_ctx *c, int steps) {
  if (!c || steps < 1 || steps > 3) return SKKR_ERR_ARG;
  c->newton = steps;
  return SKKR_OK;
}

extern "C" int skkr_gpu_set_inverse_start(skkr_ctx *c, int blocked) {
  if (!c) return SKKR_ERR_ARG;
  c->blocked_start = blocked != 0;
  return SKKR_OK;
}

extern "C" int skkr_gpu_set_fused_split(skkr_ctx *c, int on) {
  if (!c) return SKKR_ERR_ARG;
  c->fused_b = on != 0;
  return SKKR_OK;
}

extern "C" int skkr_gpu_set_graphs(skkr_ctx *c, int on) {
  if (!c) return SKKR_ERR_ARG;
  c->graphs = on != 0;
  return SKKR_OK;
}

extern "C" int skkr_gpu_set_reduce_device(skkr_ctx *c, skkr_reduce_dev_fn fn, void *user) {
  if (!c) return SKKR_ERR_ARG;
  c->red_dev_fn = fn;
  c->red_dev_user = user;
  return SKKR_OK;
}

extern "C" int skkr_gpu_set_reduce(skkr_ctx *c, skkr_reduce_fn fn, void *user) {
  if (!c) return SKKR_ERR_ARG;
  c->red_fn = fn;
  c->red_user = user;
  return SKKR_OK;
}

// G_scr(k) of every k point of the staged energy from the reference's
// k-space form, written into the structure-constant cache in batches of k
// points sized to a few GB of scratch
static int kambe_gk(skkr_ctx *c) {
  KambeDev &K = c->kd;
  const size_t bs = (size_t)c->lmmax * c->lmmax;
  int m = (int)std::max<size_t>(1, (size_t)8e9 / K.per_k());
  m = std::min(std::min(m, 65535), c->nk);
  for (int k0 = 0; k0 < c->nk; k0 += m) {
    const int mm = std::min(m, c->nk - k0);
    CKR(K.screen(c->xk.as<double>() + 2 * (size_t)k0, mm, c->st));
    launch_slab_cache(mm, K.nl, K.lm, K.centre, K.jmax, c->kblk.as<int>(), c->nbk, K.X.as<zd>(),
                      c->G.as<zd>() + (size_t)k0 * c->nbk * bs, c->st);
  }
  return SKKR_OK;
}

extern "C" int skkr_gpu_stage_kambe(skkr_ctx *c, const skkr_kambe_form *kf) {
  if (!c || !c->staged) return SKKR_ERR_ARG;
  if (!kf) {
    c->kambe_on = false;
    return SKKR_OK;
  }
  if (c->sz.mode == SKKR_BDG) return SKKR_ERR_UNSUPPORTED;
  // offset j of the staged block map -> block; every (slot, layer) must map
  // an offset to one block and a block to one offset (equivalent layers)
  const int nj = 2 * c->jmax + 1, rowlen = c->mi * nj;
  std::vector<int> blk(nj, -1);
  for (int sl = 0; sl < c->nslot; sl++)
    for (int i = 0; i < c->mi; i++)
      for (int j = 0; j < nj; j++) {
        const int b = c->blkmap[(size_t)sl * rowlen + i * nj + j];
        if (b < 0) continue;
        if (blk[j] >= 0 && blk[j] != b) return SKKR_ERR_UNSUPPORTED;
        blk[j] = b;
      }
  for (int j = 0; j < nj; j++)
    for (int j2 = 0; j2 < j; j2++)
      if (blk[j] >= 0 && blk[j] == blk[j2]) return SKKR_ERR_UNSUPPORTED;
  int rc = c->kd.setup(kf->e_re, kf->e_im, c->sz.lmax, kf->nl, kf->pos, kf->alpha, kf->centre, c->jmax, kf->gvec,
                       kf->ng, kf->rvec, kf->nr, kf->area, kf->factor, kf->gcut, kf->rcut, c->st);
  if (rc != SKKR_OK) return rc;
  CKR(c->kblk.ensure(nj * sizeof(int)));
  CK(cudaMemcpyAsync(c->kblk.p, blk.data(), nj * sizeof(int), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->kambe_on = true;
  return SKKR_OK;
}

extern "C" int skkr_gpu_run(skkr_ctx *c, skkr_status *status) {
  if (!c || !c->staged) return SKKR_ERR_ARG;
  const long long l0 = g_skkr_launches;
  cudaEvent_t ev0, ev1;
  CK(cudaEventCreate(&ev0));
  CK(cudaEventCreate(&ev1));
  CK(cudaEventRecord(ev0, c->st));
  const int n = c->n, lk = c->lk, lk2 = lk * lk, ni = c->nintfc, nk = c->nk;
  const long long MB = (long long)n * n;
  const size_t bs = (size_t)c->lmmax * c->lmmax;
  cudaStream_t st = c->st;
  c->max_dec = 0;
  c->tot_dec = 0;
  c->err_code = 0;
  c->first_bad_k = -1;
  c->max_resid = 0.0;
  c->k_fp64 = 0;
  c->alg_units = 0.0;
  c->graph_kernels = 0;
  c->graph_launches = 0;
  CKR(c->knorm.ensure((size_t)nk * sizeof(double)));
  if (c->sz.precision == SKKR_MIXED && !c->mw) {
    c->mw = mixed_create();
    if (!c->mw) return SKKR_ERR_NOMEM;
  }
  if (c->mw) {
    CKR(mixed_resid_reset(c->mw, st));
    // near the real axis the products also run on the exact-level tile
    mixed_set_precise(c->mw, c->slices_near > 0 && std::fabs(c->ce.y) < c->near_im);
    mixed_set_fused(c->mw, c->fused_b != 0);
  }
  plan_pack(c);
  CKR(c->jobs.ensure(c->jobs_h.size() * sizeof(PackJob)));
  CK(cudaMemcpyAsync(c->jobs.p, c->jobs_h.data(), c->jobs_h.size() * sizeof(PackJob),
                     cudaMemcpyHostToDevice, st));
  CKR(c->G.ensure((size_t)nk * c->nbk * bs * sizeof(zd)));
  // chunk size: keep the per-chunk work within a fixed budget
  {
    const int ncmax = 2 * c->ngeff;
    double per_k = (double)MB * sizeof(zd) * (c->nmat + 9.0 * ncmax + (5.0 * c->nprc + 1) * c->ngeff) +
                   (double)c->ngeff * ni * lk2 * sizeof(zd);
    if (use_mixed(c, false)) {
      // BF16 slice staging: up to MIXED_SLOTS operands per side, S slices of
      // the padded real embedding (A: 128-row tiles, B: 96-row tiles, K: 2n);
      // an energy that runs wholly in FP64 stages nothing
      const double Mp = 128.0 * ((n + 127) / 128), Np = 96.0 * ((2 * n + 95) / 96),
                   Kp = 32.0 * ((2 * n + 31) / 32);
      per_k += (double)ncmax * MIXED_SLOTS * c->slices_res * (Mp + Np) * Kp * 2.0;
    }
    double budget = 64.0e9;  // of the 280 GB: the estimate counts every class slot as used
    int kc = c->sz.nk_chunk > 0 ? c->sz.nk_chunk : (int)std::max(1.0, std::floor(budget / per_k));
    // grid.y of the batched kernels holds k_chunk * items-per-k (<= 2 * ngeff)
    kc = std::min(kc, 65535 / (2 * c->ngeff));
    c->kc = std::max(1, std::min(kc, nk));
  }
  CKR(c->pool.ensure((size_t)c->kc * c->nmat * MB * sizeof(zd)));

  int itcpa = 1, cpacon = 1, concpa = 1;
  double cpaerr = 0.0;
  std::vector<int> lcls, rcls, icls;
  for (;;) {
    trace_point("loop top");
    CKR(sorttmat_dev(c));
    trace_point("after sorttmat");
    CKR(check_slot_quirk(c));
    lead_classes(c, lcls, rcls);
    icls.clear();
    for (int g = 0; g < c->ngeff; g++)
      if (c->ieqg[g] == g + 1) icls.push_back(g);
    const int ncls = (int)icls.size();
    if (itcpa == 1) {
      int nLs = 0, nRs = 0;
      for (int g : lcls) nLs = std::max(nLs, c->igordl[g]);
      for (int g : rcls) nRs = std::max(nRs, c->igordr[g]);
      c->nls = nLs;
      c->nsl = nLs + nRs;
      CKR(c->sspo.ensure((size_t)nk * c->nsl * MB * sizeof(zd)));
      if (c->kambe_on) {
        CKR(kambe_gk(c));
      } else {
        launch_gk_ft(c->gR.as<zd>(), c->rvec.as<double>(), c->rstart.as<int>(), c->nbk, c->lmmax,
                     c->xk.as<double>(), nk, c->G.as<zd>(), st);
      }
    }
    CKR(c->S.ensure((size_t)ncls * ni * lk2 * sizeof(zd)));
    for (int k0 = 0; k0 < nk; k0 += c->kc) {
      const int nkc = std::min(c->kc, nk - k0);
      launch_pack(c->G.as<zd>() + (size_t)k0 * c->nbk * bs, c->nblk, c->nbk, c->blkmap_d.as<int>(),
                  c->mi, c->jmax, c->jobs.as<PackJob>(), c->nmat, lk, c->lmmax, c->sz.mode, c->fac,
                  c->fach, nkc, c->pool.as<zd>(), c->nmat, n, ehsplit(c), st);
      if (itcpa == 1) {
        const long long d0 = c->tot_dec;
        CKR(run_decimation(c, k0, nkc, lcls, rcls));
        // surfgf.f: 1 inverse + 4 triple products per iteration; dugo.f: the
        // final inverse and tripmt2
        c->alg_units += 9.0 * (double)(c->tot_dec - d0) + 3.0 * nkc * (double)(lcls.size() + rcls.size());
      }
      if (c->err_code) break;
      CKR(run_tau2d(c, k0, nkc, icls));
      c->alg_units += (7.0 * c->nprc - 6.0) * nkc * (double)ncls;  // tau2d.f per item
      launch_ksum(c->tauk.as<zd>(), nkc, (long long)ncls * ni * lk2, c->S.as<zd>(), k0 > 0, st);
      if (use_mixed(c, false) && c->dominant_frac > 0.0)
        launch_knorm(c->tauk.as<zd>(), nkc, (long long)ncls * ni * lk2, c->knorm.as<double>() + k0, st);
    }
    if (!c->err_code && use_mixed(c, false) && c->dominant_frac > 0.0)
      CKR(redo_dominant_k(c, itcpa, lcls, rcls, icls));
    if (c->err_code) {
      if (c->red_fn || c->red_dev_fn) reduce_tauc(c, true);  // tell the other ranks before returning
      break;
    }
    // rotation of the class sums: tauc = sum_g L_g S[class(g)] R_g   (cpacoord_ksave.f:382-391)
    CKR(c->T1.ensure((size_t)ni * c->ngeff * lk2 * sizeof(zd)));
    CKR(c->T2.ensure((size_t)ni * c->ngeff * lk2 * sizeof(zd)));
    CKR(c->tauc.ensure((size_t)ni * lk2 * sizeof(zd)));
    {
      int cmap[SKKR_MAPN];
      for (int g = 0; g < c->ngeff; g++) {
        int cls = c->ieqg[g] - 1;
        cmap[g] = (int)(std::find(icls.begin(), icls.end(), cls) - icls.begin());
      }
      MatRef Lm = mref(c->lg.as<zd>(), 0, lk2, lk);
      MatRef Sm = mref_map(c->S.as<zd>(), lk2, (long long)ni * lk2, lk, cmap, c->ngeff);
      MatRef T1m = mref(c->T1.as<zd>(), (long long)c->ngeff * lk2, lk2, lk);
      MatRef Rm = mref(c->rg.as<zd>(), 0, lk2, lk);
      MatRef T2m = mref(c->T2.as<zd>(), (long long)c->ngeff * lk2, lk2, lk);
      launch_zgemm(0, Lm, Sm, T1m, T1m, T1m, lk, lk, lk, ni, c->ngeff, nullptr, st);
      launch_zgemm(0, T1m, Rm, T2m, T2m, T2m, lk, lk, lk, ni, c->ngeff, nullptr, st);
      launch_gsum(c->T2.as<zd>(), c->ngeff, lk, ni, c->tauc.as<zd>(), st);
    }
    if (c->red_fn || c->red_dev_fn) {
      int rrc = reduce_tauc(c, false);
      if (rrc != SKKR_OK) {
        c->err_code = rrc;
        break;
      }
    }
    trace_point("before cpa_step");
    int rc = cpa_step(c, &itcpa, &cpacon, &concpa, &cpaerr);
    trace_point("after cpa_step");
    if (rc != SKKR_OK) {
      c->err_code = rc;
      break;
    }
    if (!(concpa && cpacon)) break;
  }
  trace_point("after CPA loop");
  c->inv_fallbacks = 0;
  c->inv_refined = 0;
  if (c->mw) CKR(mixed_resid_read(c->mw, &c->max_resid, &c->inv_fallbacks, &c->inv_refined, st));
  if (c->mw && c->err_code == 0) {
    int f = mixed_error_flag(c->mw);
    if (f != 0) {
      g_last_error = "tensor-core kernel: bounded wait expired";
      c->err_code = SKKR_ERR_CUDA;
    }
  }
  CK(cudaEventRecord(ev1, st));
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());
  float run_ms = 0.f;
  CK(cudaEventElapsedTime(&run_ms, ev0, ev1));
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  if (status) {
    status->code = c->err_code;
    status->ik = c->first_bad_k;
    status->cpa_iterations = itcpa - 1;
    status->cpa_error = cpaerr;
    status->max_dec_iters = c->max_dec;
    status->dec_iters_total = c->tot_dec;
    // host-issued launches plus the kernels run inside graphs
    status->gpu_launches = g_skkr_launches - l0 + c->graph_kernels;
    status->max_refine_resid = c->max_resid;
    status->run_ms = run_ms;
    status->inv_fallbacks = c->inv_fallbacks;
    status->inv_refined = c->inv_refined;
    status->k_fp64 = c->k_fp64;
    status->alg_flops = c->alg_units * 8.0 * (double)n * n * n;
    status->graph_launches = c->graph_launches;
    status->graph_kernels = c->graph_kernels;
  }
  return c->err_code;
}

extern "C" int skkr_gpu_fetch(skkr_ctx *c, double *tminv, double *tauc, double *taua, double *taub,
                              int ld) {
  if (!c || !c->staged || ld < c->lk) return SKKR_ERR_ARG;
  const int lk = c->lk, lk2 = lk * lk, ni = c->nintfc;
  cudaStream_t st = c->st;
  if (tminv) CKR(get_mats(tminv, c->tcat.as<zd>() + (size_t)2 * c->pl * lk2, ni, lk, ld, st));
  if (tauc) CKR(get_mats(tauc, c->tauc.as<zd>(), ni, lk, ld, st));
  zd *TAB = c->cpa.as<zd>() + (size_t)ni * 7 * lk2;
  if (taua) CKR(get_mats(taua, TAB, ni, lk, ld, st, 2LL * lk2));
  if (taub) CKR(get_mats(taub, TAB + lk2, ni, lk, ld, st, 2LL * lk2));
  return SKKR_OK;
}

extern "C" int skkr_gpu_cpacoord(skkr_ctx *c, double ce_re, double ce_im, double fac_re,
                                 double fac_im, const skkr_rtable *rt, int nk, const double *xk,
                                 const double *wk, const double *lg, const double *rg,
                                 const double *conc, const double *tminvl, const double *tminvr,
                                 double *tminv, const double *tminva, const double *tminvb,
                                 double *tauc, double *taua, double *taub, int ld,
                                 skkr_status *status) {
  int rc = skkr_gpu_stage(c, ce_re, ce_im, fac_re, fac_im, rt, nk, xk, wk, lg, rg, conc, tminvl,
                          tminvr, tminv, tminva, tminvb, ld);
  if (rc != SKKR_OK) {
    if (status) status->code = rc;
    return rc;
  }
  rc = skkr_gpu_run(c, status);
  if (rc != SKKR_OK) return rc;
  return skkr_gpu_fetch(c, tminv, tauc, taua, taub, ld);
}

extern "C" int skkr_gpu_cpacoord_bdg(skkr_ctx *c, double ce_re, double ce_im, double fac_re,
                                     double fac_im, double fach_re, double fach_im,
                                     const skkr_rtable *rt, int nk, const double *xk,
                                     const double *wk, const double *lg, const double *rg,
                                     const double *conc, const double *tminvl,
                                     const double *tminvr, double *tminv, const double *tminva,
                                     const double *tminvb, double *tauc, double *taua,
                                     double *taub, int ld, skkr_status *status) {
  if (!c || c->sz.mode != SKKR_BDG) return SKKR_ERR_ARG;
  c->fach = zmk(fach_re, fach_im);
  return skkr_gpu_cpacoord(c, ce_re, ce_im, fac_re, fac_im, rt, nk, xk, wk, lg, rg, conc, tminvl,
                           tminvr, tminv, tminva, tminvb, tauc, taua, taub, ld, status);
}

// A list of energies of one system in one call (the contour loop of
// rsp-scf/skkr.f:389-486 around cpacoord, :439): energy e runs args[e] as
// skkr_gpu_cpacoord would (BdG contexts: skkr_gpu_cpacoord_bdg), one after
// the other on the context's stream, each with its decimation graphs; st[e]
// receives its status.  Every energy runs even after one fails; the first
// nonzero code is returned.
extern "C" int skkr_gpu_contour(skkr_ctx *c, int ne, const skkr_energy_args *args, skkr_status *st) {
  if (!c || ne < 1 || !args) return SKKR_ERR_ARG;
  int first = SKKR_OK;
  for (int e = 0; e < ne; e++) {
    const skkr_energy_args &a = args[e];
    skkr_status *s = st ? st + e : nullptr;
    int rc;
    if (c->sz.mode == SKKR_BDG)
      rc = skkr_gpu_cpacoord_bdg(c, a.ce_re, a.ce_im, a.fac_re, a.fac_im, a.fach_re, a.fach_im, a.rt, a.nk, a.xk,
                                 a.wk, a.lg, a.rg, a.conc, a.tminvl, a.tminvr, a.tminv, a.tminva, a.tminvb, a.tauc,
                                 a.taua, a.taub, a.ld, s);
    else
      rc = skkr_gpu_cpacoord(c, a.ce_re, a.ce_im, a.fac_re, a.fac_im, a.rt, a.nk, a.xk, a.wk, a.lg, a.rg, a.conc,
                             a.tminvl, a.tminvr, a.tminv, a.tminva, a.tminvb, a.tauc, a.taua, a.taub, a.ld, s);
    if (s && rc != SKKR_OK) s->code = rc;
    if (rc != SKKR_OK && first == SKKR_OK) first = rc;
  }
  return first;
}

// Several systems at once: context e runs args[e] on its own stream from its
// own host thread, so the kernels of a small system fill the SMs a large one
// leaves idle.  The contexts must be distinct.
extern "C" int skkr_gpu_cpacoord_many(int n, skkr_ctx *const *ctx, const skkr_energy_args *args,
                                      skkr_status *st) {
  if (n < 1 || !ctx || !args) return SKKR_ERR_ARG;
  for (int e = 0; e < n; e++) {
    if (!ctx[e]) return SKKR_ERR_ARG;
    for (int f = 0; f < e; f++)
      if (ctx[f] == ctx[e]) return SKKR_ERR_ARG;
  }
  std::vector<int> rc(n, SKKR_OK);
  // the contexts run concurrently from their own host threads: their
  // decimation loops run from the host (graph capture from several threads
  // at once is left out), the other threads' launches fill the GPU meanwhile
  std::vector<bool> graphs(n);
  for (int e = 0; e < n; e++) {
    graphs[e] = ctx[e]->graphs;
    ctx[e]->graphs = false;
  }
  auto one = [&](int e) {
    skkr_ctx *c = ctx[e];
    const skkr_energy_args &a = args[e];
    if (cudaSetDevice(c->dev) != cudaSuccess) {
      rc[e] = SKKR_ERR_CUDA;
      return;
    }
    skkr_status *s = st ? st + e : nullptr;
    if (c->sz.mode == SKKR_BDG)
      rc[e] = skkr_gpu_cpacoord_bdg(c, a.ce_re, a.ce_im, a.fac_re, a.fac_im, a.fach_re, a.fach_im, a.rt,
                                    a.nk, a.xk, a.wk, a.lg, a.rg, a.conc, a.tminvl, a.tminvr, a.tminv,
                                    a.tminva, a.tminvb, a.tauc, a.taua, a.taub, a.ld, s);
    else
      rc[e] = skkr_gpu_cpacoord(c, a.ce_re, a.ce_im, a.fac_re, a.fac_im, a.rt, a.nk, a.xk, a.wk, a.lg,
                                a.rg, a.conc, a.tminvl, a.tminvr, a.tminv, a.tminva, a.tminvb, a.tauc,
                                a.taua, a.taub, a.ld, s);
  };
  std::vector<std::thread> th;
  for (int e = 1; e < n; e++) th.emplace_back(one, e);
  one(0);
  for (auto &t : th) t.join();
  for (int e = 0; e < n; e++) ctx[e]->graphs = graphs[e];
  for (int e = 0; e < n; e++)
    if (rc[e] != SKKR_OK) return rc[e];
  return SKKR_OK;
}

// ---------------------------------------------------------------------------
// multi-energy residency: stage several energies, run / fetch any of them
static SlotStore *get_slot(skkr_ctx *c, int slot, bool create) {
  if (slot < 0 || slot > 4096) return nullptr;
  if ((int)c->slots.size() <= slot) {
    if (!create) return nullptr;
    c->slots.resize(slot + 1, nullptr);
  }
  if (!c->slots[slot]) {
    if (!create) return nullptr;
    c->slots[slot] = new SlotStore();
  }
  return c->slots[slot];
}

extern "C" int skkr_gpu_stage_slot(skkr_ctx *c, int slot, double ce_re, double ce_im, double fac_re,
                                   double fac_im, const skkr_rtable *rt, int nk, const double *xk,
                                   const double *wk, const double *lg, const double *rg,
                                   const double *conc, const double *tminvl,
                                   const double *tminvr, const double *tminv,
                                   const double *tminva, const double *tminvb, int ld) {
  if (!c) return SKKR_ERR_ARG;
  if (c->sz.mode == SKKR_BDG) return SKKR_ERR_UNSUPPORTED;  // BdG energies go through cpacoord_bdg
  SlotStore *s = get_slot(c, slot, true);
  if (!s) return SKKR_ERR_ARG;
  swap_slot(c, *s);
  int rc = skkr_gpu_stage(c, ce_re, ce_im, fac_re, fac_im, rt, nk, xk, wk, lg, rg, conc, tminvl,
                          tminvr, tminv, tminva, tminvb, ld);
  swap_slot(c, *s);
  return rc;
}

extern "C" int skkr_gpu_run_slot(skkr_ctx *c, int slot, skkr_status *status) {
  if (!c) return SKKR_ERR_ARG;
  SlotStore *s = get_slot(c, slot, false);
  if (!s || !s->staged) return SKKR_ERR_ARG;
  swap_slot(c, *s);
  const bool kon = c->kambe_on;  // the k-space form belongs to the energy of skkr_gpu_stage
  c->kambe_on = false;
  int rc = skkr_gpu_run(c, status);
  c->kambe_on = kon;
  swap_slot(c, *s);
  return rc;
}

extern "C" int skkr_gpu_fetch_slot(skkr_ctx *c, int slot, double *tminv, double *tauc,
                                   double *taua, double *taub, int ld) {
  if (!c) return SKKR_ERR_ARG;
  SlotStore *s = get_slot(c, slot, false);
  if (!s || !s->staged) return SKKR_ERR_ARG;
  swap_slot(c, *s);
  int rc = skkr_gpu_fetch(c, tminv, tauc, taua, taub, ld);
  swap_slot(c, *s);
  return rc;
}

// ---------------------------------------------------------------------------
// Stand-alone batched entry points (tests, callers that drive their own loop).
// Each allocates its device buffers for the duration of the call.
namespace {
struct Scoped {
  std::vector<void *> ptrs;
  ~Scoped() {
    for (void *p : ptrs) cudaFree(p);
  }
  template <class T>
  int alloc(T **p, size_t count) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 16);
    if (e != cudaSuccess) {
      g_last_error = std::string("cudaMalloc: ") + cudaGetErrorString(e);
      return SKKR_ERR_NOMEM;
    }
    ptrs.push_back(q);
    *p = (T *)q;
    return SKKR_OK;
  }
};

int upload_mats(zd *dst, const double *src, int count, int n, int ld) {
  std::vector<zd> tmp((size_t)count * n * n);
  for (int m = 0; m < count; m++)
    for (int c = 0; c < n; c++)
      for (int r = 0; r < n; r++) {
        size_t s = ((size_t)m * ld * ld + r + (size_t)c * ld) * 2;
        tmp[(size_t)m * n * n + r + (size_t)c * n] = zmk(src[s], src[s + 1]);
      }
  CK(cudaMemcpy(dst, tmp.data(), tmp.size() * sizeof(zd), cudaMemcpyHostToDevice));
  return SKKR_OK;
}
int download_mats(double *dst, const zd *src, int count, int n, int ld) {
  std::vector<zd> tmp((size_t)count * n * n);
  CK(cudaMemcpy(tmp.data(), src, tmp.size() * sizeof(zd), cudaMemcpyDeviceToHost));
  for (int m = 0; m < count; m++)
    for (int c = 0; c < n; c++)
      for (int r = 0; r < n; r++) {
        zd v = tmp[(size_t)m * n * n + r + (size_t)c * n];
        size_t d = ((size_t)m * ld * ld + r + (size_t)c * ld) * 2;
        dst[d] = v.x;
        dst[d + 1] = v.y;
      }
  return SKKR_OK;
}
}  // namespace

extern "C" int skkr_gpu_gjinv_batch(int n, int batch, double *a, int ld) {
  if (n < 1 || n > 512 || batch < 1 || !a || ld < n) return SKKR_ERR_ARG;
  Scoped s;
  zd *d;
  CKR(s.alloc(&d, (size_t)batch * n * n));
  CKR(upload_mats(d, a, batch, n, ld));
  launch_zgj(mref(d, (long long)n * n, 0, n), n, batch, 1, nullptr, 0);
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  return download_mats(a, d, batch, n, ld);
}

// tau2d (main/tau2d.f:2-152) for `batch` independent items of nprc principal
// layers of n rows each, on host arrays: the forward sweep
// yy(0) = Y, yy(p) = M10(p) (M00(p-1) - yy(p-1))^-1 M01(p-1), the backward
// sweep xx(nprc-1) = X, xx(p) = M01(p) (T00(p+1) - xx(p+1))^-1 M10(p+1), and
// tau(p) = (M00(p) - xx(p) - yy(p))^-1, whose diagonal lk x lk blocks times
// wgeff are the layer taus.  M00 carries the layers' t^-1 blocks.  FP64.
extern "C" int skkr_gpu_tau2d(int batch, int nprc, int n, int lk, double wgeff, const double *m00,
                              const double *m01, const double *m10, const double *x, const double *y, double *tau) {
  if (batch < 1 || nprc < 1 || n < 1 || n > 512 || lk < 1 || n % lk || !m00 || !m01 || !m10 || !x || !y || !tau ||
      (long long)batch * nprc > 65535)
    return SKKR_ERR_ARG;
  const long long MB = (long long)n * n, per = (long long)nprc * MB;
  const int nl = n / lk;
  Scoped s;
  zd *M00, *M01, *M10, *XX, *YY, *T00, *W;
  CKR(s.alloc(&M00, batch * per));
  CKR(s.alloc(&M01, batch * per));
  CKR(s.alloc(&M10, batch * per));
  CKR(s.alloc(&XX, batch * per));
  CKR(s.alloc(&YY, batch * per));
  CKR(s.alloc(&T00, batch * per));
  CKR(s.alloc(&W, batch * MB));
  CKR(upload_mats(M00, m00, batch * nprc, n, n));
  CKR(upload_mats(M01, m01, batch * nprc, n, n));
  CKR(upload_mats(M10, m10, batch * nprc, n, n));
  // item k, PL p at base + k per + p MB; the sweeps run over k for one p
  auto pl = [&](zd *b, int p) { return mref(b + (long long)p * MB, per, 0, n); };
  const MatRef w = mref(W, MB, 0, n);
  {
    // X and Y of item k into PL nprc-1 of XX and PL 0 of YY
    Scoped t;
    zd *xs, *ys;
    CKR(t.alloc(&xs, batch * MB));
    CKR(t.alloc(&ys, batch * MB));
    CKR(upload_mats(xs, x, batch, n, n));
    CKR(upload_mats(ys, y, batch, n, n));
    launch_zaxpby(pl(XX, nprc - 1), mref(xs, MB, 0, n), nullptr, 0, nullptr, 0, n, batch, 1, nullptr, 0);
    launch_zaxpby(pl(YY, 0), mref(ys, MB, 0, n), nullptr, 0, nullptr, 0, n, batch, 1, nullptr, 0);
    CK(cudaDeviceSynchronize());
  }
  for (int p = 0; p < nprc; p++) {
    MatRef t00 = pl(T00, p), yy = pl(YY, p), m00p = pl(M00, p);
    launch_zaxpby(t00, m00p, nullptr, 0, nullptr, 0, n, batch, 1, nullptr, 0);
    if (p > 0) {
      // yy(p) holds (M00(p-1) - yy(p-1))^-1 M01(p-1): multiply by M10(p)
      launch_zgemm(0, pl(M10, p), yy, w, w, w, n, n, n, batch, 1, nullptr, 0);
      launch_zaxpby(yy, w, nullptr, 0, nullptr, 0, n, batch, 1, nullptr, 0);
    }
    if (p < nprc - 1) {
      launch_zaxpby(w, m00p, &yy, -1.0, nullptr, 0, n, batch, 1, nullptr, 0);
      launch_zgj(w, n, batch, 1, nullptr, 0);
      launch_zgemm(0, w, pl(M01, p), pl(YY, p + 1), pl(YY, p + 1), pl(YY, p + 1), n, n, n, batch, 1, nullptr, 0);
    }
  }
  for (int p = nprc - 1; p >= 0; p--) {
    MatRef xx = pl(XX, p);
    if (p < nprc - 1) {
      launch_zgemm(0, pl(M01, p), xx, w, w, w, n, n, n, batch, 1, nullptr, 0);
      launch_zaxpby(xx, w, nullptr, 0, nullptr, 0, n, batch, 1, nullptr, 0);
    }
    if (p > 0) {
      MatRef t00 = pl(T00, p);
      launch_zaxpby(w, t00, &xx, -1.0, nullptr, 0, n, batch, 1, nullptr, 0);
      launch_zgj(w, n, batch, 1, nullptr, 0);
      launch_zgemm(0, w, pl(M10, p), pl(XX, p - 1), pl(XX, p - 1), pl(XX, p - 1), n, n, n, batch, 1, nullptr, 0);
    }
  }
  for (int p = 0; p < nprc; p++) {
    MatRef t00 = pl(T00, p), xx = pl(XX, p), yy = pl(YY, p);
    launch_zaxpby(t00, t00, &xx, -1.0, &yy, -1.0, n, batch, 1, nullptr, 0);
    launch_zgj(t00, n, batch, 1, nullptr, 0);
  }
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  // layer blocks: tau[k][p nl + l] = wgeff T00[k][p] block (l, l)
  std::vector<zd> h((size_t)batch * per);
  CK(cudaMemcpy(h.data(), T00, (size_t)batch * per * sizeof(zd), cudaMemcpyDeviceToHost));
  const long long L2 = (long long)lk * lk;
  for (int k = 0; k < batch; k++)
    for (int p = 0; p < nprc; p++)
      for (int l = 0; l < nl; l++)
        for (int c = 0; c < lk; c++)
          for (int r = 0; r < lk; r++) {
            const zd v = h[(size_t)(k * per + p * MB + (long long)(l * lk + r) + (long long)(l * lk + c) * n)];
            const long long o = (((long long)k * nprc + p) * nl + l) * L2 + r + (long long)c * lk;
            tau[2 * o] = wgeff * v.x;
            tau[2 * o + 1] = wgeff * v.y;
          }
  return SKKR_OK;
}

extern "C" int skkr_gpu_gk(const skkr_rtable *rt, int lmax, int nk, const double *xk, double *out) {
  if (!rt || nk < 1 || !xk || !out || lmax < 0 || lmax > 3) return SKKR_ERR_ARG;
  const int lmmax = (lmax + 1) * (lmax + 1), nr = rt->rstart[rt->nblk];
  for (int b = 0; b < rt->nblk; b++)
    if (rt->rstart[b + 1] - rt->rstart[b] > 64) return SKKR_ERR_UNSUPPORTED;
  const size_t bs = (size_t)lmmax * lmmax;
  Scoped s;
  zd *gR, *o;
  double *rv, *kx;
  int *rs;
  CKR(s.alloc(&gR, nr * bs));
  CKR(s.alloc(&o, (size_t)nk * rt->nblk * bs));
  CKR(s.alloc(&rv, 2 * (size_t)nr));
  CKR(s.alloc(&kx, 2 * (size_t)nk));
  CKR(s.alloc(&rs, rt->nblk + 1));
  CK(cudaMemcpy(gR, rt->gR, nr * bs * sizeof(zd), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(rv, rt->rvec, 2 * (size_t)nr * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(kx, xk, 2 * (size_t)nk * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(rs, rt->rstart, (rt->nblk + 1) * sizeof(int), cudaMemcpyHostToDevice));
  launch_gk_ft(gR, rv, rs, rt->nblk, lmmax, kx, nk, o, 0);
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  CK(cudaMemcpy(out, o, (size_t)nk * rt->nblk * bs * sizeof(zd), cudaMemcpyDeviceToHost));
  return SKKR_OK;
}

extern "C" int skkr_gpu_surfgf_batch(int n, int batch, const double *ml, const double *m0,
                                     const double *mr, double *x, int ld, int itermax,
                                     double errmax, int *iters, int *stat) {
  if (n < 1 || n > 256 || batch < 1 || !ml || !m0 || !mr || !x || ld < n) return SKKR_ERR_ARG;
  const long long MB = (long long)n * n;
  Scoped s;
  zd *W;
  double *err;
  int *flags;
  CKR(s.alloc(&W, (size_t)batch * 12 * MB));
  CKR(s.alloc(&err, batch));
  CKR(s.alloc(&flags, 3 * (size_t)batch));
  // per item: 0 ml 1 m0 2 mr 3 eps 4 a0 5 a1 6 b0 7 b1 8 x 9 y1 10 P 11 Q
  auto buf = [&](int b) { return mref(W + (long long)b * MB, 12 * MB, 0, n); };
  {
    std::vector<zd> tmp((size_t)batch * 12 * MB);
    const double *srcs[3] = {ml, m0, mr};
    for (int q = 0; q < 3; q++)
      for (int m = 0; m < batch; m++)
        for (int c = 0; c < n; c++)
          for (int r = 0; r < n; r++) {
            size_t si = ((size_t)m * ld * ld + r + (size_t)c * ld) * 2;
            tmp[(size_t)m * 12 * MB + q * MB + r + (size_t)c * n] = zmk(srcs[q][si], srcs[q][si + 1]);
          }
    CK(cudaMemcpy(W, tmp.data(), tmp.size() * sizeof(zd), cudaMemcpyHostToDevice));
  }
  int *act = flags, *st = flags + batch, *it = flags + 2 * batch;
  std::vector<int> ones(batch, 1);
  CK(cudaMemcpy(act, ones.data(), batch * sizeof(int), cudaMemcpyHostToDevice));
  CK(cudaMemset(st, 0, batch * sizeof(int)));
  CK(cudaMemset(it, 0, batch * sizeof(int)));
  MatRef Ml = buf(0), M0 = buf(1), Mr = buf(2), eps = buf(3), a0 = buf(4), a1 = buf(5), b0 = buf(6),
         b1 = buf(7), X = buf(8), y1 = buf(9), P = buf(10), Q = buf(11);
  launch_zaxpby(eps, M0, nullptr, 0, nullptr, 0, n, batch, 1, nullptr, 0);
  launch_zaxpby(X, M0, nullptr, 0, nullptr, 0, n, batch, 1, nullptr, 0);
  launch_zaxpby(a0, Ml, &Ml, -2.0, nullptr, 0, n, batch, 1, nullptr, 0);
  launch_zaxpby(b0, Mr, &Mr, -2.0, nullptr, 0, n, batch, 1, nullptr, 0);
  for (int iter = 1;; iter++) {
    MatRef &ac = (iter & 1) ? a0 : a1, &an = (iter & 1) ? a1 : a0;
    MatRef &bc = (iter & 1) ? b0 : b1, &bn = (iter & 1) ? b1 : b0;
    launch_zaxpby(y1, eps, nullptr, 0, nullptr, 0, n, batch, 1, act, 0);
    launch_zgj(y1, n, batch, 1, act, 0);
    launch_zgemm(0, ac, y1, P, P, P, n, n, n, batch, 1, act, 0);
    launch_zgemm(0, bc, y1, Q, Q, Q, n, n, n, batch, 1, act, 0);
    launch_zgemm(0, P, ac, an, an, an, n, n, n, batch, 1, act, 0);
    launch_zgemm(0, Q, bc, bn, bn, bn, n, n, n, batch, 1, act, 0);
    launch_zgemm(2, P, bc, P, eps, X, n, n, n, batch, 1, act, 0);
    launch_zgemm(1, Q, ac, eps, eps, eps, n, n, n, batch, 1, act, 0);
    launch_fnorm(an, n, batch, 1, act, err, 0);
    launch_dec_state(err, act, st, it, batch, iter, itermax, errmax, 0);
    std::vector<int> h(batch);
    CK(cudaMemcpy(h.data(), act, batch * sizeof(int), cudaMemcpyDeviceToHost));
    int any = 0;
    for (int v : h) any |= v;
    if (!any || iter > itermax + 1) break;
  }
  launch_zgj(X, n, batch, 1, nullptr, 0);
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  if (iters) CK(cudaMemcpy(iters, it, batch * sizeof(int), cudaMemcpyDeviceToHost));
  if (stat) CK(cudaMemcpy(stat, st, batch * sizeof(int), cudaMemcpyDeviceToHost));
  {
    std::vector<zd> tmp((size_t)batch * 12 * MB);
    CK(cudaMemcpy(tmp.data(), W, tmp.size() * sizeof(zd), cudaMemcpyDeviceToHost));
    for (int m = 0; m < batch; m++)
      for (int c = 0; c < n; c++)
        for (int r = 0; r < n; r++) {
          zd v = tmp[(size_t)m * 12 * MB + 8 * MB + r + (size_t)c * n];
          size_t d = ((size_t)m * ld * ld + r + (size_t)c * ld) * 2;
          x[d] = v.x;
          x[d + 1] = v.y;
        }
  }
  return SKKR_OK;
}

// rsp-scf/phystau.f / nrsp-scf/phystau.f on the device
__global__ void k_phys_mats(const zd *tinv, const zd *alpha, const int *lof, int nd, zd *lmat,
                            zd *rmat, zd *cmat) {
  for (int e = threadIdx.x + blockIdx.x * blockDim.x; e < nd * nd; e += blockDim.x * gridDim.x) {
    const int a = e % nd, b = e / nd;
    zd al = alpha[lof[a]], alp = alpha[lof[b]], t = tinv[e];
    zd lv = zmul(al, t), rv = zmul(t, alp), cv = zmul(zmul(al, t), alp);
    if (a == b) {
      lv.x += 1.0;
      rv.x += 1.0;
      cv = zadd(al, cv);
    }
    lmat[e] = lv;
    rmat[e] = rv;
    cmat[e] = cv;
  }
}

// basis size, number of screening constants and the l of every basis index
// of phystau.f / phystau2.f (ldex over kappa-mu: 2 entries for l = 0, 4l+2
// for l > 0; BdG: the hole half indexes alpha_h, stored after alpha_e)
static int phys_basis(int mode, int lmax, int ld, int *nd, int *nal, std::vector<int> &lof) {
  if (lmax < 0 || lmax > 3) return SKKR_ERR_ARG;
  if (mode != SKKR_NONREL && mode != SKKR_REL && mode != SKKR_BDG) return SKKR_ERR_ARG;
  const int lmmax = (lmax + 1) * (lmax + 1);
  *nd = mode == SKKR_BDG ? 4 * lmmax : mode == SKKR_REL ? 2 * lmmax : lmmax;
  *nal = mode == SKKR_BDG ? 2 * (lmax + 1) : lmax + 1;  // BdG: alpha_e then alpha_h
  if (ld < *nd) return SKKR_ERR_ARG;
  lof.assign(*nd, 0);
  if (mode != SKKR_NONREL) {
    int k = 0;
    for (int l = 0; k < 2 * lmmax; l++)
      for (int q = 0; q < (l == 0 ? 2 : 4 * l + 2) && k < 2 * lmmax; q++) lof[k++] = l;
    for (int q = 2 * lmmax; q < *nd; q++) lof[q] = lof[q - 2 * lmmax] + lmax + 1;
  } else {
    for (int l = 0, k = 0; l <= lmax; l++)
      for (int m = -l; m <= l; m++) lof[k++] = l;
  }
  return SKKR_OK;
}

extern "C" int skkr_gpu_phystau(int mode, int lmax, double *tau, const double *tinv,
                                const double *alpha, int ld) {
  if (!tau || !tinv || !alpha) return SKKR_ERR_ARG;
  int nd, nal;
  std::vector<int> lof;
  CKR(phys_basis(mode, lmax, ld, &nd, &nal, lof));
  const long long MB = (long long)nd * nd;
  Scoped s;
  zd *T, *Ti, *Al, *Lm, *Rm, *Cm, *H;
  int *Lo;
  CKR(s.alloc(&T, MB));
  CKR(s.alloc(&Ti, MB));
  CKR(s.alloc(&Al, nal));
  CKR(s.alloc(&Lm, MB));
  CKR(s.alloc(&Rm, MB));
  CKR(s.alloc(&Cm, MB));
  CKR(s.alloc(&H, MB));
  CKR(s.alloc(&Lo, nd));
  CKR(upload_mats(T, tau, 1, nd, ld));
  CKR(upload_mats(Ti, tinv, 1, nd, ld));
  CK(cudaMemcpy(Al, alpha, nal * sizeof(zd), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(Lo, lof.data(), nd * sizeof(int), cudaMemcpyHostToDevice));
  k_phys_mats<<<4, 256>>>(Ti, Al, Lo, nd, Lm, Rm, Cm);
  SKKR_LAUNCHED();
  // tripmt(lmat, tau, rmat): (lmat tau) rmat ; then tau - cmat
  launch_zgemm(0, mref(Lm, 0, 0, nd), mref(T, 0, 0, nd), mref(H, 0, 0, nd), mref(H, 0, 0, nd),
               mref(H, 0, 0, nd), nd, nd, nd, 1, 1, nullptr, 0);
  launch_zgemm(0, mref(H, 0, 0, nd), mref(Rm, 0, 0, nd), mref(T, 0, 0, nd), mref(T, 0, 0, nd),
               mref(T, 0, 0, nd), nd, nd, nd, 1, 1, nullptr, 0);
  MatRef Tm = mref(T, 0, 0, nd), Cmm = mref(Cm, 0, 0, nd);
  launch_zaxpby(Tm, Tm, &Cmm, -1.0, nullptr, 0, nd, 1, 1, nullptr, 0);
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  return download_mats(tau, T, 1, nd, ld);
}

extern "C" int skkr_gpu_phystau2(int mode, int lmax, double *tau, const double *tinv1,
                                 const double *alpha1, const double *tinv2, const double *alpha2,
                                 int ld) {
  if (!tau || !tinv1 || !alpha1 || !tinv2 || !alpha2) return SKKR_ERR_ARG;
  int nd, nal;
  std::vector<int> lof;
  CKR(phys_basis(mode, lmax, ld, &nd, &nal, lof));
  const long long MB = (long long)nd * nd;
  Scoped s;
  zd *T, *Ti1, *Ti2, *Al1, *Al2, *Lm, *Rm, *Sc, *Cm, *H;
  int *Lo;
  CKR(s.alloc(&T, MB));
  CKR(s.alloc(&Ti1, MB));
  CKR(s.alloc(&Ti2, MB));
  CKR(s.alloc(&Al1, nal));
  CKR(s.alloc(&Al2, nal));
  CKR(s.alloc(&Lm, MB));
  CKR(s.alloc(&Rm, MB));
  CKR(s.alloc(&Sc, MB));
  CKR(s.alloc(&Cm, MB));
  CKR(s.alloc(&H, MB));
  CKR(s.alloc(&Lo, nd));
  CKR(upload_mats(T, tau, 1, nd, ld));
  CKR(upload_mats(Ti1, tinv1, 1, nd, ld));
  CKR(upload_mats(Ti2, tinv2, 1, nd, ld));
  CK(cudaMemcpy(Al1, alpha1, nal * sizeof(zd), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(Al2, alpha2, nal * sizeof(zd), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(Lo, lof.data(), nd * sizeof(int), cudaMemcpyHostToDevice));
  // lmat = 1 + alpha1 tinv1 from the row layer, rmat = 1 + tinv2 alpha2 from
  // the column layer (the other two outputs of each launch are scratch)
  k_phys_mats<<<4, 256>>>(Ti1, Al1, Lo, nd, Lm, Sc, Cm);
  SKKR_LAUNCHED();
  k_phys_mats<<<4, 256>>>(Ti2, Al2, Lo, nd, Sc, Rm, Cm);
  SKKR_LAUNCHED();
  launch_zgemm(0, mref(Lm, 0, 0, nd), mref(T, 0, 0, nd), mref(H, 0, 0, nd), mref(H, 0, 0, nd),
               mref(H, 0, 0, nd), nd, nd, nd, 1, 1, nullptr, 0);
  launch_zgemm(0, mref(H, 0, 0, nd), mref(Rm, 0, 0, nd), mref(T, 0, 0, nd), mref(T, 0, 0, nd),
               mref(T, 0, 0, nd), nd, nd, nd, 1, 1, nullptr, 0);
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  return download_mats(tau, T, 1, nd, ld);
}

extern "C" int skkr_gpu_layer_dos(int mode, int lmax, int nlay, const double *tau, int ld,
                                  const double *F, const double *G, int para, double *zmom,
                                  double *zdos_l) {
  if (!tau || !F || !G || !zmom || !zdos_l || lmax < 0 || lmax > 3 || nlay < 1) return SKKR_ERR_ARG;
  const int lmmax = (lmax + 1) * (lmax + 1), rel = mode == SKKR_REL,
            nd = rel ? 2 * lmmax : lmmax, nl = lmax + 1;
  if (ld < nd) return SKKR_ERR_ARG;
  double fac = -1.0 / 3.14159265358979323846;
  if (para && !rel) fac *= 2.0;  // spin degeneracy of the non-relativistic DOS
  Scoped s;
  zd *T, *Fd, *Gd, *Zm, *Zl;
  CKR(s.alloc(&T, (long long)nlay * nd * nd));
  CKR(s.alloc(&Fd, (long long)nlay * nd));
  CKR(s.alloc(&Gd, (long long)nlay * nd));
  CKR(s.alloc(&Zm, (long long)nlay * nd));
  CKR(s.alloc(&Zl, (long long)nlay * nl));
  CKR(upload_mats(T, tau, nlay, nd, ld));
  CK(cudaMemcpy(Fd, F, (size_t)nlay * nd * sizeof(zd), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(Gd, G, (size_t)nlay * nd * sizeof(zd), cudaMemcpyHostToDevice));
  launch_layer_dos(rel, nd, nl, nlay, T, nd, Fd, Gd, fac, Zm, Zl, 0);
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  CK(cudaMemcpy(zmom, Zm, (size_t)nlay * nd * sizeof(zd), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(zdos_l, Zl, (size_t)nlay * nl * sizeof(zd), cudaMemcpyDeviceToHost));
  return SKKR_OK;
}

// ---------------------------------------------------------------------------
// Bloch spectral function (skkr_dbogo_bsf/rsp-scf/bsf.f:2-437 with gf.f,
// pairing.f and moment.f at lambda = 0) of nlay layers at nk k points.  Per
// CPA layer (1 - conc > 1e-6): tau_c^-1, D_a = tau_a tau_c^-1 and
// D~_a = tau_c^-1 tau_a once; per k point tau(k) - tau_c and the four
// D_a (tau(k) - tau_c) D~_b; then k_bsf_reduce.  Layers without CPA use
// tau(k) itself.  Chunks of k points keep the work buffers bounded.
extern "C" int skkr_gpu_bsf(int mode, int lmax, int nk, int nlay, const double *conc, const double *tauk,
                            const double *tauc, const double *taua, const double *taub, const double *F,
                            const double *Feh, const double *pair, int para, double *out) {
  if (!conc || !tauk || !tauc || !taua || !taub || !F || !out || nk < 1 || nlay < 1 || nlay > SKKR_MAPN)
    return SKKR_ERR_ARG;
  int nd, nal;
  std::vector<int> lof;
  CKR(phys_basis(mode, lmax, 0x7fffffff, &nd, &nal, lof));
  const int bdg = mode == SKKR_BDG, nde = bdg ? nd / 2 : nd;
  if (bdg && (!Feh || !pair)) return SKKR_ERR_ARG;
  const long long MB = (long long)nd * nd, NE2 = (long long)nde * nde;
  double fac = -1.0 / 3.14159265358979323846;
  if (para && mode == SKKR_NONREL) fac *= 2.0;
  std::vector<int> cpa(nlay);
  for (int l = 0; l < nlay; l++) cpa[l] = (1.0 - conc[l]) > 1.0e-6;
  // k points per chunk: grid.y of the batched kernels holds kc * nlay, and the
  // seven per-k matrices of a chunk stay within 2 GB
  const long long per_k = 7LL * nlay * MB * (long long)sizeof(zd);
  const int kc = (int)std::max(1LL, std::min<long long>({(long long)nk, 65535LL / nlay, (2LL << 30) / per_k}));
  Scoped s;
  zd *TC, *TA, *TB, *TCI, *D4, *Fd, *Fe = nullptr, *Pd = nullptr, *DEL, *T2, *M4;
  double *Cd, *Od;
  int *Cp, *Ak;
  CKR(s.alloc(&TC, nlay * MB));
  CKR(s.alloc(&TA, nlay * MB));
  CKR(s.alloc(&TB, nlay * MB));
  CKR(s.alloc(&TCI, nlay * MB));
  CKR(s.alloc(&D4, 4 * nlay * MB));  // D_A, D_B, D~_A, D~_B
  CKR(s.alloc(&Fd, 4LL * nlay * nd));
  CKR(s.alloc(&DEL, (long long)kc * nlay * MB));
  CKR(s.alloc(&T2, 2LL * kc * nlay * MB));
  CKR(s.alloc(&M4, 4LL * kc * nlay * MB));
  CKR(s.alloc(&Cd, nlay));
  CKR(s.alloc(&Od, (long long)kc * nlay * 6));
  CKR(s.alloc(&Cp, nlay));
  CKR(s.alloc(&Ak, (long long)kc * nlay));
  CKR(upload_mats(TC, tauc, nlay, nd, nd));
  CKR(upload_mats(TA, taua, nlay, nd, nd));
  CKR(upload_mats(TB, taub, nlay, nd, nd));
  CK(cudaMemcpy(Fd, F, 4LL * nlay * nd * sizeof(zd), cudaMemcpyHostToDevice));
  if (bdg) {
    CKR(s.alloc(&Fe, 4LL * nlay * NE2));
    CKR(s.alloc(&Pd, 4 * NE2));
    CK(cudaMemcpy(Fe, Feh, 4LL * nlay * NE2 * sizeof(zd), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(Pd, pair, 4 * NE2 * sizeof(zd), cudaMemcpyHostToDevice));
  }
  CK(cudaMemcpy(Cd, conc, nlay * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(Cp, cpa.data(), nlay * sizeof(int), cudaMemcpyHostToDevice));
  {
    std::vector<int> ak((size_t)kc * nlay);
    for (size_t q = 0; q < ak.size(); q++) ak[q] = cpa[q % nlay];
    CK(cudaMemcpy(Ak, ak.data(), ak.size() * sizeof(int), cudaMemcpyHostToDevice));
  }
  // per layer (items k = 0, c = layer): tau_c^-1 and the four D matrices
  auto lay = [&](zd *b) { return mref(b, 0, MB, nd); };
  launch_zaxpby(lay(TCI), lay(TC), nullptr, 0, nullptr, 0, nd, 1, nlay, Cp, 0);
  launch_zgj(lay(TCI), nd, 1, nlay, Cp, 0);
  zd *DA = D4, *DB = D4 + nlay * MB, *DAp = D4 + 2 * nlay * MB, *DBp = D4 + 3 * nlay * MB;
  launch_zgemm(0, lay(TA), lay(TCI), lay(DA), lay(DA), lay(DA), nd, nd, nd, 1, nlay, Cp, 0);
  launch_zgemm(0, lay(TB), lay(TCI), lay(DB), lay(DB), lay(DB), nd, nd, nd, 1, nlay, Cp, 0);
  launch_zgemm(0, lay(TCI), lay(TA), lay(DAp), lay(DAp), lay(DAp), nd, nd, nd, 1, nlay, Cp, 0);
  launch_zgemm(0, lay(TCI), lay(TB), lay(DBp), lay(DBp), lay(DBp), nd, nd, nd, 1, nlay, Cp, 0);
  const long long msec = (long long)kc * nlay * MB;
  for (int k0 = 0; k0 < nk; k0 += kc) {
    const int m = std::min(kc, nk - k0);
    // items (k, layer) of this chunk
    auto per = [&](zd *b) { return mref(b, nlay * MB, MB, nd); };
    CKR(upload_mats(DEL, tauk + (size_t)k0 * nlay * MB * 2, m * nlay, nd, nd));
    MatRef tc = lay(TC);
    launch_zaxpby(per(DEL), per(DEL), &tc, -1.0, nullptr, 0, nd, m, nlay, Ak, 0);
    zd *TAk = T2, *TBk = T2 + msec;
    launch_zgemm(0, lay(DA), per(DEL), per(TAk), per(TAk), per(TAk), nd, nd, nd, m, nlay, Ak, 0);
    launch_zgemm(0, lay(DB), per(DEL), per(TBk), per(TBk), per(TBk), nd, nd, nd, m, nlay, Ak, 0);
    for (int a = 0; a < 2; a++)
      for (int b = 0; b < 2; b++) {
        zd *Mab = M4 + (a * 2 + b) * msec;
        launch_zgemm(0, per(a ? TBk : TAk), lay(b ? DBp : DAp), per(Mab), per(Mab), per(Mab), nd, nd, nd, m,
                     nlay, Ak, 0);
      }
    launch_bsf_reduce(nd, nde, bdg, nlay, m * nlay, Cd, Cp, DEL, M4, msec, TA, TB, Fd, Fe, Pd, fac, Od, 0);
    CK(cudaDeviceSynchronize());
    CK(cudaGetLastError());
    CK(cudaMemcpy(out + (size_t)k0 * nlay * 6, Od, (size_t)m * nlay * 6 * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return SKKR_OK;
}

// ---------------------------------------------------------------------------
// batched complex products and inverses on host arrays (tests, benchmarks)
extern "C" int skkr_gpu_zgemm_batch(int precision, int slices, int n, int batch, const double *a,
                                    const double *b, double *cmat, int ld) {
  if (n < 1 || n > 256 || batch < 1 || batch > 65535 || !a || !b || !cmat || ld < n) return SKKR_ERR_ARG;
  Scoped s;
  zd *A, *B, *C;
  CKR(s.alloc(&A, (size_t)batch * n * n));
  CKR(s.alloc(&B, (size_t)batch * n * n));
  CKR(s.alloc(&C, (size_t)batch * n * n));
  CKR(upload_mats(A, a, batch, n, ld));
  CKR(upload_mats(B, b, batch, n, ld));
  const long long MB = (long long)n * n;
  MatRef Am = mref(A, MB, 0, n), Bm = mref(B, MB, 0, n), Cm = mref(C, MB, 0, n);
  if (precision == SKKR_MIXED) {
    MixedWork *w = mixed_create();
    if (!w) return SKKR_ERR_NOMEM;
    int rc = mixed_zgemm(w, 0, slices, Am, Bm, Cm, Cm, Cm, n, batch, 1, nullptr, 0);
    if (rc == SKKR_OK && cudaDeviceSynchronize() != cudaSuccess) rc = SKKR_ERR_CUDA;
    if (rc == SKKR_OK && mixed_error_flag(w) != 0) rc = SKKR_ERR_CUDA;
    mixed_destroy(w);
    CKR(rc);
  } else {
    launch_zgemm(0, Am, Bm, Cm, Cm, Cm, n, n, n, batch, 1, nullptr, 0);
  }
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  return download_mats(cmat, C, batch, n, ld);
}

extern "C" int skkr_gpu_zinv_batch(int precision, int n, int batch, double *a, int ld, int newton,
                                   double *max_resid) {
  if (n < 1 || n > 256 || batch < 1 || batch > 65535 || !a || ld < n) return SKKR_ERR_ARG;
  if (precision == SKKR_MIXED && n > 128) return SKKR_ERR_UNSUPPORTED;
  Scoped s;
  zd *A;
  CKR(s.alloc(&A, (size_t)batch * n * n));
  CKR(upload_mats(A, a, batch, n, ld));
  MatRef Am = mref(A, (long long)n * n, 0, n);
  if (precision == SKKR_MIXED) {
    MixedWork *w = mixed_create();
    if (!w) return SKKR_ERR_NOMEM;
    double r = 0.0;
    int rc = mixed_resid_reset(w, 0);
    if (!rc) rc = mixed_zinv(w, Am, Am, n, batch, 1, nullptr, newton, 7, true, 0);
    if (!rc) rc = mixed_resid_read(w, &r, nullptr, nullptr, 0);
    if (rc == SKKR_OK && cudaDeviceSynchronize() != cudaSuccess) rc = SKKR_ERR_CUDA;
    if (rc == SKKR_OK && mixed_error_flag(w) != 0) rc = SKKR_ERR_CUDA;
    mixed_destroy(w);
    CKR(rc);
    if (max_resid) *max_resid = r;
  } else {
    launch_zgj(Am, n, batch, 1, nullptr, 0);
  }
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  return download_mats(a, A, batch, n, ld);
}

// ---- learned CPA warm start: the MLP on the device ----------------------
namespace {
constexpr int MLP_MAX_LAYERS = 8, MLP_MAX_DIM = 4096;

struct MlpRun {
  int nl = 0, n = 0, dmax = 0;
  std::vector<int> d;
  std::vector<long long> off;  // W_i at off[i], b_i at off[i] + d[i] d[i+1]
  long long np = 0;
  Scoped s;
  double *P = nullptr, *X = nullptr, *Y = nullptr, *buf0 = nullptr, *buf1 = nullptr, *rows = nullptr;
  double *scal = nullptr;  // [0] train loss, [1] held-out loss
  std::vector<double *> A;  // A[0] = X, A[i+1] = output of layer i
  unsigned char *sel = nullptr;
};

int mlp_sizes(int nlayer, const int *dims, int n, MlpRun &m) {
  if (nlayer < 1 || nlayer > MLP_MAX_LAYERS || !dims || n < 1) return SKKR_ERR_ARG;
  m.nl = nlayer;
  m.n = n;
  m.d.assign(dims, dims + nlayer + 1);
  m.off.resize(nlayer);
  m.np = 0;
  m.dmax = 0;
  for (int i = 0; i <= nlayer; i++) {
    if (m.d[i] < 1 || m.d[i] > MLP_MAX_DIM) return SKKR_ERR_ARG;
    m.dmax = std::max(m.dmax, m.d[i]);
  }
  for (int i = 0; i < nlayer; i++) {
    m.off[i] = m.np;
    m.np += (long long)m.d[i] * m.d[i + 1] + m.d[i + 1];
  }
  long long act = 0;
  for (int i = 0; i <= nlayer; i++) act += (long long)n * m.d[i];
  if ((act + 2LL * n * m.dmax) * 8 > (16LL << 30)) return SKKR_ERR_ARG;  // activations within 16 GB
  return SKKR_OK;
}

// device buffers; x [n][d0], y [n][d_last] (may be null), rows [n] (may be null)
int mlp_alloc(MlpRun &m, const double *params, const double *x, const double *y, const unsigned char *rows) {
  const int n = m.n;
  CKR(m.s.alloc(&m.P, m.np));
  m.A.assign(m.nl + 1, nullptr);
  for (int i = 0; i <= m.nl; i++) CKR(m.s.alloc(&m.A[i], (size_t)n * m.d[i]));
  m.X = m.A[0];
  CKR(m.s.alloc(&m.buf0, (size_t)n * m.dmax));
  CKR(m.s.alloc(&m.buf1, (size_t)n * m.dmax));
  CKR(m.s.alloc(&m.rows, n));
  CKR(m.s.alloc(&m.scal, 2));
  CK(cudaMemcpy(m.P, params, m.np * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(m.X, x, (size_t)n * m.d[0] * sizeof(double), cudaMemcpyHostToDevice));
  if (y) {
    CKR(m.s.alloc(&m.Y, (size_t)n * m.d[m.nl]));
    CK(cudaMemcpy(m.Y, y, (size_t)n * m.d[m.nl] * sizeof(double), cudaMemcpyHostToDevice));
  }
  if (rows) {
    CKR(m.s.alloc(&m.sel, n));
    CK(cudaMemcpy(m.sel, rows, n, cudaMemcpyHostToDevice));
  }
  return SKKR_OK;
}

void mlp_forward(MlpRun &m, cudaStream_t st) {
  for (int i = 0; i < m.nl; i++)
    mlp_launch_dense(m.A[i], m.n, m.d[i], m.P + m.off[i], m.P + m.off[i] + (long long)m.d[i] * m.d[i + 1],
                     m.d[i + 1], i < m.nl - 1, m.A[i + 1], st);
}

// gradient of the loss whose output gradient the loss kernel left in buf0
void mlp_backward(MlpRun &m, double *G, cudaStream_t st) {
  double *cur = m.buf0, *nxt = m.buf1;
  for (int i = m.nl - 1; i >= 0; i--) {
    if (i < m.nl - 1) mlp_launch_tanh_back(m.A[i + 1], cur, (long long)m.n * m.d[i + 1], st);
    mlp_launch_wgrad(m.A[i], cur, m.n, m.d[i], m.d[i + 1], G + m.off[i], st);
    if (i > 0) {
      mlp_launch_hgrad(cur, m.P + m.off[i], m.n, m.d[i], m.d[i + 1], nxt, st);
      std::swap(cur, nxt);
    }
  }
}

int mlp_count(const unsigned char *rows, int n, int want) {
  if (!rows) return want ? n : 0;
  int c = 0;
  for (int r = 0; r < n; r++) c += rows[r] == want;
  return c;
}
}  // namespace

extern "C" int skkr_gpu_mlp_forward(int nlayer, const int *dims, const double *params, int n, const double *x,
                                    double *y) {
  if (!params || !x || !y) return SKKR_ERR_ARG;
  MlpRun m;
  CKR(mlp_sizes(nlayer, dims, n, m));
  CKR(mlp_alloc(m, params, x, nullptr, nullptr));
  mlp_forward(m, 0);
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  CK(cudaMemcpy(y, m.A[m.nl], (size_t)n * m.d[m.nl] * sizeof(double), cudaMemcpyDeviceToHost));
  return SKKR_OK;
}

extern "C" int skkr_gpu_mlp_grad(int nlayer, const int *dims, const double *params, int n, const double *x,
                                 const double *y, const unsigned char *rows, double *loss, double *grad) {
  if (!params || !x || !y || !loss || !grad) return SKKR_ERR_ARG;
  MlpRun m;
  CKR(mlp_sizes(nlayer, dims, n, m));
  const int nsel = mlp_count(rows, n, 1);
  if (nsel < 1) return SKKR_ERR_ARG;
  CKR(mlp_alloc(m, params, x, y, rows));
  double *G;
  CKR(m.s.alloc(&G, m.np));
  const int dout = m.d[m.nl];
  mlp_forward(m, 0);
  mlp_launch_loss(m.A[m.nl], m.Y, m.sel, 1, n, dout, 1.0 / ((double)nsel * dout), m.buf0, m.rows, m.scal, 0);
  mlp_backward(m, G, 0);
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  CK(cudaMemcpy(loss, m.scal, sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(grad, G, m.np * sizeof(double), cudaMemcpyDeviceToHost));
  return SKKR_OK;
}

extern "C" int skkr_gpu_mlp_train(int nlayer, const int *dims, double *params, int n, const double *x,
                                  const double *y, const unsigned char *rows, int epochs, double lr,
                                  double weight_decay, int eval_every, double *train_loss, double *best,
                                  double *best_params) {
  if (!params || !x || !y || !train_loss || epochs < 1 || !(lr > 0.0) || weight_decay < 0.0) return SKKR_ERR_ARG;
  MlpRun m;
  CKR(mlp_sizes(nlayer, dims, n, m));
  const int ntr = mlp_count(rows, n, 1), nval = mlp_count(rows, n, 0);
  if (ntr < 1) return SKKR_ERR_ARG;
  const bool eval = eval_every > 0 && nval > 0 && best && best_params;
  CKR(mlp_alloc(m, params, x, y, rows));
  double *G, *Mo, *Vo, *losses, *bestd = nullptr, *Pbest = nullptr;
  CKR(m.s.alloc(&G, m.np));
  CKR(m.s.alloc(&Mo, m.np));
  CKR(m.s.alloc(&Vo, m.np));
  CKR(m.s.alloc(&losses, epochs));
  CK(cudaMemset(Mo, 0, m.np * sizeof(double)));
  CK(cudaMemset(Vo, 0, m.np * sizeof(double)));
  if (eval) {
    CKR(m.s.alloc(&bestd, 2));
    CKR(m.s.alloc(&Pbest, m.np));
    const double init[2] = {HUGE_VAL, HUGE_VAL};
    CK(cudaMemcpy(bestd, init, sizeof(init), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(Pbest, m.P, m.np * sizeof(double), cudaMemcpyDeviceToDevice));
  }
  const int dout = m.d[m.nl];
  const double b1 = 0.9, b2 = 0.999, eps = 1e-8;  // the AdamW defaults the host training uses
  for (int ep = 0; ep < epochs; ep++) {
    mlp_forward(m, 0);
    mlp_launch_loss(m.A[m.nl], m.Y, m.sel, 1, n, dout, 1.0 / ((double)ntr * dout), m.buf0, m.rows, losses + ep, 0);
    mlp_backward(m, G, 0);
    const double t = ep + 1.0;
    const double bc1 = 1.0 - std::pow(b1, t), bc2 = 1.0 - std::pow(b2, t);
    mlp_launch_adamw(m.P, G, Mo, Vo, m.np, lr, weight_decay, b1, b2, eps, lr / bc1, std::sqrt(bc2), 0);
    if (eval && (ep % eval_every == 0 || ep == epochs - 1)) {
      mlp_forward(m, 0);
      mlp_launch_loss(m.A[m.nl], m.Y, m.sel, 0, n, dout, 1.0 / ((double)nval * dout), nullptr, m.rows,
                      m.scal + 1, 0);
      mlp_launch_keep_best(m.scal + 1, losses + ep, bestd, m.P, Pbest, m.np, 0);
    }
  }
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  CK(cudaMemcpy(train_loss, losses, epochs * sizeof(double), cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(params, m.P, m.np * sizeof(double), cudaMemcpyDeviceToHost));
  if (eval) {
    CK(cudaMemcpy(best, bestd, 2 * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(best_params, Pbest, m.np * sizeof(double), cudaMemcpyDeviceToHost));
  } else {
    if (best) {
      best[0] = NAN;
      best[1] = train_loss[epochs - 1];
    }
    if (best_params) std::memcpy(best_params, params, m.np * sizeof(double));
  }
  return SKKR_OK;
}

// ---- the reference's k-space structure constants: Kambe lattice sums ----
extern "C" int skkr_gpu_kambe_dlm(int nitem, double e_re, double e_im, const double *kxy, const double *sep,
                                  int lmax2, const double *gvec, int ng, const double *rvec, int nr, double area,
                                  double factor, double gcut, double rcut, double *out) {
  if (nitem < 1 || !kxy || !sep || !gvec || !rvec || !out || ng < 1 || nr < 1) return SKKR_ERR_ARG;
  if (lmax2 < 0 || lmax2 > 6 || !(area > 0.0) || !(factor > 0.0) || !(gcut > 0.0) || !(rcut > 0.0))
    return SKKR_ERR_ARG;
  if (e_re == 0.0 && e_im == 0.0) return SKKR_ERR_ARG;
  const int lmmx = (lmax2 + 1) * (lmax2 + 1);
  Scoped s;
  double *K, *S, *G, *R, *O;
  CKR(s.alloc(&K, 2 * (size_t)nitem));
  CKR(s.alloc(&S, 3 * (size_t)nitem));
  CKR(s.alloc(&G, 2 * (size_t)ng));
  CKR(s.alloc(&R, 2 * (size_t)nr));
  CKR(s.alloc(&O, 2 * (size_t)nitem * lmmx));
  CK(cudaMemcpy(K, kxy, 2 * (size_t)nitem * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(S, sep, 3 * (size_t)nitem * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(G, gvec, 2 * (size_t)ng * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(R, rvec, 2 * (size_t)nr * sizeof(double), cudaMemcpyHostToDevice));
  launch_kambe_dlm(nitem, e_re, e_im, K, S, lmax2, G, ng, R, nr, area, factor, gcut, rcut, O, 0);
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  CK(cudaMemcpy(out, O, 2 * (size_t)nitem * lmmx * sizeof(double), cudaMemcpyDeviceToHost));
  return SKKR_OK;
}

// coefficient tensor of the block contraction kambe_alm (host only, no
// device call): coef[L][L'][q] = 4 pi <Y_L Y*_L' Y_q'> i^(l'-l-l_q')
// (-1)^(l_q'+m_q') at q = (l_q', -m_q'), the Gaunt integrals of the complex
// harmonics by Gauss-Legendre x uniform-phi quadrature (exact at these
// degrees), entries below 1e-13 set to zero
extern "C" int skkr_gpu_kambe_coef(int lmax, double *out) {
  if (lmax < 0 || lmax > 3 || !out) return SKKR_ERR_ARG;
  const int lm = (lmax + 1) * (lmax + 1), l2 = 2 * lmax, lm2 = (l2 + 1) * (l2 + 1);
  const int nq = (4 * lmax + l2) / 2 + 2, nph = 4 * lmax + l2 + 2;
  // Gauss-Legendre nodes and weights by Newton's method on P_nq
  std::vector<double> xg(nq), wg(nq);
  for (int i = 0; i < nq; i++) {
    double x = std::cos(M_PI * (i + 0.75) / (nq + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = x;
      for (int n = 2; n <= nq; n++) {
        const double p2 = ((2.0 * n - 1.0) * x * p1 - (n - 1.0) * p0) / n;
        p0 = p1;
        p1 = p2;
      }
      dp = nq * (x * p1 - p0) / (x * x - 1.0);
      const double dx = p1 / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    xg[i] = x;
    wg[i] = 2.0 / ((1.0 - x * x) * dp * dp);
  }
  std::vector<fcplx> C((size_t)lm * lm * lm2, fc(0.0, 0.0)), y(lm2);
  for (int i = 0; i < nq; i++) {
    const double ct = xg[i], st = std::sqrt(std::max(0.0, 1.0 - ct * ct));
    for (int p = 0; p < nph; p++) {
      const double phi = 2.0 * M_PI * p / nph, w = wg[i] * 2.0 * M_PI / nph;
      kambe_ylm(st * std::cos(phi), st * std::sin(phi), ct, l2, y.data());
      for (int a = 0; a < lm; a++)
        for (int b = 0; b < lm; b++) {
          const fcplx ab = fmulc(y[a], fconj(y[b]));
          for (int q = 0; q < lm2; q++) {
            fcplx &c = C[((size_t)a * lm + b) * lm2 + q];
            c = fadd(c, fscal(w, fmulc(ab, y[q])));
          }
        }
    }
  }
  auto lof = [](int i) { int l = 0; while ((l + 1) * (l + 1) <= i) l++; return l; };
  for (int a = 0; a < lm; a++)
    for (int b = 0; b < lm; b++)
      for (int q = 0; q < lm2; q++) {
        fcplx c = C[((size_t)a * lm + b) * lm2 + q];
        if (std::fabs(c.re) < 1e-13) c.re = 0.0;
        if (std::fabs(c.im) < 1e-13) c.im = 0.0;
        const int la = lof(a), lb = lof(b), lq = lof(q), mq = q - lq * (lq + 1);
        const fcplx t = fscal(4.0 * M_PI * (((lq + mq) % 2 + 2) % 2 ? -1.0 : 1.0), fmulc(c, fipow(lb - la - lq)));
        const int qn = lq * (lq + 1) - mq;
        double *o = out + 2 * (((size_t)a * lm + b) * lm2 + qn);
        o[0] = t.re;
        o[1] = t.im;
      }
  return SKKR_OK;
}

extern "C" int skkr_gpu_kambe_alm(int nitem, double e_re, double e_im, const double *kxy, const double *sep,
                                  int lmax, const double *gvec, int ng, const double *rvec, int nr, double area,
                                  double factor, double gcut, double rcut, double *out) {
  if (nitem < 1 || !kxy || !sep || !gvec || !rvec || !out || ng < 1 || nr < 1) return SKKR_ERR_ARG;
  if (lmax < 0 || lmax > 3 || !(area > 0.0) || !(factor > 0.0) || !(gcut > 0.0) || !(rcut > 0.0))
    return SKKR_ERR_ARG;
  if (e_re == 0.0 && e_im == 0.0) return SKKR_ERR_ARG;
  const int lm = (lmax + 1) * (lmax + 1), lm2 = (2 * lmax + 1) * (2 * lmax + 1);
  std::vector<double> coef(2 * (size_t)lm * lm * lm2);
  CKR(skkr_gpu_kambe_coef(lmax, coef.data()));
  Scoped s;
  double *K, *S, *G, *R, *Cf, *O;
  CKR(s.alloc(&K, 2 * (size_t)nitem));
  CKR(s.alloc(&S, 3 * (size_t)nitem));
  CKR(s.alloc(&G, 2 * (size_t)ng));
  CKR(s.alloc(&R, 2 * (size_t)nr));
  CKR(s.alloc(&Cf, coef.size()));
  CKR(s.alloc(&O, 2 * (size_t)nitem * lm * lm));
  CK(cudaMemcpy(K, kxy, 2 * (size_t)nitem * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(S, sep, 3 * (size_t)nitem * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(G, gvec, 2 * (size_t)ng * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(R, rvec, 2 * (size_t)nr * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(Cf, coef.data(), coef.size() * sizeof(double), cudaMemcpyHostToDevice));
  launch_kambe_alm(nitem, e_re, e_im, K, S, lmax, G, ng, R, nr, area, factor, gcut, rcut, Cf, nullptr, 1, O, 0);
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  CK(cudaMemcpy(out, O, 2 * (size_t)nitem * lm * lm * sizeof(double), cudaMemcpyDeviceToHost));
  return SKKR_OK;
}


// The reference's screened G_scr(k) on the device (gstore.f + scrstr.f): the
// layer-pair blocks of a slab of nl layers at pos [nl][3] for each k point,
// G' = G (1 - alpha G)^-1 per k (Gauss-Jordan and GEMM batched over k), and
// the blocks (centre, centre + j), j = -jmax..jmax, into
// out [nk][2 jmax + 1][lmmax][lmmax] complex (row L).  alpha [nl][lmax+1]
// complex per layer and l; the lattice arguments as for skkr_gpu_kambe_alm.
extern "C" int skkr_gpu_kambe_screened(int nk, double e_re, double e_im, const double *kxy, int nl,
                                       const double *pos, const double *alpha, int lmax, const double *gvec,
                                       int ng, const double *rvec, int nr, double area, double factor,
                                       double gcut, double rcut, int centre, int jmax, double *out) {
  if (nk < 1 || !kxy || !out) return SKKR_ERR_ARG;
  struct Own {
    KambeDev k;
    DBuf kx, o;
    ~Own() {
      k.release();
      kx.release();
      o.release();
    }
  } w;
  KambeDev &K = w.k;
  CKR(K.setup(e_re, e_im, lmax, nl, pos, alpha, centre, jmax, gvec, ng, rvec, nr, area, factor, gcut, rcut, 0));
  const int nj = 2 * jmax + 1;
  const size_t blocks = (size_t)nj * K.lm * K.lm;
  const int m = std::min(std::min((int)std::max<size_t>(1, (size_t)4e9 / K.per_k()), 65535), nk);
  CKR(w.kx.ensure(2 * (size_t)nk * sizeof(double)));
  CKR(w.o.ensure((size_t)nk * blocks * sizeof(zd)));
  CK(cudaMemcpy(w.kx.p, kxy, 2 * (size_t)nk * sizeof(double), cudaMemcpyHostToDevice));
  for (int k0 = 0; k0 < nk; k0 += m) {
    const int mm = std::min(m, nk - k0);
    CKR(K.screen(w.kx.as<double>() + 2 * (size_t)k0, mm, 0));
    launch_slab_extract(mm, nl, K.lm, centre, jmax, K.X.as<zd>(), w.o.as<zd>() + (size_t)k0 * blocks, 0);
  }
  CK(cudaDeviceSynchronize());
  CK(cudaGetLastError());
  CK(cudaMemcpy(out, w.o.p, (size_t)nk * blocks * sizeof(zd), cudaMemcpyDeviceToHost));
  return SKKR_OK;
}
