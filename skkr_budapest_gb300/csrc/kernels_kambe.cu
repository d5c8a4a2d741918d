// The reference's k-space structure constants on the device: the Kambe
// lattice sums D_L(k, s) of kambe_dev.cuh, one thread block per (k point,
// layer-pair separation) item.  The block's threads split the reciprocal
// (g) and real-space (R) terms, each accumulating all (l, m) of its terms,
// and the block sums them in a fixed order (warp shuffles, then the warps
// in index order): the transcendental per-term work (incomplete gamma and
// ilkam recursions, the Faddeeva function, harmonics) spreads over the SM
// instead of running serially in one thread.
#include "common.cuh"
#include "kernels.h"
#include "kambe_dev.cuh"

#include <algorithm>

namespace {

constexpr int KB_THREADS = 128;

// the sums of item blockIdx.x into d[lmmx] (shared): thread t takes the terms
// g = t, t + T, ... and R = t, t + T, ...; thread 0 the formula-55 self term
__device__ void kambe_block_sums(double er, double ei, const double *__restrict__ kxy,
                                 const double *__restrict__ sep, int lmax2, const double *__restrict__ gvec, int ng,
                                 const double *__restrict__ rvec, int nr, double area, double factor, double gcut,
                                 double rcut, fcplx *d) {
  __shared__ double part[KB_THREADS / 32][(SKKR_KAMBE_L2 + 1) * (SKKR_KAMBE_L2 + 1)][2];
  const int it = blockIdx.x, t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int lmmx = (lmax2 + 1) * (lmax2 + 1);
  KambeSetup K;
  kambe_setup(fc(er, ei), kxy[2 * it], kxy[2 * it + 1], sep[3 * it], sep[3 * it + 1], sep[3 * it + 2], lmax2, area,
              factor, K);
  fcplx acc[(SKKR_KAMBE_L2 + 1) * (SKKR_KAMBE_L2 + 1)];
  for (int i = 0; i < lmmx; i++) acc[i] = fc(0.0, 0.0);
  if (t == 0) kambe_self_term(K, acc);
  for (int ig = t; ig < ng; ig += blockDim.x) kambe_gterm(K, gvec[2 * ig], gvec[2 * ig + 1], gcut, acc);
  for (int ir = t; ir < nr; ir += blockDim.x) kambe_rterm(K, rvec[2 * ir], rvec[2 * ir + 1], rcut, acc);
  for (int i = 0; i < lmmx; i++) {
    double re = acc[i].re, im = acc[i].im;
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_down_sync(0xffffffffu, re, o);
      im += __shfl_down_sync(0xffffffffu, im, o);
    }
    if (lane == 0) {
      part[warp][i][0] = re;
      part[warp][i][1] = im;
    }
  }
  __syncthreads();
  for (int i = t; i < lmmx; i += blockDim.x) {
    double re = 0.0, im = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
      re += part[w][i][0];
      im += part[w][i][1];
    }
    d[i] = fc(re, im);
  }
  __syncthreads();
}

__global__ void __launch_bounds__(KB_THREADS) k_kambe_dlm_cta(double er, double ei, const double *__restrict__ kxy,
                                                              const double *__restrict__ sep, int lmax2,
                                                              const double *__restrict__ gvec, int ng,
                                                              const double *__restrict__ rvec, int nr, double area,
                                                              double factor, double gcut, double rcut,
                                                              double *__restrict__ out) {
  __shared__ fcplx d[(SKKR_KAMBE_L2 + 1) * (SKKR_KAMBE_L2 + 1)];
  kambe_block_sums(er, ei, kxy, sep, lmax2, gvec, ng, rvec, nr, area, factor, gcut, rcut, d);
  const int lmmx = (lmax2 + 1) * (lmax2 + 1);
  double *o = out + (long long)blockIdx.x * 2 * lmmx;
  for (int i = threadIdx.x; i < lmmx; i += blockDim.x) {
    o[2 * i] = d[i].re;
    o[2 * i + 1] = d[i].im;
  }
}

// the layer-pair blocks alm(k, s)[L][L'] = sum_q coef[L][L'][q] D_q(k, s):
// the block's sums, then one thread per (L, L') (kambe_alm's order over q)
__global__ void __launch_bounds__(KB_THREADS) k_kambe_alm_cta(double er, double ei, const double *__restrict__ kxy,
                                                              const double *__restrict__ sep, int lmax,
                                                              const double *__restrict__ gvec, int ng,
                                                              const double *__restrict__ rvec, int nr, double area,
                                                              double factor, double gcut, double rcut,
                                                              const double *__restrict__ coef,
                                                              const int *__restrict__ far, int nsep,
                                                              double *__restrict__ out) {
  // pairs far apart take the plane-wave form (k_directg_cta)
  if (far && far[blockIdx.x % nsep]) return;
  __shared__ fcplx d[(SKKR_KAMBE_L2 + 1) * (SKKR_KAMBE_L2 + 1)];
  kambe_block_sums(er, ei, kxy, sep, 2 * lmax, gvec, ng, rvec, nr, area, factor, gcut, rcut, d);
  const int lm = (lmax + 1) * (lmax + 1), lm2 = (2 * lmax + 1) * (2 * lmax + 1);
  fcplx *o = reinterpret_cast<fcplx *>(out + (long long)blockIdx.x * 2 * lm * lm);
  for (int e = threadIdx.x; e < lm * lm; e += blockDim.x) {
    fcplx s = fc(0.0, 0.0);
    const double *c = coef + 2 * ((long long)e * lm2);
    for (int q = 0; q < lm2; q++) s = fadd(s, fmulc(fc(c[2 * q], c[2 * q + 1]), d[q]));
    o[e] = s;
  }
}

// the plane-wave form of the blocks of items whose separation is far (far[item
// % nsep] != 0; directg.f): one block per item, one thread per (L, L').  Tiles
// of DG_TILE g vectors: the first threads form the terms (factor and the two
// harmonic vectors) in shared memory, then every thread adds the tile's
// terms to its element in g order.
constexpr int DG_TILE = 64;
__global__ void __launch_bounds__(256) k_directg_cta(double er, double ei, const double *__restrict__ kxy,
                                                    const double *__restrict__ sep, int lmax,
                                                    const double *__restrict__ gvec, int ng, double area,
                                                    const int *__restrict__ far, int nsep,
                                                    double *__restrict__ out) {
  const int it = blockIdx.x, t = threadIdx.x;
  if (!far[it % nsep]) return;
  __shared__ fcplx fs[DG_TILE], yl[DG_TILE][SKKR_DG_LM], yr[DG_TILE][SKKR_DG_LM];
  const int lm = (lmax + 1) * (lmax + 1), L = t / lm, Lp = t % lm;
  const fcplx e = fc(er, ei), kappa = fsqrtc(e);
  const double f1 = 8.0 * 3.14159265358979323846 * 3.14159265358979323846 / area;
  const double kx = kxy[2 * it], ky = kxy[2 * it + 1];
  const double sx = sep[3 * it], sy = sep[3 * it + 1], sz = sep[3 * it + 2];
  fcplx acc = fc(0.0, 0.0);
  for (int g0 = 0; g0 < ng; g0 += DG_TILE) {
    const int nt = min(DG_TILE, ng - g0);
    for (int q = t; q < nt; q += blockDim.x)
      directg_gterm(e, kappa, kx, ky, sx, sy, sz, lmax, gvec[2 * (g0 + q)], gvec[2 * (g0 + q) + 1], f1, &fs[q],
                    yl[q], yr[q]);
    __syncthreads();
    if (t < lm * lm)
      for (int q = 0; q < nt; q++) acc = fadd(acc, fmulc(fmulc(fs[q], yl[q][L]), yr[q][Lp]));
    __syncthreads();
  }
  if (t < lm * lm) {
    double *o = out + 2 * ((long long)it * lm * lm + t);
    o[0] = acc.re;
    o[1] = acc.im;
  }
}

// the slab of nl layers per k point and its 1 - alpha G (kambe_slab_elem)
__global__ void k_slab_assemble(int nk, int nl, int lm, const zd *__restrict__ alm, const int *__restrict__ pmap,
                                int nsep, const double *__restrict__ kxy, const double *__restrict__ pos,
                                const zd *__restrict__ alpha, int nal, zd *__restrict__ G, zd *__restrict__ A) {
  const long long tot = (long long)nk * nl * lm * nl * lm;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
       e += (long long)gridDim.x * blockDim.x)
    kambe_slab_elem(e, nl, lm, (const double *)alm, pmap, nsep, kxy, pos, (const double *)alpha, nal, (double *)G,
                    (double *)A);
}

// the central layer offsets (kambe_slab_extract_elem)
__global__ void k_slab_extract(int nk, int nl, int lm, int centre, int jmax, const zd *__restrict__ X,
                               zd *__restrict__ out) {
  const long long tot = (long long)nk * (2 * jmax + 1) * lm * lm;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
       e += (long long)gridDim.x * blockDim.x)
    kambe_slab_extract_elem(e, nl, lm, centre, jmax, (const double *)X, (double *)out);
}

// the central layer offsets into the structure-constant cache (kambe_slab_cache_elem)
__global__ void k_slab_cache(int nk, int nl, int lm, int centre, int jmax, const int *__restrict__ blk, int nbk,
                             const zd *__restrict__ X, zd *__restrict__ Gc) {
  const long long tot = (long long)nk * (2 * jmax + 1) * lm * lm;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
       e += (long long)gridDim.x * blockDim.x)
    kambe_slab_cache_elem(e, nl, lm, centre, jmax, blk, nbk, (const double *)X, (double *)Gc);
}

// the (k point, separation) items of the lattice sums: k of item it is
// xk[it / nsep], the separation seps[it % nsep]
__global__ void k_kambe_items(int nk, int nsep, const double *__restrict__ xk, const double *__restrict__ seps,
                              double *__restrict__ ik, double *__restrict__ is) {
  const long long tot = (long long)nk * nsep;
  for (long long it = blockIdx.x * (long long)blockDim.x + threadIdx.x; it < tot;
       it += (long long)gridDim.x * blockDim.x) {
    const long long k = it / nsep, q = it - k * nsep;
    ik[2 * it] = xk[2 * k];
    ik[2 * it + 1] = xk[2 * k + 1];
    for (int c = 0; c < 3; c++) is[3 * it + c] = seps[3 * q + c];
  }
}

}  // namespace

void launch_slab_assemble(int nk, int nl, int lm, const zd *alm, const int *pmap, int nsep, const double *kxy,
                          const double *pos, const zd *alpha, int nal, zd *G, zd *A, cudaStream_t st) {
  const long long tot = (long long)nk * nl * lm * nl * lm;
  const int blocks = (int)std::min<long long>((tot + 255) / 256, 152 * 16);
  k_slab_assemble<<<blocks, 256, 0, st>>>(nk, nl, lm, alm, pmap, nsep, kxy, pos, alpha, nal, G, A);
  SKKR_LAUNCHED();
}

void launch_slab_extract(int nk, int nl, int lm, int centre, int jmax, const zd *X, zd *out, cudaStream_t st) {
  const long long tot = (long long)nk * (2 * jmax + 1) * lm * lm;
  const int blocks = (int)std::min<long long>((tot + 255) / 256, 152 * 16);
  k_slab_extract<<<blocks, 256, 0, st>>>(nk, nl, lm, centre, jmax, X, out);
  SKKR_LAUNCHED();
}

void launch_slab_cache(int nk, int nl, int lm, int centre, int jmax, const int *blk, int nbk, const zd *X, zd *Gc,
                       cudaStream_t st) {
  const long long tot = (long long)nk * (2 * jmax + 1) * lm * lm;
  const int blocks = (int)std::min<long long>((tot + 255) / 256, 152 * 16);
  k_slab_cache<<<blocks, 256, 0, st>>>(nk, nl, lm, centre, jmax, blk, nbk, X, Gc);
  SKKR_LAUNCHED();
}

void launch_kambe_items(int nk, int nsep, const double *xk, const double *seps, double *ik, double *is,
                        cudaStream_t st) {
  const long long tot = (long long)nk * nsep;
  const int blocks = (int)std::min<long long>((tot + 255) / 256, 152 * 16);
  k_kambe_items<<<blocks, 256, 0, st>>>(nk, nsep, xk, seps, ik, is);
  SKKR_LAUNCHED();
}

// one block per item (grid.x holds up to 2^31 - 1 items)
void launch_kambe_alm(int nitem, double er, double ei, const double *kxy, const double *sep, int lmax,
                      const double *gvec, int ng, const double *rvec, int nr, double area, double factor,
                      double gcut, double rcut, const double *coef, const int *far, int nsep, double *out,
                      cudaStream_t st) {
  if (nitem <= 0) return;
  k_kambe_alm_cta<<<nitem, KB_THREADS, 0, st>>>(er, ei, kxy, sep, lmax, gvec, ng, rvec, nr, area, factor, gcut, rcut,
                                                coef, far, nsep, out);
  SKKR_LAUNCHED();
}

// one block per item; items whose separation is not far return at once
void launch_directg(int nitem, double er, double ei, const double *kxy, const double *sep, int lmax,
                    const double *gvec, int ng, double area, const int *far, int nsep, double *out,
                    cudaStream_t st) {
  if (nitem <= 0) return;
  k_directg_cta<<<nitem, 256, 0, st>>>(er, ei, kxy, sep, lmax, gvec, ng, area, far, nsep, out);
  SKKR_LAUNCHED();
}

void launch_kambe_dlm(int nitem, double er, double ei, const double *kxy, const double *sep, int lmax2,
                      const double *gvec, int ng, const double *rvec, int nr, double area, double factor,
                      double gcut, double rcut, double *out, cudaStream_t st) {
  if (nitem <= 0) return;
  k_kambe_dlm_cta<<<nitem, KB_THREADS, 0, st>>>(er, ei, kxy, sep, lmax2, gvec, ng, rvec, nr, area, factor, gcut,
                                                rcut, out);
  SKKR_LAUNCHED();
}

