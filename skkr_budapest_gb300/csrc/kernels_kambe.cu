// The reference's k-space structure constants on the device, first form:
// the Kambe lattice sums D_L(k, s) of kambe_dev.cuh, one thread per
// (k point, layer-pair separation) item running the whole sum.
#include "common.cuh"
#include "kernels.h"
#include "kambe_dev.cuh"

#include <algorithm>

namespace {

__global__ void k_kambe_dlm(int nitem, double er, double ei, const double *__restrict__ kxy,
                            const double *__restrict__ sep, int lmax2, const double *__restrict__ gvec, int ng,
                            const double *__restrict__ rvec, int nr, double area, double factor, double gcut,
                            double rcut, double *__restrict__ out) {
  const int lmmx = (lmax2 + 1) * (lmax2 + 1);
  for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < nitem; it += gridDim.x * blockDim.x) {
    fcplx d[(SKKR_KAMBE_L2 + 1) * (SKKR_KAMBE_L2 + 1)];
    kambe_dlm(fc(er, ei), kxy[2 * it], kxy[2 * it + 1], sep[3 * it], sep[3 * it + 1], sep[3 * it + 2], lmax2,
              gvec, ng, rvec, nr, area, factor, gcut, rcut, d);
    double *o = out + (long long)it * 2 * lmmx;
    for (int i = 0; i < lmmx; i++) {
      o[2 * i] = d[i].re;
      o[2 * i + 1] = d[i].im;
    }
  }
}

// the layer-pair blocks alm(k, s) = sum_q coef[L][L'][q] D_q(k, s) of each item
__global__ void k_kambe_alm(int nitem, double er, double ei, const double *__restrict__ kxy,
                            const double *__restrict__ sep, int lmax, const double *__restrict__ gvec, int ng,
                            const double *__restrict__ rvec, int nr, double area, double factor, double gcut,
                            double rcut, const double *__restrict__ coef, double *__restrict__ out) {
  const int lm = (lmax + 1) * (lmax + 1);
  for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < nitem; it += gridDim.x * blockDim.x) {
    fcplx d[(SKKR_KAMBE_L2 + 1) * (SKKR_KAMBE_L2 + 1)];
    kambe_dlm(fc(er, ei), kxy[2 * it], kxy[2 * it + 1], sep[3 * it], sep[3 * it + 1], sep[3 * it + 2], 2 * lmax,
              gvec, ng, rvec, nr, area, factor, gcut, rcut, d);
    kambe_alm(d, lmax, coef, reinterpret_cast<fcplx *>(out + (long long)it * 2 * lm * lm));
  }
}

// the slab of nl layers per k point and its 1 - alpha G (kambe_slab_elem)
__global__ void k_slab_assemble(int nk, int nl, int lm, const zd *__restrict__ alm, const double *__restrict__ kxy,
                                const double *__restrict__ pos, const zd *__restrict__ alpha, int nal,
                                zd *__restrict__ G, zd *__restrict__ A) {
  const long long tot = (long long)nk * nl * lm * nl * lm;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
       e += (long long)gridDim.x * blockDim.x)
    kambe_slab_elem(e, nl, lm, (const double *)alm, kxy, pos, (const double *)alpha, nal, (double *)G,
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

}  // namespace

void launch_slab_assemble(int nk, int nl, int lm, const zd *alm, const double *kxy, const double *pos,
                          const zd *alpha, int nal, zd *G, zd *A, cudaStream_t st) {
  const long long tot = (long long)nk * nl * lm * nl * lm;
  const int blocks = (int)std::min<long long>((tot + 255) / 256, 152 * 16);
  k_slab_assemble<<<blocks, 256, 0, st>>>(nk, nl, lm, alm, kxy, pos, alpha, nal, G, A);
  SKKR_LAUNCHED();
}

void launch_slab_extract(int nk, int nl, int lm, int centre, int jmax, const zd *X, zd *out, cudaStream_t st) {
  const long long tot = (long long)nk * (2 * jmax + 1) * lm * lm;
  const int blocks = (int)std::min<long long>((tot + 255) / 256, 152 * 16);
  k_slab_extract<<<blocks, 256, 0, st>>>(nk, nl, lm, centre, jmax, X, out);
  SKKR_LAUNCHED();
}

void launch_kambe_alm(int nitem, double er, double ei, const double *kxy, const double *sep, int lmax,
                      const double *gvec, int ng, const double *rvec, int nr, double area, double factor,
                      double gcut, double rcut, const double *coef, double *out, cudaStream_t st) {
  const int threads = 64;
  const int blocks = (nitem + threads - 1) / threads;
  k_kambe_alm<<<blocks, threads, 0, st>>>(nitem, er, ei, kxy, sep, lmax, gvec, ng, rvec, nr, area, factor, gcut,
                                          rcut, coef, out);
  SKKR_LAUNCHED();
}

void launch_kambe_dlm(int nitem, double er, double ei, const double *kxy, const double *sep, int lmax2,
                      const double *gvec, int ng, const double *rvec, int nr, double area, double factor,
                      double gcut, double rcut, double *out, cudaStream_t st) {
  const int threads = 64;
  const int blocks = (nitem + threads - 1) / threads;
  k_kambe_dlm<<<blocks, threads, 0, st>>>(nitem, er, ei, kxy, sep, lmax2, gvec, ng, rvec, nr, area, factor, gcut,
                                          rcut, out);
  SKKR_LAUNCHED();
}
