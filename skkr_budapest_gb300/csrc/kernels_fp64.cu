// FP64 batched kernels of the 2D-BZ tau path.
//
// Every kernel works on batches of small complex matrices addressed through
// MatRef (item (k, c) -> base + k*sk + map[c]*sc, column-major).  The FP64
// pipe of sm_103a (about 1.1 TFLOP/s per GPU) bounds all of them, so the
// designs favour plain data reuse in shared memory over register blocking.
#include "kernels.h"

// ---------------------------------------------------------------------------
// G_scr(k) by lattice Fourier transform of the real-space screened table.
// One CTA per (k, block); thread t owns matrix element t of the lm x lm block.
// Bytes: reads the table (L2 resident, shared by all k), writes lmmax^2*16 B.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_gk_ft(const zd *__restrict__ gR,
                                               const double *__restrict__ rvec,
                                               const int *__restrict__ rstart, int nblk, int lmmax,
                                               const double *__restrict__ xk, zd *__restrict__ out) {
  const int kk = blockIdx.y, b = blockIdx.x;
  const int r0 = rstart[b], r1 = rstart[b + 1];
  __shared__ zd ph[64];
  const double kx = xk[2 * kk], ky = xk[2 * kk + 1];
  for (int r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    double s, c;
    sincos(kx * rvec[2 * r] + ky * rvec[2 * r + 1], &s, &c);
    ph[r - r0] = make_double2(c, s);
  }
  __syncthreads();
  const int bs = lmmax * lmmax;
  for (int e = threadIdx.x; e < bs; e += blockDim.x) {
    zd acc = make_double2(0.0, 0.0);
    for (int r = r0; r < r1; r++) {
      zd g = gR[(long long)r * bs + e];
      acc = zadd(acc, zmul(ph[r - r0], g));
    }
    out[((long long)kk * nblk + b) * bs + e] = acc;
  }
}

void launch_gk_ft(const zd *gR, const double *rvec, const int *rstart, int nblk, int lmmax,
                  const double *xk, int nk, zd *out, cudaStream_t st) {
  if (nk <= 0) return;
  dim3 grid(nblk, nk);
  kstat_begin(KS_GKFT, (double)nk * nblk * lmmax * lmmax * sizeof(zd), st);
  k_gk_ft<<<grid, 256, 0, st>>>(gR, rvec, rstart, nblk, lmmax, xk, out);
  kstat_end(st);
  SKKR_LAUNCHED();
}

// ---------------------------------------------------------------------------
// packer.f + relmtrx.f: -G blocks of one principal layer, expanded to
// (kappa,mu) with the Clebsch-Gordan maps of clebsch.f when irel=1.
// ---------------------------------------------------------------------------
__constant__ double c_u1[72], c_u2[72];
__constant__ int c_ind1[72], c_ind2[72];

cudaError_t pack_set_tables(int irel, int lmax) {
  (void)lmax;
  double u1[72] = {0}, u2[72] = {0};
  int i1[72] = {0}, i2[72] = {0};
  if (irel) {
    int inr = 0;
    for (int l = 0; l <= 5; l++) {
      double tl = 2.0 * l + 1.0;
      for (int m = -l; m <= l; m++) {
        inr++;
        int kap = l, ir;
        if (kap != 0) {
          ir = 2 * kap * kap + kap + m;
          u1[ir - 1] = sqrt((l + m) / tl);
          i1[ir - 1] = inr;
          ir++;
          u2[ir - 1] = -sqrt((l - m) / tl);
          i2[ir - 1] = inr;
        }
        kap = -l - 1;
        ir = 2 * kap * kap + kap + m;
        u1[ir - 1] = sqrt((l - m + 1) / tl);
        i1[ir - 1] = inr;
        ir++;
        u2[ir - 1] = sqrt((l + m + 1) / tl);
        i2[ir - 1] = inr;
      }
    }
    for (int k = 0; k < 72; k++) {
      if (!i1[k]) i1[k] = 1;
      if (!i2[k]) i2[k] = 1;
      i1[k]--;
      i2[k]--;
      // a zero coefficient marks a spinor component outside the basis
      // (|m| > l, e.g. l = lmax + 1 for the last kappa); its index would
      // point past the lm block, so the term reads element 0 instead (it is
      // multiplied by zero either way, as in the zero-padded reference copy)
      if (u1[k] == 0.0) i1[k] = 0;
      if (u2[k] == 0.0) i2[k] = 0;
    }
  }
  cudaError_t e = cudaMemcpyToSymbol(c_u1, u1, sizeof(u1));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_u2, u2, sizeof(u2));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_ind1, i1, sizeof(i1));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_ind2, i2, sizeof(i2));
  return e;
}

// Row of component k (0..lk-1) of site i in a principal-layer matrix of nl
// sites: site-major i lk + k, or with ehsplit (BdG on the split-precision
// path) electron-first -- every site's electron half, then every site's hole
// half -- so that the two K halves of a product carry their own operand
// scales.  The two layouts are a permutation similarity of each other.
__device__ __forceinline__ int pl_row(int i, int k, int lk, int nl, int ehsplit) {
  if (!ehsplit) return i * lk + k;
  const int km = lk >> 1;
  return k < km ? i * km + k : nl * km + i * km + (k - km);
}
__device__ __forceinline__ void pl_site(int r, int lk, int nl, int ehsplit, int &i, int &k) {
  if (!ehsplit) {
    i = r / lk;
    k = r % lk;
    return;
  }
  const int km = lk >> 1, half = nl * km;
  const int h = r >= half, rr = h ? r - half : r;
  i = rr / km;
  k = rr % km + (h ? km : 0);
}

// mode 0: lm, 1: (kappa,mu), 2: BdG -- blockdiag of the electron block b
// (fac) and the hole block b + nblk (fach), each mapped to (kappa,mu)
// (skkr_dbogo_bsf main/g2d_pack.f + main/relmtrx.f).  nbk: blocks per k.
__global__ void __launch_bounds__(256) k_pack(const zd *__restrict__ G, int nblk, int nbk,
                                              const int *__restrict__ blkmap, int mi, int jmax,
                                              const PackJob *__restrict__ jobs, int lk, int lmmax,
                                              int mode, zd fac, zd fach, zd *__restrict__ pool,
                                              int nmat, int npl, int ehsplit) {
  const int kk = blockIdx.y;
  const PackJob jb = jobs[blockIdx.z];
  const int nrow = jb.ni * lk;
  const int ncol = (jb.which == 0 ? jb.ni : jb.which == 1 ? jb.nim : jb.nip) * lk;
  const int nj = 2 * jmax + 1;
  zd *out = pool + ((long long)kk * nmat + jb.dest) * (long long)npl * npl;
  const zd *Gk = G + (long long)kk * nbk * lmmax * lmmax;
  const int total = npl * npl;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int r = e % npl, c = e / npl;
    zd v = make_double2(0.0, 0.0);
    if (r < nrow && c < ncol) {
      int i, k1, jp, k2;
      pl_site(r, lk, jb.ni, ehsplit, i, k1);
      pl_site(c, lk, ncol / lk, ehsplit, jp, k2);
      i++;
      jp++;
      int j;
      bool inrange;
      if (jb.which == 0) {
        j = jp - i;
        inrange = true;
      } else if (jb.which == 1) {
        j = jp - jb.nim - i;
        int jmin = (jb.ni <= jb.nim) ? -jb.nim : -min(jb.ni, jb.nim + i - 1);
        inrange = (j >= jmin && j <= -i);
      } else {
        j = jp + jb.ni - i;
        int jmx = (jb.ni <= jb.nip) ? jb.nip : min(jb.ni, jb.nip + jb.ni - i);
        inrange = (j >= jb.ni - i + 1 && j <= jmx);
      }
      if (inrange && j >= -jmax && j <= jmax && i <= mi) {
        const int b = blkmap[(jb.slot * mi + (i - 1)) * nj + (j + jmax)];
        if (b >= 0) {
          const zd *g = Gk + (long long)b * lmmax * lmmax;
          zd val;
          if (mode == 2) {
            const int km = lk >> 1;
            if ((k1 < km) == (k2 < km)) {
              const bool h = k1 >= km;
              const zd *gg = h ? g + (long long)nblk * lmmax * lmmax : g;
              const int q1 = h ? k1 - km : k1, q2 = h ? k2 - km : k2;
              const zd f = h ? fach : fac;
              zd a1 = zmul(f, gg[c_ind1[q1] + c_ind1[q2] * lmmax]);
              zd a2 = zmul(f, gg[c_ind2[q1] + c_ind2[q2] * lmmax]);
              val = zadd(zscale(c_u1[q2], zscale(c_u1[q1], a1)), zscale(c_u2[q2], zscale(c_u2[q1], a2)));
            } else {
              val = make_double2(0.0, 0.0);
            }
          } else if (mode == 1) {
            // relmtrx.f: b = u1 (fac a) u1 + u2 (fac a) u2
            zd a1 = zmul(fac, g[c_ind1[k1] + c_ind1[k2] * lmmax]);
            zd a2 = zmul(fac, g[c_ind2[k1] + c_ind2[k2] * lmmax]);
            val = zadd(zscale(c_u1[k2], zscale(c_u1[k1], a1)), zscale(c_u2[k2], zscale(c_u2[k1], a2)));
          } else {
            val = g[k1 + k2 * lmmax];
          }
          v = make_double2(-val.x, -val.y);
        }
      }
    }
    out[e] = v;
  }
}

void launch_pack(const zd *G, int nblk, int nbk, const int *d_blkmap, int mi, int jmax,
                 const PackJob *d_jobs, int njobs, int lk, int lmmax, int mode, zd fac, zd fach, int nk,
                 zd *pool, int nmat, int npl, int ehsplit, cudaStream_t st) {
  if (nk <= 0 || njobs <= 0) return;
  int per = (npl * npl + 255) / 256;
  dim3 grid(per < 64 ? per : 64, nk, njobs);
  k_pack<<<grid, 256, 0, st>>>(G, nblk, nbk, d_blkmap, mi, jmax, d_jobs, lk, lmmax, mode, fac, fach,
                               pool, nmat, npl, ehsplit);
  SKKR_LAUNCHED();
}

// ---------------------------------------------------------------------------
// Batched complex GEMM, 32x32 output tile per CTA, 16x16 threads each owning
// a 2x2 sub-tile, K in steps of 16 through shared memory.  Each output is
// accumulated sequentially over k (the reference's loop order).
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(256) k_zgemm(MatRef A, MatRef B, MatRef C, MatRef D, MatRef E, int M,
                                               int N, int K, int nc, const int *__restrict__ act) {
  const int item = blockIdx.y;
  const int kk = item / nc, cc = item % nc;
  if (act && !act[item]) return;
  const int tilesN = (N + 31) / 32;
  const int tm = blockIdx.x / tilesN, tn = blockIdx.x % tilesN;
  const zd *a = mat_ptr(A, kk, cc);
  const zd *b = mat_ptr(B, kk, cc);
  __shared__ zd As[16][33];
  __shared__ zd Bs[16][33];
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  const int row0 = tm * 32, col0 = tn * 32;
  zd acc[2][2];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 2; j++) acc[i][j] = make_double2(0.0, 0.0);
  for (int k0 = 0; k0 < K; k0 += 16) {
#pragma unroll
    for (int q = 0; q < 2; q++) {
      int e = tid + 256 * q;
      int r = e % 32, kq = e / 32;
      int gr = row0 + r, gk = k0 + kq;
      As[kq][r] = (gr < M && gk < K) ? a[gr + (long long)gk * A.ld] : make_double2(0.0, 0.0);
      int kb = e % 16, cb = e / 16;
      int gk2 = k0 + kb, gc = col0 + cb;
      Bs[kb][cb] = (gk2 < K && gc < N) ? b[gk2 + (long long)gc * B.ld] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    const int kmax = min(16, K - k0);
    for (int q = 0; q < kmax; q++) {
      zd a0 = As[q][tx], a1 = As[q][tx + 16];
      zd b0 = Bs[q][ty], b1 = Bs[q][ty + 16];
      zfma(acc[0][0], a0, b0);
      zfma(acc[1][0], a1, b0);
      zfma(acc[0][1], a0, b1);
      zfma(acc[1][1], a1, b1);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 2; j++) {
      int r = row0 + tx + 16 * i, c = col0 + ty + 16 * j;
      if (r >= M || c >= N) continue;
      zd y = acc[i][j];
      if (MODE == 0) {
        mat_ptr(C, kk, cc)[r + (long long)c * C.ld] = y;
      } else if (MODE == 1) {
        zd *p = mat_ptr(C, kk, cc) + r + (long long)c * C.ld;
        *p = zsub(*p, y);
      } else if (MODE == 2) {
        zd *p = mat_ptr(D, kk, cc) + r + (long long)c * D.ld;
        *p = zsub(*p, y);
        zd *q2 = mat_ptr(E, kk, cc) + r + (long long)c * E.ld;
        *q2 = zsub(*q2, y);
      } else {
        zd d = mat_ptr(D, kk, cc)[r + (long long)c * D.ld];
        mat_ptr(C, kk, cc)[r + (long long)c * C.ld] = zsub(d, y);
      }
    }
}

void launch_zgemm(int mode, const MatRef &A, const MatRef &B, const MatRef &C, const MatRef &D,
                  const MatRef &E, int m, int n, int kdim, int nk, int nc, const int *act,
                  cudaStream_t st) {
  if (nk <= 0 || nc <= 0 || m <= 0 || n <= 0) return;
  dim3 grid(((m + 31) / 32) * ((n + 31) / 32), nk * nc);
  const long long items = act ? skkr_active_items((long long)nk * nc) : (long long)nk * nc;
  kstat_begin(KS_GEMM, 8.0 * m * n * kdim * (double)items, st);
  switch (mode) {
    case 0: k_zgemm<0><<<grid, 256, 0, st>>>(A, B, C, D, E, m, n, kdim, nc, act); break;
    case 1: k_zgemm<1><<<grid, 256, 0, st>>>(A, B, C, D, E, m, n, kdim, nc, act); break;
    case 2: k_zgemm<2><<<grid, 256, 0, st>>>(A, B, C, D, E, m, n, kdim, nc, act); break;
    default: k_zgemm<3><<<grid, 256, 0, st>>>(A, B, C, D, E, m, n, kdim, nc, act); break;
  }
  kstat_end(st);
  SKKR_LAUNCHED();
}

// ---------------------------------------------------------------------------
// Gauss-Jordan inversion with column pivoting (main/gjinv.f:2-59), in place
// in global memory (L1/L2 resident), one CTA per matrix, n <= 256.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(512) k_zgj(MatRef A, int n, int nc, const int *__restrict__ act) {
  const int item = blockIdx.x;
  const int kk = item / nc, cc = item % nc;
  if (act && !act[item]) return;
  zd *a = mat_ptr(A, kk, cc);
  const int ld = A.ld;
  __shared__ int ind[512];    // n <= 512
  __shared__ zd coli[512];
  __shared__ zd rowi[512];
  __shared__ double rv[32];
  __shared__ int ri[32];
  const int tid = threadIdx.x, nth = blockDim.x;
  const int lane = tid & 31, wid = tid >> 5, nw = nth >> 5;
  for (int i = 0; i < n; i++) {
    // pivot: largest |a(i,j)|, j >= i, first index on ties
    double best = -1.0;
    int bj = n;
    for (int j = i + tid; j < n; j += nth) {
      zd v = a[i + (long long)j * ld];
      double m = hypot(v.x, v.y);
      if (m > best || (m == best && j < bj)) { best = m; bj = j; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      double ob = __shfl_down_sync(0xffffffffu, best, o);
      int oj = __shfl_down_sync(0xffffffffu, bj, o);
      if (ob > best || (ob == best && oj < bj)) { best = ob; bj = oj; }
    }
    if (lane == 0) { rv[wid] = best; ri[wid] = bj; }
    __syncthreads();
    if (wid == 0) {
      best = lane < nw ? rv[lane] : -2.0;
      bj = lane < nw ? ri[lane] : n;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        double ob = __shfl_down_sync(0xffffffffu, best, o);
        int oj = __shfl_down_sync(0xffffffffu, bj, o);
        if (ob > best || (ob == best && oj < bj)) { best = ob; bj = oj; }
      }
      if (lane == 0) { ri[0] = bj < n ? bj : i; ind[i] = bj < n ? bj : i; }
    }
    __syncthreads();
    int kp = ri[0];
    if (kp >= n) kp = i;  // all candidates NaN: keep the index in range
    if (kp != i) {
      for (int r = tid; r < n; r += nth) {
        zd t = a[r + (long long)i * ld];
        a[r + (long long)i * ld] = a[r + (long long)kp * ld];
        a[r + (long long)kp * ld] = t;
      }
      __syncthreads();
    }
    const zd q = zrecip(a[i + (long long)i * ld]);
    for (int j = tid; j < n; j += nth) rowi[j] = a[i + (long long)j * ld];
    for (int r = tid; r < n; r += nth) coli[r] = (r == i) ? q : zmul(a[r + (long long)i * ld], q);
    __syncthreads();
    for (int r = tid; r < n; r += nth) a[r + (long long)i * ld] = coli[r];
    const int tot = n * n;
    for (int e = tid; e < tot; e += nth) {
      const int r = e % n, j = e / n;
      if (j == i) continue;
      zd *p = a + r + (long long)j * ld;
      zd v = (r == i) ? make_double2(0.0, 0.0) : *p;
      zfms(v, coli[r], rowi[j]);
      *p = v;
    }
    __syncthreads();
  }
  for (int i = n - 1; i >= 0; i--) {
    const int j = ind[i];
    if (j == i) continue;
    for (int c = tid; c < n; c += nth) {
      zd t = a[i + (long long)c * ld];
      a[i + (long long)c * ld] = a[j + (long long)c * ld];
      a[j + (long long)c * ld] = t;
    }
    __syncthreads();
  }
}

void launch_zgj(const MatRef &A, int n, int nk, int nc, const int *act, cudaStream_t st) {
  if (nk <= 0 || nc <= 0 || n <= 0) return;
  int th = n * n >= 4096 ? 512 : 256;
  const long long items = act ? skkr_active_items((long long)nk * nc) : (long long)nk * nc;
  kstat_begin(KS_GJ, 8.0 * n * n * (double)n * (double)items, st);
  k_zgj<<<nk * nc, th, 0, st>>>(A, n, nc, act);
  kstat_end(st);
  SKKR_LAUNCHED();
}

// ---------------------------------------------------------------------------
// elementwise helpers
// ---------------------------------------------------------------------------
__global__ void k_zaxpby(MatRef O, MatRef Aa, MatRef Bb, double s1, MatRef Dd, double s2, int hasb,
                         int hasd, int n, int nc, const int *__restrict__ act) {
  const int item = blockIdx.y;
  const int kk = item / nc, cc = item % nc;
  if (act && !act[item]) return;
  zd *o = mat_ptr(O, kk, cc);
  const zd *a = mat_ptr(Aa, kk, cc);
  const zd *b = hasb ? mat_ptr(Bb, kk, cc) : nullptr;
  const zd *d = hasd ? mat_ptr(Dd, kk, cc) : nullptr;
  const int tot = n * n;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
    const int r = e % n, c = e / n;
    zd v = a[r + (long long)c * Aa.ld];
    if (hasb) v = zadd(v, zscale(s1, b[r + (long long)c * Bb.ld]));
    if (hasd) v = zadd(v, zscale(s2, d[r + (long long)c * Dd.ld]));
    o[r + (long long)c * O.ld] = v;
  }
}

void launch_zaxpby(const MatRef &out, const MatRef &a, const MatRef *b, double s1, const MatRef *d,
                   double s2, int n, int nk, int nc, const int *act, cudaStream_t st) {
  if (nk <= 0 || nc <= 0) return;
  int per = (n * n + 255) / 256;
  dim3 grid(per < 32 ? per : 32, nk * nc);
  const long long items = act ? skkr_active_items((long long)nk * nc) : (long long)nk * nc;
  kstat_begin(KS_OTHER, (double)items * n * n * 16.0 * (2 + (b != nullptr) + (d != nullptr)), st);
  k_zaxpby<<<grid, 256, 0, st>>>(out, a, b ? *b : a, s1, d ? *d : a, s2, b != nullptr, d != nullptr,
                                 n, nc, act);
  kstat_end(st);
  SKKR_LAUNCHED();
}

__global__ void k_add_tblocks(MatRef O, MatRef In, MatRef T, int lk, int nl, int n, int nc,
                              const int *__restrict__ act, int ehsplit) {
  const int item = blockIdx.y;
  const int kk = item / nc, cc = item % nc;
  if (act && !act[item]) return;
  zd *o = mat_ptr(O, kk, cc);
  const zd *in = mat_ptr(In, kk, cc);
  const zd *t = mat_ptr(T, kk, cc);
  const int tot = n * n;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
    const int r = e % n, c = e / n;
    zd v = in[r + (long long)c * In.ld];
    int lr, kr, lc, kc;
    pl_site(r, lk, nl, ehsplit, lr, kr);
    pl_site(c, lk, nl, ehsplit, lc, kc);
    if (lr == lc && lr < nl) {
      // tau2d.f:72-78 / dugo.f:82-89: m00 = tminv + m00
      zd tv = t[(long long)lr * lk * lk + kr + kc * lk];
      v = zadd(tv, v);
    }
    o[r + (long long)c * O.ld] = v;
  }
}

void launch_add_tblocks(const MatRef &out, const MatRef &in, const MatRef &t, int lk, int nl,
                        int n, int nk, int nc, const int *act, int ehsplit, cudaStream_t st) {
  if (nk <= 0 || nc <= 0) return;
  int per = (n * n + 255) / 256;
  dim3 grid(per < 32 ? per : 32, nk * nc);
  k_add_tblocks<<<grid, 256, 0, st>>>(out, in, t, lk, nl, n, nc, act, ehsplit);
  SKKR_LAUNCHED();
}

__global__ void k_fnorm(MatRef A, int n, int nc, const int *__restrict__ act, double *out) {
  const int item = blockIdx.x;
  const int kk = item / nc, cc = item % nc;
  if (act && !act[item]) return;
  const zd *a = mat_ptr(A, kk, cc);
  double s = 0.0;
  const int tot = n * n;
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    zd v = a[(e % n) + (long long)(e / n) * A.ld];
    s += v.x * v.x + v.y * v.y;
  }
  __shared__ double red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[item] = sqrt(s);
  }
}

void launch_fnorm(const MatRef &a, int n, int nk, int nc, const int *act, double *out,
                  cudaStream_t st) {
  if (nk <= 0 || nc <= 0) return;
  k_fnorm<<<nk * nc, 256, 0, st>>>(a, n, nc, act, out);
  SKKR_LAUNCHED();
}

// surfgf.f:81-104: stop when err < errmax or iter > itermax; error > 1e10
// is "enormous"; leaving with iter > itermax is the itermax failure.
__global__ void k_dec_state(const double *err, int *act, int *stat, int *iters, int nitems, int iter,
                            int itermax, double errmax) {
  int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= nitems || !act[it]) return;
  double e = err[it];
  if (e < errmax || iter > itermax) {
    act[it] = 0;
    iters[it] = iter;
    stat[it] = (iter > itermax) ? -3 : 0;
  } else if (e > 1.0e10) {
    act[it] = 0;
    iters[it] = iter;
    stat[it] = -4;
  } else if (!(e == e)) {
    act[it] = 0;
    iters[it] = iter;
    stat[it] = -7;
  }
}

void launch_dec_state(const double *err, int *act, int *stat, int *iters, int nitems, int iter,
                      int itermax, double errmax, cudaStream_t st) {
  if (nitems <= 0) return;
  k_dec_state<<<(nitems + 255) / 256, 256, 0, st>>>(err, act, stat, iters, nitems, iter, itermax,
                                                     errmax);
  SKKR_LAUNCHED();
}

// The same update with the iteration number read from the device (*iter_p,
// the iteration just completed), counting the items left iterating in
// *nactive: the form a captured graph replays
__global__ void k_dec_state_dev(const double *err, int *act, int *stat, int *iters, int nitems,
                                const int *iter_p, int itermax, double errmax, int *nactive) {
  const int it = blockIdx.x * blockDim.x + threadIdx.x;
  const int iter = *iter_p;
  int keep = 0;
  if (it < nitems && act[it]) {
    const double e = err[it];
    keep = 1;
    if (e < errmax || iter > itermax) {
      act[it] = 0;
      iters[it] = iter;
      stat[it] = (iter > itermax) ? -3 : 0;
      keep = 0;
    } else if (e > 1.0e10) {
      act[it] = 0;
      iters[it] = iter;
      stat[it] = -4;
      keep = 0;
    } else if (!(e == e)) {
      act[it] = 0;
      iters[it] = iter;
      stat[it] = -7;
      keep = 0;
    }
  }
  keep = __syncthreads_count(keep);
  if (threadIdx.x == 0 && keep) atomicAdd(nactive, keep);
}

void launch_dec_state_dev(const double *err, int *act, int *stat, int *iters, int nitems, const int *iter_p,
                          int itermax, double errmax, int *nactive, cudaStream_t st) {
  if (nitems <= 0) return;
  k_dec_state_dev<<<(nitems + 255) / 256, 256, 0, st>>>(err, act, stat, iters, nitems, iter_p, itermax, errmax,
                                                         nactive);
  SKKR_LAUNCHED();
}

// After one decimation iteration of a captured loop: advance the iteration
// number, clear the active count, count the iteration (*runs) and set the
// loop condition (items left, within itermax, no tensor-core wait expired).  Every item retires by
// iteration itermax + 1, so the loop ends.
__global__ void k_dec_advance(int *iter_p, int *nactive, int itermax, const int *errflag,
                              cudaGraphConditionalHandle cond, int *runs) {
  const int it = *iter_p, na = *nactive;
  *iter_p = it + 1;
  *nactive = 0;
  *runs += 1;
  const bool go = na > 0 && it <= itermax && (errflag == nullptr || *errflag == 0);
  cudaGraphSetConditional(cond, go ? 1u : 0u);
}

void launch_dec_advance(int *iter_p, int *nactive, int itermax, const int *errflag, cudaGraphConditionalHandle cond,
                        int *runs, cudaStream_t st) {
  k_dec_advance<<<1, 1, 0, st>>>(iter_p, nactive, itermax, errflag, cond, runs);
  SKKR_LAUNCHED();
}

// tau2d.f:137-147: tau(l,lp,ilay) = wgeff * tau00(il0+l, il0+lp)
__global__ void k_extract_tau(MatRef W, int lk, int nl, int layer0, const double *wk, double wscale,
                              zd *out, long long out_sk, long long out_sc, int nc, int ehsplit) {
  const int item = blockIdx.y;
  const int kk = item / nc, cc = item % nc;
  const zd *w = mat_ptr(W, kk, cc);
  const double wg = wk[kk] * wscale;
  const int tot = nl * lk * lk;
  zd *o = out + (long long)kk * out_sk + (long long)cc * out_sc + (long long)layer0 * lk * lk;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
    const int l = e / (lk * lk), rem = e % (lk * lk);
    const int r = rem % lk, c = rem / lk;
    zd v = w[pl_row(l, r, lk, nl, ehsplit) + (long long)pl_row(l, c, lk, nl, ehsplit) * W.ld];
    o[e] = zscale(wg, v);
  }
}

void launch_extract_tau(const MatRef &W, int lk, int nl, int layer0, const double *wk,
                        double wscale, zd *out, long long out_sk, long long out_sc, int nk,
                        int nc, int ehsplit, cudaStream_t st) {
  if (nk <= 0 || nc <= 0) return;
  int per = (nl * lk * lk + 255) / 256;
  dim3 grid(per < 16 ? per : 16, nk * nc);
  k_extract_tau<<<grid, 256, 0, st>>>(W, lk, nl, layer0, wk, wscale, out, out_sk, out_sc, nc, ehsplit);
  SKKR_LAUNCHED();
}

// One principal-layer block (rows: PL of `rowlay0`, columns: PL of
// `collay0`) of the full Godfrin tau into its layer-pair blocks
// (skkr_dbogo_bsf/clu/tau2d_god.f:152-205): out[item][rowlay0 + a][collay0 + b]
// = wk wscale W(layer a rows, layer b columns), nl layers per PL, nintfc
// interface layers.
__global__ void k_extract_pairs(MatRef W, int lk, int nl, int rowlay0, int collay0, int nintfc,
                                const double *wk, double wscale, zd *out, long long out_sk,
                                long long out_sc, int nc, int ehsplit) {
  const int item = blockIdx.y;
  const int kk = item / nc, cc = item % nc;
  const zd *w = mat_ptr(W, kk, cc);
  const double wg = wk[kk] * wscale;
  const int lk2 = lk * lk, tot = nl * nl * lk2;
  zd *o = out + (long long)kk * out_sk + (long long)cc * out_sc;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
    const int ab = e / lk2, rem = e % lk2;
    const int a = ab / nl, b = ab % nl;
    const int r = rem % lk, c = rem / lk;
    const zd v = w[pl_row(a, r, lk, nl, ehsplit) + (long long)pl_row(b, c, lk, nl, ehsplit) * W.ld];
    o[((long long)(rowlay0 + a) * nintfc + (collay0 + b)) * lk2 + rem] = zscale(wg, v);
  }
}

void launch_extract_pairs(const MatRef &W, int lk, int nl, int rowlay0, int collay0, int nintfc,
                          const double *wk, double wscale, zd *out, long long out_sk, long long out_sc,
                          int nk, int nc, int ehsplit, cudaStream_t st) {
  if (nk <= 0 || nc <= 0) return;
  int per = (nl * nl * lk * lk + 255) / 256;
  dim3 grid(per < 16 ? per : 16, nk * nc);
  k_extract_pairs<<<grid, 256, 0, st>>>(W, lk, nl, rowlay0, collay0, nintfc, wk, wscale, out, out_sk, out_sc,
                                        nc, ehsplit);
  SKKR_LAUNCHED();
}

// Phased k sums of the pair blocks (skkr_dbogo_bsf/rsp-scf/cpacoord_ksave.f:
// 818-840) for the k points of one chunk, before the group rotation:
//   acc_ij[q][g] += sum_k e^{+i k.g v_q} tau^(class g)_{li,lj}(k)
//   acc_ji[q][g] += sum_k e^{-i k.g v_q} tau^(class g)_{lj,li}(k)
// v_q = R_q + c_li - c_lj, g(v) = a0mat[g] v (row-major 2x2).  One thread
// per matrix element of one (pair, g); the k loop runs in order.
__global__ void k_pair_sum(const zd *__restrict__ tauf, int nkc, int nc, int nintfc, int lk2,
                           const int *__restrict__ cls_of_g, int ngeff, const int *__restrict__ pairs,
                           const double *__restrict__ vecs, const double *__restrict__ a0mat,
                           const double *__restrict__ xk, zd *acc_ij, zd *acc_ji) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int q = blockIdx.y, g = blockIdx.z;
  if (e >= lk2) return;
  const int li = pairs[4 * q + 2], lj = pairs[4 * q + 3];
  const double vx = vecs[2 * q], vy = vecs[2 * q + 1];
  const double *am = a0mat + 4 * g;
  const double gx = am[0] * vx + am[1] * vy, gy = am[2] * vx + am[3] * vy;
  const int cl = cls_of_g[g];
  const long long blk = (long long)nintfc * nintfc * lk2;
  const zd *tij = tauf + (long long)cl * blk + ((long long)li * nintfc + lj) * lk2 + e;
  const zd *tji = tauf + (long long)cl * blk + ((long long)lj * nintfc + li) * lk2 + e;
  const long long sk = (long long)nc * blk;
  double sr = 0, si = 0, tr = 0, ti = 0;
  for (int k = 0; k < nkc; k++) {
    double sn, cs;
    sincos(xk[2 * k] * gx + xk[2 * k + 1] * gy, &sn, &cs);
    const zd a = tij[k * sk], b = tji[k * sk];
    sr += cs * a.x - sn * a.y;
    si += cs * a.y + sn * a.x;
    tr += cs * b.x + sn * b.y;
    ti += cs * b.y - sn * b.x;
  }
  zd *oij = acc_ij + ((long long)q * ngeff + g) * lk2 + e;
  zd *oji = acc_ji + ((long long)q * ngeff + g) * lk2 + e;
  *oij = make_double2(oij->x + sr, oij->y + si);
  *oji = make_double2(oji->x + tr, oji->y + ti);
}

void launch_pair_sum(const zd *tauf, int nkc, int nc, int nintfc, int lk, const int *cls_of_g, int ngeff,
                     int npair, const int *pairs, const double *vecs, const double *a0mat, const double *xk,
                     zd *acc_ij, zd *acc_ji, cudaStream_t st) {
  if (nkc <= 0 || npair <= 0) return;
  const int lk2 = lk * lk;
  dim3 grid((lk2 + 127) / 128, npair, ngeff);
  k_pair_sum<<<grid, 128, 0, st>>>(tauf, nkc, nc, nintfc, lk2, cls_of_g, ngeff, pairs, vecs, a0mat, xk, acc_ij,
                                   acc_ji);
  SKKR_LAUNCHED();
}

// k-sum: block (32 elements) x (32 k-slices); coalesced loads over elements,
// then a shared-memory transpose and a warp-shuffle reduction over slices.
// The summation tree is fixed, so the result is bitwise reproducible.
__global__ void __launch_bounds__(1024) k_ksum(const zd *__restrict__ tk, int nk, long long E,
                                               zd *__restrict__ S, int accumulate) {
  __shared__ zd sm[32][33];
  const long long e = (long long)blockIdx.x * 32 + threadIdx.x;
  zd acc = make_double2(0.0, 0.0);
  if (e < E)
    for (int k = threadIdx.y; k < nk; k += 32) acc = zadd(acc, tk[(long long)k * E + e]);
  sm[threadIdx.y][threadIdx.x] = acc;
  __syncthreads();
  zd v = sm[threadIdx.x][threadIdx.y];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, o);
    v.y += __shfl_down_sync(0xffffffffu, v.y, o);
  }
  const long long eo = (long long)blockIdx.x * 32 + threadIdx.y;
  if (threadIdx.x == 0 && eo < E) S[eo] = accumulate ? zadd(S[eo], v) : v;
}

void launch_ksum(const zd *tk, int nk, long long E, zd *S, int accumulate, cudaStream_t st) {
  if (E <= 0) return;
  dim3 blk(32, 32);
  k_ksum<<<(unsigned)((E + 31) / 32), blk, 0, st>>>(tk, nk, E, S, accumulate);
  SKKR_LAUNCHED();
}

// per-k Frobenius norm of the k-resolved contributions tk[k][E]
__global__ void k_knorm(const zd *__restrict__ tk, long long E, double *__restrict__ out) {
  const zd *t = tk + (long long)blockIdx.x * E;
  double s = 0.0;
  for (long long e = threadIdx.x; e < E; e += blockDim.x) s += t[e].x * t[e].x + t[e].y * t[e].y;
  __shared__ double red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[blockIdx.x] = sqrt(s);
  }
}

void launch_knorm(const zd *tk, int nk, long long E, double *out, cudaStream_t st) {
  if (nk <= 0 || E <= 0) return;
  k_knorm<<<nk, 256, 0, st>>>(tk, E, out);
  SKKR_LAUNCHED();
}

// S[e] += sign * x[e]
__global__ void k_axpy_flat(zd *__restrict__ S, const zd *__restrict__ x, long long E, double sign) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < E; e += (long long)gridDim.x * blockDim.x)
    S[e] = make_double2(S[e].x + sign * x[e].x, S[e].y + sign * x[e].y);
}

void launch_axpy_flat(zd *S, const zd *x, long long E, double sign, cudaStream_t st) {
  if (E <= 0) return;
  const long long nb = (E + 255) / 256;
  k_axpy_flat<<<(unsigned)(nb < 1024 ? nb : 1024), 256, 0, st>>>(S, x, E, sign);
  SKKR_LAUNCHED();
}

__global__ void k_gsum(const zd *T, int ng, int lk, int nl, zd *out) {
  const int tot = nl * lk * lk;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
    const int l = e / (lk * lk), rem = e % (lk * lk);
    zd acc = make_double2(0.0, 0.0);
    for (int g = 0; g < ng; g++) acc = zadd(acc, T[((long long)l * ng + g) * lk * lk + rem]);
    out[e] = acc;
  }
}

void launch_gsum(const zd *T, int ng, int lk, int nl, zd *out, cudaStream_t st) {
  int tot = nl * lk * lk;
  k_gsum<<<(tot + 255) / 256, 256, 0, st>>>(T, ng, lk, nl, out);
  SKKR_LAUNCHED();
}

// fullcpa.f:109-117: xc = c xa + (1-c) xb (per alloy layer); X is [layer][2][lk^2]
__global__ void k_cpa_mix(const zd *X, const double *conc, const int *act, int lk, zd *xc) {
  const int l = blockIdx.y;
  if (!act[l]) return;
  const double ca = conc[l], cb = 1.0 - ca;
  const int tot = lk * lk;
  const zd *xa = X + (long long)l * 2 * tot, *xb = xa + tot;
  for (int e = threadIdx.x; e < tot; e += blockDim.x)
    xc[(long long)l * tot + e] = zadd(zscale(ca, xa[e]), zscale(cb, xb[e]));
}

void launch_cpa_mix(const zd *X, const double *conc, const int *act, int lk, int nl, zd *xc,
                    cudaStream_t st) {
  dim3 grid(1, nl);
  k_cpa_mix<<<grid, 256, 0, st>>>(X, conc, act, lk, xc);
  SKKR_LAUNCHED();
}

// ---------------------------------------------------------------------------
// Layer DOS (lambda = 0 moment of nrsp-scf/moment.f:47-110, rsp-scf/moment.f:
// 60-140): zmom_i = fac (F_i tau_ii - G_i) per basis index, and per orbital l
// the sum over its indices in increasing order (locquant.f:115-122).  One CTA
// per layer; basis index i has l = floor(sqrt(i)) in the lm basis and
// floor(sqrt(i/2)) in the (kappa,mu) basis (l blocks start at 2 l^2).
__global__ void k_layer_dos(int rel, int nd, int nl, const zd *__restrict__ tau, int ld,
                            const zd *__restrict__ F, const zd *__restrict__ G, double fac,
                            zd *__restrict__ zmom, zd *__restrict__ zdos_l) {
  const int li = blockIdx.x;
  __shared__ zd z[128];
  const zd *t = tau + (long long)li * ld * ld;
  for (int i = threadIdx.x; i < nd; i += blockDim.x) {
    const long long q = (long long)li * nd + i;
    const zd v = zscale(fac, zsub(zmul(F[q], t[i + (long long)i * ld]), G[q]));
    z[i] = v;
    zmom[q] = v;
  }
  __syncthreads();
  for (int l = threadIdx.x; l < nl; l += blockDim.x) {
    const int i0 = rel ? 2 * l * l : l * l, i1 = rel ? 2 * (l + 1) * (l + 1) : (l + 1) * (l + 1);
    zd acc = make_double2(0.0, 0.0);
    for (int i = i0; i < i1 && i < nd; i++) acc = zadd(acc, z[i]);
    zdos_l[(long long)li * nl + l] = acc;
  }
}

void launch_layer_dos(int rel, int nd, int nl, int nlay, const zd *tau, int ld, const zd *F,
                      const zd *G, double fac, zd *zmom, zd *zdos_l, cudaStream_t st) {
  k_layer_dos<<<nlay, 128, 0, st>>>(rel, nd, nl, tau, ld, F, G, fac, zmom, zdos_l);
  SKKR_LAUNCHED();
}

// ---------------------------------------------------------------------------
// Bloch spectral function (skkr_dbogo_bsf/rsp-scf/bsf.f:251-418 after its
// products): one CTA per (k, layer) item.  With diagonal radial solutions
// gf.f's ggrmat(j, i) is R_ab(j, i) X(j, i); the moments at lambda = 0 read its
// diagonal (electron and hole halves) and its electron-hole block through the
// four pairing operators.  CPA layers: sum_ab c_a c_b R_ab M_ab (M_ab =
// D_a (tau(k) - tau_c) D~_b, section a*2+b of M) plus sum_a c_a R_aa tau_a;
// other layers: R_AA (tau(k)).  Six sums in a fixed order per item:
// bsfe, bsfh, then Im tr(P_x G_eh) for x = singlet, T0, T-up, T-down.
__global__ void __launch_bounds__(256) k_bsf_reduce(int nd, int nde, int bdg, int nlay, const double *conc,
                                                    const int *__restrict__ cpa, const zd *__restrict__ del,
                                                    const zd *__restrict__ M, long long msec,
                                                    const zd *__restrict__ ta, const zd *__restrict__ tb,
                                                    const zd *__restrict__ F, const zd *__restrict__ Feh,
                                                    const zd *__restrict__ P, double fac, double *out) {
  const int item = blockIdx.x, l = item % nlay;
  const long long MB = (long long)nd * nd, NE2 = (long long)nde * nde;
  const bool cp = cpa[l] != 0;
  const double cab[2] = {conc[l], 1.0 - conc[l]};
  const zd *Fl = F + (long long)l * 4 * nd;
  const zd *Fe = bdg ? Feh + (long long)l * 4 * NE2 : nullptr;
  double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  // element e of the matrices of this item, each term weighted by its radial
  // overlap R[a*2+b] (stride rs between the four species pairs)
  auto g_at = [&](long long e, const zd *R, long long rs) -> zd {
    zd g = make_double2(0.0, 0.0);
    if (cp) {
      for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++) {
          const zd m = M[(a * 2 + b) * msec + (long long)item * MB + e];
          zfma(g, zscale(cab[a] * cab[b], R[(a * 2 + b) * rs]), m);
        }
      for (int a = 0; a < 2; a++) {
        const zd t = (a ? tb : ta)[(long long)l * MB + e];
        zfma(g, zscale(cab[a], R[(a * 2 + a) * rs]), t);
      }
    } else {
      zfma(g, R[0], del[(long long)item * MB + e]);
    }
    return g;
  };
  for (int i = threadIdx.x; i < nd; i += blockDim.x) {
    const zd g = g_at(i + (long long)i * nd, Fl + i, nd);
    acc[(bdg && i >= nde) ? 1 : 0] += g.y;
  }
  if (bdg)
    for (long long idx = threadIdx.x; idx < NE2; idx += blockDim.x) {
      const int j = (int)(idx % nde), i = (int)(idx / nde);
      // G_eh(j, i) is element (j, nde + i); P_x(i, j) multiplies it in tr(P_x G_eh)
      const zd g = g_at(j + (long long)(nde + i) * nd, Fe + j + (long long)i * nde, NE2);
      for (int x = 0; x < 4; x++) acc[2 + x] += zmul(P[x * NE2 + i + (long long)j * nde], g).y;
    }
  __shared__ double red[6][256];
  for (int q = 0; q < 6; q++) red[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int q = 0; q < 6; q++) red[q][threadIdx.x] += red[q][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < 6) out[(long long)item * 6 + threadIdx.x] = fac * red[threadIdx.x][0];
}

void launch_bsf_reduce(int nd, int nde, int bdg, int nlay, int nitems, const double *conc, const int *cpa,
                       const zd *del, const zd *M, long long msec, const zd *ta, const zd *tb, const zd *F,
                       const zd *Feh, const zd *P, double fac, double *out, cudaStream_t st) {
  if (nitems <= 0) return;
  k_bsf_reduce<<<nitems, 256, 0, st>>>(nd, nde, bdg, nlay, conc, cpa, del, M, msec, ta, tb, F, Feh, P, fac, out);
  SKKR_LAUNCHED();
}
