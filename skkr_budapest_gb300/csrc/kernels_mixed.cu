// Split-precision kernels: FP64-accurate complex products on the 5th-generation
// tensor cores (tcgen05.mma, BF16 operands, FP32 accumulation in TMEM) and a
// refined inverse.
//
// Products (Ozaki-style splitting).  Every row i of A gets a power-of-two
// scale sigma_i >= max_j |A_ij| (re and im together), every column j of B a
// scale tau_j.  The scaled entries in [-1, 1] are cut into S exact slices of
// 8 significant bits by repeated rounding:
//     x/sigma = sum_p s_p 2^(-7-8(p-1)),   s_p integers, |s_p| <= 128,
// which BF16 stores exactly.  Slice p of A is stored as s_p 2^(-8(p-1)) and
// slice q of B as s_q 2^(-8(q-3)); then every slice product A_p B_q carries
// its true relative weight, and all products of one "level" p+q land in the
// same accumulator with a common factor 2^-30 sigma_i tau_j.  Each level has
// its own TMEM accumulator: the tensor core aligns addends to the largest
// exponent and truncates, so sums of one level stay exact (integer multiples
// of the level's unit, at most (c+1) K 2^14 units, within FP32's 24 bits for
// K <= 256) whereas mixing levels would drop the low bits of the smaller one.
// Products with p+q > S+1 are dropped; S = 5 keeps 15 products in 5 levels
// (5 x 96 TMEM columns) and gives about 2^-39 relative to sigma_i tau_j.
//
// Complex to real: [Cr Ci] = [Ar Ai] [[Br Bi], [-Bi Br]], i.e. a real GEMM of
// M = n, N = 2n, K = 2n; the epilogue writes column jj < n into Re C(:,jj) and
// column n+j into Im C(:,j).
//
// Staging layouts (bf16, K contiguous = K-major for both UMMA operands):
//   A'[item][s][M'][K']   M' = 128 * mtiles, K' = 64 * kblocks (zero padded)
//   B'[item][s][N'][K']   N' = NT * ntiles (zero padded)
// Tiles reach shared memory by TMA (3-D tensor maps, 128-byte swizzle).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/skkr_gpu.h"
#include "kernels.h"

namespace {

constexpr int NT = 96;            // N tile (TMEM columns per accumulator)
constexpr int MT = 128;           // M tile (UMMA M)
constexpr int KB = 64;            // K per k-block (one 128-byte swizzle row of bf16)
constexpr int NACC = 5;           // TMEM accumulators: one per level p+q = 0..4
constexpr long long WAIT_LIMIT = 1LL << 22;

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: false when the limit is reached
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  for (long long i = 0; i < WAIT_LIMIT; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *tm, int c0, int c1, int c2,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(smem_u32(dst)),
      "l"((uint64_t)tm), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
        "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
        "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// UMMA shared-memory descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (tile base 1024-byte aligned).
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;            // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset
  d |= (uint64_t)1 << 46;            // descriptor version
  d |= (uint64_t)2 << 61;            // 128-byte swizzle
  return d;
}
// instruction descriptor: BF16 x BF16 -> FP32, K-major A and B, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// ------------------------------------------------------------------ slicing
__device__ __forceinline__ double pow2_scale(double amax) {
  if (!(amax > 0.0) || !isfinite(amax)) return 1.0;
  int e;
  frexp(amax, &e);  // amax = m 2^e, m in [0.5, 1)
  return ldexp(1.0, e);
}

template <int S>
__device__ __forceinline__ void slice_store(double x, double inv_scale, int wshift, __nv_bfloat16 *dst,
                                            long long sstride) {
  double y = x * inv_scale * 128.0;
#pragma unroll
  for (int p = 0; p < S; p++) {
    double s = rint(y);
    dst[p * sstride] = __double2bfloat16(ldexp(s, wshift - 8 * p));
    y = (y - s) * 256.0;
  }
}

// A' from complex A (n x n, MatRef): one CTA per (item, 32-row block).
// Row scales over re/im of the whole row, then a shared-memory transpose so
// that both the FP64 reads (along rows i) and the bf16 writes (along kk)
// are coalesced.
template <int S>
__global__ void __launch_bounds__(256) k_split_a(MatRef A, int n, int nc, const int *__restrict__ act,
                                                 __nv_bfloat16 *__restrict__ out, int Mp, int Kp,
                                                 double *__restrict__ sigma) {
  const int item = blockIdx.y, kk0 = item / nc, cc = item % nc;
  if (act && !act[item]) return;
  const zd *a = mat_ptr(A, kk0, cc);
  const int r0 = blockIdx.x * 32, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __shared__ double red[8][32];
  __shared__ double sc[32];
  __shared__ zd T[32][33];
  double m = 0.0;
  const int row = r0 + lane;
  if (row < n)
    for (int k = w; k < n; k += 8) {
      zd v = a[row + (long long)k * A.ld];
      m = fmax(m, fmax(fabs(v.x), fabs(v.y)));
    }
  red[w][lane] = m;
  __syncthreads();
  if (w == 0) {
    double mm = 0.0;
    for (int q = 0; q < 8; q++) mm = fmax(mm, red[q][lane]);
    double s = pow2_scale(mm);
    sc[lane] = s;
    if (r0 + lane < Mp) sigma[(long long)item * Mp + r0 + lane] = s;
  }
  __syncthreads();
  const long long sstride = (long long)Mp * Kp;
  __nv_bfloat16 *base = out + (long long)item * S * sstride;
  for (int c0 = 0; c0 < n; c0 += 32) {
    for (int q = w; q < 32; q += 8) {
      int col = c0 + q;
      T[lane][q] = (row < n && col < n) ? a[row + (long long)col * A.ld] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    for (int q = w; q < 32; q += 8) {
      const int r = r0 + q, col = c0 + lane;
      if (r < n && col < n) {
        const double inv = 1.0 / sc[q];
        zd v = T[q][lane];
        slice_store<S>(v.x, inv, 0, base + (long long)r * Kp + col, sstride);
        slice_store<S>(v.y, inv, 0, base + (long long)r * Kp + n + col, sstride);
      }
    }
    __syncthreads();
  }
}

// B'^T from complex B (n x n, MatRef): one warp per column j; rows j and n+j
// of B'^T are [Re B(:,j), -Im B(:,j)] and [Im B(:,j), Re B(:,j)].
template <int S>
__global__ void __launch_bounds__(256) k_split_b(MatRef B, int n, int nc, const int *__restrict__ act,
                                                 __nv_bfloat16 *__restrict__ out, int Np, int Kp,
                                                 double *__restrict__ tau) {
  const int item = blockIdx.y, kk0 = item / nc, cc = item % nc;
  if (act && !act[item]) return;
  const int lane = threadIdx.x & 31, j = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (j >= n) return;
  const zd *b = mat_ptr(B, kk0, cc) + (long long)j * B.ld;
  double m = 0.0;
  for (int k = lane; k < n; k += 32) {
    zd v = b[k];
    m = fmax(m, fmax(fabs(v.x), fabs(v.y)));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  const double s = pow2_scale(m), inv = 1.0 / s;
  if (lane == 0) tau[(long long)item * n + j] = s;
  const long long sstride = (long long)Np * Kp;
  __nv_bfloat16 *base = out + (long long)item * S * sstride;
  __nv_bfloat16 *rj = base + (long long)j * Kp, *rjn = base + (long long)(n + j) * Kp;
  for (int k = lane; k < n; k += 32) {
    zd v = b[k];
    slice_store<S>(v.x, inv, 16, rj + k, sstride);
    slice_store<S>(-v.y, inv, 16, rj + n + k, sstride);
    slice_store<S>(v.y, inv, 16, rjn + k, sstride);
    slice_store<S>(v.x, inv, 16, rjn + n + k, sstride);
  }
}

// ------------------------------------------------------------------ the GEMM
struct OzArgs {
  int n, mtiles, ntiles, kblocks, nc, mode;
  const double *sigma;  // [item][M']
  const double *tau;    // [item][n]
  MatRef C, D, E;
  const int *act;
  int *err;
};

// accumulator of product (p, q), 0-based slices: its level p+q; levels >= 4
// share the last accumulator (they sit 2^-32 and further below the leading
// level, so the truncation of the shared sum is far below the slice error)
__host__ __device__ constexpr int level_of(int p, int q) { return p + q < NACC ? p + q : NACC - 1; }
// accumulators in use for S slices (levels 0 .. S-1)
__host__ __device__ constexpr int nlevels(int S) { return S < NACC ? S : NACC; }

template <int S>
__global__ void __launch_bounds__(128, 1) k_ozaki(const __grid_constant__ CUtensorMap tmA,
                                                  const __grid_constant__ CUtensorMap tmB, OzArgs g) {
  const int item = blockIdx.y;
  if (g.act && !g.act[item]) return;
  const int mt = blockIdx.x / g.ntiles, nt = blockIdx.x % g.ntiles;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte aligned tile area: S A tiles (MT x KB) then S B tiles (NT x KB)
  unsigned char *tiles = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr uint32_t A_BYTES = MT * KB * 2, B_BYTES = NT * KB * 2;
  unsigned char *tA = tiles, *tB = tiles + S * A_BYTES;
  __shared__ __align__(8) uint64_t bar_load, bar_mma;
  __shared__ uint32_t tmem_base;
  __shared__ int failed;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (warp == 0) {
    tmem_alloc(&tmem_base, 512);
    tmem_relinquish();
  }
  if (threadIdx.x == 0) {
    failed = 0;
    mbar_init(&bar_load, 1);
    mbar_init(&bar_mma, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tmem_base;
  constexpr uint32_t IDESC = idesc_bf16(MT, NT);

  for (int kb = 0; kb < g.kblocks; kb++) {
    const uint32_t phase = kb & 1;
    if (threadIdx.x == 0 && !failed) {
      mbar_expect_tx(&bar_load, S * (A_BYTES + B_BYTES));
#pragma unroll
      for (int s = 0; s < S; s++) {
        tma_load_3d(tA + s * A_BYTES, &tmA, kb * KB, mt * MT, item * S + s, &bar_load);
        tma_load_3d(tB + s * B_BYTES, &tmB, kb * KB, nt * NT, item * S + s, &bar_load);
      }
      if (!mbar_wait(&bar_load, phase)) {
        failed = 1;
        mbar_wait(&bar_load, phase);  // give in-flight copies a second bounded chance to land
      }
      if (!failed) {
        tc_fence_after();
        bool first[NACC] = {kb == 0, kb == 0, kb == 0, kb == 0, kb == 0};
#pragma unroll
        for (int p = 0; p < S; p++)
#pragma unroll
          for (int q = 0; q < S; q++) {
            if (p + q > S - 1) continue;  // keep p+q <= S+1 in 1-based slices
            const int lv = level_of(p, q);
            const uint32_t a0 = smem_u32(tA + p * A_BYTES), b0 = smem_u32(tB + q * B_BYTES);
#pragma unroll
            for (int k = 0; k < KB / 16; k++) {
              umma_bf16(tbase + lv * NT, sdesc_sw128(a0 + 32 * k), sdesc_sw128(b0 + 32 * k), IDESC,
                        first[lv] ? 0u : 1u);
              first[lv] = false;
            }
          }
      }
      umma_commit(&bar_mma);
      if (!mbar_wait(&bar_mma, phase)) {
        failed = 1;
        mbar_wait(&bar_mma, phase);  // MMAs must be done before TMEM is released
      }
    }
    __syncthreads();
    if (failed) break;
  }
  tc_fence_after();
  if (failed) {
    if (threadIdx.x == 0) atomicOr(g.err, 1);
  } else {
    // epilogue: warp w owns TMEM lanes 32w..32w+31 = rows of this M tile
    const int row = mt * MT + warp * 32 + lane;
    const uint32_t lane_addr = tbase + ((uint32_t)(warp * 32) << 16);
    const int kk = item / g.nc, cc = item % g.nc;
    const double srow = row < g.n ? g.sigma[(long long)item * (g.mtiles * MT) + row] * 0x1p-30 : 0.0;
    for (int c0 = 0; c0 < NT; c0 += 32) {
      float v[NACC][32];
      constexpr int NL = nlevels(S);
#pragma unroll
      for (int l = 0; l < NL; l++) tmem_ld32(lane_addr + l * NT + c0, v[l]);
      if (row >= g.n) continue;
#pragma unroll
      for (int t = 0; t < 32; t++) {
        const int jj = nt * NT + c0 + t;
        if (jj < 2 * g.n) {
          const int j = jj < g.n ? jj : jj - g.n, im = jj >= g.n;
          // smallest level first; every addend is exact in FP64
          double acc = (double)v[NL - 1][t];
#pragma unroll
          for (int l = NL - 2; l >= 0; l--) acc += (double)v[l][t];
          const double val = acc * srow * g.tau[(long long)item * g.n + j];
          const long long off = 2 * (row + (long long)j * g.C.ld) + im;
          if (g.mode == 0) {
            ((double *)mat_ptr(g.C, kk, cc))[off] = val;
          } else if (g.mode == 1) {
            ((double *)mat_ptr(g.C, kk, cc))[off] -= val;
          } else if (g.mode == 2) {
            const long long od = 2 * (row + (long long)j * g.D.ld) + im;
            const long long oe = 2 * (row + (long long)j * g.E.ld) + im;
            ((double *)mat_ptr(g.D, kk, cc))[od] -= val;
            ((double *)mat_ptr(g.E, kk, cc))[oe] -= val;
          } else if (g.mode == 3) {
            const long long od = 2 * (row + (long long)j * g.D.ld) + im;
            ((double *)mat_ptr(g.C, kk, cc))[off] = ((const double *)mat_ptr(g.D, kk, cc))[od] - val;
          } else if (g.mode == 4) {
            ((double *)mat_ptr(g.C, kk, cc))[off] = ((row == j && !im) ? 1.0 : 0.0) - val;
          } else {
            ((double *)mat_ptr(g.C, kk, cc))[off] += val;
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tbase, 512);
}

// ------------------------------------------------------------------ FP32 GJ
// Gauss-Jordan with column pivoting (main/gjinv.f) in complex FP32, matrix in
// shared memory; result written as FP64 into X.  n <= 128.
__global__ void __launch_bounds__(512) k_cgj32(MatRef A, MatRef X, int n, int nc, const int *__restrict__ act) {
  const int item = blockIdx.x, kk = item / nc, cc = item % nc;
  if (act && !act[item]) return;
  extern __shared__ float2 sa[];  // n*n column-major
  __shared__ int ind[128];
  __shared__ float2 coli[128], rowi[128];
  __shared__ float rv[16];
  __shared__ int ri[16];
  const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = nth >> 5;
  const zd *a = mat_ptr(A, kk, cc);
  for (int e = tid; e < n * n; e += nth) {
    zd v = a[(e % n) + (long long)(e / n) * A.ld];
    sa[e] = make_float2((float)v.x, (float)v.y);
  }
  __syncthreads();
  for (int i = 0; i < n; i++) {
    float best = -1.f;
    int bj = n;
    for (int j = i + tid; j < n; j += nth) {
      float2 v = sa[i + j * n];
      float m = hypotf(v.x, v.y);
      if (m > best || (m == best && j < bj)) { best = m; bj = j; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      float ob = __shfl_down_sync(0xffffffffu, best, o);
      int oj = __shfl_down_sync(0xffffffffu, bj, o);
      if (ob > best || (ob == best && oj < bj)) { best = ob; bj = oj; }
    }
    if (lane == 0) { rv[wid] = best; ri[wid] = bj; }
    __syncthreads();
    if (wid == 0) {
      best = lane < nw ? rv[lane] : -2.f;
      bj = lane < nw ? ri[lane] : n;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        float ob = __shfl_down_sync(0xffffffffu, best, o);
        int oj = __shfl_down_sync(0xffffffffu, bj, o);
        if (ob > best || (ob == best && oj < bj)) { best = ob; bj = oj; }
      }
      if (lane == 0) { ri[0] = bj; ind[i] = bj; }
    }
    __syncthreads();
    const int kp = ri[0];
    if (kp != i) {
      for (int r = tid; r < n; r += nth) {
        float2 t = sa[r + i * n];
        sa[r + i * n] = sa[r + kp * n];
        sa[r + kp * n] = t;
      }
      __syncthreads();
    }
    float2 piv = sa[i + i * n];
    float den = piv.x * piv.x + piv.y * piv.y;
    float2 q = make_float2(piv.x / den, -piv.y / den);
    for (int j = tid; j < n; j += nth) rowi[j] = sa[i + j * n];
    for (int r = tid; r < n; r += nth) {
      float2 v = sa[r + i * n];
      coli[r] = (r == i) ? q : make_float2(v.x * q.x - v.y * q.y, v.x * q.y + v.y * q.x);
    }
    __syncthreads();
    for (int r = tid; r < n; r += nth) sa[r + i * n] = coli[r];
    for (int e = tid; e < n * n; e += nth) {
      const int r = e % n, j = e / n;
      if (j == i) continue;
      float2 v = (r == i) ? make_float2(0.f, 0.f) : sa[e];
      const float2 c = coli[r], w = rowi[j];
      v.x = fmaf(-c.x, w.x, v.x);
      v.x = fmaf(c.y, w.y, v.x);
      v.y = fmaf(-c.x, w.y, v.y);
      v.y = fmaf(-c.y, w.x, v.y);
      sa[e] = v;
    }
    __syncthreads();
  }
  for (int i = n - 1; i >= 0; i--) {
    const int j = ind[i];
    if (j == i) continue;
    for (int c = tid; c < n; c += nth) {
      float2 t = sa[i + c * n];
      sa[i + c * n] = sa[j + c * n];
      sa[j + c * n] = t;
    }
    __syncthreads();
  }
  zd *x = mat_ptr(X, kk, cc);
  for (int e = tid; e < n * n; e += nth) {
    float2 v = sa[e];
    x[(e % n) + (long long)(e / n) * X.ld] = make_double2((double)v.x, (double)v.y);
  }
}

// ------------------------------------------------------------------ host side
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int get_encoder() {
  if (g_encode) return 0;
  cudaDriverEntryPointQueryResult q;
  void *fn = nullptr;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
          cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn)
    return -1;
  g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  return 0;
}

int make_map(CUtensorMap *m, void *base, int K, int rows, long long depth, int boxrows) {
  cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)depth};
  cuuint64_t strides[2] = {(cuuint64_t)K * 2, (cuuint64_t)K * 2 * rows};
  cuuint32_t box[3] = {(cuuint32_t)KB, (cuuint32_t)boxrows, 1};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -1;
}

// at least 120 KB so that only one CTA (and one 512-column TMEM allocation)
// is resident per SM
size_t oz_smem_bytes(int S) {
  size_t b = (size_t)S * (MT * KB * 2 + NT * KB * 2) + 1024;
  return b < 120 * 1024 ? 120 * 1024 : b;
}

}  // namespace

// ---------------------------------------------------------------------------
struct MixedWork {
  void *sa = nullptr, *sb = nullptr;  // slice staging
  size_t sa_cap = 0, sb_cap = 0;
  double *sigma = nullptr, *tau = nullptr;
  size_t sig_cap = 0, tau_cap = 0;
  zd *acopy = nullptr, *rbuf = nullptr;
  size_t ac_cap = 0, rb_cap = 0;
  double *rnorm = nullptr;
  size_t rn_cap = 0;
  int *err = nullptr;
  int smem_set[16] = {0};
  int last_n = -1;   // staging layout the zero padding was made for
};

static int grow(void **p, size_t *cap, size_t bytes, bool zero) {
  if (bytes <= *cap) return 0;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  if (cudaMalloc(p, bytes) != cudaSuccess) return SKKR_ERR_NOMEM;
  if (zero && cudaMemset(*p, 0, bytes) != cudaSuccess) return SKKR_ERR_NOMEM;
  *cap = bytes;
  return 0;
}

MixedWork *mixed_create() {
  MixedWork *w = new MixedWork();
  if (cudaMalloc(&w->err, sizeof(int)) != cudaSuccess) {
    delete w;
    return nullptr;
  }
  cudaMemset(w->err, 0, sizeof(int));
  return w;
}

void mixed_destroy(MixedWork *w) {
  if (!w) return;
  void *ps[] = {w->sa, w->sb, w->sigma, w->tau, w->acopy, w->rbuf, w->rnorm, w->err};
  for (void *p : ps)
    if (p) cudaFree(p);
  delete w;
}

int mixed_error_flag(MixedWork *w) {
  int h = 0;
  if (cudaMemcpy(&h, w->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  return h;
}

// dims of the staged real problem for complex n
static void oz_dims(int n, int *Mp, int *Np, int *Kp, int *mtiles, int *ntiles, int *kblocks) {
  *mtiles = (n + MT - 1) / MT;
  *Mp = *mtiles * MT;
  *ntiles = (2 * n + NT - 1) / NT;
  *Np = *ntiles * NT;
  *kblocks = (2 * n + KB - 1) / KB;
  *Kp = *kblocks * KB;
}

template <int S>
static int zgemm_s(MixedWork *w, int mode, const MatRef &A, const MatRef &B, const MatRef &C,
                   const MatRef &D, const MatRef &E, int n, int nk, int nc, const int *act,
                   cudaStream_t st) {
  if (get_encoder()) return SKKR_ERR_CUDA;
  int Mp, Np, Kp, mtiles, ntiles, kblocks;
  oz_dims(n, &Mp, &Np, &Kp, &mtiles, &ntiles, &kblocks);
  const long long items = (long long)nk * nc;
  int rc;
  // staging sized for S slices; the zero padding is redone when the layout changes
  if ((rc = grow(&w->sa, &w->sa_cap, (size_t)items * S * Mp * Kp * 2, true))) return rc;
  if ((rc = grow(&w->sb, &w->sb_cap, (size_t)items * S * Np * Kp * 2, true))) return rc;
  if (w->last_n != n * 16 + S) {
    // padding must be zero for this layout: clear what earlier layouts wrote
    if (cudaMemsetAsync(w->sa, 0, w->sa_cap, st) != cudaSuccess ||
        cudaMemsetAsync(w->sb, 0, w->sb_cap, st) != cudaSuccess)
      return SKKR_ERR_CUDA;
    w->last_n = n * 16 + S;
  }
  if ((rc = grow((void **)&w->sigma, &w->sig_cap, (size_t)items * Mp * sizeof(double), false))) return rc;
  if ((rc = grow((void **)&w->tau, &w->tau_cap, (size_t)items * n * sizeof(double), false))) return rc;
  dim3 ga((n + 31) / 32, items);
  k_split_a<S><<<ga, 256, 0, st>>>(A, n, nc, act, (__nv_bfloat16 *)w->sa, Mp, Kp, w->sigma);
  SKKR_LAUNCHED();
  dim3 gb((n + 7) / 8, items);
  k_split_b<S><<<gb, 256, 0, st>>>(B, n, nc, act, (__nv_bfloat16 *)w->sb, Np, Kp, w->tau);
  SKKR_LAUNCHED();
  CUtensorMap ma, mb;
  if (make_map(&ma, w->sa, Kp, Mp, items * S, MT) || make_map(&mb, w->sb, Kp, Np, items * S, NT))
    return SKKR_ERR_CUDA;
  const size_t smem = oz_smem_bytes(S);
  if (!w->smem_set[S]) {
    if (cudaFuncSetAttribute(k_ozaki<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return SKKR_ERR_CUDA;
    w->smem_set[S] = 1;
  }
  OzArgs g;
  g.n = n;
  g.mtiles = mtiles;
  g.ntiles = ntiles;
  g.kblocks = kblocks;
  g.nc = nc;
  g.mode = mode;
  g.sigma = w->sigma;
  g.tau = w->tau;
  g.C = C;
  g.D = D;
  g.E = E;
  g.act = act;
  g.err = w->err;
  dim3 grid(mtiles * ntiles, items);
  const long long active = act ? skkr_active_items(items) : items;
  kstat_begin(KS_GEMM, 8.0 * n * (double)n * n * (double)active, st);
  k_ozaki<S><<<grid, 128, smem, st>>>(ma, mb, g);
  kstat_end(st);
  SKKR_LAUNCHED();
  return 0;
}

int mixed_zgemm(MixedWork *w, int mode, int S, const MatRef &A, const MatRef &B, const MatRef &C,
                const MatRef &D, const MatRef &E, int n, int nk, int nc, const int *act, cudaStream_t st) {
  if (n < 1 || n > 256 || nk * (long long)nc > 65535) return SKKR_ERR_ARG;
  switch (S) {
    case 3: return zgemm_s<3>(w, mode, A, B, C, D, E, n, nk, nc, act, st);
    case 4: return zgemm_s<4>(w, mode, A, B, C, D, E, n, nk, nc, act, st);
    case 5: return zgemm_s<5>(w, mode, A, B, C, D, E, n, nk, nc, act, st);
    case 6: return zgemm_s<6>(w, mode, A, B, C, D, E, n, nk, nc, act, st);
    case 7: return zgemm_s<7>(w, mode, A, B, C, D, E, n, nk, nc, act, st);
    default: return SKKR_ERR_ARG;
  }
}

// X = A^-1: FP32 Gauss-Jordan, then `newton` steps X += X (I - A X) with the
// residual product at S = sres slices and the correction at S = 3.  X may
// alias A.
int mixed_zinv(MixedWork *w, const MatRef &A, const MatRef &X, int n, int nk, int nc, const int *act,
               int newton, int sres, double *max_resid, cudaStream_t st) {
  if (n < 1 || n > 128) return SKKR_ERR_ARG;
  const long long items = (long long)nk * nc, MB = (long long)n * n;
  int rc;
  if ((rc = grow((void **)&w->acopy, &w->ac_cap, (size_t)items * MB * sizeof(zd), false))) return rc;
  if ((rc = grow((void **)&w->rbuf, &w->rb_cap, (size_t)items * MB * sizeof(zd), false))) return rc;
  if ((rc = grow((void **)&w->rnorm, &w->rn_cap, (size_t)items * sizeof(double), false))) return rc;
  MatRef Ac = mref(w->acopy, (long long)nc * MB, MB, n);
  MatRef R = mref(w->rbuf, (long long)nc * MB, MB, n);
  launch_zaxpby(Ac, A, nullptr, 0, nullptr, 0, n, nk, nc, act, st);
  const size_t smem = (size_t)n * n * sizeof(float2);
  if (cudaFuncSetAttribute(k_cgj32, cudaFuncAttributeMaxDynamicSharedMemorySize, 128 * 128 * 8) !=
      cudaSuccess)
    return SKKR_ERR_CUDA;
  kstat_begin(KS_GJ, 8.0 * n * (double)n * n * (double)(act ? skkr_active_items(items) : items), st);
  k_cgj32<<<(unsigned)items, 512, smem, st>>>(Ac, X, n, nc, act);
  kstat_end(st);
  SKKR_LAUNCHED();
  for (int it = 0; it < newton; it++) {
    // R = I - A X
    if ((rc = mixed_zgemm(w, 4, sres, Ac, X, R, R, R, n, nk, nc, act, st))) return rc;
    if (max_resid && it == newton - 1) {
      cudaMemsetAsync(w->rnorm, 0, items * sizeof(double), st);
      launch_fnorm(R, n, nk, nc, act, w->rnorm, st);
    }
    // X = X + X R
    if ((rc = mixed_zgemm(w, 5, 3, X, R, X, X, X, n, nk, nc, act, st))) return rc;
  }
  if (max_resid) {
    std::vector<double> h(items);
    if (cudaMemcpyAsync(h.data(), w->rnorm, items * sizeof(double), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return SKKR_ERR_CUDA;
    double m = 0.0;
    for (double v : h) m = std::fmax(m, v);
    *max_resid = std::fmax(*max_resid, m);
  }
  return 0;
}
