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
// M = n, N = 2n, K' = 2K.  The real depth K' runs over groups of 16 complex
// indices, each group [Re 16 | Im 16] (kpos below), so that one 32-wide
// k-block holds both parts of 16 complex indices; B' columns 2j and 2j+1
// are Re and Im of output column j.
//
// Staging layouts (bf16, K-major for both UMMA operands, tiled by k-block so
// that one TMA box is one contiguous block):
//   A'[item][s][kb][M'][32]   M' = 128 * mtiles, kb < kblocks = ceil(K/16)
//   B'[item][s][kb][N'][32]   N' = TN * ntiles (zero padded; TN = 96, or 64
//                                 for the exact-level tile)
// A tiles reach shared memory by TMA (3-D tensor maps, 64-byte swizzle).  B
// tiles either the same way from B' or, fused, straight from the FP64 B: the
// ten warps that run the epilogue form each stage's B slices in shared
// memory while the tensor core works on the previous stage.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <string>
#include <cstring>
#include <vector>

#include "../../include/skkr_gpu.h"
#include "kernels.h"
#include "slicing.cuh"

namespace {

constexpr int NT = 96;            // N tile (TMEM columns per accumulator)
constexpr int MT = 128;           // M tile (UMMA M)
constexpr int KB = 32;            // K per k-block (one 64-byte swizzle row of bf16)
constexpr int OZ_SMEM_MAX = 232448;  // shared memory one CTA may use (opt-in)
// shared-memory pipeline stages of the sliced GEMM: three where three stages
// of S A tiles and S B tiles fit (S <= 5 at the 96-column tile), else two
__host__ __device__ constexpr int oz_stages(int S, int TN) {
  return 3 * S * (128 * 32 * 2 + TN * 32 * 2) + 1024 <= OZ_SMEM_MAX ? 3 : 2;
}
constexpr int NACC = 5;           // TMEM accumulators: one per level p+q = 0..4
constexpr long long WAIT_LIMIT = 1LL << 22;
constexpr int OZ_THREADS = 384;   // 12 warps: producer and MMA lanes in warps 0-1, all 12 run the epilogue

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
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
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
// bytes (a multiple of 16, 16-byte aligned) of global memory towards L2
__device__ __forceinline__ void bulk_prefetch_l2(const void *p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
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
// 16 consecutive accumulator columns of this warp's 32 TMEM lanes, without
// the wait (tmem_ld_wait after a batch of loads)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t *r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
        "=r"(r[15])
      : "r"(taddr)
      : "memory");
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// UMMA shared-memory descriptor: K-major, 64-byte swizzle (rows of 32 bf16),
// 8-row groups 512 bytes apart (tile base 512-byte aligned).
__device__ __forceinline__ uint64_t sdesc_sw64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;           // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(512 >> 4) << 32;  // stride byte offset: 8 rows x 64 bytes
  d |= (uint64_t)1 << 46;           // descriptor version
  d |= (uint64_t)4 << 61;           // 64-byte swizzle
  return d;
}
// instruction descriptor: BF16 x BF16 -> FP32, K-major A and B, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// ------------------------------------------------------------------ slicing
// (abs_bits, scale_exp, slice_digits, digit_bits, slice4: slicing.cuh)

// element (row r, K' index kk) of one slice region in the k-block tiled layout
__device__ __forceinline__ long long tiled(int r, int kk, int rows) {
  return ((long long)(kk >> 5) * rows + r) * 32 + (kk & 31);
}
// K' index of the real (im = 0) or imaginary (im = 1) part of complex index k
__host__ __device__ __forceinline__ int kpos(int k, int im) { return ((k >> 4) << 5) + (im << 4) + (k & 15); }

// the S words at dst + p sstride, sign bits flipped by `flip` (0 or 0x80008000)
template <int S>
__device__ __forceinline__ void store_words(const uint32_t (&w)[S][2], uint32_t flip, __nv_bfloat16 *dst,
                                            long long sstride) {
#pragma unroll
  for (int p = 0; p < S; p++)
    *reinterpret_cast<uint2 *>(dst + p * sstride) = make_uint2(w[p][0] ^ flip, w[p][1] ^ flip);
}
// one element, slices p = 0..S-1 (the shapes of no four-element group)
template <int S, int DB>
__device__ __forceinline__ void store1(const int (&dg)[S], int wshift, uint16_t flip, __nv_bfloat16 *dst,
                                       long long sstride) {
#pragma unroll
  for (int p = 0; p < S; p++) {
    const float sc = pow2f(wshift - DB * p);
    const uint16_t h = (uint16_t)(digit_bits(dg[p], sc, -12582912.0f * sc) >> 16) ^ flip;
    *reinterpret_cast<uint16_t *>(dst + p * sstride) = h;
  }
}

// A' = [Re A, Im A] (n x 2K, in the K' order) from the n x K complex A; rows scaled by their
// max over these K columns.  32 rows per block: the row maxima, then 32 x 32
// tiles transposed through shared memory, each thread taking four
// consecutive columns of one row (8-byte stores of every slice) when K is a
// multiple of four, one element otherwise.
template <int S, int DB>
__global__ void __launch_bounds__(256) k_split_a(MatRef A, int n, int K, int nc, const int *__restrict__ act,
                                                 __nv_bfloat16 *__restrict__ out, int Mp, int Kp,
                                                 int *__restrict__ sigma) {
  const int item = blockIdx.y, kk0 = item / nc, cc = item % nc;
  if (act && !act[item]) return;
  const zd *a = mat_ptr(A, kk0, cc);
  const int r0 = blockIdx.x * 32, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __shared__ unsigned long long red[8][32];
  __shared__ int sc[32];
  __shared__ zd T[32][33];
  unsigned long long m = 0;
  const int row = r0 + lane;
  if (row < n)
    for (int k = w; k < K; k += 8) {
      zd v = a[row + (long long)k * A.ld];
      const unsigned long long bx = abs_bits(v.x), by = abs_bits(v.y);
      m = bx > m ? bx : m;
      m = by > m ? by : m;
    }
  red[w][lane] = m;
  __syncthreads();
  if (w == 0) {
    unsigned long long mm = 0;
    for (int q = 0; q < 8; q++) mm = red[q][lane] > mm ? red[q][lane] : mm;
    const int es = scale_exp(mm);
    sc[lane] = es;
    if (r0 + lane < Mp) sigma[(long long)item * Mp + r0 + lane] = es;
  }
  __syncthreads();
  const long long sstride = (long long)Mp * Kp;
  __nv_bfloat16 *base = out + (long long)item * S * sstride;
  const bool vec = (K & 3) == 0;
  for (int c0 = 0; c0 < K; c0 += 32) {
    for (int q = w; q < 32; q += 8) {
      int col = c0 + q;
      T[lane][q] = (row < n && col < K) ? a[row + (long long)col * A.ld] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    if (vec) {
      // thread t: row r0 + t / 8, columns c0 + 4 (t % 8) .. +3
      const int q = threadIdx.x >> 3, c4 = (threadIdx.x & 7) * 4, r = r0 + q, col = c0 + c4;
      if (r < n && col < K) {
        double re[4], im[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
          re[e] = T[q][c4 + e].x;
          im[e] = T[q][c4 + e].y;
        }
        uint32_t wr[S][2], wi[S][2];
        slice4<S, DB>(re, im, sc[q], 0, wr, wi);
        store_words<S>(wr, 0u, base + tiled(r, kpos(col, 0), Mp), sstride);
        store_words<S>(wi, 0u, base + tiled(r, kpos(col, 1), Mp), sstride);
      }
    } else {
      for (int q = w; q < 32; q += 8) {
        const int r = r0 + q, col = c0 + lane;
        if (r < n && col < K) {
          const int es = sc[q];
          const zd v = T[q][lane];
          int dr[S], di[S];
          slice_digits<S, DB>(v.x, es, dr);
          slice_digits<S, DB>(v.y, es, di);
          store1<S, DB>(dr, 0, 0, base + tiled(r, kpos(col, 0), Mp), sstride);
          store1<S, DB>(di, 0, 0, base + tiled(r, kpos(col, 1), Mp), sstride);
        }
      }
    }
    __syncthreads();
  }
}

// B'^T from the K x n complex B: one warp per column j; rows 2j and 2j+1 of
// B'^T are [Re B(:,j), -Im B(:,j)] and [Im B(:,j), Re B(:,j)] (columns scaled
// by their max over these K rows), so that the real and imaginary parts of an
// output element land in adjacent accumulator columns of one thread.  Each
// lane takes four consecutive rows k (8-byte stores) when K is a multiple of
// four, one row otherwise; each digit is formed once and stored twice, -Im
// with its sign bit flipped.
template <int S, int DB>
__global__ void __launch_bounds__(256, 3) k_split_b(MatRef B, int n, int K, int nc, const int *__restrict__ act,
                                                 __nv_bfloat16 *__restrict__ out, int Np, int Kp,
                                                 int *__restrict__ tau) {
  const int item = blockIdx.y, kk0 = item / nc, cc = item % nc;
  if (act && !act[item]) return;
  const int lane = threadIdx.x & 31, j = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (j >= n) return;
  const zd *b = mat_ptr(B, kk0, cc) + (long long)j * B.ld;
  unsigned long long m = 0;
  for (int k = lane; k < K; k += 32) {
    zd v = b[k];
    const unsigned long long bx = abs_bits(v.x), by = abs_bits(v.y);
    m = bx > m ? bx : m;
    m = by > m ? by : m;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, m, o);
    m = t > m ? t : m;
  }
  const int es = scale_exp(m);
  if (lane == 0) tau[(long long)item * n + j] = es;
  const long long sstride = (long long)Np * Kp;
  __nv_bfloat16 *base = out + (long long)item * S * sstride;
  if ((K & 3) == 0) {
    for (int k = 4 * lane; k < K; k += 128) {
      double re[4], im[4];
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const zd v = b[k + e];
        re[e] = v.x;
        im[e] = v.y;
      }
      uint32_t wr[S][2], wi[S][2];
      slice4<S, DB>(re, im, es, 16, wr, wi);
      store_words<S>(wr, 0u, base + tiled(2 * j, kpos(k, 0), Np), sstride);
      store_words<S>(wi, 0x80008000u, base + tiled(2 * j, kpos(k, 1), Np), sstride);
      store_words<S>(wi, 0u, base + tiled(2 * j + 1, kpos(k, 0), Np), sstride);
      store_words<S>(wr, 0u, base + tiled(2 * j + 1, kpos(k, 1), Np), sstride);
    }
  } else {
    for (int k = lane; k < K; k += 32) {
      const zd v = b[k];
      int dr[S], di[S];
      slice_digits<S, DB>(v.x, es, dr);
      slice_digits<S, DB>(v.y, es, di);
      store1<S, DB>(dr, 16, 0, base + tiled(2 * j, kpos(k, 0), Np), sstride);
      store1<S, DB>(di, 16, 0x8000, base + tiled(2 * j, kpos(k, 1), Np), sstride);
      store1<S, DB>(di, 16, 0, base + tiled(2 * j + 1, kpos(k, 0), Np), sstride);
      store1<S, DB>(dr, 16, 0, base + tiled(2 * j + 1, kpos(k, 1), Np), sstride);
    }
  }
}

// ------------------------------------------------------------------ the GEMM
struct OzArgs {
  int n, mtiles, ntiles, kblocks, nc, mode;
  int eoff;             // 32 + 2 (DB - 1): result = acc 2^(sigma_i + tau_j - eoff), acc in 2^-16 units
  int db;               // digit bits DB
  const int *sigma;     // [item][M']  row scale exponents of A
  const int *tau;       // [item][n]   column scale exponents of B (staged B)
  MatRef B;             // the FP64 K x n operand B (fused B)
  int K;
  MatRef C, D, E;
  const int *act;
  int *err;
};

// FP32 accumulator value -> int64 in units of 2^-16 (bit manipulation only).
// Levels 0..3 hold exact multiples of 2^(16-DB l) >= 2^-8; the shared tail
// level is truncated at 2^-16, about 2^-53 below the leading level.
// exact level l <= 3 (its FP32 accumulator holds an integer N times
// 2^(16 - DB l), |N| < 2^24) in the same 2^-16 units: N from one conversion,
// then a shift (32 - DB l >= 0 for l <= 3); the result equals f2fix16(v)
__device__ __forceinline__ long long level_fix16(float v, int l, int db) {
  const int n = __float2int_rn(v * pow2f(db * l - 16));
  return (long long)n << (32 - db * l);
}
__device__ __forceinline__ long long f2fix16(float v) {
  const int b = __float_as_int(v);
  const int ex = (b >> 23) & 0xFF;
  if (ex == 0) return 0;
  const long long mant = (b & 0x7FFFFF) | 0x800000;
  const int sh = ex - 150 + 16;
  const long long m = sh >= 0 ? (mant << sh) : (sh > -31 ? (mant >> -sh) : 0);
  return b < 0 ? -m : m;
}
// round-to-nearest-even double of a * 2^e from integer operations only (the
// FP64 pipe of this GPU is ~1/40 of the integer rate): normalise with a
// leading-zero count, keep 53 bits, round on the dropped 11, add e to the
// exponent.  Equal to __ll2double_rn(a) * 2^e for normal results.
__device__ __forceinline__ double fix_to_double(long long a, int e) {
  if (a == 0) return 0.0;
  const unsigned long long sign = a < 0 ? 0x8000000000000000ull : 0ull;
  unsigned long long m = a < 0 ? 0ull - (unsigned long long)a : (unsigned long long)a;
  const int lz = __clzll((long long)m);
  m <<= lz;                                    // leading one at bit 63
  unsigned long long mant = m >> 11;           // 53 significant bits
  const unsigned long long rem = m & 0x7FFull;
  int ex = 63 - lz + e;
  mant += (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) ? 1ull : 0ull;
  if (mant >> 53) {                            // rounding carried into bit 53
    mant >>= 1;
    ex++;
  }
  return __longlong_as_double((long long)(sign | ((unsigned long long)(ex + 1023) << 52) |
                                          (mant & 0xFFFFFFFFFFFFFull)));
}

// accumulator of product (p, q), 0-based slices: its level p+q; levels >= 4
// share the last accumulator (they sit 2^-32 and further below the leading
// level, so the truncation of the shared sum is far below the slice error)
template <int NA>
__host__ __device__ constexpr int level_of(int p, int q) { return p + q < NA ? p + q : NA - 1; }
// accumulators in use for S slices (levels 0 .. S-1)
template <int NA>
__host__ __device__ constexpr int nlevels(int S) { return S < NA ? S : NA; }

// byte offset of bf16 (row r, column t < 32) in a K-major tile of 64-byte rows
// with the 64-byte swizzle, as TMA lays it out and the UMMA descriptor reads
// it: the 16-byte chunk index XORed with address bits 7-8 (bits 1-2 of r)
__device__ __forceinline__ uint32_t sw64_off(int r, int t) {
  return (uint32_t)(r * 64 + ((((t >> 3) ^ (r >> 1)) & 3) << 4) + ((t & 7) << 1));
}

// Fused B operand, run by the 320 threads of warps 2-11 of k_ozaki: first
// the scale exponents of the CTA's TN/2 complex columns over the whole depth
// K (into col_exp, which the epilogue reads as well), then per k-block the S
// B tiles of a stage: thread t takes column t/4 and the four complex indices
// 16 kb + 4 (t%4) .. +3, forms their digits once (as k_split_b does) and
// stores them four times (rows 2j and 2j+1, the Re and Im halves of the
// k-block, -Im with flipped sign bits).  The next k-block's values are loaded
// before the wait for the stage.  Each thread orders its stores before the
// tensor core's reads (proxy fence); lane 0 of each warp, after the warp's
// barrier, arrives on the stage's full barrier.
template <int S, int TN, int DB, int NSTAGE>
__device__ __forceinline__ void fused_b_tiles(const OzArgs &g, int item, int nt, unsigned char *sb0,
                                              uint32_t stage_bytes, uint64_t *bar_full, uint64_t *bar_empty,
                                              int *col_exp, volatile int &failed) {
  constexpr int NCT = OZ_THREADS - 64;
  constexpr uint32_t B_BYTES = TN * KB * 2;
  const int ct = threadIdx.x - 64, lane = threadIdx.x & 31;
  const zd *bsrc = mat_ptr(g.B, item / g.nc, item % g.nc);
  const int j0 = (nt * TN) >> 1;
  // warp w, four columns 4w .. 4w+3 per round (40 per round), 16 loads of
  // each lane in flight
  for (int jl0 = 4 * (ct >> 5); jl0 < TN / 2; jl0 += 4 * (NCT / 32)) {
    unsigned long long m[4] = {0, 0, 0, 0};
    for (int kc = 0; kc < g.K; kc += 128) {
      zd v[4][4];
#pragma unroll
      for (int c = 0; c < 4; c++)
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const int k = kc + lane + 32 * i, j = j0 + jl0 + c;
          v[c][i] = (k < g.K && j < g.n && jl0 + c < TN / 2) ? bsrc[k + (long long)j * g.B.ld]
                                                             : make_double2(0.0, 0.0);
        }
#pragma unroll
      for (int c = 0; c < 4; c++)
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const unsigned long long bx = abs_bits(v[c][i].x), by = abs_bits(v[c][i].y);
          m[c] = bx > m[c] ? bx : m[c];
          m[c] = by > m[c] ? by : m[c];
        }
    }
#pragma unroll
    for (int c = 0; c < 4; c++) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, m[c], o);
        m[c] = t > m[c] ? t : m[c];
      }
      const int jl = jl0 + c;
      if (lane == 0 && jl < TN / 2) col_exp[jl] = j0 + jl < g.n ? scale_exp(m[c]) : 0;
    }
  }
  asm volatile("bar.sync 1, %0;" ::"n"(NCT) : "memory");
  const int jl = ct >> 2, kq = ct & 3;
  const bool on = ct < 2 * TN;
  const bool col_ok = on && j0 + jl < g.n;
  const zd *bcol = bsrc + (long long)(col_ok ? j0 + jl : 0) * g.B.ld;
  const int es = on ? col_exp[jl] : 0;
  zd cur[4], nxt[4];
  auto fetch = [&](int kb, zd(&v)[4]) {
    const int k = 16 * kb + 4 * kq;
#pragma unroll
    for (int e = 0; e < 4; e++) v[e] = (col_ok && k + e < g.K) ? bcol[k + e] : make_double2(0.0, 0.0);
  };
  fetch(0, cur);
  const int nkb = g.kblocks;
  for (int kb = 0; kb < nkb; kb++) {
    // the warp leaves together (lane 0 reads the flag), so its barriers and
    // shuffles below always see all 32 lanes
    if (__shfl_sync(0xffffffffu, (int)failed, 0)) break;
    const int st = kb % NSTAGE;
    if (kb + 1 < nkb) fetch(kb + 1, nxt);
    // lane 0 waits for the stage, the warp follows it (its stores come after
    // the tensor core's reads of the stage)
    int ok = 1;
    if (kb >= NSTAGE && lane == 0) ok = mbar_wait(&bar_empty[st], ((kb / NSTAGE) - 1) & 1);
    if (!__shfl_sync(0xffffffffu, ok, 0)) {
      failed = 1;
      break;
    }
    if (on) {
      double re[4], im[4];
#pragma unroll
      for (int e = 0; e < 4; e++) {
        re[e] = cur[e].x;
        im[e] = cur[e].y;
      }
      uint32_t wr[S][2], wi[S][2];
      slice4<S, DB>(re, im, es, 16, wr, wi);
      unsigned char *sb = sb0 + st * stage_bytes;
      const int r = 2 * jl, t = 4 * kq;
      const uint32_t o0 = sw64_off(r, t), o1 = sw64_off(r, t + 16), o2 = sw64_off(r + 1, t),
                     o3 = sw64_off(r + 1, t + 16);
#pragma unroll
      for (int p = 0; p < S; p++) {
        unsigned char *tp = sb + p * B_BYTES;
        *reinterpret_cast<uint2 *>(tp + o0) = make_uint2(wr[p][0], wr[p][1]);
        *reinterpret_cast<uint2 *>(tp + o1) = make_uint2(wi[p][0] ^ 0x80008000u, wi[p][1] ^ 0x80008000u);
        *reinterpret_cast<uint2 *>(tp + o2) = make_uint2(wi[p][0], wi[p][1]);
        *reinterpret_cast<uint2 *>(tp + o3) = make_uint2(wr[p][0], wr[p][1]);
      }
    }
    // every lane's stores visible to the tensor core, then one arrival per warp
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncwarp();
    if (lane == 0) mbar_arrive(&bar_full[st]);
#pragma unroll
    for (int e = 0; e < 4; e++) cur[e] = nxt[e];
  }
}

// TN: N tile (TMEM columns per accumulator); NA: TMEM accumulators, one per
// level p+q = 0..NA-2 and a shared tail for the deeper levels (NA * TN <= 512).
// (96, 5) is the default tile; (64, 7) keeps levels 0..5 exact and pushes the
// truncation of the shared tail below 2^-60 of the leading level.  Four
// levels would not do: with the shared tail from level 3 on, the tensor
// core's truncating FP32 addition leaves ~2^-47 of the leading level per
// accumulation step in it (4e-12 over a 128-deep product instead of 7e-14).
// FB = 0: B tiles by TMA from the staged B'; FB = DB (7 or 8): B fused, its
// tiles formed from the FP64 g.B by warps 2-11 (tmB unused).
template <int S, int TN, int NA, int FB>
__global__ void __launch_bounds__(OZ_THREADS, 1) k_ozaki(const __grid_constant__ CUtensorMap tmA,
                                                  const __grid_constant__ CUtensorMap tmB, OzArgs g) {
  static_assert(NA * TN <= 512 && TN % 32 == 0, "accumulators must fit the 512 TMEM columns");
  constexpr int NCT = OZ_THREADS - 64;  // threads of warps 2-11
  static_assert(FB == 0 || 2 * TN <= NCT, "fused B: one (column, four k) group per thread of warps 2-11");
  const int item = blockIdx.y;
  if (g.act && !g.act[item]) return;
  const int mt = blockIdx.x / g.ntiles, nt = blockIdx.x % g.ntiles;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // NSTAGE stages, each: S A tiles (MT x KB) then S B tiles (TN x KB), 1024-byte aligned
  constexpr int NSTAGE = oz_stages(S, TN);
  unsigned char *tiles = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr uint32_t A_BYTES = MT * KB * 2, B_BYTES = TN * KB * 2;
  constexpr uint32_t STAGE_BYTES = S * (A_BYTES + B_BYTES);
  __shared__ __align__(8) uint64_t bar_full[NSTAGE], bar_empty[NSTAGE], bar_acc;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int failed, issued_kb, consumed_kb;
  __shared__ int col_exp[TN / 2];  // column scale exponents of this tile's complex columns
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (warp == 0) {
    tmem_alloc(&tmem_base, 512);
    tmem_relinquish();
  }
  if (FB > 0 && threadIdx.x >= 64 && lane == 0) {
    // fused B: start the CTA's K x TN/2 block of B towards L2 (one bulk
    // prefetch per column, lane 0 of warps 2-11)
    const zd *bsrc = mat_ptr(g.B, item / g.nc, item % g.nc);
    for (int jl = warp - 2; jl < TN / 2; jl += NCT / 32) {
      const int j = (nt * TN) / 2 + jl;
      if (j < g.n) bulk_prefetch_l2(bsrc + (long long)j * g.B.ld, (uint32_t)g.K * (uint32_t)sizeof(zd));
    }
  }
  if (FB == 0 && threadIdx.x >= 64) {  // warps 2-11: column scales of the tile (read by the epilogue)
    for (int t = threadIdx.x - 64; t < TN / 2; t += blockDim.x - 64) {
      const int j = (nt * TN) / 2 + t;
      col_exp[t] = j < g.n ? g.tau[(long long)item * g.n + j] : 0;
    }
  }
  if (threadIdx.x == 32) {
    failed = 0;
    issued_kb = -1;
    consumed_kb = -1;
    for (int i = 0; i < NSTAGE; i++) {
      mbar_init(&bar_full[i], FB ? 1 + NCT / 32 : 1);  // fused B: each converting warp arrives too
      mbar_init(&bar_empty[i], 1);
    }
    mbar_init(&bar_acc, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tbase = tmem_base;
  constexpr uint32_t IDESC = idesc_bf16(MT, TN);
  const int nkb = g.kblocks;

  if (warp == 0 && lane == 0) {
    // TMA producer
    for (int kb = 0; kb < nkb && !failed; kb++) {
      const int st = kb % NSTAGE;
      if (kb >= NSTAGE && !mbar_wait(&bar_empty[st], ((kb / NSTAGE) - 1) & 1)) {
        failed = 1;
        break;
      }
      unsigned char *sA = tiles + st * STAGE_BYTES, *sB = sA + S * A_BYTES;
      mbar_expect_tx(&bar_full[st], FB ? S * A_BYTES : STAGE_BYTES);
#pragma unroll
      for (int sl = 0; sl < S; sl++) {
        const int z = (item * S + sl) * nkb + kb;
        tma_load_3d(sA + sl * A_BYTES, &tmA, 0, mt * MT, z, &bar_full[st]);
        if (FB == 0) tma_load_3d(sB + sl * B_BYTES, &tmB, 0, nt * TN, z, &bar_full[st]);
      }
      issued_kb = kb;
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    bool first[NA];
#pragma unroll
    for (int l = 0; l < NA; l++) first[l] = true;
    for (int kb = 0; kb < nkb; kb++) {
      const int st = kb % NSTAGE;
      if (failed || !mbar_wait(&bar_full[st], (kb / NSTAGE) & 1)) {
        failed = 1;
        break;
      }
      tc_fence_after();
      const uint32_t a0 = smem_u32(tiles + st * STAGE_BYTES), b0 = a0 + S * A_BYTES;
#pragma unroll
      for (int p = 0; p < S; p++)
#pragma unroll
        for (int q = 0; q < S; q++) {
          if (p + q > S - 1) continue;  // keep p+q <= S+1 in 1-based slices
          const int lv = level_of<NA>(p, q);
#pragma unroll
          for (int k = 0; k < KB / 16; k++) {
            umma_bf16(tbase + lv * TN, sdesc_sw64(a0 + p * A_BYTES + 32 * k),
                      sdesc_sw64(b0 + q * B_BYTES + 32 * k), IDESC, first[lv] ? 0u : 1u);
            first[lv] = false;
          }
        }
      umma_commit(&bar_empty[st]);  // stage free once these MMAs have read it
      consumed_kb = kb;
    }
    umma_commit(&bar_acc);  // accumulators complete
  } else if (warp >= 2) {
    if constexpr (FB > 0) fused_b_tiles<S, TN, FB, NSTAGE>(g, item, nt, tiles + S * A_BYTES, STAGE_BYTES,
                                                           bar_full, bar_empty, col_exp, failed);
  }
  __syncthreads();
  // all MMAs (and with them every TMA load they consumed) are done once
  // bar_acc completes; a bounded wait, then a second one if the first expired
  if (!mbar_wait(&bar_acc, 0)) {
    failed = 1;
    mbar_wait(&bar_acc, 0);
  }
  tc_fence_after();
  __syncthreads();
  if (failed) {
    if (threadIdx.x == 0) {
      atomicOr(g.err, 1);
      // TMA loads issued but never consumed: let them land (bounded) before exit
      for (int kb = consumed_kb + 1; kb <= issued_kb; kb++)
        mbar_wait(&bar_full[kb % NSTAGE], (kb / NSTAGE) & 1);
    }
  } else {
    // epilogue, 12 warps: warp w reads TMEM lanes 32 (w % 4) .. +31 (rows of
    // this M tile) and the 16-column chunks part, part + 3, ... (part = w / 4)
    const int quarter = warp & 3, part = warp >> 2;
    const int row = mt * MT + quarter * 32 + lane;
    const uint32_t lane_addr = tbase + ((uint32_t)(quarter * 32) << 16);
    const int kk = item / g.nc, cc = item % g.nc;
    // accumulators carry 2^-30 sigma_i tau_j; the int64 sum is in units of 2^-16
    const int erow = row < g.n ? g.sigma[(long long)item * (g.mtiles * MT) + row] - g.eoff : 0;
    double *pc = (double *)mat_ptr(g.C, kk, cc);
    double *pd = (double *)mat_ptr(g.D, kk, cc);
    double *pe = (double *)mat_ptr(g.E, kk, cc);
    constexpr int NL = nlevels<NA>(S);
    // modes that read the old C (1, 5) or D (2, 3) load the chunk's eight
    // elements of it first, so that the loads are in flight together
    const bool rd_c = g.mode == 1 || g.mode == 5, rd_d = g.mode == 2 || g.mode == 3;
    const double2 *src = (const double2 *)(rd_c ? pc : pd);
    const long long sld = rd_c ? g.C.ld : g.D.ld;
#pragma unroll 1
    for (int c0 = part * 16; c0 < TN; c0 += 3 * 16) {
      uint32_t v[NA][16];
#pragma unroll
      for (int l = 0; l < NL; l++) tmem_ld16(lane_addr + l * TN + c0, v[l]);
      // (the seven-accumulator tile has no registers to spare for it)
      constexpr bool PF = NA <= 5;
      double2 old[PF ? 8 : 1];
      if (PF && row < g.n && (rd_c || rd_d)) {
#pragma unroll
        for (int t = 0; t < 16; t += 2) {
          const int j = (nt * TN + c0 + t) >> 1;
          if (j < g.n) old[PF ? t >> 1 : 0] = src[row + (long long)j * sld];
        }
      }
      tmem_ld_wait();
      if (row >= g.n) continue;
#pragma unroll
      for (int t = 0; t < 16; t += 2) {  // accumulator columns 2j, 2j+1 = Re, Im of column j
        const int j = (nt * TN + c0 + t) >> 1;
        if (j < g.n) {
          long long ar = 0, ai = 0;
#pragma unroll
          for (int l = 0; l < NL; l++) {
            // exact levels by conversion and shift; the shared tail bitwise
            const float vr = __uint_as_float(v[l][t]), vi = __uint_as_float(v[l][t + 1]);
            ar += (l < NA - 1 && l <= 3) ? level_fix16(vr, l, g.db) : f2fix16(vr);
            ai += (l < NA - 1 && l <= 3) ? level_fix16(vi, l, g.db) : f2fix16(vi);
          }
          const int e = erow + col_exp[(c0 + t) >> 1];
          const double2 val = make_double2(fix_to_double(ar, e), fix_to_double(ai, e));
          double2 *oc = (double2 *)pc + row + (long long)j * g.C.ld;
          double2 *od = (double2 *)pd + row + (long long)j * g.D.ld;
          const int q = t >> 1;
          double2 o = make_double2(0.0, 0.0);  // the old C or D of this element
          if constexpr (PF) {
            o = old[q];
          } else {
            if (g.mode == 1 || g.mode == 5) o = *oc;
            if (g.mode == 2 || g.mode == 3) o = *od;
          }
          if (g.mode == 0) {
            *oc = val;
          } else if (g.mode == 1) {
            *oc = make_double2(o.x - val.x, o.y - val.y);
          } else if (g.mode == 2) {
            double2 *oe = (double2 *)pe + row + (long long)j * g.E.ld;
            const double2 x = *oe;
            *od = make_double2(o.x - val.x, o.y - val.y);
            *oe = make_double2(x.x - val.x, x.y - val.y);
          } else if (g.mode == 3) {
            *oc = make_double2(o.x - val.x, o.y - val.y);
          } else if (g.mode == 4) {
            *oc = make_double2((row == j ? 1.0 : 0.0) - val.x, -val.y);
          } else {
            *oc = make_double2(o.x + val.x, o.y + val.y);
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
// Gauss-Jordan with column pivoting (main/gjinv.f: in row i the pivot is the
// largest |a(i, j)| over the columns not yet used, first index on ties) in
// complex FP32, the matrix held in registers: TY*16 threads as a TY x 16
// grid, thread (ty, tx) owning rows ty + TY a (a < RA) and columns
// tx + 16 b (b < RB); the 16 threads of one ty are one half warp.
//
// The pivot columns are not swapped into place: step i eliminates with the
// pivot (i, kp) where it lies and records sigma(i) = kp, which is Gauss-Jordan
// on A P (P the column permutation); the array then holds (A P)^-1 with its
// columns stored at the positions of A P's, so A^-1(sigma(r), c) is found at
// (r, sigma(c)) and the store permutes both indices.  With
//   c_r = a(r,kp)/piv (r != i), c_i = -1/piv,   p_j = a(i,j) (j != kp), p_kp = 1
// and row i and column kp masked to zero first, every element takes the same
// update a(r,j) <- s(r,j) a(r,j) - c_r p_j (s = 0 on row i and column kp,
// else 1): the rank-1 update, the scaled pivot row a(i,j)/piv, the pivot
// column -a(r,kp)/piv and the pivot 1/piv, as packed FP32x2 multiply-adds.
// a(r,kp) comes from the owner in the same half warp (a shuffle); the pivot
// row and the next pivot index are staged in shared memory (double-buffered)
// by the 16 threads that own row i+1 after their update: one block barrier
// per step.  The result
// (written as FP64) only seeds the Newton refinement.

__device__ __forceinline__ unsigned long long pk2(float x, float y) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
  return r;
}
__device__ __forceinline__ float2 upk2(unsigned long long r) {
  float2 v;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
  return v;
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b,
                                                   unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ unsigned long long mul2(unsigned long long a, unsigned long long b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// Pivot of row `row` among the unused columns (the row's owners: one half
// warp): the largest |a(row, j)|^2, first index on ties; the row is staged
// into `rowbuf` on the way.  Every candidate NaN: the first unused column.
template <int TY, int RA, int RB>
__device__ __forceinline__ void gj_search(const unsigned long long (&m)[RA][RB], int row, unsigned used, int tx,
                                          unsigned hmask, float2 *rowbuf, int *kp_out) {
  const int iar = row / TY;
  float best = -1.f;
  int bj = 0x7FFFFFFF, fu = 0x7FFFFFFF;
#pragma unroll
  for (int ib = 0; ib < RB; ib++) {
    unsigned long long w = m[0][ib];
#pragma unroll
    for (int ia = 1; ia < RA; ia++) w = (ia == iar) ? m[ia][ib] : w;  // static indices keep m in registers
    const float2 v = upk2(w);
    const int j = tx + 16 * ib;
    rowbuf[j] = v;
    const bool free = !((used >> ib) & 1u);
    const float mm = v.x * v.x + v.y * v.y;
    const bool ok = free && (mm > best || (mm == best && j < bj));
    best = ok ? mm : best;
    bj = ok ? j : bj;
    fu = (free && j < fu) ? j : fu;
  }
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) {
    const float ob = __shfl_xor_sync(hmask, best, o, 16);
    const int oj = __shfl_xor_sync(hmask, bj, o, 16);
    const int of = __shfl_xor_sync(hmask, fu, o, 16);
    const bool take = ob > best || (ob == best && oj < bj);
    best = take ? ob : best;
    bj = take ? oj : bj;
    fu = of < fu ? of : fu;
  }
  if (bj == 0x7FFFFFFF) bj = fu;
  if (tx == 0) *kp_out = bj;
}

// MINB: blocks per SM the register allocation must allow (the 64-row
// layouts run several matrices per SM, each block's barrier latency hidden by
// the others)
template <int TY, int RA, int RB, int MINB = 1>
__global__ void __launch_bounds__(TY * 16, MINB) k_cgj32(MatRef A, MatRef X, int n, int nc,
                                                      const int *__restrict__ act) {
  constexpr int NR = TY * RA, NCOL = 16 * RB;
  const int item = blockIdx.x, kk = item / nc, cc = item % nc;
  if (act && !act[item]) return;
  __shared__ float2 rowi[2][NCOL];
  __shared__ int sig[NR], sinv[NCOL];
  __shared__ int kpn[2];
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  const zd *a = mat_ptr(A, kk, cc);
  unsigned long long m[RA][RB];  // (re, im) pairs
#pragma unroll
  for (int ia = 0; ia < RA; ia++)
#pragma unroll
    for (int ib = 0; ib < RB; ib++) {
      const int r = ty + TY * ia, j = tx + 16 * ib;
      float2 v = make_float2(0.f, 0.f);
      if (r < n && j < n) {
        const zd w = a[r + (long long)j * A.ld];
        v = make_float2((float)w.x, (float)w.y);
      }
      m[ia][ib] = pk2(v.x, v.y);
    }
  // columns j >= n never pivot
  unsigned used = 0;
#pragma unroll
  for (int ib = 0; ib < RB; ib++)
    if (tx + 16 * ib >= n) used |= 1u << ib;
  const unsigned hmask = (ty & 1) ? 0xFFFF0000u : 0x0000FFFFu;  // the 16 threads of this ty

  if (ty == 0) gj_search<TY, RA, RB>(m, 0, used, tx, hmask, rowi[0], &kpn[0]);
  __syncthreads();
  for (int i = 0; i < n; i++) {
    const int kp = kpn[i & 1], kb = kp >> 4, kt = kp & 15;
    if (tid == 0) {
      sig[i] = kp;
      sinv[kp] = i;
    }
    if (tx == kt) used |= 1u << kb;
    const float2 *ri = rowi[i & 1];
    const float2 piv = ri[kp];
    const float rden = __frcp_rn(piv.x * piv.x + piv.y * piv.y);
    const float2 q = make_float2(piv.x * rden, -piv.y * rden);
    // multipliers c_r as the pairs (-Re c, -Re c) and (Im c, Im c); row mask
    unsigned long long ncx[RA], cy[RA];
    float f[RA];
#pragma unroll
    for (int ia = 0; ia < RA; ia++) {
      unsigned long long w = m[ia][0];
#pragma unroll
      for (int ib = 1; ib < RB; ib++) w = (ib == kb) ? m[ia][ib] : w;
      w = __shfl_sync(0xFFFFFFFFu, w, kt, 16);  // a(r, kp) from its owner in this half warp
      const float2 v = upk2(w);
      const bool isrow = ty + TY * ia == i;
      const float2 cr = isrow ? make_float2(-q.x, -q.y)
                              : make_float2(v.x * q.x - v.y * q.y, v.x * q.y + v.y * q.x);
      ncx[ia] = pk2(-cr.x, -cr.x);
      cy[ia] = pk2(cr.y, cr.y);
      f[ia] = isrow ? 0.f : 1.f;
    }
    // row i+1's owners reduce the next pivot after their update
    const bool srch = i + 1 < n && ty == ((i + 1) % TY);
#pragma unroll
    for (int ib = 0; ib < RB; ib++) {
      const int j = tx + 16 * ib;
      const bool iscol = j == kp;
      const float2 p = iscol ? make_float2(1.f, 0.f) : ri[j];
      const float g = iscol ? 0.f : 1.f;
      const unsigned long long pp = pk2(p.x, p.y), ps = pk2(p.y, -p.x);
#pragma unroll
      for (int ia = 0; ia < RA; ia++) {
        const float sm = f[ia] * g;
        const unsigned long long t = fma2(cy[ia], ps, mul2(ncx[ia], pp));
        m[ia][ib] = fma2(m[ia][ib], pk2(sm, sm), t);
      }
    }
    if (srch) gj_search<TY, RA, RB>(m, i + 1, used, tx, hmask, rowi[(i + 1) & 1], &kpn[(i + 1) & 1]);
    __syncthreads();
  }
  // storage (r, j) holds A^-1(sigma(r), sigma^-1(j))
  zd *x = mat_ptr(X, kk, cc);
#pragma unroll
  for (int ia = 0; ia < RA; ia++)
#pragma unroll
    for (int ib = 0; ib < RB; ib++) {
      const int r = ty + TY * ia, j = tx + 16 * ib;
      if (r < n && j < n) {
        const float2 v = upk2(m[ia][ib]);
        x[sig[r] + (long long)sinv[j] * X.ld] = make_double2((double)v.x, (double)v.y);
      }
    }
}

// ------------------------------------------------------------------ FP32 block products
// C = A B (m x n, depth k; m, n, k <= 64) of one item per block in complex
// FP32 from FP64 operands, for the 2 x 2 block start of the split-precision
// inverse: mode 0 C = AB, 1 C = D - AB (D read in FP64), 2 C = -AB.  Up to
// two independent products per launch (blockIdx.y picks one).  The 16 x 16
// threads each hold 4 x 4 outputs (rows ty + 16 i, columns tx + 16 j) as two
// packed FP32 pairs each (two fma.rn.f32x2 per complex multiply-add); the
// operands pass through shared memory in K chunks of 32, converted to FP32
// on the way; the sums run in a fixed order.
struct G32Job {
  MatRef A, B, C, D;
  int m, n, k, mode;
};
struct G32Jobs {
  G32Job j[2];
};

__global__ void __launch_bounds__(256, 2) k_cgemm32(G32Jobs jobs, int nc, const int *__restrict__ act) {
  const int item = blockIdx.x, kk = item / nc, cc = item % nc;
  if (act && !act[item]) return;
  const G32Job &J = jobs.j[blockIdx.y];
  const int m = J.m, n = J.n, k = J.k;
  __shared__ float2 As[32][64];  // [K index][row]
  __shared__ float2 Bs[32][65];  // [K index][column], padded against store conflicts
  const zd *a = mat_ptr(J.A, kk, cc), *b = mat_ptr(J.B, kk, cc);
  const int lda = J.A.ld, ldb = J.B.ld;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  // packed FP32 pairs: pr = (sum ar br, sum ar bi), pi = (sum ai br, sum ai bi)
  // on the (br, bi) pair as it sits in shared memory; the product is
  // (pr.x - pi.y, pr.y + pi.x)
  unsigned long long pr[4][4], pi[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) pr[i][j] = pi[i][j] = 0ull;
  for (int k0 = 0; k0 < k; k0 += 32) {
    for (int e = threadIdx.x; e < 64 * 32; e += 256) {
      const int r = e & 63, q = e >> 6, col = k0 + q;
      const zd v = (r < m && col < k) ? a[r + (long long)col * lda] : make_double2(0.0, 0.0);
      As[q][r] = make_float2((float)v.x, (float)v.y);
    }
    for (int e = threadIdx.x; e < 32 * 64; e += 256) {
      const int q = e & 31, c = e >> 5, row = k0 + q;
      const zd v = (row < k && c < n) ? b[row + (long long)c * ldb] : make_double2(0.0, 0.0);
      Bs[q][c] = make_float2((float)v.x, (float)v.y);
    }
    __syncthreads();
#pragma unroll 4
    for (int q = 0; q < 32; q++) {
      unsigned long long bv[4];
#pragma unroll
      for (int j = 0; j < 4; j++) bv[j] = *reinterpret_cast<const unsigned long long *>(&Bs[q][tx + 16 * j]);
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const float2 a = As[q][ty + 16 * i];
        const unsigned long long ar = pk2(a.x, a.x), ai = pk2(a.y, a.y);
#pragma unroll
        for (int j = 0; j < 4; j++) {
          pr[i][j] = fma2(ar, bv[j], pr[i][j]);
          pi[i][j] = fma2(ai, bv[j], pi[i][j]);
        }
      }
    }
    __syncthreads();
  }
  zd *c = mat_ptr(J.C, kk, cc);
  const int ldc = J.C.ld, mode = J.mode;
  const zd *d = mode == 1 ? mat_ptr(J.D, kk, cc) : nullptr;
  const int ldd = J.D.ld;
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int r = ty + 16 * i, col = tx + 16 * j;
      if (r < m && col < n) {
        const float2 u = upk2(pr[i][j]), v = upk2(pi[i][j]);
        const zd p = make_double2((double)(u.x - v.y), (double)(u.y + v.x));
        zd o;
        if (mode == 0) o = p;
        else if (mode == 1) {
          const zd dv = d[r + (long long)col * ldd];
          o = make_double2(dv.x - p.x, dv.y - p.y);
        } else o = make_double2(-p.x, -p.y);
        c[r + (long long)col * ldc] = o;
      }
    }
}

static G32Job g32(int mode, const MatRef &A, const MatRef &B, const MatRef &C, const MatRef &D, int m, int n,
                  int k) {
  G32Job j;
  j.A = A;
  j.B = B;
  j.C = C;
  j.D = D;
  j.m = m;
  j.n = n;
  j.k = k;
  j.mode = mode;
  return j;
}

// one or two products per launch
static void cgemm32(const G32Job &j0, const G32Job *j1, int nc, const int *act, unsigned items, cudaStream_t st) {
  G32Jobs js;
  js.j[0] = j0;
  js.j[1] = j1 ? *j1 : j0;
  k_cgemm32<<<dim3(items, j1 ? 2 : 1), 256, 0, st>>>(js, nc, act);
  SKKR_LAUNCHED();
}

// ------------------------------------------------------------------ host side

// resolved once per process (thread-safe static initialisation: contexts may
// run from several host threads)
static PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
    cudaDriverEntryPointQueryResult q;
    void *p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    return (PFN_cuTensorMapEncodeTiled_v12000)p;
  }();
  return fn;
}
int get_encoder() { return encoder() ? 0 : -1; }

// tiled staging: dims {32, rows, regions * kblocks}; one box = one contiguous block
int make_map(CUtensorMap *m, void *base, int rows, long long depth, int boxrows) {
  cuuint64_t dims[3] = {(cuuint64_t)KB, (cuuint64_t)rows, (cuuint64_t)depth};
  cuuint64_t strides[2] = {(cuuint64_t)KB * 2, (cuuint64_t)KB * 2 * rows};
  cuuint32_t box[3] = {(cuuint32_t)KB, (cuuint32_t)boxrows, 1};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = encoder()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : -1;
}

// at least 120 KB so that only one CTA (and one 512-column TMEM allocation)
// is resident per SM
size_t oz_smem_bytes(int S, int TN) {
  size_t b = (size_t)oz_stages(S, TN) * S * (MT * KB * 2 + TN * KB * 2) + 1024;
  return b < 120 * 1024 ? 120 * 1024 : b;
}

}  // namespace

// ---------------------------------------------------------------------------
// Split operands live in staging slots (MIXED_SLOTS per side) so that an
// operand used by several products is split once.  A slot records the layout
// its zero padding was made for and the slices / digit base of its contents.
struct Stage {
  void *p = nullptr;       // [item][S][kblocks][rows][32] bf16 slices
  size_t cap = 0;
  int *scale = nullptr;    // row (A) / column (B) scale exponents
  size_t scap = 0;
  int n = -1, K = -1;      // padding layout of p
  int tn = 0;              // N tile the B layout is padded to
  int S = 0, DB = 0;       // the operand held: slices, digit base, dims, items
  int cn = -1, cK = -1;
  long long items = 0;
  bool fused = false;      // B only: not split; each product forms its tiles from src
  MatRef src;
};

struct MixedWork {
  Stage A[MIXED_SLOTS], B[MIXED_SLOTS];
  zd *acopy = nullptr, *rbuf = nullptr;
  size_t ac_cap = 0, rb_cap = 0;
  double *rnorm = nullptr;
  size_t rn_cap = 0;
  int *err = nullptr;
  unsigned long long *dmax = nullptr;  // running max of accepted Newton residual norms (double bits)
  unsigned long long *nfb = nullptr;   // inverses redone in FP64 (residual above the limit)
  int *flag = nullptr;                 // per-item FP64 fallback mask
  size_t flag_cap = 0;
  int *mark = nullptr;                 // per-item mask of the further Newton steps
  size_t mark_cap = 0;
  int *cnt = nullptr;                  // count of marked items (device scalar)
  unsigned long long *nref = nullptr;  // [0] inverses that took further Newton steps, [1] kernels run by the
                                       // IF bodies of captured further steps (device counts)
  cudaStream_t side = nullptr;         // captures the bodies of conditional graph nodes
  int smem_set[64] = {0};
  bool precise = false;    // (64, 7) tile: exact levels 0..5 (mixed_set_precise)
  bool fuse_b = true;      // B operands formed inside the product (mixed_set_fused)
  bool blocked = true;     // 2 x 2 block start of inverses above 64 rows (mixed_set_blocked)
};

void mixed_set_precise(MixedWork *w, bool on) { w->precise = on; }
void mixed_set_blocked(MixedWork *w, bool on) { w->blocked = on; }
void mixed_set_fused(MixedWork *w, bool on) { w->fuse_b = on; }

// the (64, 7) tile serves products of 6 slices and more (the low-slice
// Newton corrections keep the default tile); split and multiply agree on it
static bool use_precise(const MixedWork *w, int S) { return w->precise && S >= 6; }

// the callers' streams are non-blocking: free the old buffer only once the
// device is idle (cudaFree does not wait for those streams)
static int grow(void **p, size_t *cap, size_t bytes, bool zero) {
  if (bytes <= *cap) return 0;
  std::lock_guard<std::recursive_mutex> lk(skkr_device_mutex());
  if (*p) {
    cudaDeviceSynchronize();
    cudaFree(*p);
  }
  *p = nullptr;
  *cap = 0;
  if (cudaMalloc(p, bytes) != cudaSuccess) return SKKR_ERR_NOMEM;
  // cudaMemset runs on the legacy default stream, which the non-blocking
  // streams do not wait for: finish it before the buffer is used
  if (zero && (cudaMemset(*p, 0, bytes) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess))
    return SKKR_ERR_NOMEM;
  *cap = bytes;
  return 0;
}

MixedWork *mixed_create() {
  std::lock_guard<std::recursive_mutex> lk(skkr_device_mutex());
  MixedWork *w = new MixedWork();
  if (cudaMalloc(&w->err, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&w->dmax, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&w->nfb, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&w->cnt, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&w->nref, 2 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaStreamCreateWithFlags(&w->side, cudaStreamNonBlocking) != cudaSuccess) {
    void *ps[] = {w->err, w->dmax, w->nfb, w->cnt, w->nref};
    for (void *p : ps)
      if (p) cudaFree(p);
    delete w;
    return nullptr;
  }
  cudaMemset(w->err, 0, sizeof(int));
  cudaMemset(w->dmax, 0, sizeof(unsigned long long));
  cudaMemset(w->nfb, 0, sizeof(unsigned long long));
  cudaMemset(w->nref, 0, 2 * sizeof(unsigned long long));
  cudaDeviceSynchronize();  // default-stream memsets, before the non-blocking streams use the flags
  return w;
}

int mixed_resid_reset(MixedWork *w, cudaStream_t st) {
  return (cudaMemsetAsync(w->dmax, 0, sizeof(unsigned long long), st) == cudaSuccess &&
          cudaMemsetAsync(w->nfb, 0, sizeof(unsigned long long), st) == cudaSuccess &&
          cudaMemsetAsync(w->nref, 0, 2 * sizeof(unsigned long long), st) == cudaSuccess)
             ? 0
             : SKKR_ERR_CUDA;
}

int mixed_resid_read(MixedWork *w, double *out, long long *fallbacks, long long *refined, cudaStream_t st) {
  unsigned long long h[3] = {0, 0, 0};
  if (cudaMemcpyAsync(&h[0], w->dmax, sizeof(h[0]), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(&h[1], w->nfb, sizeof(h[1]), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(&h[2], w->nref, sizeof(h[2]), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return SKKR_ERR_CUDA;
  double v;
  memcpy(&v, &h[0], sizeof(v));
  *out = v;
  if (fallbacks) *fallbacks = (long long)h[1];
  if (refined) *refined = (long long)h[2];
  return 0;
}

int *mixed_error_ptr(MixedWork *w) { return w->err; }

long long mixed_graph_kernels(MixedWork *w, cudaStream_t st) {
  unsigned long long h = 0;
  if (cudaMemcpyAsync(&h, w->nref + 1, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return 0;
  return (long long)h;
}

void mixed_destroy(MixedWork *w) {
  if (!w) return;
  std::lock_guard<std::recursive_mutex> lk(skkr_device_mutex());
  cudaDeviceSynchronize();
  for (int i = 0; i < MIXED_SLOTS; i++) {
    void *q[] = {w->A[i].p, w->A[i].scale, w->B[i].p, w->B[i].scale};
    for (void *p : q)
      if (p) cudaFree(p);
  }
  void *ps[] = {w->acopy, w->rbuf, w->rnorm, w->err, w->dmax, w->nfb, w->flag, w->mark, w->cnt, w->nref};
  for (void *p : ps)
    if (p) cudaFree(p);
  if (w->side) cudaStreamDestroy(w->side);
  delete w;
}

int mixed_error_flag(MixedWork *w) {
  int h = 0;
  if (cudaMemcpy(&h, w->err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  return h;
}

// dims of the staged real problem for complex n x K times K x n, N tile tn
static void oz_dims(int n, int K, int tn, int *Mp, int *Np, int *Kp, int *mtiles, int *ntiles, int *kblocks) {
  *mtiles = (n + MT - 1) / MT;
  *Mp = *mtiles * MT;
  *ntiles = (2 * n + tn - 1) / tn;
  *Np = *ntiles * tn;
  *kblocks = (2 * K + KB - 1) / KB;
  *Kp = *kblocks * KB;
}

// digit base for depth K: 8 bits while 2K <= 256 (8 slices then act as 7:
// the fixed-point value is limited to 62 bits), 7 bits above so that the FP32
// level sums stay exact integers
static void oz_digits(int S, int K, int *Se, int *DB) {
  *DB = K <= 128 ? 8 : 7;
  *Se = (*DB == 8 && S > 7) ? 7 : S;
}

// B operands of the default tile are fused into the product unless turned off
static bool fuses_b(const MixedWork *w, int S) { return w->fuse_b && !use_precise(w, S); }

// side 1 with fuses_b: the slot only records B (the product reads it when it
// runs: B must not change in between, which every caller keeps); `real`
// (an operand several products read) splits it all the same
template <int S, int DB>
static int split_s(MixedWork *w, int side, int slot, const MatRef &M, int n, int K, int nk, int nc,
                   const int *act, cudaStream_t st, bool real = false) {
  int Mp, Np, Kp, mtiles, ntiles, kblocks;
  const int tn = use_precise(w, S) ? 64 : NT;
  oz_dims(n, K, tn, &Mp, &Np, &Kp, &mtiles, &ntiles, &kblocks);
  const long long items = (long long)nk * nc;
  Stage &sg = side == 0 ? w->A[slot] : w->B[slot];
  sg.S = S;
  sg.DB = DB;
  sg.cn = n;
  sg.cK = K;
  sg.items = items;
  sg.fused = side == 1 && !real && fuses_b(w, S);
  if (sg.fused) {
    sg.src = M;
    return 0;
  }
  const int rows = side == 0 ? Mp : Np;
  int rc;
  // a buffer cannot be reallocated inside a captured graph: the eager run
  // before any capture sizes every slot (mixed_zinv reserves its further steps')
  if ((size_t)items * S * rows * Kp * 2 > sg.cap && stream_capturing(st)) return SKKR_ERR_CUDA;
  if ((rc = grow(&sg.p, &sg.cap, (size_t)items * S * rows * Kp * 2, true))) return rc;
  if ((rc = grow((void **)&sg.scale, &sg.scap, (size_t)items * (side == 0 ? Mp : n) * sizeof(int), false)))
    return rc;
  if (sg.n != n || sg.K != K || (side == 1 && sg.tn != tn)) {
    // padding (rows beyond the operand, K' places of complex indices >= K)
    // must be zero; a new layout clears what an earlier one wrote there
    if (cudaMemsetAsync(sg.p, 0, sg.cap, st) != cudaSuccess) return SKKR_ERR_CUDA;
    sg.n = n;
    sg.K = K;
  }
  sg.tn = side == 1 ? tn : 0;
  const long long active_s = act ? skkr_active_items(items) : items;
  // split traffic: FP64 operand read + S bf16 slices of the real embedding written
  const double split_bytes = (double)active_s * n * K * (16.0 + S * 2.0 * 2.0);
  if (side == 0) {
    dim3 ga((n + 31) / 32, items);
    kstat_begin(KS_OTHER, split_bytes, st);
    k_split_a<S, DB><<<ga, 256, 0, st>>>(M, n, K, nc, act, (__nv_bfloat16 *)sg.p, Mp, Kp, sg.scale);
  } else {
    dim3 gb((n + 7) / 8, items);
    kstat_begin(KS_OTHER, 2.0 * split_bytes, st);
    k_split_b<S, DB><<<gb, 256, 0, st>>>(M, n, K, nc, act, (__nv_bfloat16 *)sg.p, Np, Kp, sg.scale);
  }
  kstat_end(st);
  SKKR_LAUNCHED();
  return 0;
}

template <int S, int TN, int NA, int FB>
static int oz_launch(MixedWork *w, int key, dim3 grid, const CUtensorMap &ma, const CUtensorMap &mb,
                     const OzArgs &g, cudaStream_t st) {
  const size_t smem = oz_smem_bytes(S, TN);
  if (!w->smem_set[key]) {
    if (cudaFuncSetAttribute(k_ozaki<S, TN, NA, FB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
        cudaSuccess)
      return SKKR_ERR_CUDA;
    w->smem_set[key] = 1;
  }
  k_ozaki<S, TN, NA, FB><<<grid, OZ_THREADS, smem, st>>>(ma, mb, g);
  return 0;
}

template <int S, int TN, int NA>
static int gemm_s(MixedWork *w, int mode, int sa, int sb, const MatRef &C, const MatRef &D, const MatRef &E,
                  int n, int K, int nk, int nc, const int *act, cudaStream_t st) {
  if (get_encoder()) return SKKR_ERR_CUDA;
  int Mp, Np, Kp, mtiles, ntiles, kblocks;
  oz_dims(n, K, TN, &Mp, &Np, &Kp, &mtiles, &ntiles, &kblocks);
  const long long items = (long long)nk * nc;
  const Stage &A = w->A[sa];
  Stage &B = w->B[sb];
  if (A.fused || A.S != S || B.S != S || A.DB != B.DB || A.cn != n || B.cn != n || A.cK != K || B.cK != K ||
      A.items != items || B.items != items || (!B.fused && B.tn != TN))
    return SKKR_ERR_ARG;  // the slots do not hold splits of this product's operands
  // a fused B that the product writes over (C, D or E) is split first, so
  // that no CTA reads an element another one has already replaced
  if (B.fused && (mref_overlap(B.src, C, nk, nc, n) || mref_overlap(B.src, D, nk, nc, n) ||
                  mref_overlap(B.src, E, nk, nc, n))) {
    int rc;
    if constexpr (S <= 7)
      rc = A.DB == 8 ? split_s<S, 8>(w, 1, sb, B.src, n, K, nk, nc, act, st, true)
                     : split_s<S, 7>(w, 1, sb, B.src, n, K, nk, nc, act, st, true);
    else
      rc = split_s<S, 7>(w, 1, sb, B.src, n, K, nk, nc, act, st, true);
    if (rc) return rc;
  }
  CUtensorMap ma, mb;
  if (make_map(&ma, A.p, Mp, items * S * kblocks, MT)) return SKKR_ERR_CUDA;
  if (B.fused) {
    mb = ma;  // unused by the fused kernel
  } else if (make_map(&mb, B.p, Np, items * S * kblocks, TN)) {
    return SKKR_ERR_CUDA;
  }
  OzArgs g;
  g.n = n;
  g.mtiles = mtiles;
  g.ntiles = ntiles;
  g.kblocks = kblocks;
  g.nc = nc;
  g.mode = mode;
  g.eoff = 32 + 2 * (A.DB - 1);
  g.db = A.DB;
  g.sigma = A.scale;
  g.tau = B.scale;
  g.B = B.src;
  g.K = K;
  g.C = C;
  g.D = D;
  g.E = E;
  g.act = act;
  g.err = w->err;
  const long long active = act ? skkr_active_items(items) : items;
  // algorithmic BF16 tensor work: S(S+1)/2 real products of n x 2K x 2n per item
  // FP64-equivalent: one complex n x K by K x n product per item
  kstat_begin2(KS_OZAKI, (double)(S * (S + 1) / 2) * 8.0 * n * (double)n * K * (double)active,
               8.0 * n * (double)n * K * (double)active, st);
  dim3 grid(mtiles * ntiles, items);
  // shared-memory attribute keys: S + 16 x (0 staged, 1 exact-level tile, 2 / 3 fused B at 8 / 7 digit bits)
  int rc;
  if (!B.fused) {
    rc = oz_launch<S, TN, NA, 0>(w, S + (TN == NT ? 0 : 16), grid, ma, mb, g, st);
  } else if constexpr (TN == NT && NA == NACC) {
    if (A.DB == 8) {
      if constexpr (S <= 7) rc = oz_launch<S, TN, NA, 8>(w, S + 32, grid, ma, mb, g, st);
      else rc = SKKR_ERR_ARG;
    } else {
      rc = oz_launch<S, TN, NA, 7>(w, S + 48, grid, ma, mb, g, st);
    }
  } else {
    rc = SKKR_ERR_ARG;  // fused B only on the default tile
  }
  kstat_end(st);
  if (rc) return rc;
  SKKR_LAUNCHED();
  return 0;
}

int mixed_split(MixedWork *w, int side, int slot, int S, const MatRef &M, int n, int K, int nk, int nc,
                const int *act, cudaStream_t st, bool reused) {
  if (n < 1 || n > 256 || K < 1 || K > 256 || nk * (long long)nc > 65535 || slot < 0 ||
      slot >= MIXED_SLOTS || (side != 0 && side != 1))
    return SKKR_ERR_ARG;
  int Se, DB;
  oz_digits(S, K, &Se, &DB);
  if (DB == 8) {
    switch (Se) {
      case 3: return split_s<3, 8>(w, side, slot, M, n, K, nk, nc, act, st, reused);
      case 4: return split_s<4, 8>(w, side, slot, M, n, K, nk, nc, act, st, reused);
      case 5: return split_s<5, 8>(w, side, slot, M, n, K, nk, nc, act, st, reused);
      case 6: return split_s<6, 8>(w, side, slot, M, n, K, nk, nc, act, st, reused);
      case 7: return split_s<7, 8>(w, side, slot, M, n, K, nk, nc, act, st, reused);
      default: return SKKR_ERR_ARG;
    }
  }
  switch (Se) {
    case 3: return split_s<3, 7>(w, side, slot, M, n, K, nk, nc, act, st, reused);
    case 4: return split_s<4, 7>(w, side, slot, M, n, K, nk, nc, act, st, reused);
    case 5: return split_s<5, 7>(w, side, slot, M, n, K, nk, nc, act, st, reused);
    case 6: return split_s<6, 7>(w, side, slot, M, n, K, nk, nc, act, st, reused);
    case 7: return split_s<7, 7>(w, side, slot, M, n, K, nk, nc, act, st, reused);
    case 8: return split_s<8, 7>(w, side, slot, M, n, K, nk, nc, act, st, reused);
    default: return SKKR_ERR_ARG;
  }
}

int mixed_gemm_staged(MixedWork *w, int mode, int S, int sa, int sb, const MatRef &C, const MatRef &D,
                      const MatRef &E, int n, int K, int nk, int nc, const int *act, cudaStream_t st) {
  if (sa < 0 || sa >= MIXED_SLOTS || sb < 0 || sb >= MIXED_SLOTS) return SKKR_ERR_ARG;
  int Se, DB;
  oz_digits(S, K, &Se, &DB);
  if (use_precise(w, Se)) {
    switch (Se) {  // 64-column tiles, levels 0..5 in their own accumulators
      case 6: return gemm_s<6, 64, 7>(w, mode, sa, sb, C, D, E, n, K, nk, nc, act, st);
      case 7: return gemm_s<7, 64, 7>(w, mode, sa, sb, C, D, E, n, K, nk, nc, act, st);
      case 8: return gemm_s<8, 64, 7>(w, mode, sa, sb, C, D, E, n, K, nk, nc, act, st);
      default: return SKKR_ERR_ARG;
    }
  }
  switch (Se) {
    case 3: return gemm_s<3, NT, NACC>(w, mode, sa, sb, C, D, E, n, K, nk, nc, act, st);
    case 4: return gemm_s<4, NT, NACC>(w, mode, sa, sb, C, D, E, n, K, nk, nc, act, st);
    case 5: return gemm_s<5, NT, NACC>(w, mode, sa, sb, C, D, E, n, K, nk, nc, act, st);
    case 6: return gemm_s<6, NT, NACC>(w, mode, sa, sb, C, D, E, n, K, nk, nc, act, st);
    case 7: return gemm_s<7, NT, NACC>(w, mode, sa, sb, C, D, E, n, K, nk, nc, act, st);
    case 8: return gemm_s<8, NT, NACC>(w, mode, sa, sb, C, D, E, n, K, nk, nc, act, st);
    default: return SKKR_ERR_ARG;
  }
}

int mixed_zgemm_k(MixedWork *w, int mode, int S, const MatRef &A, const MatRef &B, const MatRef &C,
                  const MatRef &D, const MatRef &E, int n, int K, int nk, int nc, const int *act,
                  cudaStream_t st) {
  int rc = mixed_split(w, 0, 0, S, A, n, K, nk, nc, act, st);
  if (!rc) rc = mixed_split(w, 1, 0, S, B, n, K, nk, nc, act, st);
  if (!rc) rc = mixed_gemm_staged(w, mode, S, 0, 0, C, D, E, n, K, nk, nc, act, st);
  return rc;
}

int mixed_zgemm(MixedWork *w, int mode, int S, const MatRef &A, const MatRef &B, const MatRef &C,
                const MatRef &D, const MatRef &E, int n, int nk, int nc, const int *act, cudaStream_t st) {
  return mixed_zgemm_k(w, mode, S, A, B, C, D, E, n, n, nk, nc, act, st);
}

// Newton residual check per item: an item whose last residual norm
// |I - A X|_F is above `limit` (or not finite) is marked for an FP64
// Gauss-Jordan redo; the others fold their norm into the running maximum
// (non-negative doubles order like their bit patterns: integer atomicMax)
__global__ void k_newton_check(const double *__restrict__ rn, const int *__restrict__ act, int items,
                               double limit, int *__restrict__ flag, unsigned long long *dmax,
                               unsigned long long *nfb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= items) return;
  const int a = act ? act[i] : 1;
  const double r = rn[i];
  const int f = a && !(r <= limit);
  flag[i] = f;
  if (f) atomicAdd(nfb, 1ull);
  else if (a) atomicMax(dmax, (unsigned long long)__double_as_longlong(r));
}

// Items whose residual is above `limit` but below `basin` (Newton's
// quadratic regime) are marked for a further step.  One block: the count of
// marked items goes to *count (eager runs read it on the host), is added to
// *nref on the first further step, and, inside a captured graph, decides the
// IF node of the step (cudaGraphSetConditional).
__global__ void __launch_bounds__(1024) k_newton_select(const double *__restrict__ rn, const int *__restrict__ act,
                                                        int items, double limit, double basin, int *__restrict__ mark,
                                                        int *count, unsigned long long *nref, int first,
                                                        cudaGraphConditionalHandle cond, int use_cond,
                                                        int body_kernels) {
  __shared__ int part[32];
  int v = 0;
  for (int i = threadIdx.x; i < items; i += blockDim.x) {
    const int a = act ? act[i] : 1;
    const double r = rn[i];
    const int m = a && r > limit && r < basin;
    mark[i] = m;
    v += m;
  }
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += part[w];
    *count = t;
    if (first && t) nref[0] += (unsigned long long)t;
    if (use_cond) {
      cudaGraphSetConditional(cond, t > 0 ? 1u : 0u);
      if (t > 0) nref[1] += (unsigned long long)body_kernels;
    }
  }
}

// Inside a stream capture: an IF node whose condition a kernel captured
// before it sets, with its body captured on `side`.  cond_handle creates the
// handle on the graph being captured (the setter needs it as an argument);
// cond_if_begin appends the node after the stream's current dependencies and
// starts the capture of its body; cond_if_end closes that capture.
int cond_handle(cudaStream_t st, cudaGraphConditionalHandle *h) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g;
  if (cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, nullptr, nullptr, nullptr) != cudaSuccess ||
      cs != cudaStreamCaptureStatusActive)
    return SKKR_ERR_CUDA;
  return cudaGraphConditionalHandleCreate(h, g, 0, 0) == cudaSuccess ? 0 : SKKR_ERR_CUDA;
}

int cond_begin(cudaStream_t st, cudaStream_t side, cudaGraphConditionalHandle h, int type) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g;
  const cudaGraphNode_t *deps = nullptr;
  const cudaGraphEdgeData *ed = nullptr;
  size_t nd = 0;
  if (cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, &ed, &nd) != cudaSuccess ||
      cs != cudaStreamCaptureStatusActive)
    return SKKR_ERR_CUDA;
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = (cudaGraphConditionalNodeType)type;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  if (cudaGraphAddNode(&node, g, deps, ed, nd, &p) != cudaSuccess) return SKKR_ERR_CUDA;
  if (cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies) != cudaSuccess)
    return SKKR_ERR_CUDA;
  return cudaStreamBeginCaptureToGraph(side, p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                       cudaStreamCaptureModeRelaxed) == cudaSuccess
             ? 0
             : SKKR_ERR_CUDA;
}

int cond_end(cudaStream_t side) {
  cudaGraph_t body = nullptr;
  return cudaStreamEndCapture(side, &body) == cudaSuccess ? 0 : SKKR_ERR_CUDA;
}

bool stream_capturing(cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive;
}

// ---------------------------------------------------------------------------
// Autotuned thread layout of the FP32 Gauss-Jordan.  A size class fixes the
// columns per thread (16 RB >= n); the rows split over TY x RA threads.  Every
// layout gives the same inverse bit for bit (each element takes the same
// sequence of updates, the pivot search is deterministic), so the first
// batch of each (size class, batch size) key times the layouts once on the
// real operands and later calls use the fastest.  A capture in progress
// before a key is tuned takes the first layout.
using GjLaunch = void (*)(const MatRef &, const MatRef &, int, int, const int *, unsigned, cudaStream_t);

template <int TY, int RA, int RB, int MINB = 1>
static void gj_launch(const MatRef &A, const MatRef &X, int n, int nc, const int *act, unsigned items,
                      cudaStream_t st) {
  k_cgj32<TY, RA, RB, MINB><<<items, TY * 16, 0, st>>>(A, X, n, nc, act);
}

struct GjClass {
  int nmax;
  int nv;
  GjLaunch f[3];
  const char *name[3];
};

static const GjClass GJ_CLASSES[3] = {
    {32, 3, {gj_launch<16, 2, 2>, gj_launch<32, 1, 2>, gj_launch<8, 4, 2>}, {"16x2x2", "32x1x2", "8x4x2"}},
    {64, 3, {gj_launch<16, 4, 4, 3>, gj_launch<32, 2, 4, 2>, gj_launch<64, 1, 4>}, {"16x4x4 (3/SM)", "32x2x4 (2/SM)", "64x1x4"}},
    {128, 2, {gj_launch<32, 4, 8>, gj_launch<64, 2, 8>, nullptr}, {"32x4x8", "64x2x8", ""}},
};

namespace {
std::mutex g_tune_mu;
std::map<std::pair<int, int>, int> g_tuned;  // (class, batch bucket) -> layout
int g_tune_force = 0;                         // > 0: always layout g_tune_force - 1 (tests)
}  // namespace

static GjLaunch gj_choose(int n, long long items, const MatRef &A, const MatRef &X, int nc, const int *act,
                          cudaStream_t st) {
  const int cls = n <= 32 ? 0 : n <= 64 ? 1 : 2;
  const GjClass &C = GJ_CLASSES[cls];
  std::lock_guard<std::mutex> lk(g_tune_mu);
  if (g_tune_force > 0) return C.f[std::min(g_tune_force - 1, C.nv - 1)];
  // batches below one wave, below four waves, and larger
  const int bucket = items < 152 ? 0 : items < 608 ? 1 : 2;
  auto it = g_tuned.find({cls, bucket});
  if (it != g_tuned.end()) return C.f[it->second];
  if (stream_capturing(st)) return C.f[0];
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return C.f[0];
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return C.f[0];
  }
  // each layout: one warm run, then the best of three timed runs; a later
  // layout replaces the current choice only when it is 5 % faster (the
  // layouts are listed in order of preference)
  int best = 0;
  float tbest = 1e30f;
  for (int v = 0; v < C.nv; v++) {
    C.f[v](A, X, n, nc, act, (unsigned)items, st);  // warm (module load, caches)
    float tv = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
      cudaEventRecord(e0, st);
      C.f[v](A, X, n, nc, act, (unsigned)items, st);
      cudaEventRecord(e1, st);
      float ms = 1e30f;
      if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess)
        tv = std::min(tv, ms);
    }
    if (tv < 0.95f * tbest) {
      tbest = tv;
      best = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  g_tuned[{cls, bucket}] = best;
  return C.f[best];
}

int gj_tune_force(int v) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune_force = v;
  if (v == 0) g_tuned.clear();
  return 0;
}

std::string gj_tune_report() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  std::string r;
  static const char *bn[3] = {"<1 wave", "<4 waves", ">=4 waves"};
  for (auto &kv : g_tuned) {
    const GjClass &C = GJ_CLASSES[kv.first.first];
    r += "n<=" + std::to_string(C.nmax) + " " + bn[kv.first.second] + ": " + C.name[kv.second] + "; ";
  }
  return r;
}

// The FP32 start of an inverse above 64 rows by the 2 x 2 block form: with
// A = [[A11, A12], [A21, A22]], A11 64 x 64,
//   X11 = A11^-1, U = X11 A12, S = A22 - A21 U, Y = S^-1, T = A21 X11,
//   A^-1 = [[X11 - X12 T, X12], [-Y T, Y]],  X12 = -U Y,
// the two diagonal inverses by the FP32 Gauss-Jordan (pivoting inside each
// block) at 64 rows, where several matrices share an SM, and the six
// products by k_cgemm32.  Without pivoting across the blocks the start is
// a few times less accurate than the whole-matrix Gauss-Jordan on the
// path's matrices; the Newton steps and their acceptance test are the same.
// `scratch` holds n^2 elements per item (X11, U, S, T).
static void block_start(const MatRef &A, const MatRef &X, int n, int nc, const int *act, unsigned items,
                        zd *scratch, cudaStream_t st) {
  const int b = 64, n2 = n - 64;
  const long long MB = (long long)n * n;
  auto sub = [&](const MatRef &M, int r, int c) { return mref_offset(M, r + (long long)c * M.ld); };
  auto scr = [&](long long off, int ld) { return mref(scratch + off, (long long)nc * MB, MB, ld); };
  const MatRef X11 = scr(0, b), U = scr((long long)b * b, b), S = scr((long long)b * b + (long long)b * n2, n2),
               T = scr((long long)b * b + (long long)b * n2 + (long long)n2 * n2, n2);
  const MatRef A11 = A, A12 = sub(A, 0, b), A21 = sub(A, b, 0), A22 = sub(A, b, b);
  const MatRef Xa = X, X12 = sub(X, 0, b), X21 = sub(X, b, 0), X22 = sub(X, b, b);
  const GjLaunch g1 = gj_choose(b, items, A11, X11, nc, act, st);
  g1(A11, X11, b, nc, act, items, st);
  SKKR_LAUNCHED();
  const G32Job u = g32(0, X11, A12, U, U, b, n2, b), t = g32(0, A21, X11, T, T, n2, b, b);
  cgemm32(u, &t, nc, act, items, st);                                  // U = X11 A12, T = A21 X11
  cgemm32(g32(1, A21, U, S, A22, n2, n2, b), nullptr, nc, act, items, st);  // S = A22 - A21 U
  // Y = S^-1 straight into its place in X (the layout autotuner may run its
  // candidates on these operands: S is never overwritten)
  const GjLaunch g2 = gj_choose(n2, items, S, X22, nc, act, st);
  g2(S, X22, n2, nc, act, items, st);
  SKKR_LAUNCHED();
  const G32Job x12 = g32(2, U, X22, X12, X12, b, n2, n2), x21 = g32(2, X22, T, X21, X21, n2, b, n2);
  cgemm32(x12, &x21, nc, act, items, st);                              // X12 = -U Y, X21 = -Y T
  cgemm32(g32(1, X12, T, Xa, X11, b, b, n2), nullptr, nc, act, items, st);  // X11 - X12 T
}

// X = A^-1: FP32 Gauss-Jordan, then `newton` steps X += X (I - A X) with the
// residual product at S = sres slices and the correction at S = 3.  X may be
// A itself (`inplace`); otherwise the two must not overlap.
int mixed_zinv(MixedWork *w, const MatRef &A, const MatRef &X, int n, int nk, int nc, const int *act,
               int newton, int sres, bool inplace, cudaStream_t st) {
  if (n < 1 || n > 128 || newton < 1) return SKKR_ERR_ARG;
  const long long items = (long long)nk * nc, MB = (long long)n * n;
  int rc;
  if (inplace && (rc = grow((void **)&w->acopy, &w->ac_cap, (size_t)items * MB * sizeof(zd), false))) return rc;
  if ((rc = grow((void **)&w->rbuf, &w->rb_cap, (size_t)items * MB * sizeof(zd), false))) return rc;
  if ((rc = grow((void **)&w->rnorm, &w->rn_cap, (size_t)items * sizeof(double), false))) return rc;
  if ((rc = grow((void **)&w->flag, &w->flag_cap, (size_t)items * sizeof(int), false))) return rc;
  if ((rc = grow((void **)&w->mark, &w->mark_cap, (size_t)items * sizeof(int), false))) return rc;
  // the further Newton steps split X (and, unless B is fused, R) into slot 5
  // at sres slices (the standard correction uses 3): reserve that size, for
  // either B tile, while not capturing, so that a captured step never has to
  // grow the slot
  int Se, DB;
  oz_digits(sres, n, &Se, &DB);
  if (!stream_capturing(st)) {
    int Mp, Np, Kp, mt, ntl, kbl;
    size_t bb = 0, ba = 0;
    for (int tn : {NT, 64}) {
      oz_dims(n, n, tn, &Mp, &Np, &Kp, &mt, &ntl, &kbl);
      ba = (size_t)items * Se * Mp * Kp * 2;
      bb = std::max(bb, (size_t)items * Se * Np * Kp * 2);
    }
    if ((rc = grow(&w->A[5].p, &w->A[5].cap, ba, true))) return rc;
    if (!fuses_b(w, Se) && (rc = grow(&w->B[5].p, &w->B[5].cap, bb, true))) return rc;
  }
  // A itself serves the Gauss-Jordan start, the residuals and the FP64 redo
  // unless X overwrites it (in place): then a copy does
  const MatRef Ac = inplace ? mref(w->acopy, (long long)nc * MB, MB, n) : A;
  MatRef R = mref(w->rbuf, (long long)nc * MB, MB, n);
  if (inplace) launch_zaxpby(Ac, A, nullptr, 0, nullptr, 0, n, nk, nc, act, st);
  kstat_begin(KS_GJ, 8.0 * n * (double)n * n * (double)(act ? skkr_active_items(items) : items), st);
  if (w->blocked && n > 64) {
    block_start(Ac, X, n, nc, act, (unsigned)items, w->rbuf, st);
  } else {
    const GjLaunch gj = gj_choose(n, items, Ac, X, nc, act, st);
    gj(Ac, X, n, nc, act, (unsigned)items, st);
    SKKR_LAUNCHED();
  }
  kstat_end(st);
  // A is split once (A slot 0) for the residuals of every Newton step
  if ((rc = mixed_split(w, 0, 0, sres, Ac, n, n, nk, nc, act, st))) return rc;
  for (int it = 0; it < newton; it++) {
    // R = I - A X
    if ((rc = mixed_split(w, 1, 0, sres, X, n, n, nk, nc, act, st))) return rc;
    if ((rc = mixed_gemm_staged(w, 4, sres, 0, 0, R, R, R, n, n, nk, nc, act, st))) return rc;
    if (it == newton - 1) launch_fnorm(R, n, nk, nc, act, w->rnorm, st);
    // X = X + X R (slot 5: slot 0 keeps A)
    if ((rc = mixed_split(w, 0, 5, 3, X, n, n, nk, nc, act, st))) return rc;
    if ((rc = mixed_split(w, 1, 5, 3, R, n, n, nk, nc, act, st))) return rc;
    if ((rc = mixed_gemm_staged(w, 5, 3, 5, 5, X, X, X, n, n, nk, nc, act, st))) return rc;
  }
  // Items above the limit but inside Newton's basin (|R| < 1/2) take up to
  // NEWTON_EXTRA further steps with the correction at sres slices as well:
  // the 3-slice correction leaves about cond(A) 2^-24 |R| in the next
  // residual, which stalls ill-conditioned items.  Each step runs only if an
  // item is marked: inside a captured graph an IF node decides on the
  // device; run eagerly, the host reads the count.
  const bool cap = stream_capturing(st);
  const long long hint = skkr_active_items(-1);
  for (int e = 0; e < NEWTON_EXTRA; e++) {
    cudaGraphConditionalHandle h = 0;
    if (cap && (rc = cond_handle(st, &h))) return rc;
    // the IF body below launches 2 sliced products, 1 norm and the splits:
    // 3, or 1 with the B operands fused
    const int nbody = fuses_b(w, Se) ? 4 : 6;
    k_newton_select<<<1, 1024, 0, st>>>(w->rnorm, act, (int)items, 1e-6, 0.5, w->mark, w->cnt, w->nref, e == 0,
                                        h, cap ? 1 : 0, nbody);
    SKKR_LAUNCHED();
    const long long l_body = g_skkr_launches;
    cudaStream_t sx = st;
    if (cap) {
      if ((rc = cond_begin(st, w->side, h, cudaGraphCondTypeIf))) return rc;
      sx = w->side;
    } else {
      int marked = 0;
      if (cudaMemcpyAsync(&marked, w->cnt, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
          cudaStreamSynchronize(st) != cudaSuccess)
        return SKKR_ERR_CUDA;
      if (marked == 0) break;
      skkr_set_active_items(marked);
    }
    const int *mk = w->mark;
    auto step = [&]() -> int {
      int r;
      if ((r = mixed_split(w, 1, 0, sres, X, n, n, nk, nc, mk, sx))) return r;
      if ((r = mixed_gemm_staged(w, 4, sres, 0, 0, R, R, R, n, n, nk, nc, mk, sx))) return r;
      launch_fnorm(R, n, nk, nc, mk, w->rnorm, sx);
      if ((r = mixed_split(w, 0, 5, sres, X, n, n, nk, nc, mk, sx))) return r;
      if ((r = mixed_split(w, 1, 5, sres, R, n, n, nk, nc, mk, sx))) return r;
      return mixed_gemm_staged(w, 5, sres, 5, 5, X, X, X, n, n, nk, nc, mk, sx);
    };
    rc = step();
    if (cap) {  // close the body's capture whatever happened inside it
      const int rc2 = cond_end(w->side);
      if (!rc) rc = rc2;
      // the body's kernels are counted when they run (nref[1]), not here
      g_skkr_launches = l_body;
      g_skkr_if_captured += nbody;
    }
    if (rc) return rc;
    skkr_set_active_items(hint);
  }
  // An ill-conditioned A (cond ~ 1e7 and above) leaves the FP32 start outside
  // Newton's basin: such items are inverted again in FP64 (copy A, column-
  // pivoting Gauss-Jordan), masked so that the others are untouched.  The
  // residual before the last correction bounds the final error by its square.
  k_newton_check<<<(unsigned)((items + 255) / 256), 256, 0, st>>>(w->rnorm, act, (int)items, 1e-6, w->flag,
                                                                   w->dmax, w->nfb);
  SKKR_LAUNCHED();
  launch_zaxpby(X, Ac, nullptr, 0, nullptr, 0, n, nk, nc, w->flag, st);
  launch_zgj(X, n, nk, nc, w->flag, st);
  return 0;
}
