// Slicing of FP64 values into BF16 digit slices for the split-precision
// products, on the device and (for its CPU test) on the host.
//
// All element-wise work uses integer arithmetic on the IEEE bit patterns:
// this GPU issues about 2 FP64 operations per clock per SM against 64
// integer operations, so a single FP64 multiply per element would dominate.
//
// Scales are powers of two kept as exponents: sigma = 2^es with
// es = (biased exponent of max |x|) - 1022, i.e. sigma >= max |x| > sigma/2.
#pragma once
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define SLC_HD __host__ __device__ __forceinline__
#else
#define SLC_HD inline
#endif

SLC_HD unsigned long long slc_dbits(double x) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(x);
#else
  unsigned long long u;
  std::memcpy(&u, &x, sizeof u);
  return u;
#endif
}
SLC_HD uint32_t slc_fbits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, sizeof u);
  return u;
#endif
}
SLC_HD float slc_bitsf(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float f;
  std::memcpy(&f, &u, sizeof f);
  return f;
#endif
}
// the upper halves of a and b as one word, a's in the low half
SLC_HD uint32_t slc_hi_pair(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
  return __byte_perm(a, b, 0x7632);
#else
  return (a >> 16) | (b & 0xFFFF0000u);
#endif
}

// |x| bits of a double (non-negative doubles order like their bit patterns)
SLC_HD unsigned long long abs_bits(double x) { return slc_dbits(x) & 0x7FFFFFFFFFFFFFFFull; }
// log2 of the power-of-two scale for a max-|x| bit pattern (0 for zero)
SLC_HD int scale_exp(unsigned long long amax_bits) {
  const int ex = (int)(amax_bits >> 52);
  return ex == 0 ? 0 : ex - 1022;
}
// |round(x 2^E)| (halves away from zero) as a 64-bit integer (callers keep it
// below 2^62) and the sign of x; zero and subnormal inputs give 0
SLC_HD unsigned long long fix_round_mag(double x, int E, bool *neg) {
  const unsigned long long b = slc_dbits(x);
  *neg = (b >> 63) != 0;
  const int ex = (int)((b >> 52) & 0x7FF);
  if (ex == 0) return 0;
  const unsigned long long mant = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const int sh = ex - 1075 + E;
  if (sh >= 0) return sh >= 11 ? 0 : mant << sh;
  const int r = -sh;
  return r >= 63 ? 0 : (mant + (1ull << (r - 1))) >> r;
}
// the same with the sign applied
SLC_HD long long fix_round(double x, int E) {
  bool neg;
  const long long m = (long long)fix_round_mag(x, E, &neg);
  return neg ? -m : m;
}
SLC_HD float pow2f(int e) { return slc_bitsf((uint32_t)(127 + e) << 23); }

// sum over q < S - 1 of (2^(DB-1) - 1) 2^(DB q)
template <int S, int DB>
SLC_HD constexpr unsigned long long digit_bias() {
  unsigned long long b = 0;
  for (int q = 0; q < S - 1; q++) b |= (unsigned long long)((1 << (DB - 1)) - 1) << (DB * q);
  return b;
}

// balanced base-2^DB digits of Y = round(x 2^((DB-1) + DB(S-1)) / sigma),
// most significant first.  The lower S - 1 digits lie in
// [-(2^(DB-1) - 1), 2^(DB-1)], a set of 2^DB consecutive integers, so they
// are unique: they are the plain base-2^DB digits of |Y| + digit_bias, each
// less 2^(DB-1) - 1 (one add for the whole value, then a field extraction and
// a subtraction per digit); the top digit is what lies above them (at most
// 2^(DB-1), as |Y| <= 2^(DB-1) 2^(DB(S-1))).  Negative x negates every
// digit.  DB = 8 for K' = 2K <= 256; DB = 7 above, so that every FP32 level
// accumulator (at most 4 (p,q) pairs of |d d| <= 2^(2DB-2) over K' terms)
// stays an exact integer below 2^24.
template <int S, int DB>
SLC_HD void slice_digits(double x, int es, int *dig) {
  static_assert(DB * S <= 62, "digits must fit the 62-bit fixed-point value");
  bool neg;
  const unsigned long long v = fix_round_mag(x, (DB - 1) + DB * (S - 1) - es, &neg) + digit_bias<S, DB>();
  constexpr int LOW = (1 << (DB - 1)) - 1;
  const int sg = neg ? -1 : 0;  // d -> (d ^ sg) - sg negates when sg = -1
#pragma unroll
  for (int q = 0; q < S - 1; q++) {
    const int d = (int)((v >> (DB * q)) & ((1ull << DB) - 1)) - LOW;
    dig[S - 1 - q] = (d ^ sg) - sg;
  }
  const int top = (int)(v >> (DB * (S - 1)));  // the bias has no top part
  dig[0] = (top ^ sg) - sg;
}

// float bits of (f - 1.5 2^23) s for the float bits f of 1.5 2^23 + d (the
// integer add already done): d s, exact
SLC_HD uint32_t digit_bits_raw(uint32_t f, float s, float off) {
#ifdef __CUDA_ARCH__
  return slc_fbits(fmaf(slc_bitsf(f), s, off));
#else
  return slc_fbits(slc_bitsf(f) * s + off);
#endif
}
// float bits of d 2^k for an integer digit |d| <= 128, from one integer add
// and one FMA: (1.5 2^23 + d) 2^k - 1.5 2^23 2^k is exact, and with at most
// eight significant bits the value is a bf16 held in the upper half of the
// float (zero digits give +0).  s = 2^k, off = -1.5 2^23 2^k.
SLC_HD uint32_t digit_bits(int d, float s, float off) {
#ifdef __CUDA_ARCH__
  return slc_fbits(fmaf(slc_bitsf(0x4B400000u + (uint32_t)d), s, off));
#else
  // exact on the host as well: both terms and the sum are representable
  return slc_fbits(slc_bitsf(0x4B400000u + (uint32_t)d) * s + off);
#endif
}

// four consecutive complex values (re[e], im[e], e < 4) of one row or column
// into the slice words: wr[p] / wi[p] hold the bf16 of the digits of the real
// / imaginary parts scaled by 2^(wshift - DB p), element e in half e % 2 of
// word .x (e < 2) or .y.  The digits are those of slice_digits, formed from
// |Y| (each a field of |Y| + digit_bias less 2^(DB-1) - 1, folded into the
// bf16 construction's integer add) and negated through the bf16 sign bits,
// one XOR per word; a zero digit of a negative value becomes -0, which
// changes no product or sum
template <int S, int DB>
SLC_HD void slice4(const double (&re)[4], const double (&im)[4], int es, int wshift, uint32_t (&wr)[S][2],
                   uint32_t (&wi)[S][2]) {
  constexpr int E0 = (DB - 1) + DB * (S - 1);
  constexpr unsigned long long BIAS = digit_bias<S, DB>();
  constexpr uint32_t LOW = (1u << (DB - 1)) - 1;
#pragma unroll
  for (int h = 0; h < 2; h++) {
    bool s0, s1, t0, t1;
    const unsigned long long r0 = fix_round_mag(re[2 * h], E0 - es, &s0) + BIAS;
    const unsigned long long r1 = fix_round_mag(re[2 * h + 1], E0 - es, &s1) + BIAS;
    const unsigned long long i0 = fix_round_mag(im[2 * h], E0 - es, &t0) + BIAS;
    const unsigned long long i1 = fix_round_mag(im[2 * h + 1], E0 - es, &t1) + BIAS;
    const uint32_t sr = (s0 ? 0x8000u : 0u) | (s1 ? 0x80000000u : 0u);
    const uint32_t si = (t0 ? 0x8000u : 0u) | (t1 ? 0x80000000u : 0u);
#pragma unroll
    for (int p = 0; p < S; p++) {
      const float sc = pow2f(wshift - DB * p), off = -12582912.0f * sc;
      // digit p (most significant first): the top one is what lies above the
      // biased fields, the others a field less LOW
      const int sh = DB * (S - 1 - p);
      const uint32_t cst = p == 0 ? 0x4B400000u : 0x4B400000u - LOW;
      const uint32_t msk = p == 0 ? 0xFFFFFFFFu : (1u << DB) - 1;
      const uint32_t a0 = (uint32_t)(r0 >> sh) & msk, a1 = (uint32_t)(r1 >> sh) & msk;
      const uint32_t b0 = (uint32_t)(i0 >> sh) & msk, b1 = (uint32_t)(i1 >> sh) & msk;
      wr[p][h] = slc_hi_pair(digit_bits_raw(cst + a0, sc, off), digit_bits_raw(cst + a1, sc, off)) ^ sr;
      wi[p][h] = slc_hi_pair(digit_bits_raw(cst + b0, sc, off), digit_bits_raw(cst + b1, sc, off)) ^ si;
    }
  }
}
