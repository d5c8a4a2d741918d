// Shared device helpers of the 2D-BZ tau library.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdlib>
#include <algorithm>
#include <cstdio>

typedef double2 zd;  // complex*16, interleaved re/im

__host__ __device__ inline zd zmk(double r, double i) { return make_double2(r, i); }
__device__ inline zd zadd(zd a, zd b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ inline zd zsub(zd a, zd b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ inline zd zmul(zd a, zd b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ inline zd zscale(double s, zd a) { return make_double2(s * a.x, s * a.y); }
__device__ inline double zabs2(zd a) { return a.x * a.x + a.y * a.y; }
// c += a*b (four FMAs, real part first)
__device__ inline void zfma(zd &c, zd a, zd b) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(a.y, b.x, c.y);
}
// c -= a*b (four FMAs)
__device__ inline void zfms(zd &c, zd a, zd b) {
  c.x = fma(-a.x, b.x, c.x);
  c.x = fma(a.y, b.y, c.x);
  c.y = fma(-a.x, b.y, c.y);
  c.y = fma(-a.y, b.x, c.y);
}
// 1/q by Smith's scaled division
__device__ inline zd zrecip(zd q) {
  if (fabs(q.x) >= fabs(q.y)) {
    double r = q.y / q.x, den = q.x + q.y * r;
    return make_double2(1.0 / den, -r / den);
  }
  double r = q.x / q.y, den = q.x * r + q.y;
  return make_double2(r / den, -1.0 / den);
}

#define SKKR_MAPN 16

// A batch operand: matrix of item (k, c) starts at base + k*sk + map[c]*sc,
// column-major with leading dimension ld.
struct MatRef {
  zd *base;
  long long sk;
  long long sc;
  int ld;
  int map[SKKR_MAPN];
};

// (the map entry by static selects: a dynamic index into a kernel
// parameter's array would copy the whole MatRef to the thread's stack)
__device__ inline zd *mat_ptr(const MatRef &m, int k, int c) {
  int mc = 0;
#pragma unroll
  for (int i = 0; i < SKKR_MAPN; i++) mc = i == c ? m.map[i] : mc;
  return m.base + (long long)k * m.sk + (long long)mc * m.sc;
}

// host-side constructors
inline MatRef mref(zd *base, long long sk, long long sc, int ld) {
  MatRef r;
  r.base = base;
  r.sk = sk;
  r.sc = sc;
  r.ld = ld;
  for (int i = 0; i < SKKR_MAPN; i++) r.map[i] = i;
  return r;
}
// the same batch operand moved by `elems` elements (a sub-block of every item)
inline MatRef mref_offset(const MatRef &m, long long elems) {
  MatRef r = m;
  r.base += elems;
  return r;
}
inline MatRef mref_map(zd *base, long long sk, long long sc, int ld, const int *map, int nmap) {
  MatRef r = mref(base, sk, sc, ld);
  for (int i = 0; i < nmap && i < SKKR_MAPN; i++) r.map[i] = map[i];
  return r;
}

// element range [lo, hi) of an operand's nk x nc items (`cols` columns of at
// most ld rows each), relative to its base
inline void mref_span(const MatRef &m, int nk, int nc, int cols, long long *lo, long long *hi) {
  long long mn = 0, mx = 0;
  for (int c = 0; c < nc && c < SKKR_MAPN; c++) {
    const long long o = (long long)m.map[c] * m.sc;
    mn = c == 0 || o < mn ? o : mn;
    mx = c == 0 || o > mx ? o : mx;
  }
  const long long ks = (long long)(nk - 1) * m.sk;
  *lo = mn + std::min(0LL, ks);
  *hi = mx + std::max(0LL, ks) + (long long)cols * m.ld;
}
// whether two operands' items may share an element: no when their ranges
// are apart, or when both sit on the same lattice of item offsets (multiples
// of g = gcd(sk, sc)) with footprints of cols x ld elements that stay apart
// modulo g (buffers interleaved item by item in one allocation)
inline bool mref_overlap(const MatRef &a, const MatRef &b, int nk, int nc, int cols) {
  long long la, ha, lb, hb;
  mref_span(a, nk, nc, cols, &la, &ha);
  mref_span(b, nk, nc, cols, &lb, &hb);
  const uintptr_t a0 = (uintptr_t)(a.base + la), a1 = (uintptr_t)(a.base + ha);
  const uintptr_t b0 = (uintptr_t)(b.base + lb), b1 = (uintptr_t)(b.base + hb);
  if (!(a0 < b1 && b0 < a1)) return false;
  if (a.sk != b.sk || a.sc != b.sc || a.ld != b.ld) return true;
  long long g = std::llabs(a.sk), h = std::llabs(a.sc);
  while (h) {
    const long long t = g % h;
    g = h;
    h = t;
  }
  const long long fp = (long long)cols * a.ld;
  if (g < 2 * fp) return true;
  const long long d = ((long long)(intptr_t)((uintptr_t)b.base - (uintptr_t)a.base)) / (long long)sizeof(zd);
  const long long dm = ((d % g) + g) % g;
  return !(fp <= dm && dm + fp <= g);
}

// One process-wide lock between CUDA graph capture and the calls that may
// synchronise the device (cudaMalloc / cudaFree / cudaDeviceSynchronize of a
// growing work buffer): a capture on one host thread never overlaps such a
// call on another.  Recursive: a capture that sizes a buffer takes it again.
#include <mutex>
std::recursive_mutex &skkr_device_mutex();

// kernel launch bookkeeping (defined in capi.cu).  With SKKR_SYNC_CHECK=1 in
// the environment every launch is followed by a device synchronisation and
// the first failing launch site is recorded (diagnostics only).
extern thread_local long long g_skkr_launches;  // launches made by this host thread
// kernels captured into the IF bodies of conditional graph nodes by this
// thread (counted when they run, from device counters)
extern thread_local long long g_skkr_if_captured;
void skkr_after_launch(const char *file, int line);
#define SKKR_LAUNCHED() skkr_after_launch(__FILE__, __LINE__)

// Per-kernel-class timing with CUDA events on the launching stream (off by
// default; bench.py switches it on for the timed region).  `work` is the
// algorithmic FLOP (or byte) count of the launch.  Masked launches count the
// active items the host announced through skkr_set_active_items (-1: all).
enum { KS_GEMM = 0, KS_GJ = 1, KS_GKFT = 2, KS_OTHER = 3, KS_OZAKI = 4, KS_NCLS = 5 };
void kstat_begin(int cls, double work, cudaStream_t st);
// work2: the FP64-equivalent algorithmic count of the launch where it differs
// from `work` (a sliced product: one complex product, 8 n^2 K FLOP per item)
void kstat_begin2(int cls, double work, double work2, cudaStream_t st);
void kstat_end(cudaStream_t st);
long long skkr_active_items(long long all);
void skkr_set_active_items(long long n);
