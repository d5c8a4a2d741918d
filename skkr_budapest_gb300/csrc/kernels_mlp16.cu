// Warm-start network in the precision of the C4 surrogate: BF16 weights
// (round-to-nearest-even copies of FP32 master weights), FP32 activations,
// FP32 accumulation.  Row-major activations H[n][d]; layer i holds
// W_i[d_i][d_{i+1}] and b_i[d_{i+1}], packed W_0, b_0, W_1, ... in one FP32
// array (the masters), with a BF16 array of the same packing that the
// products read.  Every sum runs in a fixed order (the K split of the weight
// gradient is reduced split by split), so results do not depend on
// scheduling.
//
// The products are register-tiled FP32 GEMMs on the CUDA cores: at these
// widths (<= 4096, a few 10^4 rows) one epoch is a few GFLOP, and FP32
// accumulation of BF16 weights with FP32 activations has no tensor-core form
// (kind::f16 takes both operands in 16 bits).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/skkr_gpu.h"
#include "common.cuh"
#include "kernels.h"

namespace {

constexpr int TM = 64, TNB = 64, TK = 16, GT = 256;  // tile, k step, threads (16 x 16, 4 x 4 outputs each)

__device__ __forceinline__ float ld_op(const float *p, long long i) { return p[i]; }
__device__ __forceinline__ float ld_op(const __nv_bfloat16 *p, long long i) { return __bfloat162float(p[i]); }

// C[m][n] (row-major, ldc) = sum_{k in [k0, k1)} A(m, k) B(k, n), with
// A(m, k) = A[m sam + k sak] and B(k, n) = B[k sbk + n sbn]; epilogue
// (ep = 0): + bias[n] and tanh when act; ep = 1: raw partial sums into
// C + blockIdx.z * M * ldc (the K split of the weight gradient).  Each output
// sums its k in increasing order.
template <typename TB>
__global__ void __launch_bounds__(GT) k_gemm32(const float *__restrict__ A, long long sam, long long sak,
                                               const TB *__restrict__ B, long long sbk, long long sbn, int M, int N,
                                               int K, int kchunk, const float *__restrict__ bias, int act, int ep,
                                               float *__restrict__ C, int ldc) {
  __shared__ float As[TK][TM + 1], Bs[TK][TNB + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TNB;
  const int k0 = blockIdx.z * kchunk, k1 = min(K, k0 + kchunk);
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) acc[i][j] = 0.f;
  for (int kb = k0; kb < k1; kb += TK) {
    // 64 x 16 tiles of A and B, 4 elements per thread each; consecutive
    // threads walk the operand's unit-stride index (coalesced loads)
    for (int e = threadIdx.x; e < TM * TK; e += GT) {
      const int mm = sak == 1 ? e / TK : e % TM, ka = sak == 1 ? e % TK : e / TM;
      const int gm = m0 + mm, gka = kb + ka;
      As[ka][mm] = (gm < M && gka < k1) ? A[gm * sam + gka * sak] : 0.f;
      const int nn = sbn == 1 ? e % TNB : e / TK, kbb = sbn == 1 ? e / TNB : e % TK;
      const int gn = n0 + nn, gkb = kb + kbb;
      Bs[kbb][nn] = (gn < N && gkb < k1) ? ld_op(B, gkb * sbk + gn * sbn) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  float *Cb = ep == 1 ? C + (long long)blockIdx.z * M * ldc : C;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      float v = acc[i][j];
      if (ep == 0) {
        if (bias) v += bias[gn];
        if (act) v = tanhf(v);
      }
      Cb[(long long)gm * ldc + gn] = v;
    }
  }
}

// out[e] = sum over s < nsplit of part[s][e], in s order (the K-split
// partial products of the weight gradient)
__global__ void k_split_reduce(const float *__restrict__ part, int nsplit, long long m, float *__restrict__ out) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m; e += (long long)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int q = 0; q < nsplit; q++) s += part[(long long)q * m + e];
    out[e] = s;
  }
}

// db[j] = sum_r dZ[r][j], rows in order
__global__ void k_colsum(const float *__restrict__ dZ, int n, int dout, float *__restrict__ db) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < dout; j += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int r = 0; r < n; r++) s += dZ[(long long)r * dout + j];
    db[j] = s;
  }
}

// per row: squared error over the outputs on rows with sel[r] == want (sel
// null: all rows), dY = scale 2 (Yh - Y) there and 0 elsewhere
__global__ void k_loss_rows32(const float *__restrict__ Yh, const float *__restrict__ Y,
                              const unsigned char *__restrict__ sel, int want, int n, int dout, float scale,
                              float *__restrict__ dY, float *__restrict__ rowsum) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const bool on = sel ? (sel[r] == want) : true;
    float s = 0.f;
    for (int j = 0; j < dout; j++) {
      const long long e = (long long)r * dout + j;
      const float d = Yh[e] - Y[e];
      s = fmaf(d, d, s);
      if (dY) dY[e] = on ? scale * 2.f * d : 0.f;
    }
    rowsum[r] = on ? s : 0.f;
  }
}

// out[0] = scale * sum v[0..n): one block, strided per thread, then a tree
__global__ void k_sum32(const float *__restrict__ v, int n, float scale, float *__restrict__ out) {
  __shared__ float sh[1024];
  float s = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += v[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = scale * sh[0];
}

__global__ void k_tanh_back32(const float *__restrict__ A, float *__restrict__ G, long long m) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m; e += (long long)gridDim.x * blockDim.x) {
    const float a = A[e];
    G[e] *= 1.f - a * a;
  }
}

// one AdamW step (torch's formulation) of the FP32 masters, then their BF16
// copies
__global__ void k_adamw32(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                          float *__restrict__ v, __nv_bfloat16 *__restrict__ p16, long long np, float lr, float wd,
                          float b1, float b2, float eps, float step_size, float bc2_sqrt) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < np; e += (long long)gridDim.x * blockDim.x) {
    const float ge = g[e];
    const float pe = p[e] * (1.f - lr * wd);
    const float me = m[e] + (1.f - b1) * (ge - m[e]);
    const float ve = v[e] * b2 + (1.f - b2) * ge * ge;
    m[e] = me;
    v[e] = ve;
    const float pn = pe - step_size * (me / (sqrtf(ve) / bc2_sqrt + eps));
    p[e] = pn;
    p16[e] = __float2bfloat16_rn(pn);
  }
}

__global__ void k_to_bf16(const float *__restrict__ p, __nv_bfloat16 *__restrict__ q, long long np) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < np; e += (long long)gridDim.x * blockDim.x)
    q[e] = __float2bfloat16_rn(p[e]);
}

// keep the parameters of the lowest held-out loss (one block)
__global__ void k_keep_best32(const float *__restrict__ val, const float *__restrict__ train, float *__restrict__ best,
                              const float *__restrict__ p, float *__restrict__ pbest, long long np) {
  const bool better = val[0] < best[0];
  __syncthreads();
  if (better) {
    for (long long e = threadIdx.x; e < np; e += blockDim.x) pbest[e] = p[e];
    if (threadIdx.x == 0) {
      best[0] = val[0];
      best[1] = train[0];
    }
  }
}

int grid1(long long work) {
  long long g = (work + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g));
}

template <typename TB>
void gemm(const float *A, long long sam, long long sak, const TB *B, long long sbk, long long sbn, int M, int N, int K,
          int nsplit, const float *bias, int act, int ep, float *C, int ldc, cudaStream_t st) {
  const int kchunk = ((K + nsplit - 1) / nsplit + TK - 1) / TK * TK;
  const int nz = (K + kchunk - 1) / kchunk;
  dim3 grid((N + TNB - 1) / TNB, (M + TM - 1) / TM, nz);
  k_gemm32<TB><<<grid, GT, 0, st>>>(A, sam, sak, B, sbk, sbn, M, N, K, kchunk, bias, act, ep, C, ldc);
  SKKR_LAUNCHED();
}

}  // namespace

// Z = act(H W16 + b): H [n][din] FP32, W16 [din][dout] BF16
void mlp16_dense(const float *H, int n, int din, const __nv_bfloat16 *W16, const float *b, int dout, int act, float *Z,
                 cudaStream_t st) {
  gemm<__nv_bfloat16>(H, din, 1, W16, dout, 1, n, dout, din, 1, b, act, 0, Z, dout, st);
}

// dH = dZ W16^T: dZ [n][dout], W16 [din][dout]
void mlp16_hgrad(const float *dZ, int n, int din, int dout, const __nv_bfloat16 *W16, float *dH, cudaStream_t st) {
  gemm<__nv_bfloat16>(dZ, dout, 1, W16, 1, dout, n, din, dout, 1, nullptr, 0, 0, dH, din, st);
}

// g = [H^T dZ ; colsum dZ] (the packed W-then-b gradient), the row sum split
// into nsplit fixed ranges reduced in order through part [nsplit][din][dout]
void mlp16_wgrad(const float *H, const float *dZ, int n, int din, int dout, float *g, float *part, int nsplit,
                 cudaStream_t st) {
  gemm<float>(H, 1, din, dZ, dout, 1, din, dout, n, nsplit, nullptr, 0, 1, part, dout, st);
  const int kchunk = ((n + nsplit - 1) / nsplit + TK - 1) / TK * TK;
  const int nz = (n + kchunk - 1) / kchunk;
  k_split_reduce<<<grid1((long long)din * dout), 256, 0, st>>>(part, nz, (long long)din * dout, g);
  SKKR_LAUNCHED();
  k_colsum<<<(dout + 255) / 256, 256, 0, st>>>(dZ, n, dout, g + (long long)din * dout);
  SKKR_LAUNCHED();
}

void mlp16_loss(const float *Yh, const float *Y, const unsigned char *sel, int want, int n, int dout, float scale,
                float *dY, float *rowsum, float *out, cudaStream_t st) {
  k_loss_rows32<<<grid1(n), 256, 0, st>>>(Yh, Y, sel, want, n, dout, scale, dY, rowsum);
  SKKR_LAUNCHED();
  k_sum32<<<1, 1024, 0, st>>>(rowsum, n, scale, out);
  SKKR_LAUNCHED();
}

void mlp16_tanh_back(const float *A, float *G, long long m, cudaStream_t st) {
  k_tanh_back32<<<grid1(m), 256, 0, st>>>(A, G, m);
  SKKR_LAUNCHED();
}

void mlp16_adamw(float *p, const float *g, float *m, float *v, __nv_bfloat16 *p16, long long np, float lr, float wd,
                 float b1, float b2, float eps, float step_size, float bc2_sqrt, cudaStream_t st) {
  k_adamw32<<<grid1(np), 256, 0, st>>>(p, g, m, v, p16, np, lr, wd, b1, b2, eps, step_size, bc2_sqrt);
  SKKR_LAUNCHED();
}

void mlp16_to_bf16(const float *p, __nv_bfloat16 *q, long long np, cudaStream_t st) {
  k_to_bf16<<<grid1(np), 256, 0, st>>>(p, q, np);
  SKKR_LAUNCHED();
}

void mlp16_keep_best(const float *val, const float *train, float *best, const float *p, float *pbest, long long np,
                     cudaStream_t st) {
  k_keep_best32<<<1, 1024, 0, st>>>(val, train, best, p, pbest, np);
  SKKR_LAUNCHED();
}

// ---- C ABI: forward, gradient and training of the BF16-weight network ----
namespace {

struct M16 {
  int nl = 0, n = 0, dmax = 0, nsplit = 1;
  std::vector<int> d;
  std::vector<long long> off;  // W_i at off[i], b_i at off[i] + d[i] d[i+1]
  long long np = 0, wmax = 0;
  std::vector<void *> owned;
  float *P = nullptr, *Y = nullptr, *buf0 = nullptr, *buf1 = nullptr, *rows = nullptr, *scal = nullptr,
        *part = nullptr;
  __nv_bfloat16 *P16 = nullptr;
  std::vector<float *> A;  // A[0] = x, A[i+1] = output of layer i
  unsigned char *sel = nullptr;
  ~M16() {
    for (void *p : owned) cudaFree(p);
  }
  template <class T>
  int alloc(T **p, size_t count) {
    if (cudaMalloc((void **)p, (count ? count : 1) * sizeof(T)) != cudaSuccess) return SKKR_ERR_NOMEM;
    owned.push_back(*p);
    return SKKR_OK;
  }
};

#define M_CK(x)                                  \
  do {                                           \
    if ((x) != cudaSuccess) return SKKR_ERR_CUDA; \
  } while (0)
#define M_CKR(x)               \
  do {                         \
    int rc_ = (x);             \
    if (rc_) return rc_;       \
  } while (0)

int m16_sizes(int nlayer, const int *dims, int n, M16 &m) {
  if (nlayer < 1 || nlayer > 8 || !dims || n < 1) return SKKR_ERR_ARG;
  m.nl = nlayer;
  m.n = n;
  m.d.assign(dims, dims + nlayer + 1);
  m.off.resize(nlayer);
  for (int i = 0; i <= nlayer; i++) {
    if (m.d[i] < 1 || m.d[i] > 4096) return SKKR_ERR_ARG;
    m.dmax = std::max(m.dmax, m.d[i]);
  }
  for (int i = 0; i < nlayer; i++) {
    m.off[i] = m.np;
    m.np += (long long)m.d[i] * m.d[i + 1] + m.d[i + 1];
    m.wmax = std::max(m.wmax, (long long)m.d[i] * m.d[i + 1]);
  }
  long long act = 0;
  for (int i = 0; i <= nlayer; i++) act += (long long)n * m.d[i];
  if ((act + 2LL * n * m.dmax) * 4 > (16LL << 30)) return SKKR_ERR_ARG;  // activations within 16 GB
  // the weight gradient sums rows in fixed ranges of at least 256 rows
  m.nsplit = std::max(1, std::min(64, n / 256));
  return SKKR_OK;
}

int m16_alloc(M16 &m, const float *params, const float *x, const float *y, const unsigned char *rows) {
  const int n = m.n;
  M_CKR(m.alloc(&m.P, m.np));
  M_CKR(m.alloc(&m.P16, m.np));
  m.A.assign(m.nl + 1, nullptr);
  for (int i = 0; i <= m.nl; i++) M_CKR(m.alloc(&m.A[i], (size_t)n * m.d[i]));
  M_CKR(m.alloc(&m.buf0, (size_t)n * m.dmax));
  M_CKR(m.alloc(&m.buf1, (size_t)n * m.dmax));
  M_CKR(m.alloc(&m.rows, n));
  M_CKR(m.alloc(&m.scal, 2));
  M_CKR(m.alloc(&m.part, (size_t)m.nsplit * m.wmax));
  M_CK(cudaMemcpy(m.P, params, m.np * sizeof(float), cudaMemcpyHostToDevice));
  mlp16_to_bf16(m.P, m.P16, m.np, 0);
  M_CK(cudaMemcpy(m.A[0], x, (size_t)n * m.d[0] * sizeof(float), cudaMemcpyHostToDevice));
  if (y) {
    M_CKR(m.alloc(&m.Y, (size_t)n * m.d[m.nl]));
    M_CK(cudaMemcpy(m.Y, y, (size_t)n * m.d[m.nl] * sizeof(float), cudaMemcpyHostToDevice));
  }
  if (rows) {
    M_CKR(m.alloc(&m.sel, n));
    M_CK(cudaMemcpy(m.sel, rows, n, cudaMemcpyHostToDevice));
  }
  return SKKR_OK;
}

void m16_forward(M16 &m, cudaStream_t st) {
  for (int i = 0; i < m.nl; i++)
    mlp16_dense(m.A[i], m.n, m.d[i], m.P16 + m.off[i], m.P + m.off[i] + (long long)m.d[i] * m.d[i + 1], m.d[i + 1],
                i < m.nl - 1, m.A[i + 1], st);
}

// gradient of the loss whose output gradient the loss kernel left in buf0;
// the products read the BF16 weights the forward pass used
void m16_backward(M16 &m, float *G, cudaStream_t st) {
  float *cur = m.buf0, *nxt = m.buf1;
  for (int i = m.nl - 1; i >= 0; i--) {
    if (i < m.nl - 1) mlp16_tanh_back(m.A[i + 1], cur, (long long)m.n * m.d[i + 1], st);
    mlp16_wgrad(m.A[i], cur, m.n, m.d[i], m.d[i + 1], G + m.off[i], m.part, m.nsplit, st);
    if (i > 0) {
      mlp16_hgrad(cur, m.n, m.d[i], m.d[i + 1], m.P16 + m.off[i], nxt, st);
      std::swap(cur, nxt);
    }
  }
}

int m16_count(const unsigned char *rows, int n, int want) {
  if (!rows) return want ? n : 0;
  int c = 0;
  for (int r = 0; r < n; r++) c += rows[r] == want;
  return c;
}

}  // namespace

extern "C" int skkr_gpu_mlp16_forward(int nlayer, const int *dims, const float *params, int n, const float *x,
                                      float *y) {
  if (!params || !x || !y) return SKKR_ERR_ARG;
  M16 m;
  M_CKR(m16_sizes(nlayer, dims, n, m));
  M_CKR(m16_alloc(m, params, x, nullptr, nullptr));
  m16_forward(m, 0);
  M_CK(cudaDeviceSynchronize());
  M_CK(cudaGetLastError());
  M_CK(cudaMemcpy(y, m.A[m.nl], (size_t)n * m.d[m.nl] * sizeof(float), cudaMemcpyDeviceToHost));
  return SKKR_OK;
}

extern "C" int skkr_gpu_mlp16_grad(int nlayer, const int *dims, const float *params, int n, const float *x,
                                   const float *y, const unsigned char *rows, float *loss, float *grad) {
  if (!params || !x || !y || !loss || !grad) return SKKR_ERR_ARG;
  M16 m;
  M_CKR(m16_sizes(nlayer, dims, n, m));
  const int nsel = m16_count(rows, n, 1);
  if (nsel < 1) return SKKR_ERR_ARG;
  M_CKR(m16_alloc(m, params, x, y, rows));
  float *G;
  M_CKR(m.alloc(&G, m.np));
  const int dout = m.d[m.nl];
  m16_forward(m, 0);
  mlp16_loss(m.A[m.nl], m.Y, m.sel, 1, n, dout, 1.f / ((float)nsel * dout), m.buf0, m.rows, m.scal, 0);
  m16_backward(m, G, 0);
  M_CK(cudaDeviceSynchronize());
  M_CK(cudaGetLastError());
  M_CK(cudaMemcpy(loss, m.scal, sizeof(float), cudaMemcpyDeviceToHost));
  M_CK(cudaMemcpy(grad, G, m.np * sizeof(float), cudaMemcpyDeviceToHost));
  return SKKR_OK;
}

extern "C" int skkr_gpu_mlp16_train(int nlayer, const int *dims, float *params, int n, const float *x, const float *y,
                                    const unsigned char *rows, int epochs, float lr, float weight_decay,
                                    int eval_every, float *train_loss, float *best, float *best_params) {
  if (!params || !x || !y || !train_loss || epochs < 1 || !(lr > 0.f) || weight_decay < 0.f) return SKKR_ERR_ARG;
  M16 m;
  M_CKR(m16_sizes(nlayer, dims, n, m));
  const int ntr = m16_count(rows, n, 1), nval = m16_count(rows, n, 0);
  if (ntr < 1) return SKKR_ERR_ARG;
  const bool eval = eval_every > 0 && nval > 0 && best && best_params;
  M_CKR(m16_alloc(m, params, x, y, rows));
  float *G, *Mo, *Vo, *losses, *bestd = nullptr, *Pbest = nullptr;
  M_CKR(m.alloc(&G, m.np));
  M_CKR(m.alloc(&Mo, m.np));
  M_CKR(m.alloc(&Vo, m.np));
  M_CKR(m.alloc(&losses, epochs));
  M_CK(cudaMemset(Mo, 0, m.np * sizeof(float)));
  M_CK(cudaMemset(Vo, 0, m.np * sizeof(float)));
  if (eval) {
    M_CKR(m.alloc(&bestd, 2));
    M_CKR(m.alloc(&Pbest, m.np));
    const float init[2] = {HUGE_VALF, HUGE_VALF};
    M_CK(cudaMemcpy(bestd, init, sizeof(init), cudaMemcpyHostToDevice));
    M_CK(cudaMemcpy(Pbest, m.P, m.np * sizeof(float), cudaMemcpyDeviceToDevice));
  }
  const int dout = m.d[m.nl];
  const double b1 = 0.9, b2 = 0.999;
  const float eps = 1e-8f;
  for (int ep = 0; ep < epochs; ep++) {
    m16_forward(m, 0);
    mlp16_loss(m.A[m.nl], m.Y, m.sel, 1, n, dout, 1.f / ((float)ntr * dout), m.buf0, m.rows, losses + ep, 0);
    m16_backward(m, G, 0);
    const double t = ep + 1.0;
    const double bc1 = 1.0 - std::pow(b1, t), bc2 = 1.0 - std::pow(b2, t);
    mlp16_adamw(m.P, G, Mo, Vo, m.P16, m.np, lr, weight_decay, (float)b1, (float)b2, eps, (float)(lr / bc1),
                (float)std::sqrt(bc2), 0);
    if (eval && (ep % eval_every == 0 || ep == epochs - 1)) {
      m16_forward(m, 0);
      mlp16_loss(m.A[m.nl], m.Y, m.sel, 0, n, dout, 1.f / ((float)nval * dout), nullptr, m.rows, m.scal + 1, 0);
      mlp16_keep_best(m.scal + 1, losses + ep, bestd, m.P, Pbest, m.np, 0);
    }
  }
  M_CK(cudaDeviceSynchronize());
  M_CK(cudaGetLastError());
  M_CK(cudaMemcpy(train_loss, losses, epochs * sizeof(float), cudaMemcpyDeviceToHost));
  M_CK(cudaMemcpy(params, m.P, m.np * sizeof(float), cudaMemcpyDeviceToHost));
  if (eval) {
    M_CK(cudaMemcpy(best, bestd, 2 * sizeof(float), cudaMemcpyDeviceToHost));
    M_CK(cudaMemcpy(best_params, Pbest, m.np * sizeof(float), cudaMemcpyDeviceToHost));
  } else {
    if (best) {
      best[0] = NAN;
      best[1] = train_loss[epochs - 1];
    }
    if (best_params) std::memcpy(best_params, params, m.np * sizeof(float));
  }
  return SKKR_OK;
}

// ---- a network kept on the device for repeated inference ------------------
// (the warm start runs it on a few rows per energy: the parameters are
// uploaded once, inference is two small copies and one launch per layer)
struct skkr_mlp16 {
  M16 m;
  int maxrows = 0;
  cudaStream_t st = nullptr;
};

extern "C" int skkr_gpu_mlp16_load(int nlayer, const int *dims, const float *params, int maxrows, skkr_mlp16 **out) {
  if (!params || !out || maxrows < 1) return SKKR_ERR_ARG;
  skkr_mlp16 *h = new skkr_mlp16();
  int rc = m16_sizes(nlayer, dims, maxrows, h->m);
  if (rc == SKKR_OK) {
    std::vector<float> zero((size_t)maxrows * h->m.d[0], 0.f);
    rc = m16_alloc(h->m, params, zero.data(), nullptr, nullptr);
  }
  if (rc == SKKR_OK && cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess) rc = SKKR_ERR_CUDA;
  if (rc == SKKR_OK && cudaDeviceSynchronize() != cudaSuccess) rc = SKKR_ERR_CUDA;
  if (rc != SKKR_OK) {
    if (h->st) cudaStreamDestroy(h->st);
    delete h;
    return rc;
  }
  h->maxrows = maxrows;
  *out = h;
  return SKKR_OK;
}

extern "C" int skkr_gpu_mlp16_infer(skkr_mlp16 *h, int n, const float *x, float *y) {
  if (!h || !x || !y || n < 1 || n > h->maxrows) return SKKR_ERR_ARG;
  M16 &m = h->m;
  const int n0 = m.n;
  m.n = n;  // the first n rows of the buffers sized for maxrows
  M_CK(cudaMemcpyAsync(m.A[0], x, (size_t)n * m.d[0] * sizeof(float), cudaMemcpyHostToDevice, h->st));
  m16_forward(m, h->st);
  M_CK(cudaMemcpyAsync(y, m.A[m.nl], (size_t)n * m.d[m.nl] * sizeof(float), cudaMemcpyDeviceToHost, h->st));
  m.n = n0;
  M_CK(cudaStreamSynchronize(h->st));
  M_CK(cudaGetLastError());
  return SKKR_OK;
}

extern "C" int skkr_gpu_mlp16_free(skkr_mlp16 *h) {
  if (!h) return SKKR_OK;
  cudaStreamSynchronize(h->st);
  cudaStreamDestroy(h->st);
  delete h;  // M16 frees its device buffers
  return SKKR_OK;
}
