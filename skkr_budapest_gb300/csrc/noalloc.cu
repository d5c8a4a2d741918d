// Decimation (main/surfgf.f) for callers that cannot allocate device memory.
//
// Some host programs may not call cudaMalloc at all: a Fortran code whose
// device memory is owned by another layer (an OpenACC / CUDA Fortran data
// region, a pool allocator of the surrounding application), work issued
// while another library holds the allocator, or a memory budget fixed up
// front on a shared GPU.  They pass their own device buffers for inputs and
// outputs; the work matrices this routine needs live in one file-scope
// device array of fixed size (SKKR_NOALLOC_SCRATCH_BYTES), which every GPU
// that loads the library holds until the process exits.
#include <atomic>

#include "../../include/skkr_gpu.h"
#include "kernels.h"

static __device__ __align__(256) unsigned char g_sgf_scratch[SKKR_NOALLOC_SCRATCH_BYTES];

// Device address of g_sgf_scratch per device ordinal, looked up by the first
// call on that device (with the device current) and kept.  In host code the
// name g_sgf_scratch is only a host-side stand-in, never a device pointer.
// Calls may come from several host threads: the cached address is atomic
// (two threads that both find it empty look up the same value).
static std::atomic<void *> g_scratch_addr[128];

static int scratch_address(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 128) return SKKR_ERR_CUDA;
  void *p = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!p) {
    e = cudaGetSymbolAddress(&p, g_sgf_scratch);
    if (e != cudaSuccess || !p) return SKKR_ERR_CUDA;
    g_scratch_addr[dev].store(p, std::memory_order_release);
  }
  *out = p;
  return SKKR_OK;
}

__global__ void k_noalloc_init(int *act, int *stat, int *iters, int *count, int nb) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
    act[i] = 1;
    stat[i] = 0;
    iters[i] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *count = nb;
}

__global__ void k_noalloc_count(const int *act, int nb, int *count) {
  __shared__ int s[256];
  int v = 0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) v += act[i];
  s[threadIdx.x] = v;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *count = s[0];
}

#define NA_CK(x)                           \
  do {                                     \
    if ((x) != cudaSuccess) {              \
      skkr_set_active_items(-1);           \
      return SKKR_ERR_CUDA;                \
    }                                      \
  } while (0)

extern "C" int skkr_gpu_surfgf_batch_noalloc(int n, int batch, const double *ml, const double *m0,
                                             const double *mr, double *x, int ld, int itermax,
                                             double errmax, int *iters, int *stat, void *stream) {
  // the batched kernels put the item index in grid.y (at most 65535)
  if (n < 1 || n > 256 || batch < 1 || batch > 65535 || !ml || !m0 || !mr || !x || ld < n || itermax < 1)
    return SKKR_ERR_ARG;
  const size_t MB = (size_t)n * n;
  // scratch: 8 work matrices per item, then err[batch], act/stat/iters[batch], count
  const size_t mats = (size_t)batch * 8 * MB * sizeof(zd);
  const size_t need = mats + (size_t)batch * sizeof(double) + (size_t)batch * 3 * sizeof(int) + 64;
  if (need > SKKR_NOALLOC_SCRATCH_BYTES) return SKKR_ERR_NOMEM;  // over the static scratch
  void *base = nullptr;
  int rc = scratch_address(&base);
  if (rc != SKKR_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  zd *W = (zd *)base;
  double *err = (double *)((char *)base + mats);
  int *act = (int *)(err + batch), *sta = act + batch, *itr = sta + batch, *count = itr + batch;
  auto buf = [&](int b) { return mref(W + (long long)b * MB, 8LL * MB, 0, n); };
  const long long lds = (long long)ld * ld;
  MatRef Ml = mref((zd *)ml, lds, 0, ld), M0 = mref((zd *)m0, lds, 0, ld), Mr = mref((zd *)mr, lds, 0, ld);
  MatRef X = mref((zd *)x, lds, 0, ld);
  MatRef eps = buf(0), a0 = buf(1), a1 = buf(2), b0 = buf(3), b1 = buf(4), y1 = buf(5), P = buf(6), Q = buf(7);
  // every call starts from cleared flags: the scratch keeps the previous call's contents
  k_noalloc_init<<<(batch + 255) / 256, 256, 0, st>>>(act, sta, itr, count, batch);
  NA_CK(cudaGetLastError());
  // surfgf.f:37-45
  launch_zaxpby(eps, M0, nullptr, 0, nullptr, 0, n, batch, 1, nullptr, st);
  launch_zaxpby(X, M0, nullptr, 0, nullptr, 0, n, batch, 1, nullptr, st);
  launch_zaxpby(a0, Ml, &Ml, -2.0, nullptr, 0, n, batch, 1, nullptr, st);
  launch_zaxpby(b0, Mr, &Mr, -2.0, nullptr, 0, n, batch, 1, nullptr, st);
  long long active = batch;
  skkr_set_active_items(active);
  for (int iter = 1;; iter++) {
    MatRef &ac = (iter & 1) ? a0 : a1, &an = (iter & 1) ? a1 : a0;
    MatRef &bc = (iter & 1) ? b0 : b1, &bn = (iter & 1) ? b1 : b0;
    launch_zaxpby(y1, eps, nullptr, 0, nullptr, 0, n, batch, 1, act, st);
    launch_zgj(y1, n, batch, 1, act, st);
    launch_zgemm(0, ac, y1, P, P, P, n, n, n, batch, 1, act, st);
    launch_zgemm(0, bc, y1, Q, Q, Q, n, n, n, batch, 1, act, st);
    launch_zgemm(0, P, ac, an, an, an, n, n, n, batch, 1, act, st);
    launch_zgemm(0, Q, bc, bn, bn, bn, n, n, n, batch, 1, act, st);
    launch_zgemm(2, P, bc, P, eps, X, n, n, n, batch, 1, act, st);
    launch_zgemm(1, Q, ac, eps, eps, eps, n, n, n, batch, 1, act, st);
    launch_fnorm(an, n, batch, 1, act, err, st);
    launch_dec_state(err, act, sta, itr, batch, iter, itermax, errmax, st);
    k_noalloc_count<<<1, 256, 0, st>>>(act, batch, count);
    int h = 0;
    NA_CK(cudaMemcpyAsync(&h, count, sizeof(int), cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    active = h;
    skkr_set_active_items(active);
    // k_dec_state retires every item once iter > itermax, so the count
    // reaches zero by iteration itermax + 1 at the latest
    if (h == 0) break;
  }
  skkr_set_active_items(-1);
  launch_zgj(X, n, batch, 1, nullptr, st);
  if (iters) NA_CK(cudaMemcpyAsync(iters, itr, batch * sizeof(int), cudaMemcpyDeviceToHost, st));
  if (stat) NA_CK(cudaMemcpyAsync(stat, sta, batch * sizeof(int), cudaMemcpyDeviceToHost, st));
  NA_CK(cudaStreamSynchronize(st));
  NA_CK(cudaGetLastError());
  return SKKR_OK;
}
