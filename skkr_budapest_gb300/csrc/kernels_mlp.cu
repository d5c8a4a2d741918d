// Dense tanh MLP of the learned CPA warm start: forward, backward and AdamW
// on the device, FP64.  Row-major activations H[n][d]; layer i holds
// W_i[d_i][d_{i+1}] (row-major) and b_i[d_{i+1}], packed W_0, b_0, W_1, ...
// in one parameter array, the gradient array packed the same way.  Every
// reduction runs in a fixed order, so results do not depend on scheduling.
#include "common.cuh"
#include "kernels.h"
#include "mlp_dev.cuh"

namespace {

constexpr int MLP_THREADS = 256;
constexpr int MLP_RED_THREADS = 1024;

int grid_for(long long work) {
  long long g = (work + MLP_THREADS - 1) / MLP_THREADS;
  return (int)(g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g));
}

// A = act(H W + b): one output element per thread, the sum over the inputs
// in index order
__global__ void k_mlp_dense(const double *__restrict__ H, int n, int din, const double *__restrict__ W,
                            const double *__restrict__ b, int dout, int act, double *__restrict__ A) {
  const long long m = (long long)n * dout;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m;
       e += (long long)gridDim.x * blockDim.x)
    mlp_dense_elem(e, H, din, W, b, dout, act, A);
}

// per row: squared error over the outputs for the rows the selection keeps
// (sel == null: all rows), and dY = scale * 2 (Yh - Y) there, 0 elsewhere
__global__ void k_mlp_loss_rows(const double *__restrict__ Yh, const double *__restrict__ Y,
                                const unsigned char *__restrict__ sel, int want, int n, int dout, double scale,
                                double *__restrict__ dY, double *__restrict__ rowsum) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    mlp_loss_row(r, Yh, Y, sel, want, dout, scale, dY, rowsum);
}

// out[0] = scale * sum v[0..n): one block, each thread a strided subset in
// order, then a shared-memory tree
__global__ void k_mlp_sum(const double *__restrict__ v, int n, double scale, double *__restrict__ out) {
  __shared__ double sh[MLP_RED_THREADS];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += v[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = scale * sh[0];
}

// G *= 1 - A^2 (tanh layer)
__global__ void k_mlp_tanh_back(const double *__restrict__ A, double *__restrict__ G, long long m) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m;
       e += (long long)gridDim.x * blockDim.x)
    mlp_tanh_back_elem(e, A, G);
}

// g[p][j] = sum_r H[r][p] dZ[r][j] for p < din (dW), g[din][j] = sum_r dZ[r][j]
// (db): the packed W-then-b gradient of one layer, rows summed in order
__global__ void k_mlp_wgrad(const double *__restrict__ H, const double *__restrict__ dZ, int n, int din,
                            int dout, double *__restrict__ g) {
  const long long m = (long long)(din + 1) * dout;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m;
       e += (long long)gridDim.x * blockDim.x)
    mlp_wgrad_elem(e, H, dZ, n, din, dout, g);
}

// dH[r][p] = sum_j dZ[r][j] W[p][j]
__global__ void k_mlp_hgrad(const double *__restrict__ dZ, const double *__restrict__ W, int n, int din,
                            int dout, double *__restrict__ dH) {
  const long long m = (long long)n * din;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m;
       e += (long long)gridDim.x * blockDim.x)
    mlp_hgrad_elem(e, dZ, W, din, dout, dH);
}

// one AdamW step (decoupled weight decay, bias-corrected moments):
// p *= 1 - lr wd; m += (1 - b1)(g - m); v = b2 v + (1 - b2) g^2;
// p -= (lr / bc1) m / (sqrt(v) / sqrt(bc2) + eps)
__global__ void k_mlp_adamw(double *__restrict__ p, const double *__restrict__ g, double *__restrict__ m,
                            double *__restrict__ v, long long np, double lr, double wd, double b1, double b2,
                            double eps, double step_size, double bc2_sqrt) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < np;
       e += (long long)gridDim.x * blockDim.x)
    mlp_adamw_elem(e, p, g, m, v, lr, wd, b1, b2, eps, step_size, bc2_sqrt);
}

// keep the parameters of the lowest held-out loss: one block; the decision
// is read by every thread before the copy and the update of best
__global__ void k_mlp_keep_best(const double *__restrict__ val, const double *__restrict__ train,
                                double *__restrict__ best, const double *__restrict__ p,
                                double *__restrict__ pbest, long long np) {
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

}  // namespace

void mlp_launch_dense(const double *H, int n, int din, const double *W, const double *b, int dout, int act,
                      double *A, cudaStream_t st) {
  k_mlp_dense<<<grid_for((long long)n * dout), MLP_THREADS, 0, st>>>(H, n, din, W, b, dout, act, A);
  SKKR_LAUNCHED();
}

void mlp_launch_loss(const double *Yh, const double *Y, const unsigned char *sel, int want, int n, int dout,
                     double scale, double *dY, double *rowsum, double *out, cudaStream_t st) {
  k_mlp_loss_rows<<<grid_for(n), MLP_THREADS, 0, st>>>(Yh, Y, sel, want, n, dout, scale, dY, rowsum);
  SKKR_LAUNCHED();
  k_mlp_sum<<<1, MLP_RED_THREADS, 0, st>>>(rowsum, n, scale, out);
  SKKR_LAUNCHED();
}

void mlp_launch_tanh_back(const double *A, double *G, long long m, cudaStream_t st) {
  k_mlp_tanh_back<<<grid_for(m), MLP_THREADS, 0, st>>>(A, G, m);
  SKKR_LAUNCHED();
}

void mlp_launch_wgrad(const double *H, const double *dZ, int n, int din, int dout, double *g, cudaStream_t st) {
  k_mlp_wgrad<<<grid_for((long long)(din + 1) * dout), MLP_THREADS, 0, st>>>(H, dZ, n, din, dout, g);
  SKKR_LAUNCHED();
}

void mlp_launch_hgrad(const double *dZ, const double *W, int n, int din, int dout, double *dH, cudaStream_t st) {
  k_mlp_hgrad<<<grid_for((long long)n * din), MLP_THREADS, 0, st>>>(dZ, W, n, din, dout, dH);
  SKKR_LAUNCHED();
}

void mlp_launch_adamw(double *p, const double *g, double *m, double *v, long long np, double lr, double wd,
                      double b1, double b2, double eps, double step_size, double bc2_sqrt, cudaStream_t st) {
  k_mlp_adamw<<<grid_for(np), MLP_THREADS, 0, st>>>(p, g, m, v, np, lr, wd, b1, b2, eps, step_size, bc2_sqrt);
  SKKR_LAUNCHED();
}

void mlp_launch_keep_best(const double *val, const double *train, double *best, const double *p, double *pbest,
                          long long np, cudaStream_t st) {
  k_mlp_keep_best<<<1, MLP_RED_THREADS, 0, st>>>(val, train, best, p, pbest, np);
  SKKR_LAUNCHED();
}
