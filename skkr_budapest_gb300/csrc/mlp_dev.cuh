// Element logic of the warm-start network's kernels (kernels_mlp.cu), for
// host and device code: row-major activations H[n][d], W[din][dout]
// row-major, the packed W-then-b gradient of a layer.
#pragma once
#include <math.h>

#if !defined(__CUDACC__)
#define SKKR_MLP_HD
#else
#define SKKR_MLP_HD __host__ __device__
#endif

// A[e] = act(sum_i H[r][i] W[i][j] + b[j]), e = r dout + j
SKKR_MLP_HD inline void mlp_dense_elem(long long e, const double *H, int din, const double *W, const double *b,
                                       int dout, int act, double *A) {
  const long long r = e / dout;
  const int j = (int)(e - r * dout);
  const double *h = H + r * din;
  double s = b[j];
  for (int i = 0; i < din; i++) s = fma(h[i], W[(long long)i * dout + j], s);
  A[e] = act ? tanh(s) : s;
}

// row r: rowsum = squared error if the row is selected, dY = scale 2 (Yh - Y) there (0 elsewhere)
SKKR_MLP_HD inline void mlp_loss_row(int r, const double *Yh, const double *Y, const unsigned char *sel, int want,
                                     int dout, double scale, double *dY, double *rowsum) {
  const bool on = sel ? (sel[r] == want) : true;
  double s = 0.0;
  for (int j = 0; j < dout; j++) {
    const long long e = (long long)r * dout + j;
    const double d = Yh[e] - Y[e];
    s = fma(d, d, s);
    if (dY) dY[e] = on ? scale * 2.0 * d : 0.0;
  }
  rowsum[r] = on ? s : 0.0;
}

SKKR_MLP_HD inline void mlp_tanh_back_elem(long long e, const double *A, double *G) {
  const double a = A[e];
  G[e] *= 1.0 - a * a;
}

// g[e], e = p dout + j: sum_r H[r][p] dZ[r][j] (p < din), sum_r dZ[r][j] (p = din)
SKKR_MLP_HD inline void mlp_wgrad_elem(long long e, const double *H, const double *dZ, int n, int din, int dout,
                                       double *g) {
  const int p = (int)(e / dout), j = (int)(e - (long long)p * dout);
  double s = 0.0;
  if (p < din) {
    for (int r = 0; r < n; r++) s = fma(H[(long long)r * din + p], dZ[(long long)r * dout + j], s);
  } else {
    for (int r = 0; r < n; r++) s += dZ[(long long)r * dout + j];
  }
  g[e] = s;
}

// dH[e], e = r din + p: sum_j dZ[r][j] W[p][j]
SKKR_MLP_HD inline void mlp_hgrad_elem(long long e, const double *dZ, const double *W, int din, int dout,
                                       double *dH) {
  const long long r = e / din;
  const int p = (int)(e - r * din);
  const double *dz = dZ + r * dout;
  const double *w = W + (long long)p * dout;
  double s = 0.0;
  for (int j = 0; j < dout; j++) s = fma(dz[j], w[j], s);
  dH[e] = s;
}

// one AdamW step of parameter e
SKKR_MLP_HD inline void mlp_adamw_elem(long long e, double *p, const double *g, double *m, double *v, double lr,
                                       double wd, double b1, double b2, double eps, double step_size,
                                       double bc2_sqrt) {
  const double ge = g[e];
  const double pe = p[e] * (1.0 - lr * wd);
  const double me = m[e] + (1.0 - b1) * (ge - m[e]);
  const double ve = v[e] * b2 + (1.0 - b2) * ge * ge;
  m[e] = me;
  v[e] = ve;
  p[e] = pe + (-step_size) * (me / (sqrt(ve) / bc2_sqrt + eps));
}
