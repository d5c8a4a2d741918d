// Host build of the warm-start network's element logic (mlp_dev.cuh), driven
// in the order and with the packing of skkr_gpu_mlp_grad / skkr_gpu_mlp_train:
// per layer the dense products, the loss rows and their sum, then from the
// last layer down tanh', the packed W-then-b gradient and the activation
// gradient, and one AdamW step over the packed parameters.
#include <vector>
#include "../../skkr_budapest_gb300/csrc/mlp_dev.cuh"

extern "C" void mlp_grad_eval(int nl, const int *d, const double *P, int n, const double *x, const double *y,
                              const unsigned char *rows, double *loss, double *G) {
  std::vector<long long> off(nl);
  long long np = 0;
  int dmax = 0;
  for (int i = 0; i <= nl; i++) dmax = d[i] > dmax ? d[i] : dmax;
  for (int i = 0; i < nl; i++) {
    off[i] = np;
    np += (long long)d[i] * d[i + 1] + d[i + 1];
  }
  std::vector<std::vector<double>> A(nl + 1);
  A[0].assign(x, x + (size_t)n * d[0]);
  for (int i = 0; i < nl; i++) {
    A[i + 1].resize((size_t)n * d[i + 1]);
    for (long long e = 0; e < (long long)n * d[i + 1]; e++)
      mlp_dense_elem(e, A[i].data(), d[i], P + off[i], P + off[i] + (long long)d[i] * d[i + 1], d[i + 1],
                     i < nl - 1, A[i + 1].data());
  }
  int nsel = 0;
  for (int r = 0; r < n; r++) nsel += rows ? rows[r] == 1 : 1;
  const int dout = d[nl];
  const double scale = 1.0 / ((double)nsel * dout);
  std::vector<double> buf0((size_t)n * dmax), buf1((size_t)n * dmax), rs(n);
  for (int r = 0; r < n; r++) mlp_loss_row(r, A[nl].data(), y, rows, 1, dout, scale, buf0.data(), rs.data());
  double s = 0.0;
  for (int r = 0; r < n; r++) s += rs[r];
  *loss = scale * s;
  double *cur = buf0.data(), *nxt = buf1.data();
  for (int i = nl - 1; i >= 0; i--) {
    if (i < nl - 1)
      for (long long e = 0; e < (long long)n * d[i + 1]; e++) mlp_tanh_back_elem(e, A[i + 1].data(), cur);
    for (long long e = 0; e < (long long)(d[i] + 1) * d[i + 1]; e++)
      mlp_wgrad_elem(e, A[i].data(), cur, n, d[i], d[i + 1], G + off[i]);
    if (i > 0) {
      for (long long e = 0; e < (long long)n * d[i]; e++)
        mlp_hgrad_elem(e, cur, P + off[i], d[i], d[i + 1], nxt);
      double *t = cur;
      cur = nxt;
      nxt = t;
    }
  }
}

extern "C" void mlp_adamw_eval(long long np, double *p, const double *g, double *m, double *v, double lr, double wd,
                               double step_size, double bc2_sqrt) {
  for (long long e = 0; e < np; e++) mlp_adamw_elem(e, p, g, m, v, lr, wd, 0.9, 0.999, 1e-8, step_size, bc2_sqrt);
}
