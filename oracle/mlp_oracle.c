/*
 * mlp_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * FP64 restatement of the variant selector's network (12 -> 64 -> 64 -> 64 ->
 * nout, ReLU on hidden layers) and of its masked mean-squared-error loss and
 * gradient, written directly from the definitions (plain backpropagation).  The
 * reference has no learned selector (it sweeps generated variants offline,
 * generated_kernels/codegen.py:44-247), so this pins the library's own training
 * kernels: tests compare their FP32 gradients with these.  Only tests/ load it.
 *
 * Parameters: one flat array, layer by layer, W (K x N row-major) then b (N).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_API __attribute__((visibility("default")))
#define MLP_IN 12
#define MLP_HID 64
#define MLP_LAYERS 4

static void mlp_dims(int nout, int* K, int* N) {
  const int k[MLP_LAYERS] = {MLP_IN, MLP_HID, MLP_HID, MLP_HID};
  const int n[MLP_LAYERS] = {MLP_HID, MLP_HID, MLP_HID, nout};
  for (int l = 0; l < MLP_LAYERS; l++) { K[l] = k[l]; N[l] = n[l]; }
}

ORACLE_API int64_t oracle_mlp_num_params(int nout) {
  int K[MLP_LAYERS], N[MLP_LAYERS];
  mlp_dims(nout, K, N);
  int64_t n = 0;
  for (int l = 0; l < MLP_LAYERS; l++) n += (int64_t)K[l] * N[l] + N[l];
  return n;
}

/* acts[l]: B x N[l] outputs of layer l (post-ReLU for hidden layers). */
static void mlp_forward(const double* p, int nout, const double* X, int B, double** acts) {
  int K[MLP_LAYERS], N[MLP_LAYERS];
  mlp_dims(nout, K, N);
  const double* in = X;
  int64_t off = 0;
  for (int l = 0; l < MLP_LAYERS; l++) {
    const double* W = p + off;
    const double* b = W + (int64_t)K[l] * N[l];
    for (int r = 0; r < B; r++)
      for (int n = 0; n < N[l]; n++) {
        double acc = b[n];
        for (int k = 0; k < K[l]; k++) acc += in[(int64_t)r * K[l] + k] * W[(int64_t)k * N[l] + n];
        if (l + 1 < MLP_LAYERS && acc < 0.0) acc = 0.0;
        acts[l][(int64_t)r * N[l] + n] = acc;
      }
    in = acts[l];
    off += (int64_t)K[l] * N[l] + N[l];
  }
}

ORACLE_API void oracle_mlp_forward(const double* p, int nout, const double* X, int B, double* out) {
  double* acts[MLP_LAYERS];
  for (int l = 0; l < MLP_LAYERS; l++) acts[l] = (double*)malloc(sizeof(double) * (size_t)B * (l + 1 < MLP_LAYERS ? MLP_HID : nout));
  mlp_forward(p, nout, X, B, acts);
  memcpy(out, acts[MLP_LAYERS - 1], sizeof(double) * (size_t)B * nout);
  for (int l = 0; l < MLP_LAYERS; l++) free(acts[l]);
}

/* loss = sum M (O - T)^2 / sum M and its gradient with respect to every parameter. */
ORACLE_API void oracle_mlp_grad(const double* p, int nout, const double* X, int B, const double* T,
                                const double* M, double* grads, double* loss) {
  int K[MLP_LAYERS], N[MLP_LAYERS];
  mlp_dims(nout, K, N);
  double* acts[MLP_LAYERS];
  for (int l = 0; l < MLP_LAYERS; l++) acts[l] = (double*)malloc(sizeof(double) * (size_t)B * N[l]);
  mlp_forward(p, nout, X, B, acts);
  const int64_t no = (int64_t)B * nout;
  double cnt = 0.0, sq = 0.0;
  for (int64_t i = 0; i < no; i++)
    if (M[i] != 0.0) {
      const double d = acts[MLP_LAYERS - 1][i] - T[i];
      sq += d * d;
      cnt += 1.0;
    }
  if (cnt == 0.0) cnt = 1.0;
  *loss = sq / cnt;
  double* dz = (double*)malloc(sizeof(double) * (size_t)B * (nout > MLP_HID ? nout : MLP_HID));
  double* dx = (double*)malloc(sizeof(double) * (size_t)B * (nout > MLP_HID ? nout : MLP_HID));
  for (int64_t i = 0; i < no; i++) dz[i] = M[i] != 0.0 ? 2.0 * (acts[MLP_LAYERS - 1][i] - T[i]) / cnt : 0.0;
  int64_t offs[MLP_LAYERS + 1];
  offs[0] = 0;
  for (int l = 0; l < MLP_LAYERS; l++) offs[l + 1] = offs[l] + (int64_t)K[l] * N[l] + N[l];
  for (int l = MLP_LAYERS - 1; l >= 0; l--) {
    const double* Xl = l > 0 ? acts[l - 1] : X;
    const double* W = p + offs[l];
    double* dW = grads + offs[l];
    double* db = dW + (int64_t)K[l] * N[l];
    if (l + 1 < MLP_LAYERS)
      for (int64_t i = 0; i < (int64_t)B * N[l]; i++)
        if (!(acts[l][i] > 0.0)) dz[i] = 0.0;
    for (int k = 0; k < K[l]; k++)
      for (int n = 0; n < N[l]; n++) {
        double acc = 0.0;
        for (int r = 0; r < B; r++) acc += Xl[(int64_t)r * K[l] + k] * dz[(int64_t)r * N[l] + n];
        dW[(int64_t)k * N[l] + n] = acc;
      }
    for (int n = 0; n < N[l]; n++) {
      double acc = 0.0;
      for (int r = 0; r < B; r++) acc += dz[(int64_t)r * N[l] + n];
      db[n] = acc;
    }
    if (l > 0) {
      for (int r = 0; r < B; r++)
        for (int k = 0; k < K[l]; k++) {
          double acc = 0.0;
          for (int n = 0; n < N[l]; n++) acc += dz[(int64_t)r * N[l] + n] * W[(int64_t)k * N[l] + n];
          dx[(int64_t)r * K[l] + k] = acc;
        }
      double* t = dz;
      dz = dx;
      dx = t;
    }
  }
  free(dz);
  free(dx);
  for (int l = 0; l < MLP_LAYERS; l++) free(acts[l]);
}
