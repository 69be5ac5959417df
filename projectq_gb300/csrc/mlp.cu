// Cost-model network: a small MLP (F inputs -> H -> H -> 1, ReLU) with
// hand-written forward, backward and Adam kernels (FP32).  It is trained on
// kernel timings recorded by the engine and predicts the run time of a
// candidate fusion plan; the engine evaluates a host copy of the trained
// weights when it picks a planner (engine.cu, GSIM_FUSION_LEARNED).
//
// Parameter layout (one flat FP32 array):
//   W1[H][F], b1[H], W2[H][H], b2[H], W3[H], b3
// Loss: mean squared error over the batch.  Sizes are tiny (F <= 32,
// H <= 128, batch <= 65536), so every kernel maps one thread to one output
// value and loops over the reduction dimension.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gb300sim.h"

namespace gsim {
extern thread_local std::string g_last_error;
}

namespace {

struct Dims {
  int F, H;
  size_t w1() const { return 0; }
  size_t b1() const { return size_t(H) * F; }
  size_t w2() const { return b1() + H; }
  size_t b2() const { return w2() + size_t(H) * H; }
  size_t w3() const { return b2() + H; }
  size_t b3() const { return w3() + H; }
  size_t count() const { return b3() + 1; }
};

// out[b][o] = act(sum_i W[o][i] x[b][i] + bias[o])
__global__ void dense_fwd(const float *__restrict__ x, const float *__restrict__ W, const float *__restrict__ bias,
                          float *__restrict__ z, float *__restrict__ a, int B, int in, int out, int relu) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * out) return;
  const int b = idx / out, o = idx % out;
  float s = bias[o];
  for (int i = 0; i < in; ++i) s = fmaf(W[o * in + i], x[b * in + i], s);
  z[idx] = s;
  a[idx] = relu ? fmaxf(s, 0.f) : s;
}

// d_in[b][i] = sum_o W[o][i] * d_out[b][o] * (relu' of the input layer's z)
__global__ void dense_bwd_data(const float *__restrict__ dout, const float *__restrict__ W,
                               const float *__restrict__ zin, float *__restrict__ din, int B, int in, int out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= B * in) return;
  const int b = idx / in, i = idx % in;
  float s = 0.f;
  for (int o = 0; o < out; ++o) s = fmaf(W[o * in + i], dout[b * out + o], s);
  din[idx] = zin[idx] > 0.f ? s : 0.f;
}

// gW[o][i] = sum_b d_out[b][o] x[b][i] / B ; gb[o] = sum_b d_out[b][o] / B
__global__ void dense_bwd_weights(const float *__restrict__ dout, const float *__restrict__ x,
                                  float *__restrict__ gW, float *__restrict__ gb, int B, int in, int out) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= out * (in + 1)) return;
  const int o = idx / (in + 1), i = idx % (in + 1);
  double s = 0.;
  if (i < in) {
    for (int b = 0; b < B; ++b) s += double(dout[b * out + o]) * double(x[b * in + i]);
    gW[o * in + i] = float(s / B);
  } else {
    for (int b = 0; b < B; ++b) s += double(dout[b * out + o]);
    gb[o] = float(s / B);
  }
}

// d3[b] = 2 (pred[b] - y[b]) ; loss partial
__global__ void mse_grad(const float *__restrict__ pred, const float *__restrict__ y, float *__restrict__ d,
                         float *__restrict__ sq, int B) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const float e = pred[b] - y[b];
  d[b] = 2.f * e;
  sq[b] = e * e;
}

__global__ void adam_step(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                          float *__restrict__ v, size_t n, float lr, float b1, float b2, float eps, float c1,
                          float c2) {
  const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

struct Net {
  Dims d;
  float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  // activations for a batch of up to cap rows
  int cap = 0;
  float *x = nullptr, *y = nullptr, *z1 = nullptr, *a1 = nullptr, *z2 = nullptr, *a2 = nullptr, *z3 = nullptr,
        *d3 = nullptr, *d2 = nullptr, *d1 = nullptr, *sq = nullptr;
  long step = 0;
};

int err(int code, const std::string &m) {
  gsim::g_last_error = m;
  return code;
}
#define CKM(x)                                                                    \
  do {                                                                            \
    cudaError_t e_ = (x);                                                         \
    if (e_ != cudaSuccess) return err(GSIM_ERR_CUDA, std::string("mlp: ") + cudaGetErrorString(e_)); \
  } while (0)

int ensure_batch(Net *n, int B) {
  if (B <= n->cap) return GSIM_OK;
  float **bufs[] = {&n->x, &n->y, &n->z1, &n->a1, &n->z2, &n->a2, &n->z3, &n->d3, &n->d2, &n->d1, &n->sq};
  for (float **b : bufs)
    if (*b) cudaFree(*b);
  const int F = n->d.F, H = n->d.H;
  const size_t sizes[] = {size_t(B) * F, size_t(B), size_t(B) * H, size_t(B) * H, size_t(B) * H, size_t(B) * H,
                          size_t(B),     size_t(B), size_t(B) * H, size_t(B) * H, size_t(B)};
  for (int i = 0; i < 11; ++i) CKM(cudaMalloc(bufs[i], sizes[i] * sizeof(float)));
  n->cap = B;
  return GSIM_OK;
}

unsigned nb(size_t n) { return unsigned((n + 255) / 256); }

void forward(Net *n, int B) {
  const int F = n->d.F, H = n->d.H;
  const Dims &d = n->d;
  dense_fwd<<<nb(size_t(B) * H), 256>>>(n->x, n->p + d.w1(), n->p + d.b1(), n->z1, n->a1, B, F, H, 1);
  dense_fwd<<<nb(size_t(B) * H), 256>>>(n->a1, n->p + d.w2(), n->p + d.b2(), n->z2, n->a2, B, H, H, 1);
  dense_fwd<<<nb(size_t(B)), 256>>>(n->a2, n->p + d.w3(), n->p + d.b3(), n->z3, n->z3, B, H, 1, 0);
}

void backward(Net *n, int B) {
  const int F = n->d.F, H = n->d.H;
  const Dims &d = n->d;
  mse_grad<<<nb(B), 256>>>(n->z3, n->y, n->d3, n->sq, B);
  dense_bwd_weights<<<nb(size_t(H + 1)), 256>>>(n->d3, n->a2, n->g + d.w3(), n->g + d.b3(), B, H, 1);
  dense_bwd_data<<<nb(size_t(B) * H), 256>>>(n->d3, n->p + d.w3(), n->z2, n->d2, B, H, 1);
  dense_bwd_weights<<<nb(size_t(H) * (H + 1)), 256>>>(n->d2, n->a1, n->g + d.w2(), n->g + d.b2(), B, H, H);
  dense_bwd_data<<<nb(size_t(B) * H), 256>>>(n->d2, n->p + d.w2(), n->z1, n->d1, B, H, H);
  dense_bwd_weights<<<nb(size_t(H) * (F + 1)), 256>>>(n->d1, n->x, n->g + d.w1(), n->g + d.b1(), B, F, H);
}

}  // namespace

extern "C" {

GSIM_API int gsim_mlp_create(int F, int H, uint32_t seed, void **out) {
  if (F < 1 || F > 64 || H < 1 || H > 256) return err(GSIM_ERR_VALUE, "mlp: bad layer sizes");
  Net *n = new Net;
  n->d = Dims{F, H};
  const size_t cnt = n->d.count();
  CKM(cudaMalloc(&n->p, cnt * 4));
  CKM(cudaMalloc(&n->g, cnt * 4));
  CKM(cudaMalloc(&n->m, cnt * 4));
  CKM(cudaMalloc(&n->v, cnt * 4));
  CKM(cudaMemset(n->m, 0, cnt * 4));
  CKM(cudaMemset(n->v, 0, cnt * 4));
  CKM(cudaMemset(n->g, 0, cnt * 4));
  // He-uniform initialisation from a fixed LCG (reproducible across hosts).
  std::vector<float> h(cnt, 0.f);
  uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
  auto uni = [&]() {
    st = st * 6364136223846793005ull + 1442695040888963407ull;
    return float((st >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f;
  };
  const Dims &d = n->d;
  for (size_t i = 0; i < size_t(H) * F; ++i) h[d.w1() + i] = uni() * std::sqrt(6.f / F);
  for (size_t i = 0; i < size_t(H) * H; ++i) h[d.w2() + i] = uni() * std::sqrt(6.f / H);
  for (int i = 0; i < H; ++i) h[d.w3() + i] = uni() * std::sqrt(3.f / H);
  CKM(cudaMemcpy(n->p, h.data(), cnt * 4, cudaMemcpyHostToDevice));
  *out = n;
  return GSIM_OK;
}

GSIM_API int gsim_mlp_destroy(void *h) {
  Net *n = static_cast<Net *>(h);
  if (!n) return GSIM_OK;
  float *bufs[] = {n->p, n->g, n->m, n->v, n->x, n->y, n->z1, n->a1, n->z2, n->a2, n->z3, n->d3, n->d2, n->d1, n->sq};
  for (float *b : bufs)
    if (b) cudaFree(b);
  delete n;
  return GSIM_OK;
}

GSIM_API int gsim_mlp_num_params(void *h, size_t *out) {
  *out = static_cast<Net *>(h)->d.count();
  return GSIM_OK;
}

GSIM_API int gsim_mlp_get_params(void *h, float *out) {
  Net *n = static_cast<Net *>(h);
  CKM(cudaMemcpy(out, n->p, n->d.count() * 4, cudaMemcpyDeviceToHost));
  return GSIM_OK;
}

GSIM_API int gsim_mlp_set_params(void *h, const float *in) {
  Net *n = static_cast<Net *>(h);
  CKM(cudaMemcpy(n->p, in, n->d.count() * 4, cudaMemcpyHostToDevice));
  return GSIM_OK;
}

GSIM_API int gsim_mlp_predict(void *h, const float *X, int B, float *out) {
  Net *n = static_cast<Net *>(h);
  if (B < 1) return err(GSIM_ERR_VALUE, "mlp: empty batch");
  int rc = ensure_batch(n, B);
  if (rc) return rc;
  CKM(cudaMemcpy(n->x, X, size_t(B) * n->d.F * 4, cudaMemcpyHostToDevice));
  forward(n, B);
  CKM(cudaGetLastError());
  CKM(cudaMemcpy(out, n->z3, size_t(B) * 4, cudaMemcpyDeviceToHost));
  return GSIM_OK;
}

// Gradient of the mean squared error at the current parameters (no update).
GSIM_API int gsim_mlp_gradient(void *h, const float *X, const float *y, int B, float *grad, double *loss) {
  Net *n = static_cast<Net *>(h);
  if (B < 1) return err(GSIM_ERR_VALUE, "mlp: empty batch");
  int rc = ensure_batch(n, B);
  if (rc) return rc;
  CKM(cudaMemcpy(n->x, X, size_t(B) * n->d.F * 4, cudaMemcpyHostToDevice));
  CKM(cudaMemcpy(n->y, y, size_t(B) * 4, cudaMemcpyHostToDevice));
  forward(n, B);
  backward(n, B);
  CKM(cudaGetLastError());
  CKM(cudaMemcpy(grad, n->g, n->d.count() * 4, cudaMemcpyDeviceToHost));
  std::vector<float> sq(B);
  CKM(cudaMemcpy(sq.data(), n->sq, size_t(B) * 4, cudaMemcpyDeviceToHost));
  double s = 0.;
  for (float v : sq) s += v;
  *loss = s / B;
  return GSIM_OK;
}

// `epochs` full-batch Adam steps on (X, y); returns the final loss.
GSIM_API int gsim_mlp_train(void *h, const float *X, const float *y, int B, int epochs, float lr, double *loss) {
  Net *n = static_cast<Net *>(h);
  if (B < 1) return err(GSIM_ERR_VALUE, "mlp: empty batch");
  int rc = ensure_batch(n, B);
  if (rc) return rc;
  CKM(cudaMemcpy(n->x, X, size_t(B) * n->d.F * 4, cudaMemcpyHostToDevice));
  CKM(cudaMemcpy(n->y, y, size_t(B) * 4, cudaMemcpyHostToDevice));
  const size_t cnt = n->d.count();
  for (int e = 0; e < epochs; ++e) {
    forward(n, B);
    backward(n, B);
    ++n->step;
    const float c1 = 1.f - std::pow(0.9f, float(n->step)), c2 = 1.f - std::pow(0.999f, float(n->step));
    adam_step<<<nb(cnt), 256>>>(n->p, n->g, n->m, n->v, cnt, lr, 0.9f, 0.999f, 1e-8f, c1, c2);
  }
  CKM(cudaGetLastError());
  forward(n, B);
  mse_grad<<<nb(B), 256>>>(n->z3, n->y, n->d3, n->sq, B);
  std::vector<float> sq(B);
  CKM(cudaMemcpy(sq.data(), n->sq, size_t(B) * 4, cudaMemcpyDeviceToHost));
  double s = 0.;
  for (float v : sq) s += v;
  *loss = s / B;
  return GSIM_OK;
}

}  // extern "C"
