// zg_mlp.cu — the learned error-latency profile's network: 16 features -> 64 -> 64 (GELU) -> 2
// (log per-sample relative variance, log per-sample latency), BF16 weights, FP32 accumulation.
//
// Training runs in one kernel per call: a single CTA of 256 threads keeps the BF16 working
// weights and a minibatch's activations in shared memory and executes forward, backward and Adam
// for every step (the network has 5378 parameters; a step is ~1 MFLOP, so one CTA is the right
// size and no launch per step is needed).  FP32 master weights and Adam moments live in global
// memory; each step re-derives the BF16 copy from the master (round to nearest even).  The same
// device code computes one batch's gradient without updating (zg_mlp_grad) for the gradient check.
// Inference (zg_mlp_predict) is one thread per row.
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "zg_internal.cuh"

namespace {

constexpr int IN = 16, H = 64, OUT = 2;
constexpr int OW1 = 0, OB1 = OW1 + H * IN, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H, OB3 = OW3 + OUT * H;
constexpr int NP = OB3 + OUT;  // 5378 parameters
constexpr int kT = 256;        // threads of the training CTA
constexpr int kMaxB = 64;      // rows per minibatch

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.0f + erff(z * 0.70710678118654752f)) + z * 0.39894228040143268f * expf(-0.5f * z * z);
}

struct Smem {
  __nv_bfloat16 w[NP];
  float x[kMaxB][IN];
  float t[kMaxB][OUT];
  float z1[kMaxB][H], h1[kMaxB][H], z2[kMaxB][H], h2[kMaxB][H];
  float dz1[kMaxB][H], dz2[kMaxB][H];
  float y[kMaxB][OUT], dy[kMaxB][OUT];
  float red[kT / 32];
};

__device__ __forceinline__ float wv(const Smem& s, int i) { return __bfloat162float(s.w[i]); }

// One step on rows[0..B): forward, loss, backward; then either Adam on master/m/v or the raw
// gradient into grad_out.  Returns the minibatch loss (mean squared error over B x OUT).
__device__ float mlp_step(Smem& s, const float* __restrict__ X, const float* __restrict__ Y,
                          const uint32_t* __restrict__ rows, int B, float* __restrict__ master, float* __restrict__ m,
                          float* __restrict__ v, float lr, float beta1, float beta2, float eps, uint32_t t_step,
                          float* __restrict__ grad_out) {
  const int tid = threadIdx.x;
  for (int i = tid; i < NP; i += kT) s.w[i] = __float2bfloat16_rn(master[i]);
  for (int i = tid; i < B * IN; i += kT) s.x[i / IN][i % IN] = X[(size_t)rows[i / IN] * IN + i % IN];
  for (int i = tid; i < B * OUT; i += kT) s.t[i / OUT][i % OUT] = Y[(size_t)rows[i / OUT] * OUT + i % OUT];
  __syncthreads();
  // layer 1
  for (int i = tid; i < B * H; i += kT) {
    int b = i / H, j = i % H;
    float z = wv(s, OB1 + j);
    for (int k = 0; k < IN; ++k) z = fmaf(wv(s, OW1 + j * IN + k), s.x[b][k], z);
    s.z1[b][j] = z;
    s.h1[b][j] = gelu(z);
  }
  __syncthreads();
  // layer 2
  for (int i = tid; i < B * H; i += kT) {
    int b = i / H, j = i % H;
    float z = wv(s, OB2 + j);
    for (int k = 0; k < H; ++k) z = fmaf(wv(s, OW2 + j * H + k), s.h1[b][k], z);
    s.z2[b][j] = z;
    s.h2[b][j] = gelu(z);
  }
  __syncthreads();
  // output layer and loss gradient
  float lsum = 0.f;
  for (int i = tid; i < B * OUT; i += kT) {
    int b = i / OUT, o = i % OUT;
    float y = wv(s, OB3 + o);
    for (int k = 0; k < H; ++k) y = fmaf(wv(s, OW3 + o * H + k), s.h2[b][k], y);
    s.y[b][o] = y;
    float d = y - s.t[b][o];
    lsum += d * d;
    s.dy[b][o] = 2.0f * d / (float)(B * OUT);
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if ((tid & 31) == 0) s.red[tid >> 5] = lsum;
  __syncthreads();
  float loss = 0.f;
  for (int w = 0; w < kT / 32; ++w) loss += s.red[w];
  loss /= (float)(B * OUT);
  // dz2 = (dy W3) * gelu'(z2)
  for (int i = tid; i < B * H; i += kT) {
    int b = i / H, k = i % H;
    float d = 0.f;
    for (int o = 0; o < OUT; ++o) d = fmaf(s.dy[b][o], wv(s, OW3 + o * H + k), d);
    s.dz2[b][k] = d * gelu_grad(s.z2[b][k]);
  }
  __syncthreads();
  // dz1 = (dz2 W2) * gelu'(z1)
  for (int i = tid; i < B * H; i += kT) {
    int b = i / H, k = i % H;
    float d = 0.f;
    for (int j = 0; j < H; ++j) d = fmaf(s.dz2[b][j], wv(s, OW2 + j * H + k), d);
    s.dz1[b][k] = d * gelu_grad(s.z1[b][k]);
  }
  __syncthreads();
  // parameter gradients, then Adam (or export)
  const float bc1 = 1.0f - powf(beta1, (float)t_step), bc2 = 1.0f - powf(beta2, (float)t_step);
  for (int p = tid; p < NP; p += kT) {
    float g = 0.f;
    if (p < OB1) {
      int j = p / IN, k = p % IN;
      for (int b = 0; b < B; ++b) g = fmaf(s.dz1[b][j], s.x[b][k], g);
    } else if (p < OW2) {
      int j = p - OB1;
      for (int b = 0; b < B; ++b) g += s.dz1[b][j];
    } else if (p < OB2) {
      int j = (p - OW2) / H, k = (p - OW2) % H;
      for (int b = 0; b < B; ++b) g = fmaf(s.dz2[b][j], s.h1[b][k], g);
    } else if (p < OW3) {
      int j = p - OB2;
      for (int b = 0; b < B; ++b) g += s.dz2[b][j];
    } else if (p < OB3) {
      int o = (p - OW3) / H, k = (p - OW3) % H;
      for (int b = 0; b < B; ++b) g = fmaf(s.dy[b][o], s.h2[b][k], g);
    } else {
      int o = p - OB3;
      for (int b = 0; b < B; ++b) g += s.dy[b][o];
    }
    if (grad_out) {
      grad_out[p] = g;
    } else {
      float mm = beta1 * m[p] + (1.0f - beta1) * g;
      float vv = beta2 * v[p] + (1.0f - beta2) * g * g;
      m[p] = mm;
      v[p] = vv;
      master[p] -= lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
    }
  }
  __syncthreads();
  return loss;
}

__global__ void __launch_bounds__(kT) k_mlp_train(const float* __restrict__ X, const float* __restrict__ Y,
                                                  const uint32_t* __restrict__ order, uint32_t n_rows, uint32_t steps,
                                                  uint32_t batch, float lr, uint32_t step0, float* __restrict__ master,
                                                  float* __restrict__ m, float* __restrict__ v,
                                                  float* __restrict__ loss_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem& s = *reinterpret_cast<Smem*>(smem_raw);
  for (uint32_t st = 0; st < steps; ++st) {
    const uint32_t* rows = order + (uint64_t)st * batch;
    float loss = mlp_step(s, X, Y, rows, (int)batch, master, m, v, lr, 0.9f, 0.999f, 1e-8f, step0 + st + 1, nullptr);
    if (threadIdx.x == 0 && loss_out) loss_out[st] = loss;
  }
}

__global__ void __launch_bounds__(kT) k_mlp_grad(const float* __restrict__ X, const float* __restrict__ Y,
                                                 const uint32_t* __restrict__ rows, uint32_t B,
                                                 float* __restrict__ master, float* __restrict__ grad,
                                                 float* __restrict__ loss_out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem& s = *reinterpret_cast<Smem*>(smem_raw);
  float loss = mlp_step(s, X, Y, rows, (int)B, master, nullptr, nullptr, 0.f, 0.9f, 0.999f, 1e-8f, 1, grad);
  if (threadIdx.x == 0) *loss_out = loss;
}

__global__ void k_mlp_predict(const float* __restrict__ X, uint32_t n, const float* __restrict__ master,
                              float* __restrict__ Yout) {
  __shared__ __nv_bfloat16 w[NP];
  for (int i = threadIdx.x; i < NP; i += blockDim.x) w[i] = __float2bfloat16_rn(master[i]);
  __syncthreads();
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    float x[IN], h1[H];
    for (int k = 0; k < IN; ++k) x[k] = X[(size_t)r * IN + k];
    for (int j = 0; j < H; ++j) {
      float z = __bfloat162float(w[OB1 + j]);
      for (int k = 0; k < IN; ++k) z = fmaf(__bfloat162float(w[OW1 + j * IN + k]), x[k], z);
      h1[j] = gelu(z);
    }
    float y[OUT];
    for (int o = 0; o < OUT; ++o) y[o] = __bfloat162float(w[OB3 + o]);
    for (int j = 0; j < H; ++j) {
      float z = __bfloat162float(w[OB2 + j]);
      for (int k = 0; k < H; ++k) z = fmaf(__bfloat162float(w[OW2 + j * H + k]), h1[k], z);
      float h2 = gelu(z);
      for (int o = 0; o < OUT; ++o) y[o] = fmaf(__bfloat162float(w[OW3 + o * H + j]), h2, y[o]);
    }
    for (int o = 0; o < OUT; ++o) Yout[(size_t)r * OUT + o] = y[o];
  }
}

int smem_bytes() { return (int)sizeof(Smem); }

int ensure_smem() {
  static bool done = false;
  if (done) return ZG_OK;
  ZG_CUDA(cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes()));
  ZG_CUDA(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes()));
  done = true;
  return ZG_OK;
}

}  // namespace

struct zg_mlp {
  float* master;
  float* m;
  float* v;
  uint32_t step;
  float norm[2 * IN + 2 * OUT];  // x mean, x std, y mean, y std (host side)
};

extern "C" int zg_mlp_num_params(void) { return NP; }

// Xavier-uniform weights from Philox (seeded), zero biases.
extern "C" int zg_mlp_create(uint64_t seed, zg_mlp** out) {
  if (!out) return zg_set_error(ZG_ERR_INVALID_ARG, "null output"), ZG_ERR_INVALID_ARG;
  std::vector<float> h(NP, 0.f);
  auto fill = [&](int off, int fan_out, int fan_in) {
    float a = sqrtf(6.0f / (float)(fan_in + fan_out));
    for (int i = 0; i < fan_out * fan_in; ++i) {
      uint64_t r = zg_draw(seed, 0x4D4C5000u, (uint64_t)off + i, 0, 0, ~0ull);
      double u = (double)(r >> 11) * 0x1p-53;
      h[off + i] = (float)((2.0 * u - 1.0) * a);
    }
  };
  fill(OW1, H, IN);
  fill(OW2, H, H);
  fill(OW3, OUT, H);
  zg_mlp* p = new zg_mlp();
  memset(p, 0, sizeof(*p));
  for (int i = 0; i < IN; ++i) p->norm[IN + i] = 1.f;
  for (int i = 0; i < OUT; ++i) p->norm[2 * IN + OUT + i] = 1.f;
  cudaError_t e = cudaMalloc((void**)&p->master, sizeof(float) * NP * 3);
  if (e != cudaSuccess) {
    delete p;
    return zg_check_cuda(e, "mlp alloc");
  }
  p->m = p->master + NP;
  p->v = p->master + 2 * NP;
  e = cudaMemcpy(p->master, h.data(), sizeof(float) * NP, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(p->m, 0, sizeof(float) * NP * 2);
  if (e != cudaSuccess) {
    cudaFree(p->master);
    delete p;
    return zg_check_cuda(e, "mlp init");
  }
  *out = p;
  return ZG_OK;
}

extern "C" int zg_mlp_free(zg_mlp* p) {
  if (!p) return ZG_OK;
  if (p->master) cudaFree(p->master);
  delete p;
  return ZG_OK;
}

extern "C" int zg_mlp_get_params(const zg_mlp* p, float* params, float* norm) {
  if (!p) return zg_set_error(ZG_ERR_INVALID_ARG, "null mlp"), ZG_ERR_INVALID_ARG;
  if (params) ZG_CUDA(cudaMemcpy(params, p->master, sizeof(float) * NP, cudaMemcpyDeviceToHost));
  if (norm) memcpy(norm, p->norm, sizeof(p->norm));
  return ZG_OK;
}

extern "C" int zg_mlp_set_params(zg_mlp* p, const float* params, const float* norm) {
  if (!p) return zg_set_error(ZG_ERR_INVALID_ARG, "null mlp"), ZG_ERR_INVALID_ARG;
  if (params) {
    ZG_CUDA(cudaMemcpy(p->master, params, sizeof(float) * NP, cudaMemcpyHostToDevice));
    ZG_CUDA(cudaMemset(p->m, 0, sizeof(float) * NP * 2));
    p->step = 0;
  }
  if (norm) memcpy(p->norm, norm, sizeof(p->norm));
  return ZG_OK;
}

// Trains on (X, Y) given raw (un-normalised) features/targets: normalisation statistics are taken
// from this data and kept in the model.  epochs over the rows in a seeded shuffled order,
// minibatches of `batch` (<= 64) rows, Adam(lr, 0.9, 0.999, 1e-8).  loss_history: one entry per
// step (may be NULL).
extern "C" int zg_mlp_train(zg_mlp* p, const float* X, const float* Y, uint32_t n_rows, uint32_t epochs,
                            uint32_t batch, float lr, uint64_t seed, float* loss_history) {
  if (!p || !X || !Y || n_rows == 0 || batch == 0 || batch > kMaxB)
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_mlp_train: invalid argument (batch <= %d)", kMaxB), ZG_ERR_INVALID_ARG;
  int rc = ensure_smem();
  if (rc) return rc;
  // normalisation
  std::vector<float> xn((size_t)n_rows * IN), yn((size_t)n_rows * OUT);
  for (int k = 0; k < IN; ++k) {
    double s = 0, s2 = 0;
    for (uint32_t r = 0; r < n_rows; ++r) {
      s += X[(size_t)r * IN + k];
      s2 += (double)X[(size_t)r * IN + k] * X[(size_t)r * IN + k];
    }
    double mu = s / n_rows, sd = sqrt(fmax(s2 / n_rows - mu * mu, 0.0));
    p->norm[k] = (float)mu;
    p->norm[IN + k] = sd > 1e-6 ? (float)sd : 1.f;
  }
  for (int o = 0; o < OUT; ++o) {
    double s = 0, s2 = 0;
    for (uint32_t r = 0; r < n_rows; ++r) {
      s += Y[(size_t)r * OUT + o];
      s2 += (double)Y[(size_t)r * OUT + o] * Y[(size_t)r * OUT + o];
    }
    double mu = s / n_rows, sd = sqrt(fmax(s2 / n_rows - mu * mu, 0.0));
    p->norm[2 * IN + o] = (float)mu;
    p->norm[2 * IN + OUT + o] = sd > 1e-6 ? (float)sd : 1.f;
  }
  for (uint32_t r = 0; r < n_rows; ++r) {
    for (int k = 0; k < IN; ++k) xn[(size_t)r * IN + k] = (X[(size_t)r * IN + k] - p->norm[k]) / p->norm[IN + k];
    for (int o = 0; o < OUT; ++o)
      yn[(size_t)r * OUT + o] = (Y[(size_t)r * OUT + o] - p->norm[2 * IN + o]) / p->norm[2 * IN + OUT + o];
  }
  // row order: epochs of seeded permutations (Philox keys)
  std::vector<uint32_t> order;
  order.reserve((size_t)epochs * n_rows);
  std::vector<std::pair<uint64_t, uint32_t>> key(n_rows);
  for (uint32_t ep = 0; ep < epochs; ++ep) {
    for (uint32_t r = 0; r < n_rows; ++r) key[r] = {zg_draw(seed, 0x4D4C5001u, ((uint64_t)ep << 32) | r, 0, 0, ~0ull), r};
    std::sort(key.begin(), key.end());
    for (auto& kv : key) order.push_back(kv.second);
  }
  uint32_t steps = (uint32_t)(order.size() / batch);
  if (steps == 0) steps = 1;
  float *dX = nullptr, *dY = nullptr, *dL = nullptr;
  uint32_t* dO = nullptr;
  cudaError_t e = cudaMalloc((void**)&dX, sizeof(float) * xn.size());
  if (e == cudaSuccess) e = cudaMalloc((void**)&dY, sizeof(float) * yn.size());
  if (e == cudaSuccess) e = cudaMalloc((void**)&dO, sizeof(uint32_t) * order.size());
  if (e == cudaSuccess) e = cudaMalloc((void**)&dL, sizeof(float) * steps);
  if (e == cudaSuccess) e = cudaMemcpy(dX, xn.data(), sizeof(float) * xn.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dY, yn.data(), sizeof(float) * yn.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dO, order.data(), sizeof(uint32_t) * order.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_mlp_train<<<1, kT, smem_bytes()>>>(dX, dY, dO, n_rows, steps, batch, lr, p->step, p->master, p->m, p->v, dL);
    e = cudaDeviceSynchronize();
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess && loss_history) e = cudaMemcpy(loss_history, dL, sizeof(float) * steps, cudaMemcpyDeviceToHost);
  p->step += steps;
  if (dX) cudaFree(dX);
  if (dY) cudaFree(dY);
  if (dO) cudaFree(dO);
  if (dL) cudaFree(dL);
  if (e != cudaSuccess) return zg_check_cuda(e, "zg_mlp_train");
  return ZG_OK;
}

// Gradient of the mean squared error over rows [0, n_rows) (n_rows <= 64) of already-normalised
// X / Y, at the current master weights (no update).  grads: zg_mlp_num_params() floats.
extern "C" int zg_mlp_grad(const zg_mlp* p, const float* X, const float* Y, uint32_t n_rows, float* grads,
                           float* loss) {
  if (!p || !X || !Y || !grads || n_rows == 0 || n_rows > kMaxB)
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_mlp_grad: invalid argument"), ZG_ERR_INVALID_ARG;
  int rc = ensure_smem();
  if (rc) return rc;
  std::vector<uint32_t> rows(n_rows);
  for (uint32_t i = 0; i < n_rows; ++i) rows[i] = i;
  float *dX = nullptr, *dY = nullptr, *dG = nullptr;
  uint32_t* dR = nullptr;
  cudaError_t e = cudaMalloc((void**)&dX, sizeof(float) * n_rows * IN);
  if (e == cudaSuccess) e = cudaMalloc((void**)&dY, sizeof(float) * n_rows * OUT);
  if (e == cudaSuccess) e = cudaMalloc((void**)&dG, sizeof(float) * (NP + 1));
  if (e == cudaSuccess) e = cudaMalloc((void**)&dR, sizeof(uint32_t) * n_rows);
  if (e == cudaSuccess) e = cudaMemcpy(dX, X, sizeof(float) * n_rows * IN, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dY, Y, sizeof(float) * n_rows * OUT, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dR, rows.data(), sizeof(uint32_t) * n_rows, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_mlp_grad<<<1, kT, smem_bytes()>>>(dX, dY, dR, n_rows, p->master, dG, dG + NP);
    e = cudaDeviceSynchronize();
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(grads, dG, sizeof(float) * NP, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && loss) e = cudaMemcpy(loss, dG + NP, sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(dX);
  cudaFree(dY);
  cudaFree(dG);
  cudaFree(dR);
  if (e != cudaSuccess) return zg_check_cuda(e, "zg_mlp_grad");
  return ZG_OK;
}

// Predictions for raw features (normalised and de-normalised with the model's statistics).
extern "C" int zg_mlp_predict(const zg_mlp* p, const float* X, uint32_t n_rows, float* Y) {
  if (!p || !X || !Y) return zg_set_error(ZG_ERR_INVALID_ARG, "zg_mlp_predict: null argument"), ZG_ERR_INVALID_ARG;
  if (n_rows == 0) return ZG_OK;
  std::vector<float> xn((size_t)n_rows * IN);
  for (uint32_t r = 0; r < n_rows; ++r)
    for (int k = 0; k < IN; ++k) xn[(size_t)r * IN + k] = (X[(size_t)r * IN + k] - p->norm[k]) / p->norm[IN + k];
  // inputs and outputs in one block from the library's pool; stream-ordered on the legacy stream
  const cudaStream_t s = 0;
  float* d = nullptr;
  cudaError_t e = zg_malloc_async((void**)&d, sizeof(float) * (xn.size() + (size_t)n_rows * OUT), s);
  if (e != cudaSuccess) return zg_check_cuda(e, "zg_mlp_predict");
  float *dX = d, *dY = d + xn.size();
  e = cudaMemcpyAsync(dX, xn.data(), sizeof(float) * xn.size(), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    int grid = (int)std::min<uint32_t>((n_rows + 127) / 128, 1024);
    k_mlp_predict<<<grid, 128, 0, s>>>(dX, n_rows, p->master, dY);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(Y, dY, sizeof(float) * n_rows * OUT, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return zg_check_cuda(e, "zg_mlp_predict");
  for (uint32_t r = 0; r < n_rows; ++r)
    for (int o = 0; o < OUT; ++o)
      Y[(size_t)r * OUT + o] = Y[(size_t)r * OUT + o] * p->norm[2 * IN + OUT + o] + p->norm[2 * IN + o];
  return ZG_OK;
}

// ---- features of a (graph, program) query for the learned profile ------------------------
namespace {

struct DegStats {
  double s1, s2, s3, emin, esum;
  unsigned long long nz, maxd;
};

// Per-block degree statistics (no atomics: every block writes its own partial, summed on the host
// in block order, so the features are reproducible bit for bit).
constexpr int kStatBlock = 256;
__global__ void __launch_bounds__(kStatBlock) k_deg_stats(ZgDevGraph g, DegStats* __restrict__ parts) {
  double s1 = 0, s2 = 0, s3 = 0, emin = 0, esum = 0;
  unsigned long long nz = 0, maxd = 0;
  uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t v = tid; v < g.nv; v += stride) {
    double d = (double)(g.off[v + 1] - g.off[v]);
    if (d > 0) {
      nz++;
      s1 += d;
      s2 += d * d;
      s3 += d * d * d;
      maxd = max(maxd, (unsigned long long)d);
    }
  }
  for (uint64_t e = tid; e < g.m; e += stride) {
    uint4 r = zg_rec_e(g, e);
    double du = (double)(g.off[r.x + 1] - g.off[r.x]), dv = (double)(g.off[r.y + 1] - g.off[r.y]);
    emin += fmin(du, dv);
    esum += du + dv;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    s3 += __shfl_xor_sync(0xffffffffu, s3, o);
    emin += __shfl_xor_sync(0xffffffffu, emin, o);
    esum += __shfl_xor_sync(0xffffffffu, esum, o);
    nz += __shfl_xor_sync(0xffffffffu, nz, o);
    maxd = max(maxd, __shfl_xor_sync(0xffffffffu, maxd, o));
  }
  __shared__ DegStats ws[kStatBlock / 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) ws[warp] = DegStats{s1, s2, s3, emin, esum, nz, maxd};
  __syncthreads();
  if (threadIdx.x == 0) {
    DegStats t = ws[0];
    for (int w = 1; w < kStatBlock / 32; ++w) {
      t.s1 += ws[w].s1;
      t.s2 += ws[w].s2;
      t.s3 += ws[w].s3;
      t.emin += ws[w].emin;
      t.esum += ws[w].esum;
      t.nz += ws[w].nz;
      t.maxd = max(t.maxd, ws[w].maxd);
    }
    parts[blockIdx.x] = t;
  }
}

// The graph's degree statistics, computed once per graph (the graph is immutable).
int deg_stats(const zg_graph* g, cudaStream_t s) {
  if (g->deg_stats_ready) return ZG_OK;
  const int grid = zg_num_sms() * 4;
  DegStats* d = nullptr;
  ZG_CUDA(zg_malloc_async((void**)&d, sizeof(DegStats) * grid, s));
  k_deg_stats<<<grid, kStatBlock, 0, s>>>(g->d, d);
  std::vector<DegStats> h(grid);
  cudaError_t e = cudaMemcpyAsync(h.data(), d, sizeof(DegStats) * grid, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return zg_check_cuda(e, "graph features");
  DegStats t = h[0];
  for (int b = 1; b < grid; ++b) {
    t.s1 += h[b].s1;
    t.s2 += h[b].s2;
    t.s3 += h[b].s3;
    t.emin += h[b].emin;
    t.esum += h[b].esum;
    t.nz += h[b].nz;
    t.maxd = std::max(t.maxd, h[b].maxd);
  }
  double* out = g->deg_stats;
  out[0] = t.s1;
  out[1] = t.s2;
  out[2] = t.s3;
  out[3] = t.emin;
  out[4] = t.esum;
  out[5] = (double)t.nz;
  out[6] = (double)t.maxd;
  g->deg_stats_ready = true;
  return ZG_OK;
}

int pattern_slot(const zg_program* p) {
  switch (p->kind) {
    case ZG_PROG_TRIANGLE: return 0;
    case ZG_PROG_FOUR_CLIQUE:
    case ZG_PROG_FOUR_CLIQUE_UNBIASED: return 1;
    case ZG_PROG_THREE_CHAIN: return 2;
    case ZG_PROG_FOUR_CHAIN:
    case ZG_PROG_CHAIN: return 3;
    default: return p->pe + 1 == p->pv ? 4 : 5;  // tree patterns (5-star) vs cyclic ones (house)
  }
}

float lg2(double x) { return (float)log2(x > 1e-300 ? x : 1e-300); }

}  // namespace

// 16 features: log2 m, log2 non-isolated vertices, log2 max degree, log2 mean degree, log2 of the
// 2nd and 3rd degree moments, log2 mean (d_u + d_v) and mean min(d_u, d_v) over edges, the
// pattern one-hot (triangle, 4-clique, 3-chain, 4-chain/k-chain, tree pattern, cyclic pattern),
// and from a pilot run of pilot_samples estimators (stream ZG_ELP_STREAM + 1): log2 hit rate and
// log2 per-sample relative variance.
// Adaptive pilots (pilot_samples = 0): from kPilotMin estimators, 4x at a time up to kPilotMax,
// until kPilotHits hits, so rare patterns get a pilot that has seen some.
constexpr uint64_t kPilotMin = 1ull << 16, kPilotMax = 1ull << 22;
constexpr uint64_t kPilotHits = 8;

int zg_graph_max_degree(const zg_graph* g, cudaStream_t s, uint64_t* out) {
  int rc = deg_stats(g, s);
  if (rc) return rc;
  *out = (uint64_t)g->deg_stats[6];
  return ZG_OK;
}

// The graph part of the features (f[0..7]; the rest zeroed).
int zg_degree_features(const zg_graph* g, cudaStream_t s, float* f) {
  int rc = deg_stats(g, s);
  if (rc) return rc;
  const double* h = g->deg_stats;
  double m = (double)g->d.m, nz = h[5] > 0 ? h[5] : 1.0;
  for (int i = 0; i < IN; ++i) f[i] = 0.f;
  f[0] = lg2(m);
  f[1] = lg2(nz);
  f[2] = lg2(h[6]);
  f[3] = lg2(h[0] / nz);
  f[4] = lg2(h[1] / nz);
  f[5] = lg2(h[2] / nz);
  f[6] = lg2(m > 0 ? h[4] / m : 0);
  f[7] = lg2(m > 0 ? h[3] / m : 0);
  return ZG_OK;
}

// The program and pilot parts: the pattern class one-hot and, from a pilot run's counters, the
// hit rate and the per-sample relative variance.
void zg_query_features(const zg_program* p, const zg_counters& c, float* f) {
  f[8 + pattern_slot(p)] = 1.f;
  double n = (double)c.samples;
  double mean = c.estimate;
  double cv2 = (c.hits >= 2 && mean > 0) ? (c.sum_w2 / n) / (mean * mean) - 1.0 : n;
  f[14] = lg2(((double)c.hits + 0.5) / n);
  f[15] = lg2(cv2 > 1e-12 ? cv2 : 1e-12);
}

// The learned budget for a prediction: n = z^2 * 2^pred / error^2, at least 2^16.
uint64_t zg_learned_n(float pred_log2_cv2, double error, double confidence) {
  const double z = zg_normal_quantile(1.0 - (1.0 - confidence) / 2.0);
  const double n = z * z * exp2((double)pred_log2_cv2) / (error * error);
  const double lo = (double)(1ull << 16), hi = 1e18;
  return n >= hi ? (uint64_t)hi : n <= lo ? (uint64_t)lo : (uint64_t)n;
}

extern "C" int zg_graph_features(const zg_graph* g, const zg_program* p, uint64_t pilot_samples, uint64_t seed,
                                 void* cuda_stream, float* f) {
  if (!g || !p || !f) return zg_set_error(ZG_ERR_INVALID_ARG, "zg_graph_features: null argument"), ZG_ERR_INVALID_ARG;
  int rc = zg_degree_features(g, (cudaStream_t)cuda_stream, f);
  if (rc) return rc;
  zg_counters c;
  if (pilot_samples) {
    rc = zg_run(g, p, pilot_samples, 0, seed, ZG_ELP_STREAM + 1, cuda_stream, &c);
  } else {
    // adaptive: 2^16 estimators, then 2^18, 2^20, 2^22 (each from the pilot stream's first sample,
    // so a larger pilot contains the smaller) until the pilot has seen kPilotHits hits
    for (uint64_t n = kPilotMin;; n <<= 2) {
      if ((rc = zg_run(g, p, n, 0, seed, ZG_ELP_STREAM + 1, cuda_stream, &c))) break;
      if (c.hits >= kPilotHits || n >= kPilotMax) break;
    }
  }
  if (rc) return rc;
  zg_query_features(p, c, f);
  return ZG_OK;
}

// ---- learned sizing and the learned query ---------------------------------------------------
extern "C" int zg_elp_learned(const zg_mlp* net, const zg_graph* g, const zg_program* p, double error,
                              double confidence, uint64_t pilot_samples, uint64_t seed, void* cuda_stream,
                              uint64_t* n_required, float* prediction) {
  if (!net || !g || !p || !n_required)
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_elp_learned: null argument"), ZG_ERR_INVALID_ARG;
  if (!(error > 0) || !(confidence > 0 && confidence < 1))
    return zg_set_error(ZG_ERR_INVALID_ARG, "zg_elp_learned: error %g / confidence %g", error, confidence),
           ZG_ERR_INVALID_ARG;
  float f[IN], y[OUT];
  int rc = zg_graph_features(g, p, pilot_samples, seed, cuda_stream, f);
  if (rc) return rc;
  if ((rc = zg_mlp_predict(net, f, 1, y))) return rc;
  *n_required = zg_learned_n(y[0], error, confidence);
  if (prediction) {
    prediction[0] = y[0];
    prediction[1] = y[1];
  }
  return ZG_OK;
}

extern "C" int zg_query_learned(const zg_mlp* net, const zg_graph* g, const zg_program* p, double error,
                                double confidence, uint64_t max_samples, uint64_t feature_seed, uint64_t query_seed,
                                uint32_t stream_id, void* cuda_stream, uint64_t* n_required, zg_query_result* out) {
  uint64_t n = 0;
  int rc = zg_elp_learned(net, g, p, error, confidence, 0, feature_seed, cuda_stream, &n, nullptr);
  if (rc) return rc;
  if (n_required) *n_required = n;
  const uint64_t first = n > (1ull << 30) ? n / 2 : n;  // two looks for a long budget
  return zg_query(g, p, error, confidence, first, max_samples, query_seed, stream_id, cuda_stream, out);
}
