// Learned slice count: a 12 -> 64 -> 64 -> 7 MLP (ReLU, softmax over slice counts 2..8).
//
// No counterpart in the reference.  Hand-written kernels:
//   mlp_grad_kernel   FP32 forward + backward over a batch, one CTA, samples accumulated in a
//                     fixed order (deterministic), mean cross-entropy loss
//   mlp_adam_kernel   Adam update of the FP32 parameters
//   mlp_infer_kernel  BF16 inference (BF16 weights and inputs, FP32 accumulation), argmax
//   features_kernel   the 12 per-triplet features, from the digit exponents and energies
// Parameter layout (floats): W1[64][12] b1[64] W2[64][64] b2[64] W3[7][64] b3[7].
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/ccsdt.h"
#include "ccsdt_internal.cuh"

namespace {

constexpr int IN = CCSDT_MLP_IN, H = CCSDT_MLP_HIDDEN, OUT = CCSDT_MLP_OUT;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + H * IN, OFF_W2 = OFF_B1 + H, OFF_B2 = OFF_W2 + H * H,
              OFF_W3 = OFF_B2 + H, OFF_B3 = OFF_W3 + OUT * H, NPARAM = OFF_B3 + OUT;
static_assert(NPARAM == CCSDT_MLP_NPARAM, "parameter count");

constexpr int GT = 256;

// grad[NPARAM] = d(mean CE)/d(params) over samples [0, n); loss[0] = mean CE
__global__ void __launch_bounds__(GT) mlp_grad_kernel(const float* __restrict__ P, const float* __restrict__ X,
                                                       const int* __restrict__ Y, int n, float* __restrict__ grad,
                                                       float* __restrict__ loss) {
  __shared__ float g[NPARAM];
  __shared__ float x[IN], h1[H], h2[H], z[OUT], dz[OUT], da2[H], da1[H];
  __shared__ float lsum;
  const int t = threadIdx.x;
  for(int e = t; e < NPARAM; e += GT) g[e] = 0.f;
  if(t == 0) lsum = 0.f;
  __syncthreads();
  for(int s = 0; s < n; s++) {
    if(t < IN) x[t] = X[(long long) s * IN + t];
    __syncthreads();
    if(t < H) {
      float a = P[OFF_B1 + t];
      for(int f = 0; f < IN; f++) a = fmaf(P[OFF_W1 + t * IN + f], x[f], a);
      h1[t] = fmaxf(a, 0.f);
    }
    __syncthreads();
    if(t < H) {
      float a = P[OFF_B2 + t];
      for(int w = 0; w < H; w++) a = fmaf(P[OFF_W2 + t * H + w], h1[w], a);
      h2[t] = fmaxf(a, 0.f);
    }
    __syncthreads();
    if(t < OUT) {
      float a = P[OFF_B3 + t];
      for(int u = 0; u < H; u++) a = fmaf(P[OFF_W3 + t * H + u], h2[u], a);
      z[t] = a;
    }
    __syncthreads();
    if(t == 0) { // softmax, loss, dz (tiny: one thread, fixed order)
      float mx = z[0];
      for(int c = 1; c < OUT; c++) mx = fmaxf(mx, z[c]);
      float se = 0.f;
      for(int c = 0; c < OUT; c++) se += expf(z[c] - mx);
      const int y = Y[s];
      for(int c = 0; c < OUT; c++) dz[c] = (expf(z[c] - mx) / se - (c == y ? 1.f : 0.f)) / n;
      lsum += (logf(se) + mx - z[y]) / n;
    }
    __syncthreads();
    if(t < H) {
      float d = 0.f;
      for(int c = 0; c < OUT; c++) d = fmaf(P[OFF_W3 + c * H + t], dz[c], d);
      da2[t] = h2[t] > 0.f ? d : 0.f;
    }
    for(int e = t; e < OUT * H; e += GT) g[OFF_W3 + e] += dz[e / H] * h2[e % H];
    if(t < OUT) g[OFF_B3 + t] += dz[t];
    __syncthreads();
    if(t < H) {
      float d = 0.f;
      for(int u = 0; u < H; u++) d = fmaf(P[OFF_W2 + u * H + t], da2[u], d);
      da1[t] = h1[t] > 0.f ? d : 0.f;
    }
    for(int e = t; e < H * H; e += GT) g[OFF_W2 + e] += da2[e / H] * h1[e % H];
    if(t < H) g[OFF_B2 + t] += da2[t];
    __syncthreads();
    for(int e = t; e < H * IN; e += GT) g[OFF_W1 + e] += da1[e / IN] * x[e % IN];
    if(t < H) g[OFF_B1 + t] += da1[t];
    __syncthreads();
  }
  for(int e = t; e < NPARAM; e += GT) grad[e] = g[e];
  if(t == 0) *loss = lsum;
}

__global__ void mlp_adam_kernel(float* P, const float* g, float* m, float* v, int step, float lr) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - powf(b1, (float) step), c2 = 1.f - powf(b2, (float) step);
  for(int e = blockIdx.x * blockDim.x + threadIdx.x; e < NPARAM; e += gridDim.x * blockDim.x) {
    m[e] = b1 * m[e] + (1.f - b1) * g[e];
    v[e] = b2 * v[e] + (1.f - b2) * g[e] * g[e];
    P[e] -= lr * (m[e] / c1) / (sqrtf(v[e] / c2) + eps);
  }
}

__global__ void to_bf16_kernel(const float* x, __nv_bfloat16* y, int n) {
  for(int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) y[e] = __float2bfloat16_rn(x[e]);
}

// one thread per sample: BF16 weights / inputs, FP32 accumulation; slice = 2 + argmax
__global__ void mlp_infer_kernel(const __nv_bfloat16* __restrict__ P, const float* __restrict__ X, int n,
                                 int* __restrict__ slices, float* __restrict__ logits) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if(s >= n) return;
  float x[IN], a1[H], a2[H];
  for(int f = 0; f < IN; f++) x[f] = __bfloat162float(__float2bfloat16_rn(X[(long long) s * IN + f]));
  for(int u = 0; u < H; u++) {
    float a = __bfloat162float(P[OFF_B1 + u]);
    for(int f = 0; f < IN; f++) a = fmaf(__bfloat162float(P[OFF_W1 + u * IN + f]), x[f], a);
    a1[u] = __bfloat162float(__float2bfloat16_rn(fmaxf(a, 0.f)));
  }
  for(int u = 0; u < H; u++) {
    float a = __bfloat162float(P[OFF_B2 + u]);
    for(int w = 0; w < H; w++) a = fmaf(__bfloat162float(P[OFF_W2 + u * H + w]), a1[w], a);
    a2[u] = __bfloat162float(__float2bfloat16_rn(fmaxf(a, 0.f)));
  }
  int   best = 0;
  float bz   = -INFINITY;
  for(int c = 0; c < OUT; c++) {
    float a = __bfloat162float(P[OFF_B3 + c]);
    for(int u = 0; u < H; u++) a = fmaf(__bfloat162float(P[OFF_W3 + c * H + u]), a2[u], a);
    if(logits) logits[(long long) s * OUT + c] = a;
    if(a > bz) {
      bz   = a;
      best = c;
    }
  }
  slices[s] = 2 + best;
}

} // namespace

// ------------------------------------------------------------------------------ C ABI
namespace {
struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if(p) cudaFree(p);
  }
  bool alloc(size_t bytes) {
    if(ccsdt::dev_malloc(&p, bytes ? bytes : 1) != cudaSuccess) {
      p = nullptr;
      cudaGetLastError();
      return false;
    }
    return true;
  }
  template<typename T>
  T* as() {
    return static_cast<T*>(p);
  }
};
} // namespace

extern "C" ccsdt_status ccsdt_mlp_grad(const float* params, const float* X, const int* labels, int n, float* grad,
                                       float* loss) {
  if(!params || !X || !labels || !grad || !loss || n <= 0) return CCSDT_E_INVALID;
  for(int s = 0; s < n; s++)
    if(labels[s] < 0 || labels[s] >= OUT) return CCSDT_E_INVALID;
  DevBuf dp, dx, dy, dg, dl;
  if(!dp.alloc(NPARAM * 4) || !dx.alloc((size_t) n * IN * 4) || !dy.alloc((size_t) n * 4) || !dg.alloc(NPARAM * 4) ||
     !dl.alloc(4))
    return CCSDT_E_OOM;
  if(cudaMemcpy(dp.p, params, NPARAM * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
     cudaMemcpy(dx.p, X, (size_t) n * IN * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
     cudaMemcpy(dy.p, labels, (size_t) n * 4, cudaMemcpyHostToDevice) != cudaSuccess)
    return CCSDT_E_CUDA;
  mlp_grad_kernel<<<1, GT>>>(dp.as<float>(), dx.as<float>(), dy.as<int>(), n, dg.as<float>(), dl.as<float>());
  if(cudaGetLastError() != cudaSuccess || cudaMemcpy(grad, dg.p, NPARAM * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
     cudaMemcpy(loss, dl.p, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return CCSDT_E_CUDA;
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_mlp_train(const float* X, const int* labels, int n, int epochs, int batch, float lr,
                                        unsigned seed, int init, float* params, float* final_loss) {
  if(!X || !labels || !params || n <= 0 || epochs <= 0 || batch <= 0) return CCSDT_E_INVALID;
  for(int s = 0; s < n; s++)
    if(labels[s] < 0 || labels[s] >= OUT) return CCSDT_E_INVALID;
  std::vector<float> P(params, params + NPARAM);
  if(init) { // He-uniform initialisation, seeded
    std::mt19937 rng(seed);
    auto         fill = [&](int off, int rows, int cols) {
      std::uniform_real_distribution<float> u(-std::sqrt(6.f / cols), std::sqrt(6.f / cols));
      for(int e = 0; e < rows * cols; e++) P[off + e] = u(rng);
    };
    fill(OFF_W1, H, IN);
    fill(OFF_W2, H, H);
    fill(OFF_W3, OUT, H);
    for(int e = 0; e < H; e++) P[OFF_B1 + e] = P[OFF_B2 + e] = 0.f;
    for(int e = 0; e < OUT; e++) P[OFF_B3 + e] = 0.f;
  }
  DevBuf dp, dx, dy, dg, dm, dv, dl, bx, by;
  if(!dp.alloc(NPARAM * 4) || !dx.alloc((size_t) n * IN * 4) || !dy.alloc((size_t) n * 4) || !dg.alloc(NPARAM * 4) ||
     !dm.alloc(NPARAM * 4) || !dv.alloc(NPARAM * 4) || !dl.alloc(4) || !bx.alloc((size_t) batch * IN * 4) ||
     !by.alloc((size_t) batch * 4))
    return CCSDT_E_OOM;
  cudaMemcpy(dp.p, P.data(), NPARAM * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dx.p, X, (size_t) n * IN * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dy.p, labels, (size_t) n * 4, cudaMemcpyHostToDevice);
  cudaMemset(dm.p, 0, NPARAM * 4);
  cudaMemset(dv.p, 0, NPARAM * 4);
  std::mt19937     rng(seed ^ 0x5bd1e995u);
  std::vector<int> order(n);
  for(int s = 0; s < n; s++) order[s] = s;
  std::vector<float> hx((size_t) batch * IN);
  std::vector<int>   hy(batch);
  int                step = 0;
  for(int ep = 0; ep < epochs; ep++) {
    std::shuffle(order.begin(), order.end(), rng);
    for(int b0 = 0; b0 < n; b0 += batch) {
      const int nb = std::min(batch, n - b0);
      for(int q = 0; q < nb; q++) {
        std::memcpy(&hx[(size_t) q * IN], X + (size_t) order[b0 + q] * IN, IN * 4);
        hy[q] = labels[order[b0 + q]];
      }
      cudaMemcpy(bx.p, hx.data(), (size_t) nb * IN * 4, cudaMemcpyHostToDevice);
      cudaMemcpy(by.p, hy.data(), (size_t) nb * 4, cudaMemcpyHostToDevice);
      mlp_grad_kernel<<<1, GT>>>(dp.as<float>(), bx.as<float>(), by.as<int>(), nb, dg.as<float>(), dl.as<float>());
      mlp_adam_kernel<<<22, 256>>>(dp.as<float>(), dg.as<float>(), dm.as<float>(), dv.as<float>(), ++step, lr);
    }
  }
  // loss on the whole set with the final parameters
  mlp_grad_kernel<<<1, GT>>>(dp.as<float>(), dx.as<float>(), dy.as<int>(), n, dg.as<float>(), dl.as<float>());
  if(cudaGetLastError() != cudaSuccess || cudaMemcpy(params, dp.p, NPARAM * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return CCSDT_E_CUDA;
  if(final_loss && cudaMemcpy(final_loss, dl.p, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return CCSDT_E_CUDA;
  return CCSDT_OK;
}

extern "C" ccsdt_status ccsdt_mlp_predict(const float* params, const float* X, int n, int* slices, float* logits) {
  if(!params || !X || !slices || n <= 0) return CCSDT_E_INVALID;
  DevBuf dp, db, dx, ds, dl;
  if(!dp.alloc(NPARAM * 4) || !db.alloc(NPARAM * 2) || !dx.alloc((size_t) n * IN * 4) || !ds.alloc((size_t) n * 4) ||
     (logits && !dl.alloc((size_t) n * OUT * 4)))
    return CCSDT_E_OOM;
  cudaMemcpy(dp.p, params, NPARAM * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(dx.p, X, (size_t) n * IN * 4, cudaMemcpyHostToDevice);
  to_bf16_kernel<<<22, 256>>>(dp.as<float>(), db.as<__nv_bfloat16>(), NPARAM);
  mlp_infer_kernel<<<(n + 127) / 128, 128>>>(db.as<__nv_bfloat16>(), dx.as<float>(), n, ds.as<int>(),
                                             logits ? dl.as<float>() : nullptr);
  if(cudaGetLastError() != cudaSuccess || cudaMemcpy(slices, ds.p, (size_t) n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return CCSDT_E_CUDA;
  if(logits && cudaMemcpy(logits, dl.p, (size_t) n * OUT * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return CCSDT_E_CUDA;
  return CCSDT_OK;
}

// Device-side BF16 inference for the LEARNED mode (inputs already on the device).
void ccsdt_mlp_infer_device(const void* params_bf16, const float* X, long n, int* slices, cudaStream_t st) {
  if(n <= 0) return;
  mlp_infer_kernel<<<(unsigned) ((n + 127) / 128), 128, 0, st>>>(static_cast<const __nv_bfloat16*>(params_bf16), X,
                                                                 (int) n, slices, nullptr);
}
