// mlp.cu — training of the turn scheduler's MLP on the GPU.
//
// The policy (policy.cuh) is a 16 -> 64 -> 64 -> 3 FP32 MLP with ReLU hidden
// layers and sigmoid outputs. Its training data are per-turn records of the
// evaluator (features, and the parameters the fastest run chose next); the
// loss is the weighted mean squared error of the outputs.
//
// mlp_grad_kernel: each block walks tiles of 64 rows. Per tile it runs the
// forward pass and the backward pass in shared memory (one row x unit per
// thread and step), then every thread adds the tile's contribution to the
// parameters it owns (parameter p = thread + k * 256) to registers; the block
// adds its sums to the global gradient once at the end.
// adam_kernel: one block applies an Adam step to all 5443 parameters, clears
// the gradient and advances the step counter, so one training epoch is two
// launches that are captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "policy.cuh"
#include "hvm_gb300.h"

namespace hvm {

constexpr int MLP_TILE = 64, MLP_THREADS = 256;
constexpr int MLP_OWN = (POLICY_PARAMS + MLP_THREADS - 1) / MLP_THREADS;  // parameters per thread
constexpr int HP = POLICY_HID + 1;  // padded row of a hidden-layer tile

struct MlpShared {
  float w[POLICY_PARAMS];
  float w1t[POLICY_IN][POLICY_HID];   // W1 transposed: lanes of a warp read consecutive units
  float w2t[POLICY_HID][POLICY_HID];  // W2 transposed
  float x[MLP_TILE][POLICY_IN];
  float t[MLP_TILE][POLICY_OUT];
  float sw[MLP_TILE];
  float h1[MLP_TILE][HP];
  float h2[MLP_TILE][HP];
  float d1[MLP_TILE][HP];
  float d2[MLP_TILE][HP];
  float d3[MLP_TILE][POLICY_OUT];
  float red[MLP_THREADS / 32];
};

__device__ __forceinline__ float sigmoidf_(float z) { return 1.0f / (1.0f + expf(-z)); }

// Forward pass of one tile; rows past `n` have zero weight.
__device__ void tile_forward(MlpShared& S, const float* x, const float* t, const float* sw, size_t row0, size_t n) {
  const int tid = threadIdx.x;
  for (int k = tid; k < MLP_TILE * POLICY_IN; k += MLP_THREADS) {
    const int s = k / POLICY_IN, i = k % POLICY_IN;
    const size_t r = row0 + s;
    S.x[s][i] = r < n ? x[r * POLICY_IN + i] : 0.f;
  }
  for (int k = tid; k < MLP_TILE * POLICY_OUT; k += MLP_THREADS) {
    const int s = k / POLICY_OUT, o = k % POLICY_OUT;
    const size_t r = row0 + s;
    S.t[s][o] = r < n ? t[r * POLICY_OUT + o] : 0.f;
  }
  for (int s = tid; s < MLP_TILE; s += MLP_THREADS) S.sw[s] = row0 + s < n ? sw[row0 + s] : 0.f;
  __syncthreads();
  for (int k = tid; k < MLP_TILE * POLICY_HID; k += MLP_THREADS) {
    const int s = k / POLICY_HID, j = k % POLICY_HID;
    float z = S.w[POLICY_B1 + j];
    #pragma unroll
    for (int i = 0; i < POLICY_IN; i++) z = fmaf(S.w1t[i][j], S.x[s][i], z);
    S.h1[s][j] = z > 0.f ? z : 0.f;
  }
  __syncthreads();
  for (int k = tid; k < MLP_TILE * POLICY_HID; k += MLP_THREADS) {
    const int s = k / POLICY_HID, j = k % POLICY_HID;
    float z = S.w[POLICY_B2 + j];
    #pragma unroll 8
    for (int i = 0; i < POLICY_HID; i++) z = fmaf(S.w2t[i][j], S.h1[s][i], z);
    S.h2[s][j] = z > 0.f ? z : 0.f;
  }
  __syncthreads();
}

// Loss and gradient over all rows. `scale` = 1 / sum(sw). `grad` and `loss`
// accumulate (the caller clears them); block 0 also advances `*step`.
__global__ void __launch_bounds__(MLP_THREADS) mlp_grad_kernel(const float* __restrict__ w, const float* x,
                                                                const float* t, const float* sw, size_t n,
                                                                float scale, float* grad, float* loss) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  MlpShared& S = *reinterpret_cast<MlpShared*>(smem_raw);
  const int tid = threadIdx.x;
  for (int k = tid; k < POLICY_PARAMS; k += MLP_THREADS) S.w[k] = w[k];
  __syncthreads();
  for (int k = tid; k < POLICY_HID * POLICY_IN; k += MLP_THREADS) {
    const int j = k / POLICY_IN, i = k % POLICY_IN;
    S.w1t[i][j] = S.w[POLICY_W1 + k];
  }
  for (int k = tid; k < POLICY_HID * POLICY_HID; k += MLP_THREADS) {
    const int j = k / POLICY_HID, i = k % POLICY_HID;
    S.w2t[i][j] = S.w[POLICY_W2 + k];
  }
  float acc[MLP_OWN];
  #pragma unroll
  for (int k = 0; k < MLP_OWN; k++) acc[k] = 0.f;
  float lsum = 0.f;
  const size_t tiles = (n + MLP_TILE - 1) / MLP_TILE;
  for (size_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    __syncthreads();
    tile_forward(S, x, t, sw, tile * MLP_TILE, n);
    // Output layer and the error at its pre-activation.
    for (int k = tid; k < MLP_TILE * POLICY_OUT; k += MLP_THREADS) {
      const int s = k / POLICY_OUT, o = k % POLICY_OUT;
      float z = S.w[POLICY_B3 + o];
      for (int j = 0; j < POLICY_HID; j++) z = fmaf(S.w[POLICY_W3 + o * POLICY_HID + j], S.h2[s][j], z);
      const float y = sigmoidf_(z), e = y - S.t[s][o];
      lsum += S.sw[s] * e * e;
      S.d3[s][o] = 2.f * scale * S.sw[s] * e * y * (1.f - y);
    }
    __syncthreads();
    for (int k = tid; k < MLP_TILE * POLICY_HID; k += MLP_THREADS) {
      const int s = k / POLICY_HID, j = k % POLICY_HID;
      float g = 0.f;
      #pragma unroll
      for (int o = 0; o < POLICY_OUT; o++) g = fmaf(S.w[POLICY_W3 + o * POLICY_HID + j], S.d3[s][o], g);
      S.d2[s][j] = S.h2[s][j] > 0.f ? g : 0.f;
    }
    __syncthreads();
    for (int k = tid; k < MLP_TILE * POLICY_HID; k += MLP_THREADS) {
      const int s = k / POLICY_HID, i = k % POLICY_HID;
      float g = 0.f;
      #pragma unroll 8
      for (int j = 0; j < POLICY_HID; j++) g = fmaf(S.w[POLICY_W2 + j * POLICY_HID + i], S.d2[s][j], g);
      S.d1[s][i] = S.h1[s][i] > 0.f ? g : 0.f;
    }
    __syncthreads();
    // Each thread's parameters: sum over the tile's rows.
    #pragma unroll
    for (int k = 0; k < MLP_OWN; k++) {
      const int p = tid + k * MLP_THREADS;
      if (p >= POLICY_PARAMS) break;
      float g = 0.f;
      if (p < POLICY_B1) {
        const int j = (p - POLICY_W1) / POLICY_IN, i = (p - POLICY_W1) % POLICY_IN;
        for (int s = 0; s < MLP_TILE; s++) g = fmaf(S.d1[s][j], S.x[s][i], g);
      } else if (p < POLICY_W2) {
        const int j = p - POLICY_B1;
        for (int s = 0; s < MLP_TILE; s++) g += S.d1[s][j];
      } else if (p < POLICY_B2) {
        const int j = (p - POLICY_W2) / POLICY_HID, i = (p - POLICY_W2) % POLICY_HID;
        for (int s = 0; s < MLP_TILE; s++) g = fmaf(S.d2[s][j], S.h1[s][i], g);
      } else if (p < POLICY_W3) {
        const int j = p - POLICY_B2;
        for (int s = 0; s < MLP_TILE; s++) g += S.d2[s][j];
      } else if (p < POLICY_B3) {
        const int o = (p - POLICY_W3) / POLICY_HID, j = (p - POLICY_W3) % POLICY_HID;
        for (int s = 0; s < MLP_TILE; s++) g = fmaf(S.d3[s][o], S.h2[s][j], g);
      } else {
        const int o = p - POLICY_B3;
        for (int s = 0; s < MLP_TILE; s++) g += S.d3[s][o];
      }
      acc[k] += g;
    }
  }
  #pragma unroll
  for (int k = 0; k < MLP_OWN; k++) {
    const int p = tid + k * MLP_THREADS;
    if (p < POLICY_PARAMS && acc[k] != 0.f) atomicAdd(&grad[p], acc[k]);
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xFFFFFFFFu, lsum, o);
  if ((tid & 31) == 0) S.red[tid >> 5] = lsum;
  __syncthreads();
  if (tid == 0) {
    float v = 0.f;
    for (int i = 0; i < MLP_THREADS / 32; i++) v += S.red[i];
    atomicAdd(loss, v * scale);
  }
}

// One Adam step (Kingma & Ba, 2015) over all parameters by one block. state:
// [0] step count, [1] loss of the step, [2] loss accumulator.
__global__ void adam_kernel(float* w, float* grad, float* m, float* v, float* state, float lr) {
  __shared__ float t_sh;
  if (threadIdx.x == 0) t_sh = state[0] + 1.f;
  __syncthreads();
  const float t = t_sh, b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - powf(b1, t), c2 = 1.f - powf(b2, t);
  for (int p = threadIdx.x; p < POLICY_PARAMS; p += blockDim.x) {
    const float g = grad[p];
    const float mm = b1 * m[p] + (1.f - b1) * g, vv = b2 * v[p] + (1.f - b2) * g * g;
    m[p] = mm;
    v[p] = vv;
    w[p] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    grad[p] = 0.f;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    state[0] = t;
    state[1] = state[2];
    state[2] = 0.f;
  }
}

// Runs the turn kernel's inference routine on each row (one block per row).
__global__ void policy_forward_kernel(const float* w, const float* x, size_t n, float* y) {
  __shared__ float feat[POLICY_IN], h1[POLICY_HID], h2[POLICY_HID], out[POLICY_OUT];
  for (size_t r = blockIdx.x; r < n; r += gridDim.x) {
    if (threadIdx.x < POLICY_IN) feat[threadIdx.x] = x[r * POLICY_IN + threadIdx.x];
    __syncthreads();
    policy_infer_block(w, feat, h1, h2, out);
    if (threadIdx.x < POLICY_OUT) y[r * POLICY_OUT + threadIdx.x] = out[threadIdx.x];
    __syncthreads();
  }
}

namespace {

void set_err(char* err, size_t cap, const std::string& m) {
  if (err && cap) {
    size_t k = m.size() < cap - 1 ? m.size() : cap - 1;
    memcpy(err, m.data(), k);
    err[k] = 0;
  }
}

// Device buffers of one training problem, freed on scope exit.
struct Buffers {
  float *w = nullptr, *x = nullptr, *t = nullptr, *sw = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr,
        *state = nullptr, *y = nullptr;
  ~Buffers() {
    float* ps[] = {w, x, t, sw, grad, m, v, state, y};
    for (float* p : ps) if (p) cudaFree(p);
  }
};

#define MLP_CK(call)                                                                     \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) {                                                             \
      set_err(err, err_cap, std::string(#call) + ": " + cudaGetErrorString(e_));         \
      return -1;                                                                         \
    }                                                                                    \
  } while (0)

int grad_grid(int device) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  return sms > 0 ? sms : 1;
}

int upload(Buffers& b, const float* weights, const float* x, const float* t, const float* sw, size_t n, char* err,
           size_t err_cap) {
  MLP_CK(cudaMalloc((void**)&b.w, POLICY_PARAMS * sizeof(float)));
  MLP_CK(cudaMalloc((void**)&b.grad, POLICY_PARAMS * sizeof(float)));
  MLP_CK(cudaMalloc((void**)&b.state, 4 * sizeof(float)));
  MLP_CK(cudaMalloc((void**)&b.x, n * POLICY_IN * sizeof(float)));
  MLP_CK(cudaMalloc((void**)&b.t, n * POLICY_OUT * sizeof(float)));
  MLP_CK(cudaMalloc((void**)&b.sw, n * sizeof(float)));
  MLP_CK(cudaMemcpy(b.w, weights, POLICY_PARAMS * sizeof(float), cudaMemcpyHostToDevice));
  MLP_CK(cudaMemcpy(b.x, x, n * POLICY_IN * sizeof(float), cudaMemcpyHostToDevice));
  MLP_CK(cudaMemcpy(b.t, t, n * POLICY_OUT * sizeof(float), cudaMemcpyHostToDevice));
  MLP_CK(cudaMemcpy(b.sw, sw, n * sizeof(float), cudaMemcpyHostToDevice));
  MLP_CK(cudaMemset(b.grad, 0, POLICY_PARAMS * sizeof(float)));
  MLP_CK(cudaMemset(b.state, 0, 4 * sizeof(float)));
  MLP_CK(cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MlpShared)));
  return 0;
}

int check_rows(const float* x, const float* t, const float* sw, size_t n, double* wsum, char* err, size_t err_cap) {
  if (!x || !t || !sw || n == 0) { set_err(err, err_cap, "empty training set"); return -1; }
  double s = 0;
  for (size_t i = 0; i < n; i++) {
    if (!(sw[i] >= 0.f) || !std::isfinite(sw[i])) { set_err(err, err_cap, "row weights must be finite and >= 0"); return -1; }
    s += sw[i];
  }
  if (!(s > 0)) { set_err(err, err_cap, "row weights sum to zero"); return -1; }
  *wsum = s;
  return 0;
}

}  // namespace
}  // namespace hvm

using namespace hvm;

extern "C" int hvm_gb300_policy_forward(int device, const float* weights, const float* x, size_t n, float* y,
                                        char* err, size_t err_cap) {
  if (!weights || !x || !y) { set_err(err, err_cap, "null argument"); return -1; }
  if (n == 0) return 0;
  MLP_CK(cudaSetDevice(device));
  Buffers b;
  MLP_CK(cudaMalloc((void**)&b.w, POLICY_PARAMS * sizeof(float)));
  MLP_CK(cudaMalloc((void**)&b.x, n * POLICY_IN * sizeof(float)));
  MLP_CK(cudaMalloc((void**)&b.y, n * POLICY_OUT * sizeof(float)));
  MLP_CK(cudaMemcpy(b.w, weights, POLICY_PARAMS * sizeof(float), cudaMemcpyHostToDevice));
  MLP_CK(cudaMemcpy(b.x, x, n * POLICY_IN * sizeof(float), cudaMemcpyHostToDevice));
  unsigned grid = (unsigned)(n < 4096 ? n : 4096);
  policy_forward_kernel<<<grid, 128>>>(b.w, b.x, n, b.y);
  MLP_CK(cudaGetLastError());
  MLP_CK(cudaMemcpy(y, b.y, n * POLICY_OUT * sizeof(float), cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int hvm_gb300_policy_grad(int device, const float* weights, const float* x, const float* t,
                                     const float* sw, size_t n, float* grad, float* loss, char* err,
                                     size_t err_cap) {
  if (!weights || !grad || !loss) { set_err(err, err_cap, "null argument"); return -1; }
  double wsum = 0;
  if (check_rows(x, t, sw, n, &wsum, err, err_cap)) return -1;
  MLP_CK(cudaSetDevice(device));
  Buffers b;
  if (upload(b, weights, x, t, sw, n, err, err_cap)) return -1;
  mlp_grad_kernel<<<grad_grid(device), MLP_THREADS, sizeof(MlpShared)>>>(b.w, b.x, b.t, b.sw, n,
                                                                          (float)(1.0 / wsum), b.grad, b.state + 2);
  MLP_CK(cudaGetLastError());
  MLP_CK(cudaMemcpy(grad, b.grad, POLICY_PARAMS * sizeof(float), cudaMemcpyDeviceToHost));
  MLP_CK(cudaMemcpy(loss, b.state + 2, sizeof(float), cudaMemcpyDeviceToHost));
  return 0;
}

extern "C" int hvm_gb300_policy_train(int device, float* weights, const float* x, const float* t, const float* sw,
                                      size_t n, uint32_t epochs, float lr, float* loss, char* err, size_t err_cap) {
  if (!weights) { set_err(err, err_cap, "null argument"); return -1; }
  if (!(lr > 0.f) || !std::isfinite(lr)) { set_err(err, err_cap, "learning rate must be > 0"); return -1; }
  double wsum = 0;
  if (check_rows(x, t, sw, n, &wsum, err, err_cap)) return -1;
  MLP_CK(cudaSetDevice(device));
  Buffers b;
  if (upload(b, weights, x, t, sw, n, err, err_cap)) return -1;
  MLP_CK(cudaMalloc((void**)&b.m, POLICY_PARAMS * sizeof(float)));
  MLP_CK(cudaMalloc((void**)&b.v, POLICY_PARAMS * sizeof(float)));
  MLP_CK(cudaMemset(b.m, 0, POLICY_PARAMS * sizeof(float)));
  MLP_CK(cudaMemset(b.v, 0, POLICY_PARAMS * sizeof(float)));
  // One epoch = gradient + Adam step, captured once and replayed.
  cudaStream_t s = nullptr;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ge = nullptr;
  MLP_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  int rc = 0;
  const int grid = grad_grid(device);
  const float scale = (float)(1.0 / wsum);
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    mlp_grad_kernel<<<grid, MLP_THREADS, sizeof(MlpShared), s>>>(b.w, b.x, b.t, b.sw, n, scale, b.grad, b.state + 2);
    adam_kernel<<<1, 1024, 0, s>>>(b.w, b.grad, b.m, b.v, b.state, lr);
    e = cudaStreamEndCapture(s, &g);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&ge, g, 0);
  for (uint32_t i = 0; e == cudaSuccess && i < epochs; i++) e = cudaGraphLaunch(ge, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess) e = cudaMemcpy(weights, b.w, POLICY_PARAMS * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && loss) e = cudaMemcpy(loss, b.state + 1, sizeof(float), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    set_err(err, err_cap, std::string("policy training: ") + cudaGetErrorString(e));
    rc = -1;
  }
  if (ge) cudaGraphExecDestroy(ge);
  if (g) cudaGraphDestroy(g);
  cudaStreamDestroy(s);
  return rc;
}
