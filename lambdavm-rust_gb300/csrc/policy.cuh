// policy.cuh — the turn scheduler's decision, fixed or learned.
//
// At the end of every turn the last block picks the next turn's parameters:
//   budget       rounds a warp may run before the turn ends
//   stop frac    the turn ends once busy threads fall below (1 - frac) of the
//                initially busy ones (threads that ran dry hand their share
//                back through the ring)
//   static share input redexes each thread takes at turn start (the rest is
//                claimed dynamically)
// The fixed policy (runtime.cu, fixed_policy) is the GB300 counterpart of the
// reference's SEED/GROW/WORK mode machine (src/hvm.cu:1509-1548). The learned
// policy is a small FP32 MLP (16 features -> 64 -> 64 -> 3, ReLU, sigmoid
// outputs) evaluated by the last block with warp-level dot products; it only
// changes the order of reduction, never the normal form or the interaction
// count. The fixed policy remains the fallback (mode 0, or a non-finite
// output).
#pragma once
#include <stdint.h>
#include "hvm_defs.h"

HVM_NS_BEGIN

constexpr int POLICY_IN = 16, POLICY_HID = 64, POLICY_OUT = 3;
// Packed weights: W1[64][16] b1[64] W2[64][64] b2[64] W3[3][64] b3[3].
constexpr int POLICY_W1 = 0;
constexpr int POLICY_B1 = POLICY_W1 + POLICY_HID * POLICY_IN;
constexpr int POLICY_W2 = POLICY_B1 + POLICY_HID;
constexpr int POLICY_B2 = POLICY_W2 + POLICY_HID * POLICY_HID;
constexpr int POLICY_W3 = POLICY_B2 + POLICY_HID;
constexpr int POLICY_B3 = POLICY_W3 + POLICY_OUT * POLICY_HID;
constexpr int POLICY_PARAMS = POLICY_B3 + POLICY_OUT;

// POLICY_SCRIPT: the decision at the close of turn k is script[3k .. 3k+2]
// (Ctl::policy_w, Ctl::policy_script_len turns; -1 or past the end: fixed).
enum : uint32_t { POLICY_FIXED = 0, POLICY_LEARNED = 1, POLICY_CONSTANT = 2, POLICY_SCRIPT = 3 };

__device__ __forceinline__ float policy_sigmoid(float x) { return 1.0f / (1.0f + __expf(-x)); }

// Forward pass by one block: feat[16] -> out[3] (all in shared memory).
// Layers 1 and 2: one hidden unit per thread; layer 3: each output is a
// 64-long dot product by warp 0 (two inputs per lane, shuffle reduction).
__device__ __forceinline__ void policy_infer_block(const float* __restrict__ w, const float* feat, float* h1,
                                                   float* h2, float* out) {
  for (int j = threadIdx.x; j < POLICY_HID; j += blockDim.x) {
    float z = __ldg(&w[POLICY_B1 + j]);
    #pragma unroll
    for (int i = 0; i < POLICY_IN; i++) z = fmaf(__ldg(&w[POLICY_W1 + j * POLICY_IN + i]), feat[i], z);
    h1[j] = z > 0.f ? z : 0.f;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < POLICY_HID; j += blockDim.x) {
    float z = __ldg(&w[POLICY_B2 + j]);
    for (int i = 0; i < POLICY_HID; i++) z = fmaf(__ldg(&w[POLICY_W2 + j * POLICY_HID + i]), h1[i], z);
    h2[j] = z > 0.f ? z : 0.f;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int l = threadIdx.x;
    for (int o = 0; o < POLICY_OUT; o++) {
      float p = __ldg(&w[POLICY_W3 + o * POLICY_HID + l]) * h2[l] +
                __ldg(&w[POLICY_W3 + o * POLICY_HID + l + 32]) * h2[l + 32];
      for (int s = 16; s > 0; s >>= 1) p += __shfl_down_sync(0xFFFFFFFFu, p, s);
      if (l == 0) out[o] = policy_sigmoid(p + __ldg(&w[POLICY_B3 + o]));
    }
  }
  __syncthreads();
}

HVM_NS_END
