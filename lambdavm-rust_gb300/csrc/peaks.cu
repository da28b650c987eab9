// peaks.cu — a measured denominator for the evaluator's second roofline.
//
// The evaluator's net operations are 32-bit atomic exchanges on var words
// (the linker) and 64-bit node takes, scattered over the net. Their ceiling
// is the L2's atomic throughput, which no vendor table states for this
// access pattern, so it is measured: every thread of a full grid issues
// independent atomicExch operations at pseudo-random word addresses of a
// region (xorshift32 per thread), and the rate is operations per second of
// device time (CUDA events, after a warm-up launch).
#include <cuda_runtime.h>
#include <cstdint>
#include <cstring>
#include <string>

#include "hvm_gb300.h"

namespace {

__global__ void atomic_exch_probe(uint32_t* buf, uint64_t mask, uint32_t iters, uint32_t* sink) {
  uint32_t x = 0x9E3779B9u ^ (blockIdx.x * blockDim.x + threadIdx.x) * 0x85EBCA6Bu;
  uint32_t acc = 0;
  for (uint32_t i = 0; i < iters; i++) {
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    acc += atomicExch(&buf[x & mask], x);
  }
  if (acc == 0x12345678u) *sink = acc;  // keeps the results live
}

void set_err(char* err, size_t cap, const std::string& m) {
  if (err && cap) {
    size_t k = m.size() < cap - 1 ? m.size() : cap - 1;
    memcpy(err, m.data(), k);
    err[k] = 0;
  }
}

}  // namespace

extern "C" int hvm_gb300_atomic_peak(int device, uint64_t region_words, double* exch_per_s, char* err,
                                     size_t err_cap) {
  if (!exch_per_s || region_words < 1024 || (region_words & (region_words - 1))) {
    set_err(err, err_cap, "region_words must be a power of two >= 1024");
    return -1;
  }
  cudaError_t e = cudaSetDevice(device);
  int sms = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  uint32_t* buf = nullptr;
  uint32_t* sink = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  if (e == cudaSuccess) e = cudaMalloc((void**)&buf, region_words * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc((void**)&sink, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(buf, 0, region_words * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  const uint32_t blocks = (uint32_t)sms * 8, threads = 256, iters = 256;
  float ms = 0.f;
  if (e == cudaSuccess) {
    atomic_exch_probe<<<blocks, threads>>>(buf, region_words - 1, iters, sink);  // warm-up
    cudaEventRecord(a);
    atomic_exch_probe<<<blocks, threads>>>(buf, region_words - 1, iters, sink);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (buf) cudaFree(buf);
  if (sink) cudaFree(sink);
  if (e != cudaSuccess) {
    set_err(err, err_cap, std::string("atomic peak probe: ") + cudaGetErrorString(e));
    return -1;
  }
  *exch_per_s = (double)blocks * threads * iters / (ms * 1e-3);
  return 0;
}
