// Measured ceilings for the march's roofline.  The march kernels keep the
// snapshot in L2 and are bound by L2 latency, instruction issue and the SFU
// rather than by HBM, so the benchmark reports each kernel against the
// ceiling that binds it.  Three small kernels measure those ceilings on the
// device at hand:
//
//  * l2_stream: float4 reads (ld.global.cg: L2, not L1) of a buffer that fits
//    in L2, over and over: the L2 read bandwidth;
//  * l2_gather: float4 reads at pseudo-random positions of the same buffer,
//    four independent chains per thread: the rate of 16-byte gathers that hit
//    L2, the access pattern of the march's candidate and payload loads
//    (useful bytes: 16 per gather, although each brings a 32-byte sector);
//  * ex2: ex2.approx.ftz.f32 in eight independent chains per thread: the SFU's
//    throughput, which bounds the emission pass (one ex2 per lambda bin, line
//    and run of equal neighbours).
//
// Nothing here is on a render path; fomo_measure_ceilings runs them on request.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fomo_gpu.h"
#include "fomo_device.cuh"
#include "runtime_internal.h"

namespace fomo {
namespace {

__global__ void l2_stream_kernel(const float4* __restrict__ buf, int64_t n4, int reps, float* sink) {
  float acc = 0.0f;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int r = 0; r < reps; ++r)
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4; i += stride) {
      const float4 v = __ldcg(buf + i);
      acc += (v.x + v.y) + (v.z + v.w);
    }
  if (acc == 1.2345f) sink[0] = acc;  // never true for the zero buffer; keeps the loads
}

__global__ void l2_gather_kernel(const float4* __restrict__ buf, uint32_t mask, int iters, float* sink) {
  uint32_t s0 = 0x9e3779b9u * (blockIdx.x * blockDim.x + threadIdx.x + 1);
  uint32_t s1 = s0 ^ 0x85ebca6bu, s2 = s0 ^ 0xc2b2ae35u, s3 = s0 ^ 0x27d4eb2fu;
  float acc = 0.0f;
  for (int it = 0; it < iters; ++it) {
    // xorshift positions, four independent gathers in flight per thread
    s0 ^= s0 << 13; s0 ^= s0 >> 17; s0 ^= s0 << 5;
    s1 ^= s1 << 13; s1 ^= s1 >> 17; s1 ^= s1 << 5;
    s2 ^= s2 << 13; s2 ^= s2 >> 17; s2 ^= s2 << 5;
    s3 ^= s3 << 13; s3 ^= s3 >> 17; s3 ^= s3 << 5;
    const float4 a = __ldg(buf + (s0 & mask)), b = __ldg(buf + (s1 & mask));
    const float4 c = __ldg(buf + (s2 & mask)), d = __ldg(buf + (s3 & mask));
    acc += (a.x + b.y) + (c.z + d.w);
  }
  if (acc == 1.2345f) sink[0] = acc;
}

__global__ void ex2_kernel(int iters, float* sink) {
  float x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = -0.001f * (float)((threadIdx.x + k) & 63);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = ex2_approx(x[k]) - 1.5f;  // stays in [-1.5, -0.5]
  }
  float acc = 0.0f;
#pragma unroll
  for (int k = 0; k < 8; ++k) acc += x[k];
  if (acc == 1.2345f) sink[0] = acc;
}

// Median of three timed launches (CUDA events on the context's stream).
template <typename F>
float time_ms(cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1, F launch) {
  launch();  // warm-up
  float t[3];
  for (int k = 0; k < 3; ++k) {
    cudaEventRecord(e0, s);
    launch();
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&t[k], e0, e1);
  }
  if (t[0] > t[1]) { const float u = t[0]; t[0] = t[1]; t[1] = u; }
  if (t[1] > t[2]) { const float u = t[1]; t[1] = t[2]; t[2] = u; }
  if (t[0] > t[1]) { const float u = t[0]; t[0] = t[1]; t[1] = u; }
  return t[1];
}

}  // namespace
}  // namespace fomo

using namespace fomo;

extern "C" int fomo_measure_ceilings(fomo_ctx* ctx, fomo_ceilings* out) {
  if (!ctx || !out) return FOMO_EINVAL;
  cudaSetDevice(ctx->device);
  const size_t bytes = size_t(64) << 20;  // fits the 126 MB L2 with room to spare
  void* buf = nullptr;
  int rc = dev_alloc(ctx, &buf, bytes + 256);
  if (rc) return rc;
  cudaStream_t s = ctx->stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaMemsetAsync(buf, 0, bytes + 256, s);
  if (e != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    dev_free(ctx, buf);
    return cuda_err(ctx, e, "ceilings set-up");
  }
  const float4* b4 = static_cast<const float4*>(buf);
  float* sink = reinterpret_cast<float*>(static_cast<char*>(buf) + bytes);
  const int64_t n4 = (int64_t)(bytes / sizeof(float4));
  const int threads = 256;
  const int blocks = ctx->sm_count * 8;  // 64 warps per SM
  const int reps = 64;
  const float ms_stream = time_ms(s, e0, e1, [&] { l2_stream_kernel<<<blocks, threads, 0, s>>>(b4, n4, reps, sink); });
  const int giters = 256;
  const float ms_gather = time_ms(s, e0, e1, [&] {
    l2_gather_kernel<<<blocks, threads, 0, s>>>(b4, (uint32_t)(n4 - 1), giters, sink);
  });
  const int xiters = 1024;
  const float ms_ex2 = time_ms(s, e0, e1, [&] { ex2_kernel<<<blocks, threads, 0, s>>>(xiters, sink); });
  e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  dev_free(ctx, buf);
  if (e != cudaSuccess) return cuda_err(ctx, e, "ceilings kernels");
  const double nthreads = (double)blocks * threads;
  out->l2_read_gbs = (double)bytes * reps / (ms_stream * 1e-3) / 1e9;
  out->l2_gather_gbs = nthreads * giters * 4.0 * 16.0 / (ms_gather * 1e-3) / 1e9;
  out->ex2_per_s = nthreads * xiters * 8.0 / (ms_ex2 * 1e-3);
  out->sm_count = ctx->sm_count;
  return FOMO_OK;
}
