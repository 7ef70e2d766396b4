// Live peak probes for the roofline denominators of the pivot kernels.
//
// The pivot update is bound by shared-memory bandwidth (FP32 tableau) or by
// the FP64 FMA pipe (FP64 tableau, one FMA per element per pivot).  Neither
// figure is a published GB300 constant, so blpg_measure_peaks times three
// synthetic kernels on the running device:
//   smem:  every thread streams float4 loads and stores over a shared buffer
//          (bytes read + written per second);
//   fp64 / fp32: independent FMA chains per thread (2 flops per FMA).
#include <cuda_runtime.h>

#include <cstdint>

#include "blpg_internal.h"

namespace {

__device__ __forceinline__ float4 lds4(unsigned addr) {
  float4 v;
  asm volatile("ld.volatile.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"(addr)
               : "memory");
  return v;
}
__device__ __forceinline__ void sts4(unsigned addr, float4 v) {
  asm volatile("st.volatile.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(v.x), "f"(v.y),
               "f"(v.z), "f"(v.w)
               : "memory");
}

// Volatile 16-byte shared loads and stores (they cannot be forwarded or
// removed), four independent streams per thread, bank-conflict free.
__global__ void __launch_bounds__(512) smem_probe(float* sink, int iters) {
  extern __shared__ float4 buf[];  // 2048 float4 (32 KB) per CTA
  const int t = threadIdx.x;
  for (int i = t; i < 2048; i += 512) buf[i] = make_float4(i, i + 1, i + 2, i + 3);
  __syncthreads();
  const unsigned base_addr = (unsigned)__cvta_generic_to_shared(buf);
  float acc = 0.f;
  for (int it = 0; it < iters; ++it) {
    const int base = (it & 3) * 512;
    const unsigned a0 = base_addr + 16u * ((base + t) & 2047);
    const unsigned a1 = base_addr + 16u * ((base + 512 + t) & 2047);
    const unsigned a2 = base_addr + 16u * ((base + 1024 + t) & 2047);
    const unsigned a3 = base_addr + 16u * ((base + 1536 + t) & 2047);
    float4 v0 = lds4(a0), v1 = lds4(a1), v2 = lds4(a2), v3 = lds4(a3);
    acc += v0.x + v1.y + v2.z + v3.w;
    v0.y += 1.f;
    v1.z += 1.f;
    v2.w += 1.f;
    v3.x += 1.f;
    sts4(a2, v0);
    sts4(a3, v1);
    sts4(a0, v2);
    sts4(a1, v3);
  }
  if (acc == -1.0f) sink[t] = acc;
}

template <typename T>
__global__ void __launch_bounds__(256) fma_probe(T* sink, int iters, T a) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
    x6 = x0 + 6, x7 = x0 + 7;
  const T b = (T)0.5;
  for (int it = 0; it < iters; ++it) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (T)-1) sink[threadIdx.x] = s;
}

float time_ms(cudaEvent_t e0, cudaEvent_t e1) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  return ms;
}

}  // namespace

extern "C" int32_t blpg_measure_peaks(int32_t device, double* smem_gbs, double* fp64_tflops,
                                      double* fp32_tflops) {
  using blpg::fail;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess || cudaSetDevice(device) != cudaSuccess)
    return fail(BLPG_ENODEV, "blpg_measure_peaks: no device %d", device);
  const int sms = prop.multiProcessorCount;
  float* sink = nullptr;
  if (cudaMalloc(&sink, 4096 * sizeof(double)) != cudaSuccess)
    return fail(BLPG_ENOMEM, "blpg_measure_peaks: cudaMalloc");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best_smem = 0, best64 = 0, best32 = 0;
  const int smem_iters = 1 << 12;
  const int blocks = sms * 4;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    smem_probe<<<blocks, 512, 2048 * sizeof(float4)>>>(sink, smem_iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    double bytes = (double)blocks * 512 * smem_iters * 128.0;  // 4 x (16 B load + 16 B store)
    double gbs = bytes / (time_ms(e0, e1) * 1e-3) / 1e9;
    if (rep > 0 && gbs > best_smem) best_smem = gbs;
  }
  for (int rep = 0; rep < 3; ++rep) {
    const int it64 = 1 << 11, it32 = 1 << 12, fb = sms * 8;
    cudaEventRecord(e0);
    fma_probe<double><<<fb, 256>>>((double*)sink, it64, 0.999);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    double t64 = (double)fb * 256 * it64 * 8 * 2 / (time_ms(e0, e1) * 1e-3) / 1e12;
    cudaEventRecord(e0);
    fma_probe<float><<<fb, 256>>>(sink, it32, 0.999f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    double t32 = (double)fb * 256 * it32 * 8 * 2 / (time_ms(e0, e1) * 1e-3) / 1e12;
    if (rep > 0) {
      if (t64 > best64) best64 = t64;
      if (t32 > best32) best32 = t32;
    }
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (err != cudaSuccess)
    return fail(BLPG_ECUDA, "blpg_measure_peaks: %s", cudaGetErrorString(err));
  if (smem_gbs) *smem_gbs = best_smem;
  if (fp64_tflops) *fp64_tflops = best64;
  if (fp32_tflops) *fp32_tflops = best32;
  return BLPG_OK;
}
