// Peak issue rates of the current GPU for the pipes the step uses: FP64 FMA
// (the phi-FFTs and the dense FP64 kernels) and bf16 mma.sync m16n8k16 with
// fp32 accumulation (the tensor-core stage).  Each probe keeps eight
// independent accumulation chains per thread (or four MMA chains per warp)
// in flight on 8 blocks of 256 threads per SM, long enough (tens of ms) for
// launch costs to vanish.
#include <cuda_runtime.h>

#include "pizza_gpu.h"

namespace {

__global__ void k_probe_dfma(double* out, int iters, double a) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
         x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      x0 = fma(x0, a, 1.0); x1 = fma(x1, a, 1.0); x2 = fma(x2, a, 1.0); x3 = fma(x3, a, 1.0);
      x4 = fma(x4, a, 1.0); x5 = fma(x5, a, 1.0); x6 = fma(x6, a, 1.0); x7 = fma(x7, a, 1.0);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_probe_mma(float* out, int iters) {
  const unsigned a0 = 0x3f803f80u + threadIdx.x, b0 = 0x3f003f00u;
  float c[4][4] = {};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 8; ++u) {
#pragma unroll
      for (int q = 0; q < 4; ++q)
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
            "{%0,%1,%2,%3};\n"
            : "+f"(c[q][0]), "+f"(c[q][1]), "+f"(c[q][2]), "+f"(c[q][3])
            : "r"(a0), "r"(a0), "r"(a0), "r"(a0), "r"(b0), "r"(b0));
    }
  }
  float s = 0.f;
  for (int q = 0; q < 4; ++q) s += c[q][0] + c[q][1] + c[q][2] + c[q][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

extern "C" int pz_probe_peaks(double* dfma_tflops, double* mma_bf16_tflops) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (!e) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e) return PZ_E_CUDA;
  const int blocks = 8 * sms, threads = 256;
  void* buf = nullptr;
  if (cudaMalloc(&buf, (size_t)blocks * threads * sizeof(double))) return PZ_E_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float ms = 0.f;
  int rc = PZ_OK;
  for (int rep = 0; rep < 2 && rc == PZ_OK; ++rep) {   // the first launch of each is a warm-up
    const int it_d = 2000, it_m = 4000;
    cudaEventRecord(e0);
    k_probe_dfma<<<blocks, threads>>>(static_cast<double*>(buf), it_d, 0.999999);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) || cudaGetLastError()) { rc = PZ_E_CUDA; break; }
    cudaEventElapsedTime(&ms, e0, e1);
    if (dfma_tflops) *dfma_tflops = 2.0 * 64.0 * it_d * (double)blocks * threads / (ms * 1e-3) / 1e12;
    cudaEventRecord(e0);
    k_probe_mma<<<blocks, threads>>>(static_cast<float*>(buf), it_m);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) || cudaGetLastError()) { rc = PZ_E_CUDA; break; }
    cudaEventElapsedTime(&ms, e0, e1);
    if (mma_bf16_tflops)
      *mma_bf16_tflops = 4096.0 * 32.0 * it_m * (double)blocks * (threads / 32) / (ms * 1e-3) / 1e12;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  return rc;
}
