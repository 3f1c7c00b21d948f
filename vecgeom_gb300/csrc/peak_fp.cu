// peak_fp.cu -- FMA throughput probe for the compute roofline (libvgpeak.so).
//
// The navigation kernels are bound by the FP64 and FP32/integer pipes, not by
// HBM; their roofline denominators are the pipes' measured peaks.  Each thread
// runs eight independent fused multiply-add chains, enough to keep the pipe
// busy at full occupancy; the result is written so the chains stay live.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

template <typename T>
__device__ __forceinline__ T fma_rn(T a, T b, T c);
template <>
__device__ __forceinline__ double fma_rn<double>(double a, double b, double c)
{
  return __fma_rn(a, b, c);
}
template <>
__device__ __forceinline__ float fma_rn<float>(float a, float b, float c)
{
  return __fmaf_rn(a, b, c);
}

template <typename T>
__global__ void __launch_bounds__(256) fma_chains(int iters, T seed, T *out)
{
  T a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + (T)(threadIdx.x + k);
  const T b = (T)0.999999, c = (T)1e-7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma_rn<T>(a[k], b, c);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <typename T>
int run(int device, int iters, float *ms, double *flops)
{
  int sms = 0;
  if (cudaSetDevice(device) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 1;
  const int block = 256, grid = sms * 8;
  T *out          = nullptr;
  if (cudaMalloc(&out, sizeof(T) * (size_t)grid * block) != cudaSuccess) return 2;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chains<T><<<grid, block>>>(iters / 8, (T)1, out);  // warm-up
  cudaEventRecord(e0);
  fma_chains<T><<<grid, block>>>(iters, (T)1, out);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float t       = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return 3;
  *ms    = t;
  *flops = 2.0 * 8.0 * (double)iters * (double)grid * (double)block;
  return 0;
}

}  // namespace

// Times one launch of the FMA chains on `device` (fp64 != 0: double, else float).
// Returns 0 and the launch time and FLOPs performed, or a non-zero code.
extern "C" int vgp_fma_peak(int device, int fp64, int iters, float *ms, double *flops)
{
  if (!ms || !flops || iters < 8) return 1;
  return fp64 ? run<double>(device, iters, ms, flops) : run<float>(device, iters, ms, flops);
}
