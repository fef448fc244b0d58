// Measured device rates that bound the element kernels: the FP64 FMA rate
// (pxg_fp64_rate) and the rate of FP64 reductions in L2 by lane pattern (pxg_red_rate).
//
// Every thread runs kChains independent FMA chains (x <- x a + b) for `iters`
// iterations, so the FP64 pipe always has independent work; the grid holds several
// blocks per SM.  The rate is the number of FMAs divided by the event-timed duration of
// one launch (after a warm-up launch), taken as the best of a few launches.
#include "pxg_internal.h"

namespace pxg
{
namespace
{
constexpr int kChains = 8;

__global__ void __launch_bounds__(256) kFp64Fma(double a, double b, int iters, double * out)
{
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c)
    x[c] = (threadIdx.x + c) * 1e-9;
#pragma unroll 4
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int c = 0; c < kChains; ++c)
      x[c] = fma(x[c], a, b);
  double s = 0.;
#pragma unroll
  for (int c = 0; c < kChains; ++c)
    s += x[c];
  // a store the compiler cannot drop; the value never equals the sentinel in practice
  if (s == -1.0)
    out[blockIdx.x] = s;
}

__device__ __forceinline__ uint32_t mix32(uint32_t x)
{
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

// every warp instruction adds 1.0 to 32 doubles: `per` consecutive lanes share one
// 32-byte sector (spread over it), the sectors are hashed over the array (nsect sectors,
// a power of two), so that the pattern is the scatter's, not a stream
template <int PER>
__global__ void __launch_bounds__(256) kRedRate(double * p, uint32_t nsect, int reps)
{
  uint32_t const lane = threadIdx.x & 31, warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  uint32_t const group = lane / PER, sub = lane % PER;
  for (int r = 0; r < reps; ++r)
  {
    uint32_t const s = mix32(warp * 1315423911u + (uint32_t)r * 2654435761u + group * 97u) & (nsect - 1);
    atomicAdd(p + 4ull * s + sub * (4 / PER), 1.0);
  }
}
} // namespace
} // namespace pxg

using namespace pxg;

extern "C" pxg_status pxg_red_rate(int device, int lanes_per_sector, int64_t bytes, double * red_per_s, double * ms_out)
{
  if (!red_per_s || (lanes_per_sector != 1 && lanes_per_sector != 2 && lanes_per_sector != 4) || bytes < 4096 ||
      (bytes & (bytes - 1)) || bytes > (int64_t)1 << 35)
    return PXG_ERR_INVALID_ARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
  {
    cudaGetLastError();
    return PXG_ERR_NO_DEVICE;
  }
  if (cudaSetDevice(device) != cudaSuccess)
    return PXG_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return PXG_ERR_CUDA;
  int const threads = 256, blocks = sms * 8, reps = 64;
  uint32_t const nsect = (uint32_t)(bytes / 32);
  double * p = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  pxg_status st = PXG_OK;
  if (cudaMalloc(&p, (size_t)bytes) != cudaSuccess || cudaMemset(p, 0, (size_t)bytes) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    st = PXG_ERR_CUDA;
  double best = 1e300;
  for (int rep = 0; rep < 4 && st == PXG_OK; ++rep)
  {
    cudaEventRecord(e0);
    if (lanes_per_sector == 1)
      kRedRate<1><<<blocks, threads>>>(p, nsect, reps);
    else if (lanes_per_sector == 2)
      kRedRate<2><<<blocks, threads>>>(p, nsect, reps);
    else
      kRedRate<4><<<blocks, threads>>>(p, nsect, reps);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess)
    {
      st = PXG_ERR_CUDA;
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) // the first launch warms up
      best = ms;
  }
  if (st == PXG_OK && cudaGetLastError() != cudaSuccess)
    st = PXG_ERR_CUDA;
  if (e0)
    cudaEventDestroy(e0);
  if (e1)
    cudaEventDestroy(e1);
  if (p)
    cudaFree(p);
  if (st != PXG_OK)
    return st;
  *red_per_s = (double)blocks * threads * reps / (best * 1e-3);
  if (ms_out)
    *ms_out = best;
  return PXG_OK;
}

extern "C" pxg_status pxg_fp64_rate(int device, double * fma_per_s, double * ms_out)
{
  if (!fma_per_s)
    return PXG_ERR_INVALID_ARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
  {
    cudaGetLastError();
    return PXG_ERR_NO_DEVICE;
  }
  if (cudaSetDevice(device) != cudaSuccess)
    return PXG_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return PXG_ERR_CUDA;
  int const threads = 256, blocks = sms * 4, iters = 1 << 15;
  double * out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  pxg_status st = PXG_OK;
  if (cudaMalloc(&out, sizeof(double) * blocks) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
      cudaEventCreate(&e1) != cudaSuccess)
    st = PXG_ERR_CUDA;
  double best = 1e300;
  for (int rep = 0; rep < 4 && st == PXG_OK; ++rep)
  {
    cudaEventRecord(e0);
    kFp64Fma<<<blocks, threads>>>(0.9999999, 1e-7, iters, out);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess)
    {
      st = PXG_ERR_CUDA;
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) // the first launch warms up
      best = ms;
  }
  if (st == PXG_OK && cudaGetLastError() != cudaSuccess)
    st = PXG_ERR_CUDA;
  if (e0)
    cudaEventDestroy(e0);
  if (e1)
    cudaEventDestroy(e1);
  if (out)
    cudaFree(out);
  if (st != PXG_OK)
    return st;
  *fma_per_s = (double)blocks * threads * kChains * (double)iters / (best * 1e-3);
  if (ms_out)
    *ms_out = best;
  return PXG_OK;
}
