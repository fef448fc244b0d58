// pxg_prune_csr_noalloc: the closeMatrix prune/compact (|v| <= 1e-16 dropped) of a
// CSR matrix, for callers that cannot allocate GPU memory.
//
// Who needs it: code that runs where cudaMalloc is not allowed or not safe, for
// example inside a host callback or a memory-pool-managed runtime that forbids
// driver allocations, a signal-safe or real-time section, or a plugin whose host
// application owns every device allocation.  Such a caller passes its own input and
// output buffers; the intermediate per-row counts and scan partials live in a
// fixed-size device array that is part of this library's image.
//
// Limits and behaviour:
//   - at most kMaxRows rows (4,194,304); larger matrices are rejected with
//     PXG_ERR_INVALID_ARG before anything runs;
//   - the scratch array (16.8 MB) is held on every GPU that loads the library until
//     the process exits;
//   - the first call on a device looks up the array's device address (set-up once per
//     device, with that device current);
//   - every call copies the kept count back to the host and synchronises `stream`
//     before it returns, so a call cannot be captured into a CUDA graph;
//   - every call shares the one array: calls that overlap on the GPU (different
//     streams or threads) race and corrupt each other's result; serialise them;
//   - the array keeps the last call's contents; each call writes every entry it later
//     reads, so nothing has to start at zero;
//   - no cudaMalloc, cudaFree or allocating library routine is called.
#include <cub/block/block_scan.cuh>

#include <mutex>

#include "pxg_internal.h"

namespace
{

constexpr int64_t kMaxRows = int64_t(1) << 22;
constexpr int kRowsPerBlock = 1024;
constexpr int64_t kMaxBlocks = kMaxRows / kRowsPerBlock;
// [0, kMaxRows): per-row exclusive prefix inside its block
// [kMaxRows, kMaxRows + kMaxBlocks): per-block totals, then their exclusive prefix
// [kMaxRows + kMaxBlocks]: total number of kept entries
constexpr int64_t kScratchWords = kMaxRows + kMaxBlocks + 64;

static __device__ __align__(256) int32_t gPruneScratch[kScratchWords];

__device__ __forceinline__ bool keep(double v) { return !(fabs(v) <= 1e-16); }

__global__ void __launch_bounds__(kRowsPerBlock)
    kNaCount(int32_t const * __restrict__ rowPtr, double const * __restrict__ vals, int64_t n,
             int32_t * __restrict__ scratch)
{
  using BS = cub::BlockScan<int32_t, kRowsPerBlock>;
  __shared__ typename BS::TempStorage ts;
  int64_t const r = blockIdx.x * (int64_t)kRowsPerBlock + threadIdx.x;
  int32_t cnt = 0;
  if (r < n)
    for (int32_t p = rowPtr[r]; p < rowPtr[r + 1]; ++p)
      cnt += keep(vals[p]) ? 1 : 0;
  int32_t pre, tot;
  BS(ts).ExclusiveSum(cnt, pre, tot);
  if (r < n)
    scratch[r] = pre;
  if (threadIdx.x == 0)
    scratch[kMaxRows + blockIdx.x] = tot;
}

// exclusive scan of the block totals (at most kMaxBlocks = 4 per thread)
__global__ void __launch_bounds__(kRowsPerBlock) kNaScanBlocks(int64_t nb, int32_t * __restrict__ scratch)
{
  using BS = cub::BlockScan<int32_t, kRowsPerBlock>;
  __shared__ typename BS::TempStorage ts;
  constexpr int PER = (int)(kMaxBlocks / kRowsPerBlock);
  int32_t v[PER];
  int32_t s = 0;
#pragma unroll
  for (int k = 0; k < PER; ++k)
  {
    int64_t const b = (int64_t)threadIdx.x * PER + k;
    v[k] = (b < nb) ? scratch[kMaxRows + b] : 0;
    s += v[k];
  }
  int32_t pre, tot;
  BS(ts).ExclusiveSum(s, pre, tot);
#pragma unroll
  for (int k = 0; k < PER; ++k)
  {
    int64_t const b = (int64_t)threadIdx.x * PER + k;
    if (b < nb)
      scratch[kMaxRows + b] = pre;
    pre += v[k];
  }
  if (threadIdx.x == 0)
    scratch[kMaxRows + kMaxBlocks] = tot;
}

__global__ void kNaCompact(int32_t const * __restrict__ rowPtr, int32_t const * __restrict__ col,
                           double const * __restrict__ vals, int64_t n, int32_t const * __restrict__ scratch,
                           int32_t * __restrict__ rowPtrOut, int32_t * __restrict__ colOut,
                           double * __restrict__ valOut)
{
  int64_t const r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n)
    return;
  int32_t o = scratch[r] + scratch[kMaxRows + r / kRowsPerBlock];
  rowPtrOut[r] = o;
  for (int32_t p = rowPtr[r]; p < rowPtr[r + 1]; ++p)
    if (keep(vals[p]))
    {
      colOut[o] = col[p];
      valOut[o] = vals[p];
      ++o;
    }
  if (r == n - 1)
    rowPtrOut[n] = scratch[kMaxRows + kMaxBlocks];
}

std::mutex gSetupMutex;
int32_t * gScratchPtr[64] = {nullptr};

} // namespace

extern "C" pxg_status pxg_prune_csr_noalloc(int32_t const * row_ptr, int32_t const * col_idx,
                                            double const * vals, int64_t nrows, int32_t * row_ptr_out,
                                            int32_t * col_idx_out, double * vals_out, int64_t * nnz_out,
                                            void * stream)
{
  if (!row_ptr || !col_idx || !vals || !row_ptr_out || !col_idx_out || !vals_out || !nnz_out)
    return PXG_ERR_INVALID_ARG;
  if (nrows <= 0 || nrows > kMaxRows)
    return PXG_ERR_INVALID_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
  {
    cudaGetLastError();
    return PXG_ERR_NO_DEVICE;
  }
  int32_t * scratch = nullptr;
  {
    // set-up once per device: the host-side name of the array is not a device
    // address; ask the runtime for the address on the current device
    std::lock_guard<std::mutex> lock(gSetupMutex);
    if (!gScratchPtr[dev])
    {
      void * p = nullptr;
      cudaError_t const e = cudaGetSymbolAddress(&p, gPruneScratch);
      if (e != cudaSuccess || !p)
      {
        cudaGetLastError();
        return PXG_ERR_CUDA;
      }
      gScratchPtr[dev] = static_cast<int32_t *>(p);
    }
    scratch = gScratchPtr[dev];
  }
  cudaStream_t const s = (cudaStream_t)stream;
  int64_t const nb = (nrows + kRowsPerBlock - 1) / kRowsPerBlock;
  kNaCount<<<(unsigned)nb, kRowsPerBlock, 0, s>>>(row_ptr, vals, nrows, scratch);
  kNaScanBlocks<<<1, kRowsPerBlock, 0, s>>>(nb, scratch);
  kNaCompact<<<(unsigned)((nrows + 255) / 256), 256, 0, s>>>(row_ptr, col_idx, vals, nrows, scratch, row_ptr_out,
                                                             col_idx_out, vals_out);
  if (cudaGetLastError() != cudaSuccess)
    return PXG_ERR_CUDA;
  int32_t total = 0;
  if (cudaMemcpyAsync(&total, scratch + kMaxRows + kMaxBlocks, sizeof(int32_t), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
  {
    cudaGetLastError();
    return PXG_ERR_CUDA;
  }
  *nnz_out = total;
  return PXG_OK;
}
