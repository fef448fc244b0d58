// Element colouring for the colour-ordered scatter.
//
// Two elements that share a vertex share DOFs (an edge or face DOF lies on shared
// vertices), so colouring the vertex-adjacency graph of the elements gives colour
// classes whose elements touch disjoint DOF sets.  Assembled one class per launch,
// every CSR entry then receives at most one contribution per launch, and the sums are
// formed in a fixed order (colour by colour): the values are bitwise reproducible,
// unlike reductions whose order depends on timing.
//
// The colouring is the greedy parallel method of Jones and Plassmann ("A parallel
// graph coloring heuristic", SIAM J. Sci. Comput. 14(3), 1993): in each round an
// uncoloured element whose hash priority beats every uncoloured neighbour takes the
// smallest colour no coloured neighbour has.  Each round reads the previous round's
// colours and writes a new array, so the result does not depend on timing.  Elements
// are then sorted by (colour, element id).
#include <cub/cub.cuh>

#include <vector>

#include "pxg_internal.h"

namespace pxg
{
namespace
{

constexpr int kMaxColours = 128;

__global__ void kNodeCount(uint32_t const * __restrict__ conn, int64_t n, int32_t * __restrict__ cnt)
{
  int64_t const k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < n)
    atomicAdd(cnt + conn[k], 1);
}

__global__ void kNodeFill(uint32_t const * __restrict__ conn, int64_t n, int nv, int32_t * __restrict__ cur,
                          uint32_t * __restrict__ elems)
{
  int64_t const k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < n)
    elems[atomicAdd(cur + conn[k], 1)] = (uint32_t)(k / nv);
}

// priority of an element: a 32-bit integer hash (the finaliser of MurmurHash3)
__device__ __forceinline__ uint32_t prio(uint32_t e)
{
  uint32_t h = e;
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}

__global__ void kColourRound(uint32_t const * __restrict__ conn, int64_t nelem, int nv,
                             int32_t const * __restrict__ nStart, uint32_t const * __restrict__ nElems,
                             int16_t const * __restrict__ colIn, int16_t * __restrict__ colOut,
                             unsigned long long * __restrict__ left, int * __restrict__ overflow)
{
  int64_t const e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= nelem)
    return;
  int16_t const c0 = colIn[e];
  if (c0 >= 0)
  {
    colOut[e] = c0;
    return;
  }
  uint32_t const pe = prio((uint32_t)e);
  unsigned long long used[2] = {0ull, 0ull};
  bool best = true;
  for (int v = 0; v < nv && best; ++v)
  {
    uint32_t const n = conn[e * nv + v];
    for (int32_t k = nStart[n]; k < nStart[n + 1]; ++k)
    {
      uint32_t const f = nElems[k];
      if (f == (uint32_t)e)
        continue;
      int const cf = colIn[f];
      if (cf < 0)
      {
        uint32_t const pf = prio(f);
        if (pf > pe || (pf == pe && f > (uint32_t)e))
        {
          best = false;
          break;
        }
      }
      else
        used[cf >> 6] |= 1ull << (cf & 63);
    }
  }
  if (!best)
  {
    colOut[e] = -1;
    atomicAdd(left, 1ull);
    return;
  }
  int c;
  if (~used[0])
    c = __ffsll((long long)~used[0]) - 1;
  else if (~used[1])
    c = 64 + __ffsll((long long)~used[1]) - 1;
  else
  {
    atomicExch(overflow, 1);
    c = kMaxColours - 1;
  }
  colOut[e] = (int16_t)c;
}

__global__ void kIota(uint32_t * __restrict__ v, int64_t n)
{
  int64_t const k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < n)
    v[k] = (uint32_t)k;
}

__global__ void kColourHist(int16_t const * __restrict__ col, int64_t n, int32_t * __restrict__ hist)
{
  int64_t const k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k < n)
    atomicAdd(hist + col[k], 1);
}

unsigned blocksOf(int64_t n) { return (unsigned)((n + 255) / 256); }

} // namespace

pxg_status buildColouring(pxg_ctx * c)
{
  if (c->colour.built)
    return PXG_OK;
  if (!c->conn.p || c->nelem <= 0)
    return fail(c, PXG_ERR_INVALID_ARG, "colouring needs a mesh");
  int64_t const E = c->nelem, nv = c->nv, nn = c->nnodes, ni = E * nv;
  if (ni >= (int64_t)1 << 31)
    return fail(c, PXG_ERR_UNSUPPORTED, "colouring: more than 2^31 element-vertex incidences");
  // vertex -> elements
  DevBuf<int32_t> nStart, cur;
  DevBuf<uint32_t> nElems;
  PXG_CUDA(c, nStart.alloc(nn + 1));
  PXG_CUDA(c, cur.alloc(nn + 1));
  PXG_CUDA(c, nElems.alloc(ni));
  PXG_CUDA(c, cudaMemset(cur.p, 0, (nn + 1) * 4));
  kNodeCount<<<blocksOf(ni), 256>>>(c->conn.p, ni, cur.p);
  size_t tb = 0;
  PXG_CUDA(c, cub::DeviceScan::ExclusiveSum(nullptr, tb, cur.p, nStart.p, nn + 1));
  DevBuf<unsigned char> tmp;
  PXG_CUDA(c, tmp.alloc(tb));
  PXG_CUDA(c, cub::DeviceScan::ExclusiveSum(tmp.p, tb, cur.p, nStart.p, nn + 1));
  PXG_CUDA(c, cudaMemcpy(cur.p, nStart.p, (nn + 1) * 4, cudaMemcpyDeviceToDevice));
  kNodeFill<<<blocksOf(ni), 256>>>(c->conn.p, ni, (int)nv, cur.p, nElems.p);
  PXG_CUDA(c, cudaGetLastError());
  // rounds
  DevBuf<int16_t> col[2];
  PXG_CUDA(c, col[0].alloc(E));
  PXG_CUDA(c, col[1].alloc(E));
  PXG_CUDA(c, cudaMemset(col[0].p, 0xff, E * 2));
  DevBuf<unsigned long long> left;
  DevBuf<int> overflow;
  PXG_CUDA(c, left.alloc(1));
  PXG_CUDA(c, overflow.alloc(1));
  PXG_CUDA(c, cudaMemset(overflow.p, 0, 4));
  int in = 0;
  for (int round = 0;; ++round)
  {
    if (round > 10000)
      return fail(c, PXG_ERR_NUMERIC, "colouring did not finish");
    PXG_CUDA(c, cudaMemset(left.p, 0, 8));
    kColourRound<<<blocksOf(E), 256>>>(c->conn.p, E, (int)nv, nStart.p, nElems.p, col[in].p, col[in ^ 1].p, left.p,
                                       overflow.p);
    PXG_CUDA(c, cudaGetLastError());
    in ^= 1;
    unsigned long long h = 0;
    PXG_CUDA(c, cudaMemcpy(&h, left.p, 8, cudaMemcpyDeviceToHost));
    if (h == 0)
      break;
  }
  int ovf = 0;
  PXG_CUDA(c, cudaMemcpy(&ovf, overflow.p, 4, cudaMemcpyDeviceToHost));
  if (ovf)
    return fail(c, PXG_ERR_UNSUPPORTED, "colouring needs more than %d colours", kMaxColours);
  // histogram and the element order (colour, element id): a stable radix sort by colour
  DevBuf<int32_t> hist;
  PXG_CUDA(c, hist.alloc(kMaxColours));
  PXG_CUDA(c, cudaMemset(hist.p, 0, kMaxColours * 4));
  kColourHist<<<blocksOf(E), 256>>>(col[in].p, E, hist.p);
  std::vector<int32_t> h(kMaxColours);
  PXG_CUDA(c, cudaMemcpy(h.data(), hist.p, kMaxColours * 4, cudaMemcpyDeviceToHost));
  int ncol = 0;
  for (int k = 0; k < kMaxColours; ++k)
    if (h[k])
      ncol = k + 1;
  DevBuf<uint32_t> iota, permOut;
  DevBuf<int16_t> keysOut;
  PXG_CUDA(c, iota.alloc(E));
  PXG_CUDA(c, keysOut.alloc(E));
  PXG_CUDA(c, c->colour.perm.alloc(E));
  kIota<<<blocksOf(E), 256>>>(iota.p, E);
  tb = 0;
  auto * keysIn = reinterpret_cast<uint16_t *>(col[in].p); // colours are >= 0 now
  auto * keysSorted = reinterpret_cast<uint16_t *>(keysOut.p);
  PXG_CUDA(c, cub::DeviceRadixSort::SortPairs(nullptr, tb, keysIn, keysSorted, iota.p, c->colour.perm.p, E, 0, 8));
  PXG_CUDA(c, tmp.alloc(tb));
  PXG_CUDA(c, cub::DeviceRadixSort::SortPairs(tmp.p, tb, keysIn, keysSorted, iota.p, c->colour.perm.p, E, 0, 8));
  PXG_CUDA(c, cudaDeviceSynchronize());
  c->colour.start.assign(ncol + 1, 0);
  for (int k = 0; k < ncol; ++k)
    c->colour.start[k + 1] = c->colour.start[k] + h[k];
  c->colour.ncol = ncol;
  c->colour.built = true;
  return PXG_OK;
}

} // namespace pxg
