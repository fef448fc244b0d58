// Device construction of the DOF map and of the structural CSR pattern.
//
// DOF map: proxpde numbers DOFs by first touch (include/dof.hpp:111-329): the element
// loop visits the local DOF slots s = e * N + l in increasing order (points, then
// edges, then faces, then the element) and a DOF entity gets the next id the first
// time one of its slots is met.  The id of an entity is therefore the number of
// "first-touch" slots before its own first slot, which the device computes in
// parallel: first slot of every entity (atomicMin for points, a stable sort by entity
// key for edges and faces), a flag per slot, an exclusive scan.
//
// Pattern: the element loop emits every pair (emap[e][i], emap[e][j])
// (include/builder.hpp:131-152); Eigen's setFromTriplets keeps one entry per distinct
// pair, sorted by column inside each outer vector (builder.hpp:368).  The device sorts
// the pair keys, keeps the unique ones and derives row_ptr/col_idx.  The scatter map
// rank[e][i][j] = position of column emap[e][j] in row emap[e][i] lets the element
// kernels add into the CSR values without searching.
#include <cub/cub.cuh>

#include <vector>

#include "pxg_internal.h"

namespace pxg
{
namespace
{

constexpr int TPB = 256;

inline unsigned blocksFor(int64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

__global__ void kNodeFirstTouch(uint32_t const * __restrict__ conn, int64_t n, int nv, int N,
                                uint32_t * __restrict__ ft)
{
  int64_t const k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n)
    return;
  int64_t const e = k / nv;
  int const a = (int)(k - e * nv);
  atomicMin(&ft[conn[k]], (uint32_t)(e * N + a));
}

// Edge (kind 0) and face (kind 1) keys.  An edge is the unordered pair of its
// vertices; a quadrilateral face of a conforming hexahedral mesh is identified by its
// smallest vertex and the vertex opposite to it in the face cycle.
__global__ void kEntityKeys(uint32_t const * __restrict__ conn, int64_t nelem, int etype,
                            int kind, uint64_t * __restrict__ keys, uint32_t * __restrict__ slots)
{
  int const per = (kind == 1) ? 6 : (etype == P2TET ? 6 : 12);
  int64_t const k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nelem * per)
    return;
  int64_t const e = k / per;
  int const l = (int)(k - e * per);
  int const nv = (etype == P2TET) ? 4 : 8;
  int const N = (etype == P2TET) ? 10 : 27;
  uint32_t const * v = conn + e * nv;
  uint64_t key;
  int local;
  if (kind == 0)
  {
    uint32_t a, b;
    if (etype == P2TET)
    {
      a = v[tetEdgeV(l, 0)];
      b = v[tetEdgeV(l, 1)];
      local = 4 + l;
    }
    else
    {
      a = v[hexEdgeV(l, 0)];
      b = v[hexEdgeV(l, 1)];
      local = 8 + l;
    }
    uint32_t const lo = a < b ? a : b, hi = a < b ? b : a;
    key = ((uint64_t)lo << 32) | hi;
  }
  else
  {
    uint32_t f[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
      f[i] = v[hexFaceV(l, i)];
    int m = 0;
#pragma unroll
    for (int i = 1; i < 4; ++i)
      if (f[i] < f[m])
        m = i;
    key = ((uint64_t)f[m] << 32) | f[(m + 2) & 3];
    local = 20 + l;
  }
  keys[k] = key;
  slots[k] = (uint32_t)(e * N + local);
}

__global__ void kSegmentHead(uint64_t const * __restrict__ keys, int64_t n, uint32_t * __restrict__ head)
{
  int64_t const k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n)
    return;
  head[k] = (k == 0 || keys[k] != keys[k - 1]) ? (uint32_t)k : 0u;
}

__global__ void kEntityFirst(uint32_t const * __restrict__ sortedSlots, uint32_t const * __restrict__ segStart,
                             int64_t n, uint32_t * __restrict__ first)
{
  int64_t const k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= n)
    return;
  first[sortedSlots[k]] = sortedSlots[segStart[k]];
}

// first slot of point and element DOFs
__global__ void kPointElemFirst(uint32_t const * __restrict__ conn, uint32_t const * __restrict__ ft,
                                int64_t nelem, int nv, int N, int hasElemDof, uint32_t * __restrict__ first)
{
  int64_t const k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nelem * nv)
    return;
  int64_t const e = k / nv;
  int const a = (int)(k - e * nv);
  first[e * N + a] = ft[conn[k]];
  if (hasElemDof && a == 0)
    first[e * N + N - 1] = (uint32_t)(e * N + N - 1);
}

__global__ void kFlag(uint32_t const * __restrict__ first, int64_t n, uint32_t * __restrict__ flag)
{
  int64_t const s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n)
    return;
  flag[s] = (first[s] == (uint32_t)s) ? 1u : 0u;
}

__global__ void kElemMap(uint32_t const * __restrict__ first, uint32_t const * __restrict__ ids,
                         int64_t n, uint32_t * __restrict__ emap)
{
  int64_t const s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n)
    return;
  emap[s] = ids[first[s]];
}

__global__ void kPairKeys(uint32_t const * __restrict__ emap, int64_t nelem, int N, uint64_t ndof,
                          uint64_t * __restrict__ keys)
{
  int64_t const k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t const NN = (int64_t)N * N;
  if (k >= nelem * NN)
    return;
  int64_t const e = k / NN;
  int const r = (int)(k - e * NN);
  int const i = r / N, j = r - (r / N) * N;
  keys[k] = (uint64_t)emap[e * N + i] * ndof + emap[e * N + j];
}

__global__ void kCsrFromKeys(uint64_t const * __restrict__ ukeys, int64_t nnz, uint64_t ndof,
                             int32_t * __restrict__ col, int32_t * __restrict__ rowPtr)
{
  int64_t const k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= nnz)
    return;
  uint64_t const key = ukeys[k];
  int64_t const r = (int64_t)(key / ndof);
  col[k] = (int32_t)(key - (uint64_t)r * ndof);
  int64_t const rprev = (k == 0) ? -1 : (int64_t)(ukeys[k - 1] / ndof);
  for (int64_t rr = rprev + 1; rr <= r; ++rr)
    rowPtr[rr] = (int32_t)k;
  if (k == nnz - 1)
    for (int64_t rr = r + 1; rr <= (int64_t)ndof; ++rr)
      rowPtr[rr] = (int32_t)nnz;
}

__global__ void kMaxRowLen(int32_t const * __restrict__ rowPtr, int64_t n, unsigned long long * out)
{
  int64_t const r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  unsigned const len = (r < n) ? (unsigned)(rowPtr[r + 1] - rowPtr[r]) : 0u;
  unsigned const m = __reduce_max_sync(0xffffffffu, len);
  if ((threadIdx.x & 31) == 0 && m)
    atomicMax(out, (unsigned long long)m);
}

__global__ void kRank(uint32_t const * __restrict__ emap, int64_t nelem, int N,
                      int32_t const * __restrict__ rowPtr, int32_t const * __restrict__ col,
                      uint16_t * __restrict__ rank)
{
  int64_t const k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t const NN = (int64_t)N * N;
  if (k >= nelem * NN)
    return;
  int64_t const e = k / NN;
  int const r = (int)(k - e * NN);
  int const i = r / N, j = r - (r / N) * N;
  uint32_t const ri = emap[e * N + i];
  int32_t const cj = (int32_t)emap[e * N + j];
  int32_t lo = rowPtr[ri], hi = rowPtr[ri + 1];
  int32_t const base = lo;
  while (lo < hi)
  {
    int32_t const mid = (lo + hi) >> 1;
    if (col[mid] < cj)
      lo = mid + 1;
    else
      hi = mid;
  }
  rank[k] = (uint16_t)(lo - base);
}

struct MaxU32
{
  __device__ __forceinline__ uint32_t operator()(uint32_t a, uint32_t b) const { return a > b ? a : b; }
};

// Sort (key, slot) pairs of one entity kind and record the first slot of each entity.
pxg_status entityFirst(pxg_ctx * c, int kind, DevBuf<uint32_t> & first)
{
  int const per = (kind == 1) ? 6 : (c->etype == P2TET ? 6 : 12);
  int64_t const n = c->nelem * per;
  DevBuf<uint64_t> k0, k1;
  DevBuf<uint32_t> s0, s1, head;
  PXG_CUDA(c, k0.alloc(n));
  PXG_CUDA(c, k1.alloc(n));
  PXG_CUDA(c, s0.alloc(n));
  PXG_CUDA(c, s1.alloc(n));
  PXG_CUDA(c, head.alloc(n));
  kEntityKeys<<<blocksFor(n), TPB>>>(c->conn.p, c->nelem, c->etype, kind, k0.p, s0.p);
  PXG_CUDA(c, cudaGetLastError());
  size_t tb = 0;
  PXG_CUDA(c, cub::DeviceRadixSort::SortPairs(nullptr, tb, k0.p, k1.p, s0.p, s1.p, n));
  DevBuf<unsigned char> tmp;
  PXG_CUDA(c, tmp.alloc(tb));
  PXG_CUDA(c, cub::DeviceRadixSort::SortPairs(tmp.p, tb, k0.p, k1.p, s0.p, s1.p, n));
  kSegmentHead<<<blocksFor(n), TPB>>>(k1.p, n, head.p);
  PXG_CUDA(c, cudaGetLastError());
  size_t tb2 = 0;
  PXG_CUDA(c, cub::DeviceScan::InclusiveScan(nullptr, tb2, head.p, s0.p, MaxU32{}, n));
  if (tb2 > tb)
    PXG_CUDA(c, tmp.alloc(tb2));
  PXG_CUDA(c, cub::DeviceScan::InclusiveScan(tmp.p, tb2, head.p, s0.p, MaxU32{}, n));
  kEntityFirst<<<blocksFor(n), TPB>>>(s1.p, s0.p, n, first.p);
  PXG_CUDA(c, cudaGetLastError());
  return PXG_OK;
}

} // namespace

pxg_status buildDofmap(pxg_ctx * c)
{
  int64_t const S = c->nelem * c->N;
  DevBuf<uint32_t> ft, first, flag, ids;
  PXG_CUDA(c, ft.alloc(c->nnodes));
  PXG_CUDA(c, first.alloc(S));
  PXG_CUDA(c, flag.alloc(S));
  PXG_CUDA(c, ids.alloc(S));
  PXG_CUDA(c, cudaMemset(ft.p, 0xff, ft.bytes()));
  int64_t const nslotV = c->nelem * c->nv;
  kNodeFirstTouch<<<blocksFor(nslotV), TPB>>>(c->conn.p, nslotV, c->nv, c->N, ft.p);
  PXG_CUDA(c, cudaGetLastError());
  kPointElemFirst<<<blocksFor(nslotV), TPB>>>(c->conn.p, ft.p, c->nelem, c->nv, c->N,
                                              c->etype == Q2HEX, first.p);
  PXG_CUDA(c, cudaGetLastError());
  pxg_status s;
  if (c->etype == P2TET || c->etype == Q2HEX)
    if ((s = entityFirst(c, 0, first)) != PXG_OK)
      return s;
  if (c->etype == Q2HEX)
    if ((s = entityFirst(c, 1, first)) != PXG_OK)
      return s;
  kFlag<<<blocksFor(S), TPB>>>(first.p, S, flag.p);
  PXG_CUDA(c, cudaGetLastError());
  size_t tb = 0;
  PXG_CUDA(c, cub::DeviceScan::ExclusiveSum(nullptr, tb, flag.p, ids.p, S));
  DevBuf<unsigned char> tmp;
  PXG_CUDA(c, tmp.alloc(tb));
  PXG_CUDA(c, cub::DeviceScan::ExclusiveSum(tmp.p, tb, flag.p, ids.p, S));
  uint32_t lastId = 0, lastFlag = 0;
  PXG_CUDA(c, cudaMemcpy(&lastId, ids.p + (S - 1), 4, cudaMemcpyDeviceToHost));
  PXG_CUDA(c, cudaMemcpy(&lastFlag, flag.p + (S - 1), 4, cudaMemcpyDeviceToHost));
  int64_t const ndof = (int64_t)lastId + lastFlag;
  if (ndof > 0x7fffffffll)
    return fail(c, PXG_ERR_INVALID_ARG, "ndof %lld exceeds int32 CSR indices", (long long)ndof);
  PXG_CUDA(c, c->emap.alloc(S));
  kElemMap<<<blocksFor(S), TPB>>>(first.p, ids.p, S, c->emap.p);
  PXG_CUDA(c, cudaGetLastError());
  PXG_CUDA(c, cudaDeviceSynchronize());
  c->ndof = ndof;
  c->bcMask.reset();
  c->bcVal.reset();
  c->nbc = 0;
  return PXG_OK;
}

pxg_status buildPattern(pxg_ctx * c)
{
  int64_t const NN = (int64_t)c->N * c->N;
  int64_t const n = c->nelem * NN;
  uint64_t const ndof = (uint64_t)c->ndof;
  int endBit = 1;
  while (endBit < 64 && ((ndof * ndof) >> endBit) != 0)
    ++endBit;
  DevBuf<uint64_t> k0, k1;
  PXG_CUDA(c, k0.alloc(n));
  PXG_CUDA(c, k1.alloc(n));
  kPairKeys<<<blocksFor(n), TPB>>>(c->emap.p, c->nelem, c->N, ndof, k0.p);
  PXG_CUDA(c, cudaGetLastError());
  size_t tb = 0;
  PXG_CUDA(c, cub::DeviceRadixSort::SortKeys(nullptr, tb, k0.p, k1.p, n, 0, endBit));
  DevBuf<unsigned char> tmp;
  PXG_CUDA(c, tmp.alloc(tb));
  PXG_CUDA(c, cub::DeviceRadixSort::SortKeys(tmp.p, tb, k0.p, k1.p, n, 0, endBit));
  DevBuf<int64_t> nsel;
  PXG_CUDA(c, nsel.alloc(1));
  size_t tb2 = 0;
  PXG_CUDA(c, cub::DeviceSelect::Unique(nullptr, tb2, k1.p, k0.p, nsel.p, n));
  if (tb2 > tb)
    PXG_CUDA(c, tmp.alloc(tb2));
  PXG_CUDA(c, cub::DeviceSelect::Unique(tmp.p, tb2, k1.p, k0.p, nsel.p, n));
  int64_t nnz = 0;
  PXG_CUDA(c, cudaMemcpy(&nnz, nsel.p, 8, cudaMemcpyDeviceToHost));
  if (nnz > 0x7fffffffll)
    return fail(c, PXG_ERR_INVALID_ARG, "nnz %lld exceeds int32 CSR indices", (long long)nnz);
  k1.reset();
  PXG_CUDA(c, c->rowPtr.alloc(c->ndof + 1));
  PXG_CUDA(c, c->colIdx.alloc(nnz));
  kCsrFromKeys<<<blocksFor(nnz), TPB>>>(k0.p, nnz, ndof, c->colIdx.p, c->rowPtr.p);
  PXG_CUDA(c, cudaGetLastError());
  k0.reset();
  PXG_CUDA(c, cudaMemset(c->counter.p, 0, 8));
  kMaxRowLen<<<blocksFor(c->ndof), TPB>>>(c->rowPtr.p, c->ndof, c->counter.p);
  unsigned long long mrl = 0;
  PXG_CUDA(c, cudaMemcpy(&mrl, c->counter.p, 8, cudaMemcpyDeviceToHost));
  if (mrl > 65535)
    return fail(c, PXG_ERR_UNSUPPORTED, "a CSR row has %llu entries (> 65535)", mrl);
  PXG_CUDA(c, c->rank.alloc(n));
  kRank<<<blocksFor(n), TPB>>>(c->emap.p, c->nelem, c->N, c->rowPtr.p, c->colIdx.p, c->rank.p);
  PXG_CUDA(c, cudaGetLastError());
  PXG_CUDA(c, cudaDeviceSynchronize());
  c->nnz = nnz;
  c->maxRowLen = (int)mrl;
  return PXG_OK;
}

} // namespace pxg
