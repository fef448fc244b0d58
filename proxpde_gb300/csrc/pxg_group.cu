// Warp-group scatter map of the P2 FP64 element kernel.
//
// The element kernels add every local entry into the CSR values with an FP64 reduction
// in L2.  For P2 tetrahedra that is 200 reductions per element (K and M, both
// triangles) to positions scattered over ten rows, and the L2 reduction rate bounds
// the kernel.  The 32 consecutive elements of a warp share many positions (a DOF
// belongs to up to ~24 of them), so the kernel can sum a warp's contributions per
// distinct position first and add each sum once, in ascending position order, so
// that neighbouring lanes reduce into the same 32-byte sectors.
//
// The map, built once per mesh and pattern on the device:
//   item t = e * 100 + i * 10 + j   position rowPtr[emap[e][i]] + rank[e][i][j]
//   key    = (e / 32) << 32 | position, sorted (stable) with the item's code; then,
//            with c the number of items of the item's position in the group,
//            (e / 32) << 38 | c << 32 | position, sorted again (stable), so that a
//            group's positions come by count, ascending inside each count
//   off[g] first distinct index of group g; pos[d] the position of distinct index d and
//   beg[d] the offset of its first contribution among the group's 3,200 items (the
//   contributions of d end where those of d + 1, or the group's items, begin); item[]
//   the codes in sorted order, padded by 8 entries for the 16-byte loads of the last
//   group.
// A code is lane | pair index << 5 | mass class << 11 (p2GroupCode): where the kernel
// finds the lane's stiffness and mass values in shared memory.  The contributions of
// one position are summed in element order, the order of the stable sorts.  The sums
// are FP64 additions on the SMs, whose FP64 rate is low: ordering the positions by
// count makes the 32 lanes of a warp sum runs of the same length, so that no lane
// idles through a longer neighbour's additions.
#include <cub/cub.cuh>

#include "pxg_internal.h"

namespace pxg
{
namespace
{

constexpr int TPB = 256;

inline unsigned blocksFor(int64_t n) { return (unsigned)((n + TPB - 1) / TPB); }

__global__ void kGroupKeys(uint32_t const * __restrict__ emap, int64_t nitems, int32_t const * __restrict__ rowPtr,
                           uint16_t const * __restrict__ rank, uint64_t * __restrict__ keys,
                           uint16_t * __restrict__ codes)
{
  int64_t const t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nitems)
    return;
  int64_t const e = t / 100;
  int const q = (int)(t - e * 100), i = q / 10, j = q - i * 10;
  int32_t const pos = rowPtr[emap[e * 10 + i]] + rank[t];
  keys[t] = ((uint64_t)(e >> 5) << 32) | (uint32_t)pos;
  codes[t] = p2GroupCode((int)(e & 31), i, j);
}

// the count of each item's position: one thread per run head writes it for the run
__global__ void kGroupCountKeys(uint64_t const * __restrict__ keys, int64_t n, uint64_t * __restrict__ keys2)
{
  int64_t const t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n || (t > 0 && keys[t] == keys[t - 1]))
    return;
  uint64_t const k = keys[t];
  int64_t u = t + 1;
  while (u < n && u - t < 63 && keys[u] == k)
    ++u;
  uint64_t const k2 = ((k >> 32) << 38) | ((uint64_t)(u - t) << 32) | (k & 0xffffffffu);
  for (int64_t v = t; v < u; ++v)
    keys2[v] = k2;
}

__global__ void kGroupFlags(uint64_t const * __restrict__ keys, int64_t n, int32_t * __restrict__ flag)
{
  int64_t const t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n)
    return;
  flag[t] = (t == 0 || keys[t] != keys[t - 1]) ? 1 : 0;
}

// distinct index d = idx[t] at the first item t of each run of equal keys
__global__ void kGroupDistinct(uint64_t const * __restrict__ keys, int32_t const * __restrict__ idx, int64_t n,
                               int64_t groupItems, int32_t * __restrict__ pos, uint16_t * __restrict__ beg)
{
  int64_t const t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= n || (t > 0 && keys[t] == keys[t - 1]))
    return;
  int32_t const d = idx[t];
  pos[d] = (int32_t)(uint32_t)(keys[t] & 0xffffffffu);
  beg[d] = (uint16_t)(t % groupItems);
}

__global__ void kGroupOff(int32_t const * __restrict__ idx, int64_t ngroups, int64_t groupItems, int32_t ndistinct,
                          int32_t * __restrict__ off)
{
  int64_t const g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (g > ngroups)
    return;
  off[g] = g == ngroups ? ndistinct : idx[g * groupItems];
}

} // namespace

pxg_status buildScatterGroups(pxg_ctx * c)
{
  auto & G = c->groups;
  G.reset();
  if (c->etype != P2TET || !c->rank.p)
    return fail(c, PXG_ERR_INVALID_ARG, "the warp-group scatter map is built for P2 tetrahedra");
  int64_t const n = c->nelem * 100;
  if (n <= 0 || n > 0x7fffffffll)
    return fail(c, PXG_ERR_UNSUPPORTED, "%lld element entries exceed the warp-group map's int32 indices",
                (long long)n);
  int64_t const ngroups = (c->nelem + 31) / 32;
  int gbits = 0;
  while (gbits < 26 && (uint64_t)(ngroups - 1) >> gbits)
    ++gbits;
  if ((uint64_t)(ngroups - 1) >> gbits)
    return fail(c, PXG_ERR_UNSUPPORTED, "too many element groups for the warp-group map");
  DevBuf<uint64_t> k0, k1;
  DevBuf<uint16_t> v0;
  PXG_CUDA(c, k0.alloc(n));
  PXG_CUDA(c, k1.alloc(n));
  PXG_CUDA(c, v0.alloc(n));
  PXG_CUDA(c, G.item.alloc(n + 8));
  PXG_CUDA(c, cudaMemset(G.item.p + n, 0, 16));
  kGroupKeys<<<blocksFor(n), TPB>>>(c->emap.p, n, c->rowPtr.p, c->rank.p, k0.p, v0.p);
  PXG_CUDA(c, cudaGetLastError());
  size_t tb = 0;
  PXG_CUDA(c, cub::DeviceRadixSort::SortPairs(nullptr, tb, k0.p, k1.p, v0.p, G.item.p, (int)n, 0, 38 + gbits));
  DevBuf<unsigned char> tmp;
  PXG_CUDA(c, tmp.alloc(tb));
  // by group and position
  PXG_CUDA(c, cub::DeviceRadixSort::SortPairs(tmp.p, tb, k0.p, k1.p, v0.p, G.item.p, (int)n, 0, 32 + gbits));
  // by group, count and position
  kGroupCountKeys<<<blocksFor(n), TPB>>>(k1.p, n, k0.p);
  PXG_CUDA(c, cudaGetLastError());
  PXG_CUDA(c, cub::DeviceRadixSort::SortPairs(tmp.p, tb, k0.p, k1.p, G.item.p, v0.p, (int)n, 0, 38 + gbits));
  PXG_CUDA(c, cudaMemcpy(G.item.p, v0.p, n * sizeof(uint16_t), cudaMemcpyDeviceToDevice));
  v0.reset();
  // flags and their exclusive scan (k0 reused as two int32 arrays)
  int32_t * flag = reinterpret_cast<int32_t *>(k0.p);
  int32_t * idx = flag + n;
  kGroupFlags<<<blocksFor(n), TPB>>>(k1.p, n, flag);
  PXG_CUDA(c, cudaGetLastError());
  size_t tb2 = 0;
  PXG_CUDA(c, cub::DeviceScan::ExclusiveSum(nullptr, tb2, flag, idx, (int)n));
  if (tb2 > tb)
    PXG_CUDA(c, tmp.alloc(tb2));
  PXG_CUDA(c, cub::DeviceScan::ExclusiveSum(tmp.p, tb2, flag, idx, (int)n));
  int32_t last[2] = {0, 0};
  PXG_CUDA(c, cudaMemcpy(&last[0], idx + n - 1, 4, cudaMemcpyDeviceToHost));
  PXG_CUDA(c, cudaMemcpy(&last[1], flag + n - 1, 4, cudaMemcpyDeviceToHost));
  int32_t const nd = last[0] + last[1];
  PXG_CUDA(c, G.pos.alloc(nd));
  PXG_CUDA(c, G.beg.alloc(nd));
  PXG_CUDA(c, G.off.alloc(ngroups + 1));
  kGroupDistinct<<<blocksFor(n), TPB>>>(k1.p, idx, n, 32 * 100, G.pos.p, G.beg.p);
  PXG_CUDA(c, cudaGetLastError());
  kGroupOff<<<blocksFor(ngroups + 1), TPB>>>(idx, ngroups, 32 * 100, nd, G.off.p);
  PXG_CUDA(c, cudaGetLastError());
  PXG_CUDA(c, cudaDeviceSynchronize());
  G.ngroups = ngroups;
  G.ndistinct = nd;
  G.built = true;
  return PXG_OK;
}

} // namespace pxg
