// Boundary facets, their markers and Dirichlet constraints built on the device
// (proxpde: buildFacets / markFacetsCube, include/mesh.hpp:226-498; BCEss::setupDofMap,
// include/bc.hpp:252-295).
//
// Facets: every face of every element, keyed by its three smallest vertex ids (a
// triangle by its vertices; a quadrilateral of a conforming hexahedral mesh by three of
// its four).  Two stable radix sorts order the keys; a face whose key occurs once is a
// boundary facet.  The facets are kept in key order as (element, local face).
// Markers: either from the caller (one per facet, in that order) or from the planes of
// a box, as markFacetsCube does.
// Constraints: the DOFs of a Lagrange facet are the element DOFs that lie on it (its
// vertices, edges and, for Q2, the face DOF); each condition (marker, function id,
// coefficient) constrains them with value coef * f(DOF point).  Later conditions win on
// shared DOFs, as in pxg_set_bc.
#include <cub/cub.cuh>

#include <vector>

#include "pxg_internal.h"

namespace pxg
{
namespace
{

unsigned blocksOf(int64_t n) { return (unsigned)((n + 255) / 256); }

// local vertices of face lf: tetrahedron face i is opposite vertex i; hexahedron faces
// follow hexFaceV
__host__ __device__ inline int faceVerts(bool hex, int lf, int (&fv)[4])
{
  if (hex)
  {
    for (int k = 0; k < 4; ++k)
      fv[k] = hexFaceV(lf, k);
    return 4;
  }
  int n = 0;
  for (int v = 0; v < 4; ++v)
    if (v != lf)
      fv[n++] = v;
  return 3;
}

// local DOFs on face lf (at most 9: Q2)
template <int T>
__device__ int faceDofs(int lf, int (&out)[9])
{
  int fv[4];
  int const nfv = faceVerts(Elem<T>::hex, lf, fv);
  auto in = [&](int v) {
    for (int k = 0; k < nfv; ++k)
      if (fv[k] == v)
        return true;
    return false;
  };
  int n = 0;
  for (int k = 0; k < nfv; ++k)
    out[n++] = fv[k];
  if constexpr (T == P2TET)
    for (int e = 0; e < 6; ++e)
      if (in(tetEdgeV(e, 0)) && in(tetEdgeV(e, 1)))
        out[n++] = 4 + e;
  if constexpr (T == Q2HEX)
  {
    for (int e = 0; e < 12; ++e)
      if (in(hexEdgeV(e, 0)) && in(hexEdgeV(e, 1)))
        out[n++] = 8 + e;
    out[n++] = 20 + lf;
  }
  return n;
}

__global__ void kFaceKeys(uint32_t const * __restrict__ conn, int64_t nfaces, bool hex, int nv, int nf,
                          unsigned long long * __restrict__ keyHi, uint32_t * __restrict__ keyLo,
                          uint32_t * __restrict__ idx)
{
  int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nfaces)
    return;
  int64_t const e = i / nf;
  int const lf = (int)(i % nf);
  int fv[4];
  int const n = faceVerts(hex, lf, fv);
  uint32_t v[4];
  for (int k = 0; k < n; ++k)
    v[k] = conn[e * nv + fv[k]];
  // the three smallest ids in increasing order
  for (int a = 0; a < n; ++a)
    for (int b = a + 1; b < n; ++b)
      if (v[b] < v[a])
      {
        uint32_t const t = v[a];
        v[a] = v[b];
        v[b] = t;
      }
  keyHi[i] = (unsigned long long)v[0] << 32 | v[1];
  keyLo[i] = v[2];
  idx[i] = (uint32_t)i;
}

__global__ void kGather64(unsigned long long const * __restrict__ src, uint32_t const * __restrict__ idx, int64_t n,
                          unsigned long long * __restrict__ dst)
{
  int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n)
    dst[i] = src[idx[i]];
}

__global__ void kBoundaryFlag(unsigned long long const * __restrict__ hiSorted, uint32_t const * __restrict__ keyLo,
                              uint32_t const * __restrict__ idx, int64_t n, uint8_t * __restrict__ flag)
{
  int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  unsigned long long const h = hiSorted[i];
  uint32_t const l = keyLo[idx[i]];
  bool const dup = (i > 0 && hiSorted[i - 1] == h && keyLo[idx[i - 1]] == l) ||
                   (i + 1 < n && hiSorted[i + 1] == h && keyLo[idx[i + 1]] == l);
  flag[i] = dup ? 0 : 1;
}

// markFacetsCube (mesh.hpp:443-481): the first matching plane of the facet's bounding box
__global__ void kMarkBox(uint32_t const * __restrict__ facets, int64_t nb, uint32_t const * __restrict__ conn,
                         double const * __restrict__ xyz, bool hex, int nv, int nf, double3 o, double3 L,
                         int32_t * __restrict__ marker)
{
  int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nb)
    return;
  int64_t const e = facets[i] / nf;
  int const lf = (int)(facets[i] % nf);
  int fv[4];
  int const n = faceVerts(hex, lf, fv);
  double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
  for (int k = 0; k < n; ++k)
  {
    int64_t const v = conn[e * nv + fv[k]];
    for (int d = 0; d < 3; ++d)
    {
      double const x = xyz[3 * v + d];
      mn[d] = fmin(mn[d], x);
      mx[d] = fmax(mx[d], x);
    }
  }
  int m = 0; // side::NONE
  if (fabs(mx[1] - o.y) < 1e-6 * L.y)
    m = 1; // BOTTOM
  else if (fabs(mn[0] - o.x - L.x) < 1e-6 * L.x)
    m = 2; // RIGHT
  else if (fabs(mn[1] - o.y - L.y) < 1e-6 * L.y)
    m = 3; // TOP
  else if (fabs(mx[0] - o.x) < 1e-6 * L.x)
    m = 4; // LEFT
  else if (fabs(mx[2] - o.z) < 1e-6 * L.z)
    m = 5; // BACK
  else if (fabs(mn[2] - o.z - L.z) < 1e-6 * L.z)
    m = 6; // FRONT
  marker[i] = m;
}

// one condition: constrain the DOFs of the facets with marker m, value coef * f(point)
template <int T>
__global__ void kBcFacets(uint32_t const * __restrict__ facets, int32_t const * __restrict__ marker, int64_t nb,
                          uint32_t const * __restrict__ conn, uint32_t const * __restrict__ emap,
                          double const * __restrict__ xyz, int nf, int m, int fn, double coef,
                          uint8_t * __restrict__ mask, double * __restrict__ val)
{
  constexpr int NV = Elem<T>::NV, N = Elem<T>::N;
  int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nb || marker[i] != m)
    return;
  int64_t const e = facets[i] / nf;
  int const lf = (int)(facets[i] % nf);
  double X[NV][3], P[N][3];
  for (int v = 0; v < NV; ++v)
  {
    int64_t const id = conn[e * NV + v];
    for (int d = 0; d < 3; ++d)
      X[v][d] = xyz[3 * id + d];
  }
  mappingPoints<T>(X, P);
  int loc[9];
  int const n = faceDofs<T>(lf, loc);
  for (int k = 0; k < n; ++k)
  {
    uint32_t const dof = emap[e * N + loc[k]];
    mask[dof] = 1;
    val[dof] = evalFn(fn, coef, P[loc[k]][0], P[loc[k]][1], P[loc[k]][2]);
  }
}

__global__ void kCountMask(uint8_t const * __restrict__ mask, int64_t n, unsigned long long * __restrict__ out)
{
  unsigned long long c = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    c += mask[i];
  for (int o = 16; o > 0; o >>= 1)
    c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c)
    atomicAdd(out, c);
}

} // namespace
} // namespace pxg

using namespace pxg;

namespace
{
int facesPerElem(int etype) { return isHex(etype) ? 6 : 4; }
} // namespace

extern "C"
{

pxg_status pxg_build_facets(pxg_ctx * c, int64_t * nfacets)
{
  if (!c || !nfacets)
    return PXG_ERR_INVALID_ARG;
  if (!c->conn.p)
    return fail(c, PXG_ERR_INVALID_ARG, "set the mesh first");
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  if (c->facets.built)
  {
    *nfacets = c->facets.n;
    return PXG_OK;
  }
  int const nf = facesPerElem(c->etype);
  int64_t const nfaces = c->nelem * nf;
  if (nfaces >= ((int64_t)1 << 32))
    return fail(c, PXG_ERR_UNSUPPORTED, "more than 2^32 element faces");
  bool const hex = isHex(c->etype);
  DevBuf<unsigned long long> hi, hi2, hiSorted;
  DevBuf<uint32_t> lo, idx, idx1, idx2;
  PXG_CUDA(c, hi.alloc(nfaces));
  PXG_CUDA(c, lo.alloc(nfaces));
  PXG_CUDA(c, idx.alloc(nfaces));
  PXG_CUDA(c, idx1.alloc(nfaces));
  kFaceKeys<<<blocksOf(nfaces), 256>>>(c->conn.p, nfaces, hex, c->nv, nf, hi.p, lo.p, idx.p);
  PXG_CUDA(c, cudaGetLastError());
  // stable sorts: by the low key, then by the high key
  DevBuf<uint32_t> loSorted;
  PXG_CUDA(c, loSorted.alloc(nfaces));
  size_t tb = 0, tb2 = 0;
  PXG_CUDA(c, cub::DeviceRadixSort::SortPairs(nullptr, tb, lo.p, loSorted.p, idx.p, idx1.p, nfaces));
  PXG_CUDA(c, hi2.alloc(nfaces));
  PXG_CUDA(c, hiSorted.alloc(nfaces));
  PXG_CUDA(c, idx2.alloc(nfaces));
  PXG_CUDA(c, cub::DeviceRadixSort::SortPairs(nullptr, tb2, hi2.p, hiSorted.p, idx1.p, idx2.p, nfaces));
  DevBuf<unsigned char> tmp;
  PXG_CUDA(c, tmp.alloc(tb > tb2 ? tb : tb2));
  PXG_CUDA(c, cub::DeviceRadixSort::SortPairs(tmp.p, tb, lo.p, loSorted.p, idx.p, idx1.p, nfaces));
  kGather64<<<blocksOf(nfaces), 256>>>(hi.p, idx1.p, nfaces, hi2.p);
  PXG_CUDA(c, cub::DeviceRadixSort::SortPairs(tmp.p, tb2, hi2.p, hiSorted.p, idx1.p, idx2.p, nfaces));
  loSorted.reset();
  hi.reset();
  hi2.reset();
  // boundary = key occurs once; keep them in key order
  DevBuf<uint8_t> flag;
  PXG_CUDA(c, flag.alloc(nfaces));
  kBoundaryFlag<<<blocksOf(nfaces), 256>>>(hiSorted.p, lo.p, idx2.p, nfaces, flag.p);
  PXG_CUDA(c, cudaGetLastError());
  DevBuf<uint32_t> sel;
  DevBuf<int64_t> nsel;
  PXG_CUDA(c, sel.alloc(nfaces));
  PXG_CUDA(c, nsel.alloc(1));
  tb = 0;
  PXG_CUDA(c, cub::DeviceSelect::Flagged(nullptr, tb, idx2.p, flag.p, sel.p, nsel.p, nfaces));
  PXG_CUDA(c, tmp.alloc(tb));
  PXG_CUDA(c, cub::DeviceSelect::Flagged(tmp.p, tb, idx2.p, flag.p, sel.p, nsel.p, nfaces));
  int64_t nb = 0;
  PXG_CUDA(c, cudaMemcpy(&nb, nsel.p, 8, cudaMemcpyDeviceToHost));
  PXG_CUDA(c, c->facets.face.alloc(nb > 0 ? nb : 1));
  PXG_CUDA(c, c->facets.marker.alloc(nb > 0 ? nb : 1));
  if (nb > 0)
  {
    PXG_CUDA(c, cudaMemcpy(c->facets.face.p, sel.p, nb * 4, cudaMemcpyDeviceToDevice));
    PXG_CUDA(c, cudaMemset(c->facets.marker.p, 0, nb * 4));
  }
  c->facets.n = nb;
  c->facets.built = true;
  *nfacets = nb;
  return PXG_OK;
}

pxg_status pxg_get_facets(pxg_ctx * c, uint32_t * faces, int32_t * markers)
{
  if (!c)
    return PXG_ERR_INVALID_ARG;
  if (!c->facets.built)
    return fail(c, PXG_ERR_INVALID_ARG, "build the facets first");
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  if (faces && c->facets.n)
    PXG_CUDA(c, cudaMemcpy(faces, c->facets.face.p, c->facets.n * 4, cudaMemcpyDeviceToHost));
  if (markers && c->facets.n)
    PXG_CUDA(c, cudaMemcpy(markers, c->facets.marker.p, c->facets.n * 4, cudaMemcpyDeviceToHost));
  return PXG_OK;
}

pxg_status pxg_set_facet_markers(pxg_ctx * c, int32_t const * markers)
{
  if (!c || !markers)
    return PXG_ERR_INVALID_ARG;
  if (!c->facets.built)
    return fail(c, PXG_ERR_INVALID_ARG, "build the facets first");
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  if (c->facets.n)
    PXG_CUDA(c, cudaMemcpy(c->facets.marker.p, markers, c->facets.n * 4, cudaMemcpyHostToDevice));
  return PXG_OK;
}

pxg_status pxg_mark_facets_box(pxg_ctx * c, double const * origin, double const * length)
{
  if (!c || !origin || !length || !(length[0] > 0.) || !(length[1] > 0.) || !(length[2] > 0.))
    return PXG_ERR_INVALID_ARG;
  int64_t nb = 0;
  pxg_status st = pxg_build_facets(c, &nb);
  if (st != PXG_OK)
    return st;
  if (nb)
  {
    kMarkBox<<<blocksOf(nb), 256>>>(c->facets.face.p, nb, c->conn.p, c->xyz.p, isHex(c->etype), c->nv,
                                    facesPerElem(c->etype), make_double3(origin[0], origin[1], origin[2]),
                                    make_double3(length[0], length[1], length[2]), c->facets.marker.p);
    PXG_CUDA(c, cudaGetLastError());
  }
  return PXG_OK;
}

pxg_status pxg_set_bc_markers(pxg_ctx * c, int32_t const * markers, int32_t const * fns, double const * coefs,
                              int nbc, double diag)
{
  if (c)
    ++c->bcVer;
  if (!c || nbc < 0 || (nbc > 0 && (!markers || !fns || !coefs)))
    return PXG_ERR_INVALID_ARG;
  if (c->ndof <= 0)
    return fail(c, PXG_ERR_INVALID_ARG, "build or set the DOF map first");
  if (!c->facets.built)
    return fail(c, PXG_ERR_INVALID_ARG, "build and mark the facets first");
  for (int k = 0; k < nbc; ++k)
    if (fns[k] < 0 || fns[k] > PXG_FN_COORD_Z)
      return fail(c, PXG_ERR_INVALID_ARG, "condition %d: unknown function %d", k, fns[k]);
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  c->bcDiag = diag;
  PXG_CUDA(c, c->bcMask.alloc(c->ndof));
  PXG_CUDA(c, c->bcVal.alloc(c->ndof));
  PXG_CUDA(c, cudaMemset(c->bcMask.p, 0, c->ndof));
  PXG_CUDA(c, cudaMemset(c->bcVal.p, 0, c->ndof * 8));
  int64_t const nb = c->facets.n;
  int const nf = facesPerElem(c->etype);
  for (int k = 0; k < nbc && nb > 0; ++k)
  {
    auto go = [&](auto kern) {
      kern<<<blocksOf(nb), 256>>>(c->facets.face.p, c->facets.marker.p, nb, c->conn.p, c->emap.p, c->xyz.p, nf,
                                  markers[k], fns[k], coefs[k], c->bcMask.p, c->bcVal.p);
    };
    switch (c->etype)
    {
    case P1TET:
      go(kBcFacets<P1TET>);
      break;
    case P2TET:
      go(kBcFacets<P2TET>);
      break;
    case Q1HEX:
      go(kBcFacets<Q1HEX>);
      break;
    case Q2HEX:
      go(kBcFacets<Q2HEX>);
      break;
    }
    PXG_CUDA(c, cudaGetLastError());
  }
  PXG_CUDA(c, cudaMemset(c->counter.p, 0, 8));
  kCountMask<<<152 * 4, 256>>>(c->bcMask.p, c->ndof, c->counter.p);
  unsigned long long n = 0;
  PXG_CUDA(c, cudaMemcpy(&n, c->counter.p, 8, cudaMemcpyDeviceToHost));
  c->nbc = (int64_t)n;
  if (n == 0)
  {
    c->bcMask.reset();
    c->bcVal.reset();
  }
  return PXG_OK;
}

} // extern "C"
