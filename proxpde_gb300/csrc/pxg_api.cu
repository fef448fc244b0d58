// Context lifecycle, inputs (mesh, DOF map, coefficient, BCs) and outputs of the
// C ABI declared in include/pxg.h.
#include <cstdarg>
#include <cstdlib>
#include <vector>

#include "pxg_internal.h"

namespace pxg
{

pxg_status fail(pxg_ctx * c, pxg_status s, char const * fmt, ...)
{
  if (c)
  {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    c->err = buf;
  }
  return s;
}

pxg_status cudaFail(pxg_ctx * c, cudaError_t e, char const * what)
{
  pxg_status const s = (e == cudaErrorMemoryAllocation) ? PXG_ERR_OOM : PXG_ERR_CUDA;
  cudaGetLastError(); // clear a non-sticky error so the context stays usable
  return fail(c, s, "%s: %s", what, cudaGetErrorString(e));
}

pxg_status ensureDevice(pxg_ctx * c)
{
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess)
    return cudaFail(c, e, "cudaSetDevice");
  return PXG_OK;
}

// Copy `count` elements from a host or device source into a device buffer.
template <typename T>
pxg_status upload(pxg_ctx * c, DevBuf<T> & dst, T const * src, size_t count, int mem,
                  cudaStream_t s = nullptr)
{
  if (dst.n != count)
    PXG_CUDA(c, dst.alloc(count));
  if (count == 0)
    return PXG_OK;
  PXG_CUDA(c, cudaMemcpyAsync(dst.p, src, count * sizeof(T),
                              mem == PXG_MEM_HOST ? cudaMemcpyHostToDevice
                                                  : cudaMemcpyDeviceToDevice,
                              s));
  if (mem == PXG_MEM_HOST)
    PXG_CUDA(c, cudaStreamSynchronize(s));
  return PXG_OK;
}

template <typename T>
pxg_status download(pxg_ctx * c, T * dst, T const * src, size_t count, int mem)
{
  if (count == 0)
    return PXG_OK;
  PXG_CUDA(c, cudaMemcpy(dst, src, count * sizeof(T),
                         mem == PXG_MEM_HOST ? cudaMemcpyDeviceToHost
                                             : cudaMemcpyDeviceToDevice));
  return PXG_OK;
}

} // namespace pxg

using namespace pxg;

extern "C"
{

int pxg_version(void) { return 10000; }

char const * pxg_status_string(pxg_status s)
{
  switch (s)
  {
  case PXG_OK:
    return "ok";
  case PXG_ERR_INVALID_ARG:
    return "invalid argument";
  case PXG_ERR_OOM:
    return "out of memory";
  case PXG_ERR_CUDA:
    return "CUDA error";
  case PXG_ERR_TIMEOUT:
    return "timeout";
  case PXG_ERR_NOT_CONVERGED:
    return "not converged";
  case PXG_ERR_UNSUPPORTED:
    return "unsupported";
  case PXG_ERR_NO_DEVICE:
    return "no CUDA device";
  case PXG_ERR_NUMERIC:
    return "numerical error";
  }
  return "unknown status";
}

char const * pxg_last_error(pxg_ctx const * ctx) { return ctx ? ctx->err.c_str() : "null context"; }

pxg_status pxg_create(pxg_ctx ** out, int device)
{
  if (!out)
    return PXG_ERR_INVALID_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
  {
    cudaGetLastError();
    return PXG_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n)
    return PXG_ERR_NO_DEVICE;
  auto * c = new pxg_ctx;
  c->device = device;
  auto envOn = [](char const * name) {
    char const * v = getenv(name);
    return v && v[0] == '1';
  };
  c->q1Generic = envOn("PXG_Q1_GENERIC");
  c->q1Thread = envOn("PXG_Q1_THREAD");
  c->q1Group = envOn("PXG_Q1_GROUP");
  c->tetGeneric = envOn("PXG_TET_GENERIC");
  c->q2Generic = envOn("PXG_Q2_GENERIC");
  c->groupScatter = !envOn("PXG_NO_GROUP_SCATTER");
  c->zeroOverlap = !envOn("PXG_NO_ZERO_OVERLAP");
  if (char const * r = getenv("PXG_GROUP_RED_MAX"))
    c->groupRedMax = atoi(r);
  pxg_status s = ensureDevice(c);
  if (s == PXG_OK && cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    s = cudaFail(c, cudaGetLastError(), "SM count");
  if (s == PXG_OK)
    s = initTables(c);
  if (s == PXG_OK)
  {
    cudaError_t e = c->counter.alloc(8);
    if (e != cudaSuccess)
      s = cudaFail(c, e, "counter alloc");
  }
  if (s != PXG_OK)
  {
    delete c;
    return s;
  }
  *out = c;
  return PXG_OK;
}

pxg_status pxg_destroy(pxg_ctx * ctx)
{
  if (!ctx)
    return PXG_ERR_INVALID_ARG;
  cudaSetDevice(ctx->device);
  delete ctx;
  return PXG_OK;
}

pxg_status pxg_set_mesh(pxg_ctx * c, int etype, double const * xyz, int64_t nnodes,
                        uint32_t const * conn, int64_t nelem, int mem)
{
  if (c)
  {
    ++c->meshVer;
    c->recipes.clear();
    c->dofElemPtr.reset();
    c->dofElem.reset();
  }
  if (!c)
    return PXG_ERR_INVALID_ARG;
  if (etype < PXG_P1TET || etype > PXG_Q2HEX)
    return fail(c, PXG_ERR_UNSUPPORTED, "element type %d not provided", etype);
  if (nnodes <= 0 || nelem <= 0 || !xyz || !conn)
    return fail(c, PXG_ERR_INVALID_ARG, "empty mesh or null pointer");
  if (nnodes > 0xfffffffell)
    return fail(c, PXG_ERR_INVALID_ARG, "too many nodes for 32-bit ids");
  int const nv = numVerts(etype), N = numDofs(etype);
  if ((int64_t)nelem * N > 0x7fffffffll)
    return fail(c, PXG_ERR_INVALID_ARG, "nelem * dofs per element exceeds 2^31");
  if (mem == PXG_MEM_HOST)
  {
    // connectivity is checked on the host (a device check runs for device input)
    for (int64_t k = 0; k < nelem * nv; ++k)
      if ((int64_t)conn[k] >= nnodes)
        return fail(c, PXG_ERR_INVALID_ARG, "element %lld references node %u >= %lld",
                    (long long)(k / nv), conn[k], (long long)nnodes);
  }
  pxg_status s = ensureDevice(c);
  if (s != PXG_OK)
    return s;
  c->emap.reset();
  c->rowPtr.reset();
  c->colIdx.reset();
  c->rank.reset();
  c->groups.reset();
  c->kE.reset();
  c->hasCoef = false;
  c->colour.perm.reset();
  c->colour.start.clear();
  c->colour.ncol = 0;
  c->colour.built = false;
  c->facets.face.reset();
  c->facets.marker.reset();
  c->facets.n = 0;
  c->facets.built = false;
  c->scatter = PXG_SCATTER_REDUCE;
  c->threads = 0;
  c->bcMask.reset();
  c->bcVal.reset();
  c->nbc = 0;
  c->ndof = 0;
  c->nnz = 0;
  c->etype = etype;
  c->nv = nv;
  c->N = N;
  c->nnodes = nnodes;
  c->nelem = nelem;
  if ((s = upload(c, c->xyz, xyz, (size_t)nnodes * 3, mem)) != PXG_OK)
    return s;
  if ((s = upload(c, c->conn, conn, (size_t)nelem * nv, mem)) != PXG_OK)
    return s;
  if (mem == PXG_MEM_DEVICE)
  {
    // device-side bounds check of the connectivity
    std::vector<uint32_t> h((size_t)nelem * nv);
    PXG_CUDA(c, cudaMemcpy(h.data(), c->conn.p, h.size() * 4, cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < h.size(); ++k)
      if ((int64_t)h[k] >= nnodes)
        return fail(c, PXG_ERR_INVALID_ARG, "element %lld references node %u >= %lld",
                    (long long)(k / nv), h[k], (long long)nnodes);
  }
  return PXG_OK;
}

pxg_status pxg_set_coords(pxg_ctx * c, double const * xyz, int mem, void * stream)
{
  if (c)
  {
    ++c->meshVer;
  }
  if (!c || !xyz)
    return PXG_ERR_INVALID_ARG;
  if (c->etype < 0)
    return fail(c, PXG_ERR_INVALID_ARG, "no mesh set");
  pxg_status s = ensureDevice(c);
  if (s != PXG_OK)
    return s;
  PXG_CUDA(c, cudaMemcpyAsync(c->xyz.p, xyz, c->xyz.bytes(),
                              mem == PXG_MEM_HOST ? cudaMemcpyHostToDevice
                                                  : cudaMemcpyDeviceToDevice,
                              (cudaStream_t)stream));
  if (mem == PXG_MEM_HOST)
    PXG_CUDA(c, cudaStreamSynchronize((cudaStream_t)stream));
  return PXG_OK;
}

pxg_status pxg_build_dofmap(pxg_ctx * c, int64_t * ndof)
{
  if (c)
  {
    ++c->meshVer;
    c->recipes.clear();
    c->dofElemPtr.reset();
    c->dofElem.reset();
  }
  if (!c)
    return PXG_ERR_INVALID_ARG;
  if (c->etype < 0)
    return fail(c, PXG_ERR_INVALID_ARG, "no mesh set");
  pxg_status s = ensureDevice(c);
  if (s != PXG_OK)
    return s;
  c->rowPtr.reset();
  c->colIdx.reset();
  c->rank.reset();
  c->groups.reset();
  c->nnz = 0;
  if ((s = buildDofmap(c)) != PXG_OK)
    return s;
  if (ndof)
    *ndof = c->ndof;
  return PXG_OK;
}

pxg_status pxg_set_dofmap(pxg_ctx * c, uint32_t const * em, int64_t ndof, int mem)
{
  if (c)
  {
    ++c->meshVer;
    c->recipes.clear();
    c->dofElemPtr.reset();
    c->dofElem.reset();
  }
  if (!c || !em || ndof <= 0)
    return PXG_ERR_INVALID_ARG;
  if (c->etype < 0)
    return fail(c, PXG_ERR_INVALID_ARG, "no mesh set");
  if (ndof > 0x7fffffffll)
    return fail(c, PXG_ERR_INVALID_ARG, "ndof exceeds int32 CSR indices");
  size_t const n = (size_t)c->nelem * c->N;
  std::vector<uint32_t> h;
  uint32_t const * hp = em;
  if (mem == PXG_MEM_DEVICE)
  {
    h.resize(n);
    PXG_CUDA(c, cudaMemcpy(h.data(), em, n * 4, cudaMemcpyDeviceToHost));
    hp = h.data();
  }
  for (size_t k = 0; k < n; ++k)
    if ((int64_t)hp[k] >= ndof)
      return fail(c, PXG_ERR_INVALID_ARG, "DOF id %u >= ndof %lld", hp[k], (long long)ndof);
  pxg_status s = ensureDevice(c);
  if (s != PXG_OK)
    return s;
  if ((s = upload(c, c->emap, hp, n, PXG_MEM_HOST)) != PXG_OK)
    return s;
  c->ndof = ndof;
  c->rowPtr.reset();
  c->colIdx.reset();
  c->rank.reset();
  c->groups.reset();
  c->nnz = 0;
  c->bcMask.reset();
  c->bcVal.reset();
  c->nbc = 0;
  return PXG_OK;
}

pxg_status pxg_get_dofmap(pxg_ctx * c, uint32_t * em, int mem)
{
  if (!c || !em)
    return PXG_ERR_INVALID_ARG;
  if (!c->emap.p)
    return fail(c, PXG_ERR_INVALID_ARG, "no DOF map");
  pxg_status s = ensureDevice(c);
  if (s != PXG_OK)
    return s;
  return download(c, em, c->emap.p, (size_t)c->nelem * c->N, mem);
}

pxg_status pxg_build_pattern(pxg_ctx * c, int64_t * nnz)
{
  if (!c)
    return PXG_ERR_INVALID_ARG;
  if (!c->emap.p)
    return fail(c, PXG_ERR_INVALID_ARG, "build or set the DOF map first");
  pxg_status s = ensureDevice(c);
  if (s != PXG_OK)
    return s;
  if ((s = buildPattern(c)) != PXG_OK)
    return s;
  if (nnz)
    *nnz = c->nnz;
  return PXG_OK;
}

pxg_status pxg_get_pattern(pxg_ctx * c, int32_t * rp, int32_t * ci, int mem)
{
  if (!c || !rp || !ci)
    return PXG_ERR_INVALID_ARG;
  if (!c->rowPtr.p)
    return fail(c, PXG_ERR_INVALID_ARG, "no pattern built");
  pxg_status s = ensureDevice(c);
  if (s != PXG_OK)
    return s;
  if ((s = download(c, rp, c->rowPtr.p, (size_t)c->ndof + 1, mem)) != PXG_OK)
    return s;
  return download(c, ci, c->colIdx.p, (size_t)c->nnz, mem);
}

pxg_status pxg_pattern_device(pxg_ctx * c, int32_t const ** rp, int32_t const ** ci)
{
  if (!c || !rp || !ci)
    return PXG_ERR_INVALID_ARG;
  if (!c->rowPtr.p)
    return fail(c, PXG_ERR_INVALID_ARG, "no pattern built");
  *rp = c->rowPtr.p;
  *ci = c->colIdx.p;
  return PXG_OK;
}

pxg_status pxg_set_coef(pxg_ctx * c, double const * k, int mem, void * stream)
{
  if (c)
  {
    ++c->coefVer;
  }
  if (!c || !k)
    return PXG_ERR_INVALID_ARG;
  if (c->etype < 0)
    return fail(c, PXG_ERR_INVALID_ARG, "no mesh set");
  pxg_status s = ensureDevice(c);
  if (s != PXG_OK)
    return s;
  if (c->kE.n != (size_t)c->nelem)
    PXG_CUDA(c, c->kE.alloc(c->nelem));
  PXG_CUDA(c, cudaMemcpyAsync(c->kE.p, k, c->kE.bytes(),
                              mem == PXG_MEM_HOST ? cudaMemcpyHostToDevice
                                                  : cudaMemcpyDeviceToDevice,
                              (cudaStream_t)stream));
  if (mem == PXG_MEM_HOST)
    PXG_CUDA(c, cudaStreamSynchronize((cudaStream_t)stream));
  c->hasCoef = true;
  return PXG_OK;
}

pxg_status pxg_set_bc(pxg_ctx * c, uint32_t const * dofs, double const * vals, int64_t n,
                      double diag, int mem)
{
  if (c)
  {
    ++c->bcVer;
  }
  if (!c || n < 0 || (n > 0 && (!dofs || !vals)))
    return PXG_ERR_INVALID_ARG;
  if (c->ndof <= 0)
    return fail(c, PXG_ERR_INVALID_ARG, "build or set the DOF map first");
  pxg_status s = ensureDevice(c);
  if (s != PXG_OK)
    return s;
  c->bcDiag = diag;
  if (n == 0)
  {
    c->bcMask.reset();
    c->bcVal.reset();
    c->nbc = 0;
    return PXG_OK;
  }
  std::vector<uint32_t> hd;
  std::vector<double> hv;
  uint32_t const * pd = dofs;
  double const * pv = vals;
  if (mem == PXG_MEM_DEVICE)
  {
    hd.resize(n);
    hv.resize(n);
    PXG_CUDA(c, cudaMemcpy(hd.data(), dofs, n * 4, cudaMemcpyDeviceToHost));
    PXG_CUDA(c, cudaMemcpy(hv.data(), vals, n * 8, cudaMemcpyDeviceToHost));
    pd = hd.data();
    pv = hv.data();
  }
  std::vector<uint8_t> mask(c->ndof, 0);
  std::vector<double> val(c->ndof, 0.);
  for (int64_t k = 0; k < n; ++k)
  {
    if ((int64_t)pd[k] >= c->ndof)
      return fail(c, PXG_ERR_INVALID_ARG, "BC DOF %u >= ndof %lld", pd[k], (long long)c->ndof);
    mask[pd[k]] = 1;
    val[pd[k]] = pv[k]; // last value wins, as the last constraining BC does
  }
  if ((s = upload(c, c->bcMask, mask.data(), mask.size(), PXG_MEM_HOST)) != PXG_OK)
    return s;
  if ((s = upload(c, c->bcVal, val.data(), val.size(), PXG_MEM_HOST)) != PXG_OK)
    return s;
  c->nbc = n;
  return PXG_OK;
}

pxg_status pxg_device_alloc(pxg_ctx * c, uint64_t bytes, void ** ptr)
{
  if (!c || !ptr)
    return PXG_ERR_INVALID_ARG;
  *ptr = nullptr;
  pxg_status s = ensureDevice(c);
  if (s != PXG_OK)
    return s;
  if (bytes == 0)
    return PXG_OK;
  PXG_CUDA(c, cudaMalloc(ptr, bytes));
  return PXG_OK;
}

pxg_status pxg_device_free(pxg_ctx * c, void * ptr)
{
  if (!c)
    return PXG_ERR_INVALID_ARG;
  pxg_status s = ensureDevice(c);
  if (s != PXG_OK)
    return s;
  if (ptr)
    PXG_CUDA(c, cudaFree(ptr));
  return PXG_OK;
}

pxg_status pxg_memcpy(pxg_ctx * c, void * dst, void const * src, uint64_t bytes, int dir, void * stream)
{
  if (!c || (bytes && (!dst || !src)) || dir < 0 || dir > 2)
    return c ? fail(c, PXG_ERR_INVALID_ARG, "pxg_memcpy: bad argument") : PXG_ERR_INVALID_ARG;
  pxg_status s = ensureDevice(c);
  if (s != PXG_OK)
    return s;
  if (bytes == 0)
    return PXG_OK;
  cudaMemcpyKind const k = dir == 0 ? cudaMemcpyHostToDevice : dir == 1 ? cudaMemcpyDeviceToHost
                                                                        : cudaMemcpyDeviceToDevice;
  if (stream)
    PXG_CUDA(c, cudaMemcpyAsync(dst, src, bytes, k, (cudaStream_t)stream));
  else
    PXG_CUDA(c, cudaMemcpy(dst, src, bytes, k));
  return PXG_OK;
}

} // extern "C"
