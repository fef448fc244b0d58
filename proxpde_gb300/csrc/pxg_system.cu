// Systems of FE spaces on one mesh: vector spaces and the coupling blocks of mixed
// problems (proxpde: FESpace<..., dim> with its offset, include/fespace.hpp:15-60;
// Builder::buildLhs on vector spaces and Builder::buildCoupling, include/builder.hpp:
// 31-277; AssemblyTensorStiffness, include/assembly_lhs.hpp:116-161; AssemblyGrad /
// AssemblyDiv, include/assembly_coupling.hpp:42-132).
//
// Layout: the spaces' DOFs are concatenated with offsets; inside a vector space the DOF
// ordering is BLOCK (component d of DOF k is k + d * ndof, include/dof.hpp:312-327).
// Pattern: the union over the elements of all pairs of the element's DOFs in every
// space.  Blocks the reference never assembles (e.g. pressure-pressure) are structural
// zeros there, which closeMatrix's prune removes, so the closed matrix has the
// reference's pattern.
// Assembly: one call = one Builder call over a (row space, column space) pair.  One
// CUDA block per element: the geometry and the mapped gradients at the quadrature points
// of the row space's rule go to shared memory, then the threads take the (row, column)
// entries, apply the call's Dirichlet condensation (rows and columns, the diagonal and
// h on constrained rows for buildLhs) and add into the CSR values (FP64 reductions; the
// column position by binary search in the sorted row).
#include <cub/cub.cuh>

#include <map>
#include <memory>
#include <vector>

#include "pxg_internal.h"

struct pxg_sys
{
  int device = 0;
  std::vector<pxg_ctx *> sp;
  std::vector<int> dim, qr;
  std::vector<int64_t> off;
  int64_t ntot = 0, nnz = 0;
  pxg::DevBuf<int32_t> rowPtr, colIdx;
  std::vector<std::unique_ptr<pxg::DevBuf<uint8_t>>> bcMask;
  std::vector<std::unique_ptr<pxg::DevBuf<double>>> bcVal;
  double diag = 1.0;
  // tables per (row, column) pair: w, vertex gradients, row / column phi and dphi on
  // the reference element at the row space's quadrature points
  struct Tables
  {
    int nq = 0;
    pxg::DevBuf<double> t;
  };
  std::map<std::pair<int, int>, std::unique_ptr<Tables>> tables;
};

namespace pxg
{
namespace
{

constexpr int kSysThreads = 128;

struct SysArgs
{
  int64_t nelem;
  int nv;
  uint32_t const * conn;
  double const * xyz;
  int Nr, Nc, dr, dc;
  int64_t ndr, ndc, offr, offc;
  uint32_t const * emr;
  uint32_t const * emc;
  uint8_t const * maskr;
  double const * valr;
  uint8_t const * maskc;
  double const * valc;
  int diagCall;
  double diag;
  int nq;
  double const * tab; // w[nq], dV[nq][nv][3], phr[nq][Nr], dpr[nq][Nr][3], phc[nq][Nc], dpc[nq][Nc][3]
  int nops;
  int kind[4];
  double coef[4];
  int pairPath; // one space, stiffness / tensor stiffness / mass only: the block path
  int32_t const * rowPtr;
  int32_t const * colIdx;
  double * vals;
  double * b;
};

__device__ __forceinline__ int64_t position(int32_t const * rp, int32_t const * ci, int64_t row, int32_t col)
{
  int32_t lo = rp[row], hi = rp[row + 1] - 1;
  while (lo < hi)
  {
    int32_t const mid = (lo + hi) >> 1;
    if (ci[mid] < col)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// Entry (I, J) = (row DOF i, component d1; column DOF j, component d2) of element e:
// the call's Dirichlet condensation, or the FP64 reduction at its CSR position
__device__ __forceinline__ void sysEmit(SysArgs const & a, int64_t e, int I, int J, double v,
                                       unsigned char const * consR, unsigned char const * consC, double const * h)
{
  int const i = I % a.Nr, d1 = I / a.Nr, j = J % a.Nc, d2 = J / a.Nc;
  int64_t const gI = a.offr + a.emr[e * a.Nr + i] + (int64_t)d1 * a.ndr;
  int64_t const gJ = a.offc + a.emc[e * a.Nc + j] + (int64_t)d2 * a.ndc;
  bool const cI = consR[I], cJ = consC[J];
  if (cI || cJ)
  {
    if (!cI && a.b && h[J] != 0.)
      atomicAdd(a.b + gI, -v * h[J]); // lift: Fe = -C Ke h
    if (a.diagCall && I == J)
    {
      // buildLhs: constrained diagonal = diag, Fe = h (builder.hpp:105-124)
      atomicAdd(a.vals + position(a.rowPtr, a.colIdx, gI, (int32_t)gI), a.diag);
      if (a.b)
        atomicAdd(a.b + gI, h[J]);
    }
    return;
  }
  atomicAdd(a.vals + position(a.rowPtr, a.colIdx, gI, (int32_t)gJ), v);
}

__global__ void __launch_bounds__(kSysThreads) kSysAssemble(SysArgs a)
{
  extern __shared__ double sm[];
  int const nq = a.nq, Nr = a.Nr, Nc = a.Nc, Lr = Nr * a.dr, Lc = Nc * a.dc, nv = a.nv;
  double * X = sm;                  // nv * 3
  double * Jinv = X + 24;           // nq * 9
  double * JxW = Jinv + 9 * nq;     // nq
  double * dRr = JxW + nq;          // nq * Nr * 3
  double * dRc = dRr + nq * Nr * 3; // nq * Nc * 3
  double * h = dRc + nq * Nc * 3;   // Lc
  double * wph = h + Lc;            // nq * Nr: JxW phi (block path)
  auto * consR = reinterpret_cast<unsigned char *>(wph + nq * Nr);
  unsigned char * consC = consR + Lr;
  double const * W = a.tab;
  double const * dV = W + nq;
  double const * phr = dV + nq * nv * 3;
  double const * dpr = phr + nq * Nr;
  double const * phc = dpr + nq * Nr * 3;
  double const * dpc = phc + nq * Nc;
  for (int64_t e = blockIdx.x; e < a.nelem; e += gridDim.x)
  {
    __syncthreads(); // the previous element's entries are done with the shared data
    for (int k = threadIdx.x; k < nv * 3; k += blockDim.x)
      X[k] = a.xyz[3 * (int64_t)a.conn[e * nv + k / 3] + k % 3];
    __syncthreads();
    for (int q = threadIdx.x; q < nq; q += blockDim.x)
    {
      double J[3][3] = {};
      for (int v = 0; v < nv; ++v)
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c)
            J[r][c] += X[3 * v + r] * dV[(q * nv + v) * 3 + c];
      double C[3][3]; // adj(J)
      C[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
      C[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
      C[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
      C[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
      C[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
      C[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
      C[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
      C[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
      C[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
      double const det = J[0][0] * C[0][0] + J[0][1] * C[1][0] + J[0][2] * C[2][0];
      for (int k = 0; k < 9; ++k)
        Jinv[9 * q + k] = C[k / 3][k % 3] / det;
      JxW[q] = fabs(det) * W[q];
    }
    __syncthreads();
    // mapped gradients: dphi_c = sum_k dphiRef_k Jinv[k][c]
    for (int k = threadIdx.x; k < nq * Nr; k += blockDim.x)
    {
      int const q = k / Nr;
      double const * g = dpr + 3 * k;
      for (int c = 0; c < 3; ++c)
        dRr[3 * k + c] = g[0] * Jinv[9 * q + c] + g[1] * Jinv[9 * q + 3 + c] + g[2] * Jinv[9 * q + 6 + c];
    }
    for (int k = threadIdx.x; k < nq * Nc; k += blockDim.x)
    {
      int const q = k / Nc;
      double const * g = dpc + 3 * k;
      for (int c = 0; c < 3; ++c)
        dRc[3 * k + c] = g[0] * Jinv[9 * q + c] + g[1] * Jinv[9 * q + 3 + c] + g[2] * Jinv[9 * q + 6 + c];
    }
    // constraints of the call: rows from the row space, columns (and h) from the column space
    for (int I = threadIdx.x; I < Lr; I += blockDim.x)
    {
      int64_t const id = a.emr[e * Nr + I % Nr] + (int64_t)(I / Nr) * a.ndr;
      consR[I] = a.maskr ? a.maskr[id] : 0;
    }
    for (int J = threadIdx.x; J < Lc; J += blockDim.x)
    {
      int64_t const id = a.emc[e * Nc + J % Nc] + (int64_t)(J / Nc) * a.ndc;
      bool const cj = a.maskc && a.maskc[id];
      consC[J] = cj;
      h[J] = cj ? a.valc[id] : 0.;
    }
    __syncthreads();
    if (a.pairPath)
    {
      // one space: B_d1d2(i, j) = sum_q JxW grad_d1 phi_i grad_d2 phi_j for the pairs
      // i <= j gives all nine component blocks of (i, j) and, transposed, of (j, i); the
      // stiffness is the trace of B
      for (int k = threadIdx.x; k < nq * Nr; k += blockDim.x)
      {
        double const w = JxW[k / Nr];
        dRc[3 * k] = w * dRr[3 * k];
        dRc[3 * k + 1] = w * dRr[3 * k + 1];
        dRc[3 * k + 2] = w * dRr[3 * k + 2];
        wph[k] = w * phr[k];
      }
      __syncthreads();
      bool needM = false;
      for (int k = 0; k < a.nops; ++k)
        needM = needM || a.kind[k] == PXG_OP_MASS;
      for (int p = threadIdx.x; p < Nr * (Nr + 1) / 2; p += blockDim.x)
      {
        int i = 0, rem = p;
        while (rem >= Nr - i)
        {
          rem -= Nr - i;
          ++i;
        }
        int const j = i + rem;
        double B[3][3] = {{0., 0., 0.}, {0., 0., 0.}, {0., 0., 0.}}, M = 0.;
        for (int q = 0; q < nq; ++q)
        {
          double const * gi = dRr + 3 * (q * Nr + i);
          double const * wj = dRc + 3 * (q * Nr + j);
#pragma unroll
          for (int d1 = 0; d1 < 3; ++d1)
#pragma unroll
            for (int d2 = 0; d2 < 3; ++d2)
              B[d1][d2] = fma(gi[d1], wj[d2], B[d1][d2]);
          if (needM)
            M = fma(phr[q * Nr + i], wph[q * Nr + j], M);
        }
        double const K = B[0][0] + B[1][1] + B[2][2];
        for (int d1 = 0; d1 < a.dr; ++d1)
          for (int d2 = 0; d2 < a.dr; ++d2)
          {
            double v = 0., vt = 0.; // entries (i d1, j d2) and (j d1, i d2)
            for (int k = 0; k < a.nops; ++k)
            {
              double const c = a.coef[k];
              switch (a.kind[k])
              {
              case PXG_OP_STIFFNESS:
                if (d1 == d2)
                {
                  v += c * K;
                  vt += c * K;
                }
                break;
              case PXG_OP_TENSOR_STIFFNESS:
              {
                double const dk = d1 == d2 ? K : 0.;
                v += c * (dk + B[d1][d2]);
                vt += c * (dk + B[d2][d1]);
                break;
              }
              case PXG_OP_MASS:
                if (d1 == d2)
                {
                  v += c * M;
                  vt += c * M;
                }
                break;
              }
            }
            sysEmit(a, e, d1 * Nr + i, d2 * Nr + j, v, consR, consC, h);
            if (i != j)
              sysEmit(a, e, d1 * Nr + j, d2 * Nr + i, vt, consR, consC, h);
          }
      }
      continue;
    }
    for (int p = threadIdx.x; p < Lr * Lc; p += blockDim.x)
    {
      int const I = p / Lc, J = p % Lc;
      int const i = I % Nr, d1 = I / Nr, j = J % Nc, d2 = J / Nc;
      double v = 0.;
      for (int k = 0; k < a.nops; ++k)
      {
        double s = 0.;
        switch (a.kind[k])
        {
        case PXG_OP_STIFFNESS:
        case PXG_OP_TENSOR_STIFFNESS:
          for (int q = 0; q < nq; ++q)
          {
            double const * gi = dRr + 3 * (q * Nr + i);
            double const * gj = dRc + 3 * (q * Nc + j);
            double t = d1 == d2 ? gi[0] * gj[0] + gi[1] * gj[1] + gi[2] * gj[2] : 0.;
            if (a.kind[k] == PXG_OP_TENSOR_STIFFNESS)
              t += gi[d1] * gj[d2];
            s += JxW[q] * t;
          }
          break;
        case PXG_OP_MASS:
          if (d1 == d2)
            for (int q = 0; q < nq; ++q)
              s += JxW[q] * phr[q * Nr + i] * phc[q * Nc + j];
          break;
        case PXG_OP_GRAD:
          for (int q = 0; q < nq; ++q)
            s += JxW[q] * dRr[3 * (q * Nr + i) + d1] * phc[q * Nc + j];
          break;
        case PXG_OP_DIV:
          for (int q = 0; q < nq; ++q)
            s += JxW[q] * phr[q * Nr + i] * dRc[3 * (q * Nc + j) + d2];
          break;
        }
        v += a.coef[k] * s;
      }
      sysEmit(a, e, I, J, v, consR, consC, h);
    }
  }
}

// keys of all pairs of an element's DOFs over all spaces
struct SpaceDev
{
  uint32_t const * em;
  int N, dim;
  int64_t ndof, off;
};
struct KeyArgs
{
  int nsp;
  SpaceDev s[4];
  int L;
  int64_t nelem, ntot;
};

__device__ __forceinline__ int64_t globalDof(KeyArgs const & a, int64_t e, int A)
{
  for (int k = 0; k < a.nsp; ++k)
  {
    int const Lk = a.s[k].N * a.s[k].dim;
    if (A < Lk)
      return a.s[k].off + a.s[k].em[e * a.s[k].N + A % a.s[k].N] + (int64_t)(A / a.s[k].N) * a.s[k].ndof;
    A -= Lk;
  }
  return 0;
}

__global__ void kSysKeys(KeyArgs a, unsigned long long * __restrict__ keys)
{
  int64_t const n = a.nelem * a.L * a.L;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
  {
    int64_t const e = k / ((int64_t)a.L * a.L);
    int const r = (int)(k % ((int64_t)a.L * a.L));
    keys[k] = (unsigned long long)globalDof(a, e, r / a.L) * (unsigned long long)a.ntot +
              (unsigned long long)globalDof(a, e, r % a.L);
  }
}

__global__ void kSysCsr(unsigned long long const * __restrict__ keys, int64_t nk, int64_t ntot,
                        int32_t * __restrict__ rowCount, int32_t * __restrict__ col)
{
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nk; k += (int64_t)gridDim.x * blockDim.x)
  {
    atomicAdd(rowCount + keys[k] / ntot, 1);
    col[k] = (int32_t)(keys[k] % ntot);
  }
}

unsigned gridOf(int64_t n) { return (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16); }

} // namespace
} // namespace pxg

using namespace pxg;

extern "C"
{

pxg_status pxg_sys_create(pxg_sys ** out, pxg_ctx * const * spaces, int const * dims, int const * qr_types,
                          int nspaces, int64_t * ntot, int64_t * nnz)
{
  if (!out || !spaces || !dims || nspaces < 1 || nspaces > 4)
    return PXG_ERR_INVALID_ARG;
  *out = nullptr;
  pxg_ctx * c0 = spaces[0];
  for (int s = 0; s < nspaces; ++s)
  {
    pxg_ctx * c = spaces[s];
    if (!c || c->ndof <= 0 || !c->emap.p)
      return c ? fail(c, PXG_ERR_INVALID_ARG, "space %d: set the mesh and build the DOF map first", s)
               : PXG_ERR_INVALID_ARG;
    if (dims[s] < 1 || dims[s] > 3)
      return fail(c0, PXG_ERR_INVALID_ARG, "space %d: dim %d", s, dims[s]);
    if (c->device != c0->device || c->nelem != c0->nelem || c->nnodes != c0->nnodes ||
        isHex(c->etype) != isHex(c0->etype))
      return fail(c0, PXG_ERR_INVALID_ARG, "space %d is not on the mesh of space 0", s);
    int const q = qr_types ? qr_types[s] : c->etype;
    if (q < 0 || q > 3 || isHex(q) != isHex(c->etype))
      return fail(c0, PXG_ERR_INVALID_ARG, "space %d: quadrature type %d", s, q);
  }
  pxg_status st = ensureDevice(c0);
  if (st != PXG_OK)
    return st;
  auto S = std::make_unique<pxg_sys>();
  S->device = c0->device;
  int64_t o = 0;
  KeyArgs ka{};
  ka.nsp = nspaces;
  for (int s = 0; s < nspaces; ++s)
  {
    S->sp.push_back(spaces[s]);
    S->dim.push_back(dims[s]);
    S->qr.push_back(qr_types ? qr_types[s] : spaces[s]->etype);
    S->off.push_back(o);
    S->bcMask.emplace_back(new DevBuf<uint8_t>);
    S->bcVal.emplace_back(new DevBuf<double>);
    ka.s[s] = SpaceDev{spaces[s]->emap.p, spaces[s]->N, dims[s], spaces[s]->ndof, o};
    ka.L += spaces[s]->N * dims[s];
    o += spaces[s]->ndof * dims[s];
  }
  S->ntot = o;
  if (o >= ((int64_t)1 << 31))
    return fail(c0, PXG_ERR_UNSUPPORTED, "system of 2^31 DOFs or more");
  ka.nelem = c0->nelem;
  ka.ntot = o;
  // pattern: sort the pair keys, keep the unique ones, count rows
  int64_t const nk = ka.nelem * ka.L * ka.L;
  DevBuf<unsigned long long> keys, sorted, uniq;
  DevBuf<int64_t> nu;
  PXG_CUDA(c0, keys.alloc(nk));
  PXG_CUDA(c0, sorted.alloc(nk));
  PXG_CUDA(c0, uniq.alloc(nk));
  PXG_CUDA(c0, nu.alloc(1));
  kSysKeys<<<gridOf(nk), 256>>>(ka, keys.p);
  PXG_CUDA(c0, cudaGetLastError());
  size_t tb = 0, tb2 = 0;
  PXG_CUDA(c0, cub::DeviceRadixSort::SortKeys(nullptr, tb, keys.p, sorted.p, nk));
  PXG_CUDA(c0, cub::DeviceSelect::Unique(nullptr, tb2, sorted.p, uniq.p, nu.p, nk));
  DevBuf<unsigned char> tmp;
  PXG_CUDA(c0, tmp.alloc(std::max(tb, tb2)));
  PXG_CUDA(c0, cub::DeviceRadixSort::SortKeys(tmp.p, tb, keys.p, sorted.p, nk));
  PXG_CUDA(c0, cub::DeviceSelect::Unique(tmp.p, tb2, sorted.p, uniq.p, nu.p, nk));
  int64_t nz = 0;
  PXG_CUDA(c0, cudaMemcpy(&nz, nu.p, 8, cudaMemcpyDeviceToHost));
  PXG_CUDA(c0, S->colIdx.alloc(nz));
  DevBuf<int32_t> cnt;
  PXG_CUDA(c0, cnt.alloc(o + 1));
  PXG_CUDA(c0, cudaMemset(cnt.p, 0, (o + 1) * 4));
  kSysCsr<<<gridOf(nz), 256>>>(uniq.p, nz, o, cnt.p, S->colIdx.p);
  PXG_CUDA(c0, S->rowPtr.alloc(o + 1));
  tb = 0;
  PXG_CUDA(c0, cub::DeviceScan::ExclusiveSum(nullptr, tb, cnt.p, S->rowPtr.p, o + 1));
  PXG_CUDA(c0, tmp.alloc(tb));
  PXG_CUDA(c0, cub::DeviceScan::ExclusiveSum(tmp.p, tb, cnt.p, S->rowPtr.p, o + 1));
  PXG_CUDA(c0, cudaDeviceSynchronize());
  S->nnz = nz;
  if (ntot)
    *ntot = o;
  if (nnz)
    *nnz = nz;
  *out = S.release();
  return PXG_OK;
}

pxg_status pxg_sys_destroy(pxg_sys * s)
{
  if (s)
  {
    cudaSetDevice(s->device);
    delete s;
  }
  return PXG_OK;
}

pxg_status pxg_sys_get_pattern(pxg_sys * s, int32_t * row_ptr, int32_t * col_idx)
{
  if (!s || !row_ptr || !col_idx)
    return PXG_ERR_INVALID_ARG;
  pxg_ctx * c0 = s->sp[0];
  pxg_status st = ensureDevice(c0);
  if (st != PXG_OK)
    return st;
  PXG_CUDA(c0, cudaMemcpy(row_ptr, s->rowPtr.p, (s->ntot + 1) * 4, cudaMemcpyDeviceToHost));
  PXG_CUDA(c0, cudaMemcpy(col_idx, s->colIdx.p, s->nnz * 4, cudaMemcpyDeviceToHost));
  return PXG_OK;
}

pxg_status pxg_sys_close_matrix(pxg_sys * s, double const * vals, int32_t * row_ptr, int32_t * col_idx,
                                double * vals_out, int64_t * nnz_out, void * stream)
{
  if (!s || !vals || !row_ptr || !col_idx || !vals_out || !nnz_out)
    return PXG_ERR_INVALID_ARG;
  return closeCsr(s->sp[0], s->rowPtr.p, s->colIdx.p, s->ntot, vals, row_ptr, col_idx, vals_out, nnz_out,
                  (cudaStream_t)stream);
}

pxg_status pxg_sys_pattern_device(pxg_sys * s, int32_t const ** row_ptr, int32_t const ** col_idx)
{
  if (!s || !row_ptr || !col_idx)
    return PXG_ERR_INVALID_ARG;
  *row_ptr = s->rowPtr.p;
  *col_idx = s->colIdx.p;
  return PXG_OK;
}

pxg_status pxg_sys_set_bc(pxg_sys * s, int space, uint32_t const * dofs, double const * vals, int64_t n,
                          double diag)
{
  if (!s || space < 0 || space >= (int)s->sp.size() || n < 0 || (n > 0 && (!dofs || !vals)))
    return PXG_ERR_INVALID_ARG;
  pxg_ctx * c = s->sp[space];
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  int64_t const m = c->ndof * s->dim[space];
  s->diag = diag;
  if (n == 0)
  {
    s->bcMask[space]->reset();
    s->bcVal[space]->reset();
    return PXG_OK;
  }
  std::vector<uint8_t> mask(m, 0);
  std::vector<double> v(m, 0.);
  for (int64_t k = 0; k < n; ++k)
  {
    if ((int64_t)dofs[k] >= m)
      return fail(c, PXG_ERR_INVALID_ARG, "BC DOF %u >= %lld component DOFs", dofs[k], (long long)m);
    mask[dofs[k]] = 1;
    v[dofs[k]] = vals[k]; // the last value wins
  }
  PXG_CUDA(c, s->bcMask[space]->alloc(m));
  PXG_CUDA(c, s->bcVal[space]->alloc(m));
  PXG_CUDA(c, cudaMemcpy(s->bcMask[space]->p, mask.data(), m, cudaMemcpyHostToDevice));
  PXG_CUDA(c, cudaMemcpy(s->bcVal[space]->p, v.data(), m * 8, cudaMemcpyHostToDevice));
  return PXG_OK;
}

pxg_status pxg_sys_assemble(pxg_sys * s, int row, int col, int const * kinds, double const * coefs, int nops,
                            double * vals, double * b, unsigned flags, void * stream)
{
  if (!s || row < 0 || col < 0 || row >= (int)s->sp.size() || col >= (int)s->sp.size() || !kinds || !coefs ||
      nops < 1 || nops > 4 || !vals)
    return PXG_ERR_INVALID_ARG;
  pxg_ctx * cr = s->sp[row];
  pxg_ctx * cc = s->sp[col];
  for (int k = 0; k < nops; ++k)
  {
    int const kd = kinds[k];
    bool ok = kd >= PXG_OP_STIFFNESS && kd <= PXG_OP_DIV;
    if (ok && (kd == PXG_OP_STIFFNESS || kd == PXG_OP_TENSOR_STIFFNESS || kd == PXG_OP_MASS))
      ok = row == col;
    if (ok && kd == PXG_OP_GRAD)
      ok = row != col && s->dim[col] == 1;
    if (ok && kd == PXG_OP_DIV)
      ok = row != col && s->dim[row] == 1;
    if (!ok)
      return fail(cr, PXG_ERR_INVALID_ARG, "operator %d (kind %d) does not fit spaces (%d, %d)", k, kd, row, col);
  }
  if (s->qr[row] != s->qr[col])
    return fail(cr, PXG_ERR_INVALID_ARG, "coupled spaces need the same quadrature rule");
  pxg_status st = ensureDevice(cr);
  if (st != PXG_OK)
    return st;
  // tables of the pair
  auto & T = s->tables[{row, col}];
  int const nv = cr->nv, Nr = cr->N, Nc = cc->N;
  if (!T)
  {
    std::vector<double> xi, w;
    hostRule(s->qr[row], xi, w);
    int const nq = (int)w.size();
    int const vt = isHex(cr->etype) ? Q1HEX : P1TET;
    std::vector<double> tab;
    tab.insert(tab.end(), w.begin(), w.end());
    std::vector<double> phi(27), dphi(27 * 3);
    for (int q = 0; q < nq; ++q) // vertex gradients (the geometry)
    {
      hostShape(vt, &xi[3 * q], phi.data(), dphi.data());
      tab.insert(tab.end(), dphi.begin(), dphi.begin() + 3 * nv);
    }
    for (int pass = 0; pass < 2; ++pass)
    {
      int const t = pass == 0 ? cr->etype : cc->etype, N = pass == 0 ? Nr : Nc;
      std::vector<double> ph, dp;
      for (int q = 0; q < nq; ++q)
      {
        hostShape(t, &xi[3 * q], phi.data(), dphi.data());
        ph.insert(ph.end(), phi.begin(), phi.begin() + N);
        dp.insert(dp.end(), dphi.begin(), dphi.begin() + 3 * N);
      }
      tab.insert(tab.end(), ph.begin(), ph.end());
      tab.insert(tab.end(), dp.begin(), dp.end());
    }
    T.reset(new pxg_sys::Tables);
    T->nq = nq;
    PXG_CUDA(cr, T->t.alloc(tab.size()));
    PXG_CUDA(cr, cudaMemcpy(T->t.p, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice));
  }
  cudaStream_t const st0 = (cudaStream_t)stream;
  if (!(flags & PXG_ACCUMULATE))
  {
    PXG_CUDA(cr, cudaMemsetAsync(vals, 0, s->nnz * 8, st0));
    if (b)
      PXG_CUDA(cr, cudaMemsetAsync(b, 0, s->ntot * 8, st0));
  }
  SysArgs a{};
  a.nelem = cr->nelem;
  a.nv = nv;
  a.conn = cr->conn.p;
  a.xyz = cr->xyz.p;
  a.Nr = Nr;
  a.Nc = Nc;
  a.dr = s->dim[row];
  a.dc = s->dim[col];
  a.ndr = cr->ndof;
  a.ndc = cc->ndof;
  a.offr = s->off[row];
  a.offc = s->off[col];
  a.emr = cr->emap.p;
  a.emc = cc->emap.p;
  a.maskr = s->bcMask[row]->p;
  a.valr = s->bcVal[row]->p;
  a.maskc = s->bcMask[col]->p;
  a.valc = s->bcVal[col]->p;
  a.diagCall = row == col;
  a.diag = s->diag;
  a.nq = T->nq;
  a.tab = T->t.p;
  a.nops = nops;
  for (int k = 0; k < nops; ++k)
  {
    a.kind[k] = kinds[k];
    a.coef[k] = coefs[k];
  }
  a.rowPtr = s->rowPtr.p;
  a.colIdx = s->colIdx.p;
  a.vals = vals;
  a.b = b;
  a.pairPath = row == col;
  for (int k = 0; k < nops; ++k)
    a.pairPath = a.pairPath && (kinds[k] == PXG_OP_STIFFNESS || kinds[k] == PXG_OP_TENSOR_STIFFNESS ||
                                kinds[k] == PXG_OP_MASS);
  int const Lr = Nr * a.dr, Lc = Nc * a.dc;
  size_t const smem =
      (24 + 10 * (size_t)a.nq + 3 * (size_t)a.nq * (Nr + Nc) + Lc + (size_t)a.nq * Nr) * 8 + Lr + Lc;
  unsigned const grid = (unsigned)std::min<int64_t>(a.nelem, 152 * 8);
  kSysAssemble<<<grid, kSysThreads, smem, st0>>>(a);
  PXG_CUDA(cr, cudaGetLastError());
  return PXG_OK;
}

} // extern "C"
