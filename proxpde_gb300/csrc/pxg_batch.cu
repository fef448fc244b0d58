// Batched adjoint gradients: many independent problems assembled, solved and
// differentiated together.
//
// A batch is the disjoint union of the problems of one element type, given to a
// context as one mesh whose elements are grouped by problem.  proxpde's first-touch
// numbering (include/dof.hpp:111-329) over such a union gives every problem a
// contiguous DOF range, and the union's pattern is block diagonal, so assembly and
// the gradient kernel need nothing new: one launch covers every problem.
//
// The solves need per-problem scalars.  kBatchSolve is one persistent cooperative
// kernel that, for every problem of up to two batches at once, runs Jacobi-PCG on
// K u = b, forms J_p = 1/2 (u - u_t)^T M (u - u_t) and M (u - u_t), and runs the
// adjoint CG K lambda = M (u - u_t); each problem stops at its own tolerance.  Grid
// barriers between the CG stages are bounded spins: when a wait exceeds its limit the
// kernel sets an error flag and every block returns (PXG_ERR_TIMEOUT on the host).
// pxg_batch_adjoint captures the assembly, the persistent solve and the gradient
// kernels in one CUDA graph and replays it.
#include <cooperative_groups.h>

#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <vector>

#include "pxg_internal.h"

namespace pxg
{
namespace
{

constexpr int kBt = 256;               // threads per block of the persistent kernel
constexpr unsigned kSpinLimit = 1u << 22; // polls of a barrier before giving up (x ~256 ns)

// per-problem accumulator slots
enum : int
{
  A_PQ0 = 0,
  A_PQ1,
  A_RZ0,
  A_RZ1,
  A_RR0,
  A_RR1,
  A_BB,
  A_J,
  A_N
};

struct SysDev
{
  int32_t const * rp;
  int32_t const * ci;
  double const * K;
  double const * M;
  double const * b;
  double const * ut;
  int32_t const * rowProb; // global problem id of each row
  double * u;
  double * lam;
  double * r;
  double * z;
  double * p;
  double * q;
  double * dinv;
  double * w;
  double * Mw;
  int64_t nrows;
};

struct BatchDev
{
  SysDev sys[2];
  int nsys;
  int64_t total;  // rows of all systems
  int nprob;      // problems of all systems
  double * acc;   // [nprob][A_N]
  int * done;     // [nprob] 0 = running, else iterations + 1
  int * itF;      // [nprob] forward CG iterations
  int * itA;      // [nprob] adjoint CG iterations
  unsigned * bar; // [0] arrivals, [1] generation
  int * err;      // [0] barrier timeout
  unsigned extra; // arrivals expected beyond the grid (0; >0 only to test the timeout path)
  double tol2;
  int maxIter;
};

// Grid barrier with a bounded wait.  Returns false (and sets err) on timeout.
__device__ bool gridSync(BatchDev const & d)
{
  __syncthreads();
  __shared__ int ok;
  if (threadIdx.x == 0)
  {
    ok = 1;
    volatile unsigned * gen = d.bar + 1;
    unsigned const g = *gen;
    __threadfence();
    if (atomicAdd(d.bar, 1u) == gridDim.x - 1 + d.extra)
    {
      d.bar[0] = 0;
      __threadfence();
      atomicAdd(d.bar + 1, 1u);
    }
    else
    {
      unsigned spins = 0;
      while (*gen == g)
      {
        if (++spins > kSpinLimit || *(volatile int *)d.err)
        {
          atomicExch(d.err, 1);
          ok = 0;
          break;
        }
        __nanosleep(256);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok && !*(volatile int *)d.err;
}

// row g of the virtual concatenation -> (system, local row)
__device__ __forceinline__ int sysOf(BatchDev const & d, int64_t g, int64_t & lr)
{
  if (d.nsys > 1 && g >= d.sys[0].nrows)
  {
    lr = g - d.sys[0].nrows;
    return 1;
  }
  lr = g;
  return 0;
}

__device__ __forceinline__ int probOf(BatchDev const & d, int64_t g)
{
  int64_t lr;
  int const sy = sysOf(d, g, lr);
  return d.sys[sy].rowProb[lr];
}

// Per-block accumulation of per-problem sums.  Every block owns one contiguous range
// of rows, so it meets a contiguous range of problem ids [pmin, pmin + nslot); each
// lane keeps running sums while its problem does not change and flushes them into
// shared-memory slots, and the block adds its slots into the global accumulators at
// the end of the phase: one global atomic per block, problem and quantity.
constexpr int kMaxSlot = 128;

template <int NV>
struct BlockAcc
{
  int pmin, nslot;
  double v[kMaxSlot][NV];
};

template <int NV>
__device__ __forceinline__ void baBegin(BlockAcc<NV> & ba, BatchDev const & d, int64_t r0, int64_t r1)
{
  __syncthreads(); // the previous phase's flush has finished reading the slots
  if (threadIdx.x == 0)
  {
    if (r0 < r1)
    {
      ba.pmin = probOf(d, r0);
      ba.nslot = probOf(d, r1 - 1) - ba.pmin + 1;
    }
    else
    {
      ba.pmin = 0;
      ba.nslot = 0;
    }
  }
  for (int k = threadIdx.x; k < kMaxSlot * NV; k += blockDim.x)
    ba.v[k / NV][k % NV] = 0.;
  __syncthreads();
}

template <int NV>
struct LaneAcc
{
  int prob = -1;
  double v[NV];
};

template <int NV>
__device__ __forceinline__ void laFlush(LaneAcc<NV> & la, BlockAcc<NV> & ba, double * acc, int const (&slot)[NV])
{
  if (la.prob < 0)
    return;
  int const k = la.prob - ba.pmin;
#pragma unroll
  for (int q = 0; q < NV; ++q)
    if (la.v[q] != 0.)
    {
      if (k >= 0 && k < ba.nslot && k < kMaxSlot)
        atomicAdd(&ba.v[k][q], la.v[q]);
      else
        atomicAdd(acc + (int64_t)la.prob * A_N + slot[q], la.v[q]);
    }
  la.prob = -1;
}

template <int NV>
__device__ __forceinline__ void laAdd(LaneAcc<NV> & la, BlockAcc<NV> & ba, double * acc, int const (&slot)[NV],
                                      int prob, double const (&v)[NV])
{
  if (prob != la.prob)
  {
    laFlush<NV>(la, ba, acc, slot);
    la.prob = prob;
#pragma unroll
    for (int q = 0; q < NV; ++q)
      la.v[q] = 0.;
  }
#pragma unroll
  for (int q = 0; q < NV; ++q)
    la.v[q] += v[q];
}

template <int NV>
__device__ __forceinline__ void baEnd(BlockAcc<NV> & ba, LaneAcc<NV> & la, double * acc, int const (&slot)[NV])
{
  laFlush<NV>(la, ba, acc, slot);
  __syncthreads();
  int const n = ba.nslot < kMaxSlot ? ba.nslot : kMaxSlot;
  for (int k = threadIdx.x; k < n * NV; k += blockDim.x)
  {
    double const x = ba.v[k / NV][k % NV];
    if (x != 0.)
      atomicAdd(acc + (int64_t)(ba.pmin + k / NV) * A_N + slot[k % NV], x);
  }
}

// rows of this block
__device__ __forceinline__ void blockRows(BatchDev const & d, int64_t & r0, int64_t & r1)
{
  int64_t const per = (d.total + gridDim.x - 1) / gridDim.x;
  r0 = (int64_t)blockIdx.x * per;
  if (r0 > d.total)
    r0 = d.total;
  r1 = r0 + per;
  if (r1 > d.total)
    r1 = d.total;
}

// One batched PCG solve: x = K^-1 rhs per problem.  `forward` selects (b -> u) or
// (Mw -> lam).  Returns false on a barrier timeout.
__device__ bool batchCg(BatchDev const & d, bool forward, BlockAcc<2> & ba2, BlockAcc<1> & ba1)
{
  int64_t const nthr = (int64_t)gridDim.x * blockDim.x;
  int64_t const tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t r0, r1;
  blockRows(d, r0, r1);
  constexpr int RPW = 32 / kLpr;
  int const lane = threadIdx.x & 31, warp = threadIdx.x / 32, nwarps = blockDim.x / 32;
  // reset accumulators and flags
  for (int64_t k = tid; k < (int64_t)d.nprob * A_N; k += nthr)
    if ((k % A_N) != A_J)
      d.acc[k] = 0.;
  for (int64_t k = tid; k < d.nprob; k += nthr)
  {
    d.done[k] = 0;
    (forward ? d.itF : d.itA)[k] = 0;
  }
  if (!gridSync(d))
    return false;
  // init: x = 0, r = rhs, z = D^-1 r, p = z; r.z into RZ1 (the slot iteration 0 reads), b.b
  {
    int const sl[2] = {A_RZ1, A_BB};
    baBegin<2>(ba2, d, r0, r1);
    LaneAcc<2> la;
    for (int64_t g = r0 + threadIdx.x; g < r1; g += blockDim.x)
    {
      int64_t lr;
      SysDev const & s = d.sys[sysOf(d, g, lr)];
      double const bi = forward ? s.b[lr] : __ldcg(s.Mw + lr);
      double dd = 0.;
      for (int32_t k = s.rp[lr]; k < s.rp[lr + 1]; ++k)
        if (s.ci[k] == (int32_t)lr)
          dd = s.K[k];
      double const di = dd != 0. ? 1.0 / dd : 1.0;
      s.dinv[lr] = di;
      double const zi = di * bi;
      __stcg((forward ? s.u : s.lam) + lr, 0.);
      __stcg(s.r + lr, bi);
      __stcg(s.z + lr, zi);
      __stcg(s.p + lr, zi);
      double const v[2] = {bi * zi, bi * bi};
      laAdd<2>(la, ba2, d.acc, sl, s.rowProb[lr], v);
    }
    baEnd<2>(ba2, la, d.acc, sl);
  }
  if (!gridSync(d))
    return false;
  for (int64_t k = tid; k < d.nprob; k += nthr)
    if (d.acc[k * A_N + A_BB] == 0.)
      d.done[k] = 1;
  if (!gridSync(d))
    return false;
  for (int it = 0; it < d.maxIter; ++it)
  {
    int const par = it & 1;
    // S1: q = K p, p.q ; zero the slots reused next
    if (blockIdx.x == 0)
      for (int k = threadIdx.x; k < d.nprob; k += blockDim.x)
      {
        d.acc[(int64_t)k * A_N + A_PQ0 + (par ^ 1)] = 0.;
        d.acc[(int64_t)k * A_N + A_RR0 + (par ^ 1)] = 0.;
        d.acc[(int64_t)k * A_N + A_RZ0 + par] = 0.;
      }
    {
      int const sl[1] = {A_PQ0 + par};
      baBegin<1>(ba1, d, r0, r1);
      LaneAcc<1> la;
      for (int64_t g0 = r0 + (int64_t)warp * RPW; g0 < r1; g0 += (int64_t)nwarps * RPW)
      {
        int64_t const g = g0 + lane / kLpr;
        int64_t lr = 0;
        int sy = 0, pr = -1;
        bool act = false;
        if (g < r1)
        {
          sy = sysOf(d, g, lr);
          pr = d.sys[sy].rowProb[lr];
          act = !__ldcg(d.done + pr);
        }
        SysDev const & s = d.sys[sy];
        double const t = rowDot<true>(s.rp, s.ci, s.K, s.p, lr, act);
        if (act && (lane & (kLpr - 1)) == 0)
        {
          __stcg(s.q + lr, t);
          double const v[1] = {__ldcg(s.p + lr) * t};
          laAdd<1>(la, ba1, d.acc, sl, pr, v);
        }
      }
      baEnd<1>(ba1, la, d.acc, sl);
    }
    if (!gridSync(d))
      return false;
    // S2: x += alpha p, r -= alpha q, z = D^-1 r ; r.z, r.r
    {
      int const sl[2] = {A_RZ0 + par, A_RR0 + par};
      baBegin<2>(ba2, d, r0, r1);
      LaneAcc<2> la;
      for (int64_t g = r0 + threadIdx.x; g < r1; g += blockDim.x)
      {
        int64_t lr;
        SysDev const & s = d.sys[sysOf(d, g, lr)];
        int const pr = s.rowProb[lr];
        if (__ldcg(d.done + pr))
          continue;
        double const * a = d.acc + (int64_t)pr * A_N;
        double const al = __ldcg(a + A_RZ0 + (par ^ 1)) / __ldcg(a + A_PQ0 + par);
        double * x = forward ? s.u : s.lam;
        __stcg(x + lr, __ldcg(x + lr) + al * __ldcg(s.p + lr));
        double const ri = __ldcg(s.r + lr) - al * __ldcg(s.q + lr);
        __stcg(s.r + lr, ri);
        double const zi = s.dinv[lr] * ri;
        __stcg(s.z + lr, zi);
        double const v[2] = {ri * zi, ri * ri};
        laAdd<2>(la, ba2, d.acc, sl, pr, v);
      }
      baEnd<2>(ba2, la, d.acc, sl);
    }
    if (!gridSync(d))
      return false;
    // S3: convergence per problem, p = z + beta p
    for (int64_t g = r0 + threadIdx.x; g < r1; g += blockDim.x)
    {
      int64_t lr;
      SysDev const & s = d.sys[sysOf(d, g, lr)];
      int const pr = s.rowProb[lr];
      if (__ldcg(d.done + pr))
        continue;
      double const * a = d.acc + (int64_t)pr * A_N;
      if (!(__ldcg(a + A_RR0 + par) <= d.tol2 * __ldcg(a + A_BB)))
      {
        double const be = __ldcg(a + A_RZ0 + par) / __ldcg(a + A_RZ0 + (par ^ 1));
        __stcg(s.p + lr, __ldcg(s.z + lr) + be * __ldcg(s.p + lr));
      }
    }
    // bookkeeping by block 0 (other blocks only read `done` after the barrier)
    if (blockIdx.x == 0)
      for (int k = threadIdx.x; k < d.nprob; k += blockDim.x)
        if (!d.done[k])
        {
          double const * a = d.acc + (int64_t)k * A_N;
          if (__ldcg(a + A_RR0 + par) <= d.tol2 * __ldcg(a + A_BB) || it + 1 >= d.maxIter)
          {
            d.done[k] = it + 2;
            (forward ? d.itF : d.itA)[k] = it + 1;
          }
        }
    if (!gridSync(d))
      return false;
    // all problems done?
    __shared__ int running;
    if (threadIdx.x == 0)
      running = 0;
    __syncthreads();
    for (int k = threadIdx.x; k < d.nprob; k += blockDim.x)
      if (!__ldcg(d.done + k))
        running = 1;
    __syncthreads();
    if (!running)
      break;
  }
  return gridSync(d);
}

__global__ void __launch_bounds__(kBt) kBatchSolve(BatchDev d)
{
  __shared__ BlockAcc<2> ba2;
  __shared__ BlockAcc<1> ba1;
  if (!batchCg(d, true, ba2, ba1))
    return;
  // loss: w = u - u_t, Mw = M w, J_p = 1/2 w.Mw
  int64_t r0, r1;
  blockRows(d, r0, r1);
  for (int64_t g = r0 + threadIdx.x; g < r1; g += blockDim.x)
  {
    int64_t lr;
    SysDev const & s = d.sys[sysOf(d, g, lr)];
    __stcg(s.w + lr, __ldcg(s.u + lr) - s.ut[lr]);
  }
  if (!gridSync(d))
    return;
  {
    constexpr int RPW = 32 / kLpr;
    int const lane = threadIdx.x & 31, warp = threadIdx.x / 32, nwarps = blockDim.x / 32;
    int const sl[1] = {A_J};
    baBegin<1>(ba1, d, r0, r1);
    LaneAcc<1> la;
    for (int64_t g0 = r0 + (int64_t)warp * RPW; g0 < r1; g0 += (int64_t)nwarps * RPW)
    {
      int64_t const g = g0 + lane / kLpr;
      int64_t lr = 0;
      int sy = 0;
      bool const valid = g < r1;
      if (valid)
        sy = sysOf(d, g, lr);
      SysDev const & s = d.sys[sy];
      double const t = rowDot<true>(s.rp, s.ci, s.M, s.w, lr, valid);
      if (valid && (lane & (kLpr - 1)) == 0)
      {
        __stcg(s.Mw + lr, t);
        double const v[1] = {0.5 * __ldcg(s.w + lr) * t};
        laAdd<1>(la, ba1, d.acc, sl, s.rowProb[lr], v);
      }
    }
    baEnd<1>(ba1, la, d.acc, sl);
  }
  if (!gridSync(d))
    return;
  batchCg(d, false, ba2, ba1);
}

// DOF range of problem p: from the DOF of its first element's first slot (the first
// DOF it touches) to the next problem's
__global__ void kDofOff(uint32_t const * __restrict__ emap, int64_t const * __restrict__ elemOff, int nprob, int N,
                        int64_t ndof, int64_t * __restrict__ dofOff)
{
  int const p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > nprob)
    return;
  dofOff[p] = (p == nprob) ? ndof : (int64_t)emap[elemOff[p] * N];
}

__global__ void kFillRowProb(int64_t const * __restrict__ dofOff, int nprob, int probBase, int32_t * __restrict__ rowProb)
{
  int const p = blockIdx.x;
  if (p >= nprob)
    return;
  for (int64_t r = dofOff[p] + threadIdx.x; r < dofOff[p + 1]; r += blockDim.x)
    rowProb[r] = probBase + p;
}

} // namespace
} // namespace pxg

using namespace pxg;

extern "C"
{

pxg_status pxg_batch_set(pxg_ctx * c, int64_t const * elem_offsets, int64_t nprob)
{
  if (!c || !elem_offsets || nprob <= 0)
    return PXG_ERR_INVALID_ARG;
  if (!c->rowPtr.p)
    return fail(c, PXG_ERR_INVALID_ARG, "build the pattern of the union mesh first");
  if (elem_offsets[0] != 0 || elem_offsets[nprob] != c->nelem)
    return fail(c, PXG_ERR_INVALID_ARG, "element offsets must run from 0 to nelem");
  for (int64_t p = 0; p < nprob; ++p)
    if (elem_offsets[p + 1] <= elem_offsets[p])
      return fail(c, PXG_ERR_INVALID_ARG, "problem %lld has no element", (long long)p);
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  BatchState & B = c->batch;
  int64_t const n = c->ndof, nnz = c->nnz;
  B.nprob = nprob;
  PXG_CUDA(c, B.elemOff.alloc(nprob + 1));
  PXG_CUDA(c, B.dofOff.alloc(nprob + 1));
  PXG_CUDA(c, cudaMemcpy(B.elemOff.p, elem_offsets, (nprob + 1) * 8, cudaMemcpyHostToDevice));
  PXG_CUDA(c, B.rowProb.alloc(n));
  kDofOff<<<(unsigned)((nprob + 1 + 255) / 256), 256>>>(c->emap.p, B.elemOff.p, (int)nprob, c->N, n, B.dofOff.p);
  kFillRowProb<<<(unsigned)nprob, 256>>>(B.dofOff.p, (int)nprob, 0, B.rowProb.p);
  PXG_CUDA(c, cudaGetLastError());
  // the DOF ranges must be contiguous and increasing (elements grouped by problem, no
  // node shared between problems)
  std::vector<int64_t> h(nprob + 1);
  PXG_CUDA(c, cudaMemcpy(h.data(), B.dofOff.p, (nprob + 1) * 8, cudaMemcpyDeviceToHost));
  for (int64_t p = 0; p < nprob; ++p)
    if (h[p + 1] <= h[p])
      return fail(c, PXG_ERR_INVALID_ARG, "problems share DOFs or are not grouped (problem %lld)", (long long)p);
  B.dofOffHost = h;
  for (DevBuf<double> * v : {&B.K, &B.M})
    PXG_CUDA(c, v->alloc(nnz));
  for (DevBuf<double> * v : {&B.b, &B.u, &B.lam, &B.r, &B.z, &B.p, &B.q, &B.dinv, &B.w, &B.Mw})
    PXG_CUDA(c, v->alloc(n));
  B.ready = true;
  return PXG_OK;
}

pxg_status pxg_batch_adjoint(pxg_ctx * const * ctxs, int nctx, pxg_rhs_op const * rhs,
                             double const * const * u_targets, double rtol, int max_iter, double * losses,
                             double * const * grads, int * iters, int use_graph, void * stream)
{
  if (!ctxs || nctx < 1 || nctx > 2 || !rhs || !u_targets || !losses || !grads || !(rtol > 0.) || max_iter <= 0)
    return PXG_ERR_INVALID_ARG;
  pxg_ctx * c0 = ctxs[0];
  for (int i = 0; i < nctx; ++i)
  {
    if (!ctxs[i] || !ctxs[i]->batch.ready || !ctxs[i]->hasCoef || !u_targets[i] || !grads[i])
      return ctxs[i] ? fail(ctxs[i], PXG_ERR_INVALID_ARG, "batch %d: pxg_batch_set, the coefficient, the target "
                                                            "and the gradient output are required", i)
                     : PXG_ERR_INVALID_ARG;
    if (ctxs[i]->device != c0->device)
      return fail(c0, PXG_ERR_INVALID_ARG, "batches must live on one GPU");
  }
  pxg_status st = ensureDevice(c0);
  if (st != PXG_OK)
    return st;
  BatchShared & S = c0->bshared;
  int nprob = 0;
  for (int i = 0; i < nctx; ++i)
    nprob += (int)ctxs[i]->batch.nprob;
  if (S.nprob < nprob)
  {
    PXG_CUDA(c0, S.acc.alloc((size_t)nprob * A_N));
    PXG_CUDA(c0, S.done.alloc(nprob));
    PXG_CUDA(c0, S.itF.alloc(nprob));
    PXG_CUDA(c0, S.itA.alloc(nprob));
    PXG_CUDA(c0, S.bar.alloc(2));
    PXG_CUDA(c0, S.err.alloc(1));
    S.nprob = nprob;
  }
  // second batch: its problems follow the first one's
  if (nctx == 2)
  {
    BatchState & B1 = ctxs[1]->batch;
    int const base = (int)ctxs[0]->batch.nprob;
    if (B1.probBase != base)
    {
      kFillRowProb<<<(unsigned)B1.nprob, 256>>>(B1.dofOff.p, (int)B1.nprob, base, B1.rowProb.p);
      PXG_CUDA(c0, cudaGetLastError());
      B1.probBase = base;
    }
  }
  else if (ctxs[0]->batch.probBase != 0)
  {
    kFillRowProb<<<(unsigned)ctxs[0]->batch.nprob, 256>>>(ctxs[0]->batch.dofOff.p, (int)ctxs[0]->batch.nprob, 0,
                                                          ctxs[0]->batch.rowProb.p);
    ctxs[0]->batch.probBase = 0;
  }
  BatchDev d{};
  d.nsys = nctx;
  d.total = 0;
  for (int i = 0; i < nctx; ++i)
  {
    pxg_ctx * c = ctxs[i];
    BatchState & B = c->batch;
    d.sys[i] = SysDev{c->rowPtr.p, c->colIdx.p, B.K.p, B.M.p, B.b.p, u_targets[i], B.rowProb.p, B.u.p, B.lam.p,
                      B.r.p, B.z.p, B.p.p, B.q.p, B.dinv.p, B.w.p, B.Mw.p, c->ndof};
    d.total += c->ndof;
  }
  d.nprob = nprob;
  d.acc = S.acc.p;
  d.done = S.done.p;
  d.itF = S.itF.p;
  d.itA = S.itA.p;
  d.bar = S.bar.p;
  d.err = S.err.p;
  d.tol2 = rtol * rtol;
  d.maxIter = max_iter;
  {
    // PXG_TEST_BARRIER_SHORTFALL=1 makes every grid barrier wait for one block more
    // than the grid has, so the bounded waits run out (tests of the timeout path)
    char const * t = getenv("PXG_TEST_BARRIER_SHORTFALL");
    d.extra = (t && t[0] == '1') ? 1u : 0u;
  }

  int dev = c0->device, sms = 0, perSm = 0;
  PXG_CUDA(c0, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  PXG_CUDA(c0, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kBatchSolve, kBt, 0));
  if (perSm < 1)
    return fail(c0, PXG_ERR_CUDA, "persistent solver does not fit on an SM");
  int const blocks = sms * (perSm < 8 ? perSm : 8);

  cudaStream_t const s = (cudaStream_t)stream;
  auto record = [&](cudaStream_t rs) -> pxg_status {
    pxg_lhs_op const opK{2, 1.0, 0, 0.0, 1};
    pxg_lhs_op const opM{0, 0.0, 1, 1.0, 0};
    pxg_rhs_op r = *rhs;
    r.apply_bc = 1;
    for (int i = 0; i < nctx; ++i)
    {
      pxg_status e = pxg_assemble(ctxs[i], &opK, ctxs[i]->batch.K.p, &opM, ctxs[i]->batch.M.p, &r,
                                  ctxs[i]->batch.b.p, 0u, rs);
      if (e != PXG_OK)
        return e;
    }
    PXG_CUDA(c0, cudaMemsetAsync(S.acc.p, 0, (size_t)nprob * A_N * 8, rs));
    PXG_CUDA(c0, cudaMemsetAsync(S.bar.p, 0, 8, rs));
    PXG_CUDA(c0, cudaMemsetAsync(S.err.p, 0, 4, rs));
    void * args[] = {&d};
    PXG_CUDA(c0, cudaLaunchCooperativeKernel((void const *)kBatchSolve, dim3(blocks), dim3(kBt), args, 0, rs));
    for (int i = 0; i < nctx; ++i)
    {
      pxg_status e = launchAdjointGrad(ctxs[i], ctxs[i]->batch.u.p, ctxs[i]->batch.lam.p, grads[i], rs);
      if (e != PXG_OK)
        return e;
    }
    return PXG_OK;
  };

  if (use_graph)
  {
    // the graph is rebuilt when the arguments change; replayed otherwise
    GraphKey key{};
    key.nctx = nctx;
    for (int i = 0; i < nctx; ++i)
    {
      key.ctx[i] = ctxs[i];
      key.ut[i] = u_targets[i];
      key.grad[i] = grads[i];
    }
    key.rhs = *rhs;
    key.rtol = rtol;
    key.maxIter = max_iter;
    if (!S.exec || !(S.key == key))
    {
      if (S.exec)
        cudaGraphExecDestroy(S.exec);
      S.exec = nullptr;
      cudaStream_t cs = nullptr;
      PXG_CUDA(c0, cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      PXG_CUDA(c0, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      pxg_status e = record(cs);
      cudaGraph_t graph = nullptr;
      cudaError_t ce = cudaStreamEndCapture(cs, &graph);
      cudaStreamDestroy(cs);
      if (e != PXG_OK)
      {
        if (graph)
          cudaGraphDestroy(graph);
        return e;
      }
      if (ce == cudaSuccess)
        ce = cudaGraphInstantiate(&S.exec, graph, 0);
      if (graph)
        cudaGraphDestroy(graph);
      if (ce != cudaSuccess)
        return cudaFail(c0, ce, "batch graph capture");
      S.key = key;
    }
    PXG_CUDA(c0, cudaGraphLaunch(S.exec, s));
  }
  else
  {
    if ((st = record(s)) != PXG_OK)
      return st;
  }
  // per-problem results
  std::vector<double> acc((size_t)nprob * A_N);
  std::vector<int> itf(nprob), ita(nprob);
  int err = 0;
  PXG_CUDA(c0, cudaMemcpyAsync(acc.data(), S.acc.p, acc.size() * 8, cudaMemcpyDeviceToHost, s));
  PXG_CUDA(c0, cudaMemcpyAsync(itf.data(), S.itF.p, nprob * 4, cudaMemcpyDeviceToHost, s));
  PXG_CUDA(c0, cudaMemcpyAsync(ita.data(), S.itA.p, nprob * 4, cudaMemcpyDeviceToHost, s));
  PXG_CUDA(c0, cudaMemcpyAsync(&err, S.err.p, 4, cudaMemcpyDeviceToHost, s));
  PXG_CUDA(c0, cudaStreamSynchronize(s));
  if (err)
    return fail(c0, PXG_ERR_TIMEOUT, "persistent batch solver: a grid barrier wait ran out");
  int worst = 0;
  bool conv = true;
  for (int p = 0; p < nprob; ++p)
  {
    losses[p] = acc[(size_t)p * A_N + A_J];
    worst = std::max(worst, std::max(itf[p], ita[p]));
    if (itf[p] >= max_iter || ita[p] >= max_iter)
      conv = false;
  }
  if (iters)
    *iters = worst;
  if (!conv)
    return fail(c0, PXG_ERR_NOT_CONVERGED, "a batched CG reached %d iterations", max_iter);
  return PXG_OK;
}

} // extern "C"
