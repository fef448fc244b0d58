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
#include <cstdio>
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
  int shortRows; // 1: rows of at most 16 entries (2 lanes per row in the products)
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
  int chunksPerBlock; // about this many chunks of rows per block and iteration
  double tol2;
  int maxIter;
  // problem table and the chunk tables of alternate iterations
  int const * probSys;
  int64_t const * probRow0;
  int64_t const * probRows;
  int * chunkProb[2];
  int64_t * chunkRow0[2];
  int * chunkRows[2];
  int * nchunk; // [2]
  // optional timeline (PXG_BATCH_TRACE): per CG iteration the global timer after each
  // phase and the chunk count, written by block 0; nullptr when off
  unsigned long long * trace;
  int traceCap;
};

__device__ __forceinline__ unsigned long long globalTimer()
{
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// record slot k of the timeline (block 0, thread 0)
__device__ __forceinline__ void traceMark(BatchDev const & d, int k, unsigned long long v)
{
  if (d.trace && blockIdx.x == 0 && threadIdx.x == 0 && k < d.traceCap)
    d.trace[k] = v;
}

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

// Sum NV per-thread values over the block and add them to dst[slot[q]] (one atomic
// per quantity).  Every thread of the block calls it.
template <int NV>
__device__ __forceinline__ void blockAddTo(double (&v)[NV], double * dst, int const (&slot)[NV])
{
  __shared__ double red[kBt / 32][NV];
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q)
  {
    double x = v[q];
    for (int o = 16; o > 0; o >>= 1)
      x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0)
      red[warp][q] = x;
  }
  __syncthreads();
  if (warp == 0)
  {
#pragma unroll
    for (int q = 0; q < NV; ++q)
    {
      double x = lane < kBt / 32 ? red[lane][q] : 0.;
      for (int o = 16; o > 0; o >>= 1)
        x += __shfl_xor_sync(0xffffffffu, x, o);
      if (lane == 0 && x != 0.)
        atomicAdd(dst + slot[q], x);
    }
  }
  __syncthreads();
}

// Exclusive prefix sum over the block of one int per thread; returns the thread's
// offset and sets total.  Every thread of the block calls it.
__device__ __forceinline__ int blockExclusiveScan(int x, int & total)
{
  __shared__ int wsum[kBt / 32];
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int inc = x;
  for (int o = 1; o < 32; o <<= 1)
  {
    int const y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o)
      inc += y;
  }
  if (lane == 31)
    wsum[warp] = inc;
  __syncthreads();
  int base = 0, tot = 0;
  for (int w = 0; w < kBt / 32; ++w)
  {
    base += w < warp ? wsum[w] : 0;
    tot += wsum[w];
  }
  __syncthreads();
  total = tot;
  return base + inc - x;
}

// Block 0: cut the rows of the running problems into chunks of equal size (at least
// 256 rows, about d.chunksPerBlock = 4 per block) for the iterations of parity `par`.
// The chunks are dealt round-robin to the blocks, so the work of an iteration follows
// the running problems instead of a fixed row partition.
__device__ void buildChunks(BatchDev const & d, int par)
{
  __shared__ long long sRows;
  if (threadIdx.x == 0)
    sRows = 0;
  __syncthreads();
  long long mine = 0;
  for (int k = threadIdx.x; k < d.nprob; k += blockDim.x)
    if (!__ldcg(d.done + k))
      mine += d.probRows[k];
  atomicAdd(reinterpret_cast<unsigned long long *>(&sRows), (unsigned long long)mine);
  __syncthreads();
  long long const rows = sRows;
  long long const per = d.chunksPerBlock;
  long long csize = (rows + per * gridDim.x - 1) / (per * gridDim.x);
  csize = csize < 256 ? 256 : csize;
  int running = 0;
  for (int base = 0; base < d.nprob; base += blockDim.x)
  {
    int const k = base + threadIdx.x;
    int64_t const nr = (k < d.nprob && !__ldcg(d.done + k)) ? d.probRows[k] : 0;
    int const nc = (int)((nr + csize - 1) / csize);
    int tot;
    int const off = running + blockExclusiveScan(nc, tot);
    for (int c = 0; c < nc; ++c)
    {
      d.chunkProb[par][off + c] = k;
      d.chunkRow0[par][off + c] = d.probRow0[k] + c * csize;
      d.chunkRows[par][off + c] = (int)(nr - c * csize < csize ? nr - c * csize : csize);
    }
    running += tot;
  }
  if (threadIdx.x == 0)
    d.nchunk[par] = running;
  __threadfence();
}

// q = K p over the rows [c0, c0 + nr) of one chunk; returns the thread's share of p.q.
// A warp takes 32 rows at a time, LPR batches of 32 / LPR rows (LPR lanes per row), and
// reduces the lane partials with transposeReduce, so that every lane ends with one
// row's value: the FP64 pipe, which bounds this phase with the matrix stream, spends
// LPR - 1 additions and one p.q FMA per lane on 32 rows instead of log2(LPR) additions
// per batch and a p.q FMA that only one lane in LPR uses.
template <int LPR, int UNR>
__device__ __forceinline__ double spmvChunk(SysDev const & s, int64_t c0, int nr)
{
  constexpr int RPW = 32 / LPR;
  int const lane = threadIdx.x & 31, warp = threadIdx.x / 32, nwarps = blockDim.x / 32;
  int const sub = lane & (LPR - 1);
  double pq = 0.;
  for (int v0 = warp * 32; v0 < nr; v0 += nwarps * 32)
  {
    double t[LPR];
#pragma unroll
    for (int k = 0; k < LPR; ++k)
    {
      int const v = v0 + k * RPW + lane / LPR;
      bool const act = v < nr;
      t[k] = rowDot<true, LPR, UNR, false>(s.rp, s.ci, s.K, s.p, c0 + (act ? v : 0), act);
    }
    double const qv = transposeReduce<LPR>(t, sub);
    int const v = v0 + sub * RPW + lane / LPR; // the row whose value this lane holds
    if (v < nr)
    {
      __stcg(s.q + c0 + v, qv);
      pq += __ldcg(s.p + c0 + v) * qv;
    }
  }
  return pq;
}

constexpr int kRu = 4;  // rows per thread whose loads are issued before any store (p update)
constexpr int kRu2 = 2; // the same for the x, r, z update (five loads a row)

// One batched PCG solve: x = K^-1 rhs per problem.  `forward` selects (b -> u) or
// (Mw -> lam).  Returns false on a barrier timeout.
__device__ bool batchCg(BatchDev const & d, bool forward, BlockAcc<2> & ba2)
{
  int const tb = forward ? 0 : d.traceCap / 2; // timeline: [iteration][S1 end, S2 end, S3 end, chunks]
  int64_t const nthr = (int64_t)gridDim.x * blockDim.x;
  int64_t const tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t r0, r1;
  blockRows(d, r0, r1);
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
  if (blockIdx.x == 0)
  {
    for (int k = threadIdx.x; k < d.nprob; k += blockDim.x)
      if (__ldcg(d.acc + (int64_t)k * A_N + A_BB) == 0.)
        d.done[k] = 1;
    __syncthreads();
    buildChunks(d, 0);
  }
  if (!gridSync(d))
    return false;
  traceMark(d, d.traceCap / 2 - 1 + tb, globalTimer()); // start of the iterations
  for (int it = 0; it < d.maxIter; ++it)
  {
    int const par = it & 1;
    int const nch = __ldcg(d.nchunk + par);
    if (nch == 0)
      break; // every problem has converged
    int const * cProb = d.chunkProb[par];
    int64_t const * cRow0 = d.chunkRow0[par];
    int const * cRows = d.chunkRows[par];
    // S1: q = K p, p.q ; zero the slots reused next
    if (blockIdx.x == 0)
      for (int k = threadIdx.x; k < d.nprob; k += blockDim.x)
      {
        d.acc[(int64_t)k * A_N + A_PQ0 + (par ^ 1)] = 0.;
        d.acc[(int64_t)k * A_N + A_RR0 + (par ^ 1)] = 0.;
        d.acc[(int64_t)k * A_N + A_RZ0 + par] = 0.;
      }
    for (int c = blockIdx.x; c < nch; c += gridDim.x)
    {
      int const pr = __ldcg(cProb + c);
      int64_t const c0 = __ldcg(cRow0 + c);
      int const nr = __ldcg(cRows + c);
      SysDev const & s = d.sys[d.probSys[pr]];
      double pq[1] = {s.shortRows ? spmvChunk<2, 8>(s, c0, nr) : spmvChunk<4, 7>(s, c0, nr)};
      int const sl[1] = {A_PQ0 + par};
      blockAddTo<1>(pq, d.acc + (int64_t)pr * A_N, sl);
    }
    if (!gridSync(d))
      return false;
    if (4 * it + 3 < d.traceCap / 2 - 1)
      traceMark(d, tb + 4 * it, globalTimer());
    // S2: x += alpha p, r -= alpha q, z = D^-1 r ; r.z, r.r
    for (int c = blockIdx.x; c < nch; c += gridDim.x)
    {
      int const pr = __ldcg(cProb + c);
      int64_t const c0 = __ldcg(cRow0 + c);
      int const nr = __ldcg(cRows + c);
      SysDev const & s = d.sys[d.probSys[pr]];
      double const * a = d.acc + (int64_t)pr * A_N;
      double const al = __ldcg(a + A_RZ0 + (par ^ 1)) / __ldcg(a + A_PQ0 + par);
      double * x = forward ? s.u : s.lam;
      double v2[2] = {0., 0.};
      for (int v = threadIdx.x; v < nr; v += kRu2 * blockDim.x)
      {
        double xv[kRu2], pv[kRu2], rv[kRu2], qv[kRu2], dv[kRu2];
#pragma unroll
        for (int u = 0; u < kRu2; ++u)
        {
          int const vv = v + u * blockDim.x;
          int64_t const lr = c0 + (vv < nr ? vv : 0);
          xv[u] = __ldcg(x + lr);
          pv[u] = __ldcg(s.p + lr);
          rv[u] = __ldcg(s.r + lr);
          qv[u] = __ldcg(s.q + lr);
          dv[u] = s.dinv[lr];
        }
#pragma unroll
        for (int u = 0; u < kRu2; ++u)
        {
          int const vv = v + u * blockDim.x;
          if (vv >= nr)
            break;
          int64_t const lr = c0 + vv;
          __stcg(x + lr, xv[u] + al * pv[u]);
          double const ri = rv[u] - al * qv[u];
          __stcg(s.r + lr, ri);
          double const zi = dv[u] * ri;
          __stcg(s.z + lr, zi);
          v2[0] += ri * zi;
          v2[1] += ri * ri;
        }
      }
      int const sl[2] = {A_RZ0 + par, A_RR0 + par};
      blockAddTo<2>(v2, d.acc + (int64_t)pr * A_N, sl);
    }
    if (!gridSync(d))
      return false;
    if (4 * it + 3 < d.traceCap / 2 - 1)
      traceMark(d, tb + 4 * it + 1, globalTimer());
    // S3: convergence per problem, p = z + beta p
    for (int c = blockIdx.x; c < nch; c += gridDim.x)
    {
      int const pr = __ldcg(cProb + c);
      double const * a = d.acc + (int64_t)pr * A_N;
      if (__ldcg(a + A_RR0 + par) <= d.tol2 * __ldcg(a + A_BB))
        continue;
      int64_t const c0 = __ldcg(cRow0 + c);
      int const nr = __ldcg(cRows + c);
      SysDev const & s = d.sys[d.probSys[pr]];
      double const be = __ldcg(a + A_RZ0 + par) / __ldcg(a + A_RZ0 + (par ^ 1));
      for (int v = threadIdx.x; v < nr; v += kRu * blockDim.x)
      {
        double zv[kRu], pv[kRu];
#pragma unroll
        for (int u = 0; u < kRu; ++u)
        {
          int const vv = v + u * blockDim.x;
          int64_t const lr = c0 + (vv < nr ? vv : 0);
          zv[u] = __ldcg(s.z + lr);
          pv[u] = __ldcg(s.p + lr);
        }
#pragma unroll
        for (int u = 0; u < kRu; ++u)
        {
          int const vv = v + u * blockDim.x;
          if (vv < nr)
            __stcg(s.p + c0 + vv, zv[u] + be * pv[u]);
        }
      }
    }
    // bookkeeping and the next iteration's chunks, by block 0 (the other blocks read
    // them after the barrier)
    if (blockIdx.x == 0)
    {
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
      __syncthreads();
      buildChunks(d, par ^ 1);
    }
    if (!gridSync(d))
      return false;
    if (4 * it + 3 < d.traceCap / 2 - 1)
    {
      traceMark(d, tb + 4 * it + 2, globalTimer());
      traceMark(d, tb + 4 * it + 3, (unsigned long long)nch);
    }
  }
  return gridSync(d);
}

__global__ void __launch_bounds__(kBt, 4) kBatchSolve(BatchDev d)
{
  __shared__ BlockAcc<2> ba2;
  __shared__ BlockAcc<1> ba1;
  if (!batchCg(d, true, ba2))
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
  batchCg(d, false, ba2);
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
  int64_t totalRows = 0;
  for (int i = 0; i < nctx; ++i)
    totalRows += ctxs[i]->ndof;
  int64_t const capChunks = totalRows / 256 + nprob + 16;
  auto dropGraph = [&] {
    if (S.exec)
      cudaGraphExecDestroy(S.exec);
    S.exec = nullptr;
  };
  if (S.nprob < nprob)
  {
    dropGraph(); // the graph holds the old buffers
    PXG_CUDA(c0, S.acc.alloc((size_t)nprob * A_N));
    PXG_CUDA(c0, S.done.alloc(nprob));
    PXG_CUDA(c0, S.itF.alloc(nprob));
    PXG_CUDA(c0, S.itA.alloc(nprob));
    PXG_CUDA(c0, S.bar.alloc(2));
    PXG_CUDA(c0, S.err.alloc(1));
    PXG_CUDA(c0, S.probSys.alloc(nprob));
    PXG_CUDA(c0, S.probRow0.alloc(nprob));
    PXG_CUDA(c0, S.probRows.alloc(nprob));
    S.nprob = nprob;
  }
  if (S.capChunks < capChunks)
  {
    dropGraph();
    for (int k = 0; k < 2; ++k)
    {
      PXG_CUDA(c0, S.chunkProb[k].alloc(capChunks));
      PXG_CUDA(c0, S.chunkRows[k].alloc(capChunks));
      PXG_CUDA(c0, S.chunkRow0[k].alloc(capChunks));
    }
    PXG_CUDA(c0, S.nchunk.alloc(2));
    S.capChunks = capChunks;
  }
  {
    // problem table: system, first row and rows of every problem, in global order
    std::vector<int> ps;
    std::vector<int64_t> p0, pn;
    for (int i = 0; i < nctx; ++i)
    {
      std::vector<int64_t> const & off = ctxs[i]->batch.dofOffHost;
      for (int64_t q = 0; q < ctxs[i]->batch.nprob; ++q)
      {
        ps.push_back(i);
        p0.push_back(off[q]);
        pn.push_back(off[q + 1] - off[q]);
      }
    }
    PXG_CUDA(c0, cudaMemcpy(S.probSys.p, ps.data(), ps.size() * sizeof(int), cudaMemcpyHostToDevice));
    PXG_CUDA(c0, cudaMemcpy(S.probRow0.p, p0.data(), p0.size() * 8, cudaMemcpyHostToDevice));
    PXG_CUDA(c0, cudaMemcpy(S.probRows.p, pn.data(), pn.size() * 8, cudaMemcpyHostToDevice));
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
                      B.r.p, B.z.p, B.p.p, B.q.p, B.dinv.p, B.w.p, B.Mw.p, c->ndof, c->maxRowLen <= 16 ? 1 : 0};
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
  d.probSys = S.probSys.p;
  d.probRow0 = S.probRow0.p;
  d.probRows = S.probRows.p;
  for (int k = 0; k < 2; ++k)
  {
    d.chunkProb[k] = S.chunkProb[k].p;
    d.chunkRow0[k] = S.chunkRow0[k].p;
    d.chunkRows[k] = S.chunkRows[k].p;
  }
  d.nchunk = S.nchunk.p;
  // optional timeline of the persistent solver (not with graph replay: the buffer is
  // read back after the launch)
  char const * traceFile = getenv("PXG_BATCH_TRACE");
  DevBuf<unsigned long long> trace;
  if (traceFile && traceFile[0])
  {
    d.traceCap = 2 * (4 * std::min(max_iter, 4096) + 1);
    PXG_CUDA(c0, trace.alloc(d.traceCap));
    PXG_CUDA(c0, cudaMemset(trace.p, 0, d.traceCap * 8));
    d.trace = trace.p;
    use_graph = 0;
  }
  {
    // PXG_TEST_BARRIER_SHORTFALL=1 makes every grid barrier wait for one block more
    // than the grid has, so the bounded waits run out (tests of the timeout path)
    char const * t = getenv("PXG_TEST_BARRIER_SHORTFALL");
    d.extra = (t && t[0] == '1') ? 1u : 0u;
    // chunks per block and iteration: 4 measured best on the 256-problem batch (2: 410,
    // 4: 361, 8: 368, 16: 411 ms); PXG_BATCH_CHUNKS overrides
    char const * cpb = getenv("PXG_BATCH_CHUNKS");
    d.chunksPerBlock = (cpb && atoi(cpb) > 0) ? atoi(cpb) : 4;
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
      key.scatter[i] = ctxs[i]->scatter;
      key.threads[i] = ctxs[i]->threads;
      key.arith[i] = ctxs[i]->arith;
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
  if (d.trace)
  {
    // text: one line per CG iteration, "solve iteration ns_S1 ns_S2 ns_S3 chunks"
    std::vector<unsigned long long> t(d.traceCap);
    PXG_CUDA(c0, cudaMemcpy(t.data(), d.trace, t.size() * 8, cudaMemcpyDeviceToHost));
    if (FILE * f = fopen(traceFile, "a"))
    {
      int const half = d.traceCap / 2;
      for (int sv = 0; sv < 2; ++sv)
      {
        unsigned long long prev = t[sv * half + half - 1];
        for (int it = 0; 4 * it + 3 < half - 1 && t[sv * half + 4 * it + 2]; ++it)
        {
          unsigned long long const * r = &t[sv * half + 4 * it];
          fprintf(f, "%d %d %llu %llu %llu %llu\n", sv, it, r[0] - prev, r[1] - r[0], r[2] - r[1], r[3]);
          prev = r[2];
        }
      }
      fclose(f);
    }
  }
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
