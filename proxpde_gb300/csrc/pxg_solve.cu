// Device Jacobi-preconditioned CG and the adjoint gradient of the diffusion loss
//   K(k) u = b,   J(u) = 1/2 (u - u_t)^T M (u - u_t),   dJ/d log k_e = -(C u)_e^T K_e (C lambda)_e
// with K lambda = M (u - u_t), K_e = k_e K0_e the element stiffness and C zeroing the
// DOFs constrained by the essential BCs (the derivative of the condensed matrix
// C K C + D is C K0_e C).  proxpde itself solves with UmfPackLU
// (include/sparse_matrix.hpp:44); the CG here is plain and not an optimisation
// target.
//
// CG design: every scalar (alpha, beta, r.z, residual, done flag, iteration count)
// stays in device memory; dot products are reduced in two deterministic passes
// (per-block partials, then a fixed-order sum that every block of the next kernel does
// itself, so that an iteration is three kernels: the product, the update of x, r and z,
// the update of p); a chunk of iterations is captured once in a CUDA graph and
// replayed, and the host reads the done flag once per chunk.  Kernels after
// convergence return immediately, so a partly used chunk costs launches only.
// GB300's FP64 rate (1/64 of FP32) makes the product about as FP64-bound as it is
// HBM-bound: every entry is one FMA, and every unused slot of a row's last round and
// every shuffle addition costs a slot too, so the lanes per row and entries per lane
// follow the matrix's mean row length.
#include <cub/block/block_reduce.cuh>

#include <algorithm>
#include <cmath>
#include <vector>

#include "pxg_internal.h"

namespace pxg
{
namespace
{

constexpr int kTpb = 256;
constexpr int kMaxPartBlocks = 1024;
constexpr int kChunk = 16; // CG iterations per captured graph

enum : int
{
  S_RZ = 0, // r.z of the iterations of even index (S_RZNEW: odd)
  S_PQ,
  S_RZNEW,
  S_RR,
  S_BB,
  S_ALPHA,
  S_BETA,
  S_DONE,
  S_ITER,
  S_TOL2,
  S_MAXIT,
  S_COUNT
};

inline int partBlocks(int64_t n)
{
  int64_t b = (n + kTpb - 1) / kTpb;
  return (int)(b < kMaxPartBlocks ? b : kMaxPartBlocks);
}

template <int NV>
__device__ __forceinline__ void blockSum(double (&v)[NV], double * out)
{
  using BR = cub::BlockReduce<double, kTpb>;
  __shared__ typename BR::TempStorage ts;
#pragma unroll
  for (int k = 0; k < NV; ++k)
  {
    double const s = BR(ts).Sum(v[k]);
    if (threadIdx.x == 0)
      out[k] = s;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kTpb) kDiagInv(int32_t const * __restrict__ rp, int32_t const * __restrict__ ci,
                                                 double const * __restrict__ a, int64_t n, double * __restrict__ dinv)
{
  int64_t const r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n)
    return;
  double d = 0.;
  for (int32_t p = rp[r]; p < rp[r + 1]; ++p)
    if (ci[p] == (int32_t)r)
      d = a[p];
  dinv[r] = (d != 0.) ? 1.0 / d : 1.0;
}

__global__ void __launch_bounds__(kTpb) kCgInit(double const * __restrict__ b, double const * __restrict__ dinv,
                                                int64_t n, double * __restrict__ x, double * __restrict__ r,
                                                double * __restrict__ z, double * __restrict__ p,
                                                double * __restrict__ part)
{
  double acc[2] = {0., 0.};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
  {
    double const bi = b[i], zi = dinv[i] * bi;
    x[i] = 0.;
    r[i] = bi;
    z[i] = zi;
    p[i] = zi;
    acc[0] += bi * zi;
    acc[1] += bi * bi;
  }
  blockSum<2>(acc, part + 2 * blockIdx.x);
}

// Sum the per-block partials with one block (deterministic for a fixed grid).
template <int NV>
__device__ __forceinline__ void sumPartials(double const * __restrict__ part, int nb, double (&out)[NV])
{
  double v[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k)
    v[k] = 0.;
  for (int b = threadIdx.x; b < nb; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < NV; ++k)
      v[k] += part[NV * b + k];
  __shared__ double res[NV];
  blockSum<NV>(v, res);
#pragma unroll
  for (int k = 0; k < NV; ++k)
    out[k] = res[k];
}

__global__ void __launch_bounds__(kTpb) kFinalInit(double const * __restrict__ part, int nb, double * __restrict__ s,
                                                   double tol2, double maxit)
{
  double t[2];
  sumPartials<2>(part, nb, t);
  if (threadIdx.x != 0)
    return;
  s[S_RZ] = t[0];
  s[S_BB] = t[1];
  s[S_RR] = t[1];
  s[S_ITER] = 0.;
  s[S_TOL2] = tol2;
  s[S_MAXIT] = maxit;
  s[S_DONE] = (t[1] == 0.) ? 1. : 0.;
}

// q = A p and the partials of p.q; LPR lanes per row, UNR entries per lane and round
template <int LPR, int UNR>
__global__ void __launch_bounds__(kTpb) kSpmvDot(int32_t const * __restrict__ rp, int32_t const * __restrict__ ci,
                                                 double const * __restrict__ a, double const * __restrict__ p,
                                                 int64_t n, double * __restrict__ q, double * __restrict__ part,
                                                 double const * __restrict__ s)
{
  if (s[S_DONE] != 0.)
    return;
  double acc[1] = {0.};
  constexpr int RPW = 32 / LPR; // rows per warp step
  int64_t const warps = (int64_t)gridDim.x * (blockDim.x / 32);
  int64_t const w = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  int const lane = threadIdx.x & 31;
  for (int64_t r0 = w * RPW; r0 < n; r0 += warps * RPW)
  {
    int64_t const row = r0 + lane / LPR;
    bool const valid = row < n;
    double const t = rowDot<false, LPR, UNR>(rp, ci, a, p, row, valid);
    if (valid && (lane & (LPR - 1)) == 0)
    {
      q[row] = t;
      acc[0] += p[row] * t;
    }
  }
  blockSum<1>(acc, part + blockIdx.x);
}

__device__ __forceinline__ int rzSlot(int parity) { return parity ? S_RZNEW : S_RZ; }

// x += alpha p, r -= alpha q, z = D^-1 r and the partials of r.z and r.r, with
// alpha = r.z / p.q from the product's partials (every block sums them in the same
// order, so all use the same alpha); `parity` is the iteration index's
__global__ void __launch_bounds__(kTpb) kCgUpdate(double * __restrict__ x, double * __restrict__ r,
                                                  double const * __restrict__ p, double const * __restrict__ q,
                                                  double const * __restrict__ dinv, double * __restrict__ z,
                                                  int64_t n, double const * __restrict__ partPQ, int nb,
                                                  double * __restrict__ part, double * __restrict__ s, int parity)
{
  if (s[S_DONE] != 0.)
    return;
  double pq[1];
  sumPartials<1>(partPQ, nb, pq);
  double const al = s[rzSlot(parity)] / pq[0];
  if (blockIdx.x == 0 && threadIdx.x == 0)
  {
    s[S_PQ] = pq[0];
    s[S_ALPHA] = al;
  }
  double acc[2] = {0., 0.};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
  {
    x[i] += al * p[i];
    double const ri = r[i] - al * q[i];
    r[i] = ri;
    double const zi = dinv[i] * ri;
    z[i] = zi;
    acc[0] += ri * zi;
    acc[1] += ri * ri;
  }
  blockSum<2>(acc, part + 2 * blockIdx.x);
}

// p = z + beta p with beta = r.z (new) / r.z (old) from the update's partials (every
// block sums them in the same order); block 0 stores the new r.z in the other parity's
// slot, counts the iteration and raises the done flag.  The flag is read once per
// block (a block that sees it raised by block 0 skips an update nobody reads).
__global__ void __launch_bounds__(kTpb) kPUpdate(double * __restrict__ p, double const * __restrict__ z, int64_t n,
                                                 double const * __restrict__ part, int nb, double * __restrict__ s,
                                                 int parity)
{
  __shared__ int done;
  if (threadIdx.x == 0)
    done = s[S_DONE] != 0.;
  __syncthreads();
  if (done)
    return;
  double t[2];
  sumPartials<2>(part, nb, t);
  double const rz = t[0], rr = t[1];
  double const be = rz / s[rzSlot(parity)];
  if (blockIdx.x == 0 && threadIdx.x == 0)
  {
    s[rzSlot(parity ^ 1)] = rz;
    s[S_RR] = rr;
    s[S_BETA] = be;
    double const it = s[S_ITER] + 1.;
    s[S_ITER] = it;
    if (rr <= s[S_TOL2] * s[S_BB] || it >= s[S_MAXIT] || !(rr == rr))
      s[S_DONE] = 1.;
  }
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = z[i] + be * p[i];
}

// y = A x and the dot x^T y (deterministic), for the loss
__global__ void __launch_bounds__(kTpb) kSpmvPlainDot(int32_t const * __restrict__ rp, int32_t const * __restrict__ ci,
                                                      double const * __restrict__ a, double const * __restrict__ x,
                                                      int64_t n, double * __restrict__ y, double * __restrict__ part)
{
  double acc[1] = {0.};
  constexpr int RPW = 32 / kLpr;
  int64_t const warps = (int64_t)gridDim.x * (blockDim.x / 32);
  int64_t const w = (int64_t)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  int const lane = threadIdx.x & 31;
  for (int64_t r0 = w * RPW; r0 < n; r0 += warps * RPW)
  {
    int64_t const row = r0 + lane / kLpr;
    bool const valid = row < n;
    double const t = rowDot<false>(rp, ci, a, x, row, valid);
    if (valid && (lane & (kLpr - 1)) == 0)
    {
      y[row] = t;
      acc[0] += x[row] * t;
    }
  }
  blockSum<1>(acc, part + blockIdx.x);
}

__global__ void kSub(double const * __restrict__ a, double const * __restrict__ b, int64_t n, double * __restrict__ c)
{
  int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n)
    c[i] = a[i] - b[i];
}

__global__ void kScale(double * __restrict__ v, int64_t n, double s)
{
  int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n)
    v[i] *= s;
}

} // namespace

// ------------------------------------------------------------------ CG driver
pxg_status cgSolve(pxg_ctx * c, int32_t const * rp, int32_t const * ci, double const * a, int64_t n,
                   double const * b, double * x, double rtol, int maxIter, int * itersOut, double * relOut,
                   cudaStream_t user)
{
  CgWork & w = c->cg;
  if (w.n < n)
  {
    PXG_CUDA(c, w.r.alloc(n));
    PXG_CUDA(c, w.z.alloc(n));
    PXG_CUDA(c, w.p.alloc(n));
    PXG_CUDA(c, w.q.alloc(n));
    PXG_CUDA(c, w.dinv.alloc(n));
    PXG_CUDA(c, w.part.alloc(3 * kMaxPartBlocks)); // p.q, then r.z and r.r
    PXG_CUDA(c, w.scal.alloc(S_COUNT));
    w.n = n;
  }
  if (!w.stream)
    PXG_CUDA(c, cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking));
  if (!w.evIn)
  {
    PXG_CUDA(c, cudaEventCreateWithFlags(&w.evIn, cudaEventDisableTiming));
    PXG_CUDA(c, cudaEventCreateWithFlags(&w.evOut, cudaEventDisableTiming));
  }
  cudaStream_t const s = w.stream;
  PXG_CUDA(c, cudaEventRecord(w.evIn, user));
  PXG_CUDA(c, cudaStreamWaitEvent(s, w.evIn, 0));
  int const nb = partBlocks(n);
  unsigned const rows = (unsigned)((n + kTpb - 1) / kTpb);
  kDiagInv<<<rows, kTpb, 0, s>>>(rp, ci, a, n, w.dinv.p);
  kCgInit<<<nb, kTpb, 0, s>>>(b, w.dinv.p, n, x, w.r.p, w.z.p, w.p.p, w.part.p);
  kFinalInit<<<1, kTpb, 0, s>>>(w.part.p, nb, w.scal.p, rtol * rtol, (double)maxIter);
  PXG_CUDA(c, cudaGetLastError());

  // the product's row split from the mean row length (P1 tetrahedra ~15, Q1 hexahedra
  // ~27, longer rows several rounds of 32)
  int32_t nnz = 0;
  PXG_CUDA(c, cudaMemcpyAsync(&nnz, rp + n, sizeof(nnz), cudaMemcpyDeviceToHost, s));
  PXG_CUDA(c, cudaStreamSynchronize(s));
  double const meanRow = n > 0 ? (double)nnz / (double)n : 0.;
  auto spmv = meanRow <= 16. ? kSpmvDot<2, 8> : meanRow <= 28. ? kSpmvDot<2, 14> : kSpmvDot<4, 8>;
  // the product's grid: one wave of resident blocks (its register use limits them),
  // so that no second, partial wave trails
  int perSm = 0;
  PXG_CUDA(c, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, spmv, kTpb, 0));
  int64_t const rowsPerBlock = kTpb / 2;
  int const nbS = (int)std::max<int64_t>(1, std::min<int64_t>({(int64_t)kMaxPartBlocks, (int64_t)perSm * c->sms,
                                                                (n + rowsPerBlock - 1) / rowsPerBlock}));
  double * const partPQ = w.part.p;
  double * const partRZ = w.part.p + kMaxPartBlocks;

  // capture one chunk of iterations (an even number, so that the parity of an
  // iteration's index is its position's in the chunk)
  static_assert(kChunk % 2 == 0, "r.z slots alternate by iteration");
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  PXG_CUDA(c, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
  for (int k = 0; k < kChunk; ++k)
  {
    spmv<<<nbS, kTpb, 0, s>>>(rp, ci, a, w.p.p, n, w.q.p, partPQ, w.scal.p);
    kCgUpdate<<<nb, kTpb, 0, s>>>(x, w.r.p, w.p.p, w.q.p, w.dinv.p, w.z.p, n, partPQ, nbS, partRZ, w.scal.p, k & 1);
    kPUpdate<<<nb, kTpb, 0, s>>>(w.p.p, w.z.p, n, partRZ, nb, w.scal.p, k & 1);
  }
  cudaError_t ce = cudaStreamEndCapture(s, &graph);
  if (ce == cudaSuccess)
    ce = cudaGraphInstantiate(&exec, graph, 0);
  if (graph)
    cudaGraphDestroy(graph);
  if (ce != cudaSuccess)
    return cudaFail(c, ce, "CG graph capture");
  double h[S_COUNT];
  pxg_status st = PXG_OK;
  for (int launched = 0;; launched += kChunk)
  {
    ce = cudaGraphLaunch(exec, s);
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(h, w.scal.p, sizeof(h), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess)
      ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess)
    {
      st = cudaFail(c, ce, "CG iterations");
      break;
    }
    if (h[S_DONE] != 0. || launched + kChunk >= maxIter)
      break;
  }
  cudaGraphExecDestroy(exec);
  if (st != PXG_OK)
    return st;
  PXG_CUDA(c, cudaEventRecord(w.evOut, s));
  PXG_CUDA(c, cudaStreamWaitEvent(user, w.evOut, 0));
  double const rel = h[S_BB] > 0. ? std::sqrt(h[S_RR] / h[S_BB]) : 0.;
  if (itersOut)
    *itersOut = (int)h[S_ITER];
  if (relOut)
    *relOut = rel;
  if (!(rel <= rtol))
    return fail(c, PXG_ERR_NOT_CONVERGED, "CG stopped after %d iterations at relative residual %.3e (tol %.1e)",
                (int)h[S_ITER], rel, rtol);
  return PXG_OK;
}

} // namespace pxg

using namespace pxg;

extern "C"
{

pxg_status pxg_cg(pxg_ctx * c, int32_t const * row_ptr, int32_t const * col_idx, double const * vals, int64_t n,
                  double const * b, double * x, double rtol, int max_iter, int * iters, double * rel_res,
                  void * stream)
{
  if (!c || !row_ptr || !col_idx || !vals || !b || !x || n <= 0 || !(rtol > 0.) || max_iter <= 0)
    return c ? fail(c, PXG_ERR_INVALID_ARG, "pxg_cg: bad argument") : PXG_ERR_INVALID_ARG;
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  return cgSolve(c, row_ptr, col_idx, vals, n, b, x, rtol, max_iter, iters, rel_res, (cudaStream_t)stream);
}

pxg_status pxg_adjoint_grad(pxg_ctx * c, double const * u, double const * lambda, double * g, void * stream)
{
  if (!c || !u || !lambda || !g)
    return PXG_ERR_INVALID_ARG;
  if (!c->emap.p || !c->hasCoef)
    return fail(c, PXG_ERR_INVALID_ARG, "adjoint gradient needs the DOF map and the coefficient");
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  return launchAdjointGrad(c, u, lambda, g, (cudaStream_t)stream);
}

pxg_status pxg_adjoint_forward(pxg_ctx * c, pxg_rhs_op const * rhs, double const * u_target, double rtol,
                               int max_iter, double * u_out, double * loss, int * iters, void * stream)
{
  if (!c || !rhs || !u_target || !loss)
    return PXG_ERR_INVALID_ARG;
  if (!c->rowPtr.p || !c->hasCoef)
    return fail(c, PXG_ERR_INVALID_ARG, "forward needs the pattern and the coefficient");
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  cudaStream_t const s = (cudaStream_t)stream;
  AdjState & A = c->adj;
  int64_t const n = c->ndof, nnz = c->nnz;
  if (A.n != n || A.nnz != nnz)
  {
    PXG_CUDA(c, A.K.alloc(nnz));
    PXG_CUDA(c, A.M.alloc(nnz));
    PXG_CUDA(c, A.b.alloc(n));
    PXG_CUDA(c, A.u.alloc(n));
    PXG_CUDA(c, A.w.alloc(n));
    PXG_CUDA(c, A.Mw.alloc(n));
    PXG_CUDA(c, A.lam.alloc(n));
    PXG_CUDA(c, A.part.alloc(kMaxPartBlocks));
    A.n = n;
    A.nnz = nnz;
  }
  A.valid = false;
  // K(k) with BCs, M without, b = rhs with BCs (and the BC lift of K)
  pxg_lhs_op const opK{2, 1.0, 0, 0.0, 1};
  pxg_lhs_op const opM{0, 0.0, 1, 1.0, 0};
  pxg_rhs_op r = *rhs;
  r.apply_bc = 1;
  if ((st = pxg_assemble(c, &opK, A.K.p, &opM, A.M.p, &r, A.b.p, 0u, stream)) != PXG_OK)
    return st;
  if ((st = cgSolve(c, c->rowPtr.p, c->colIdx.p, A.K.p, n, A.b.p, A.u.p, rtol, max_iter, iters, nullptr, s)) !=
      PXG_OK)
    return st;
  unsigned const blocks = (unsigned)((n + kTpb - 1) / kTpb);
  kSub<<<blocks, kTpb, 0, s>>>(A.u.p, u_target, n, A.w.p);
  int const nb = partBlocks(n);
  kSpmvPlainDot<<<nb, kTpb, 0, s>>>(c->rowPtr.p, c->colIdx.p, A.M.p, A.w.p, n, A.Mw.p, A.part.p);
  PXG_CUDA(c, cudaGetLastError());
  std::vector<double> hp(nb);
  PXG_CUDA(c, cudaMemcpyAsync(hp.data(), A.part.p, nb * sizeof(double), cudaMemcpyDeviceToHost, s));
  PXG_CUDA(c, cudaStreamSynchronize(s));
  double J = 0.;
  for (double v : hp)
    J += v;
  *loss = 0.5 * J;
  if (u_out)
    PXG_CUDA(c, cudaMemcpyAsync(u_out, A.u.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  A.rtol = rtol;
  A.maxIter = max_iter;
  A.valid = true;
  return PXG_OK;
}

pxg_status pxg_adjoint_backward(pxg_ctx * c, double dloss, double * grad, double * lambda_out, int * iters,
                                void * stream)
{
  if (!c || !grad)
    return PXG_ERR_INVALID_ARG;
  AdjState & A = c->adj;
  if (!A.valid)
    return fail(c, PXG_ERR_INVALID_ARG, "pxg_adjoint_backward needs a preceding pxg_adjoint_forward");
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  cudaStream_t const s = (cudaStream_t)stream;
  // K lambda = M (u - u_t)  (K symmetric)
  if ((st = cgSolve(c, c->rowPtr.p, c->colIdx.p, A.K.p, A.n, A.Mw.p, A.lam.p, A.rtol, A.maxIter, iters, nullptr,
                    s)) != PXG_OK)
    return st;
  if ((st = launchAdjointGrad(c, A.u.p, A.lam.p, grad, s)) != PXG_OK)
    return st;
  if (dloss != 1.0)
    kScale<<<(unsigned)((c->nelem + kTpb - 1) / kTpb), kTpb, 0, s>>>(grad, c->nelem, dloss);
  if (lambda_out)
    PXG_CUDA(c, cudaMemcpyAsync(lambda_out, A.lam.p, A.n * sizeof(double), cudaMemcpyDeviceToDevice, s));
  PXG_CUDA(c, cudaGetLastError());
  return PXG_OK;
}

} // extern "C"
