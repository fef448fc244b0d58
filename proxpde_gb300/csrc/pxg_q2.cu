// Q2 hexahedra in double-float arithmetic.
//
// The FP64 element loop of kAssemble<Q2HEX> runs one element per thread with ~37k
// FP64 operations per element, bound by the FP64 pipe at 1/64 of the FP32 rate.
// Here a block of 128 threads assembles one element at a time (persistent grid,
// elements strided over the blocks), with the Q2 reference tables held once per block
// in shared memory as hi/lo float pairs (double-float, pxg_dfl.h):
//   1. the 12 edge differences of the element's vertices (FP64, exact conversions) and
//      its vertex average (the hexahedron's origin, geo.hpp:721-728);
//   2. thread q < 27 = Gauss point q: J_q of the trilinear map as half the bilinear
//      interpolation of the edge differences along each axis (the same J as the
//      mapping over the 27 Lagrange points, which lie on the trilinear image), adj(J_q),
//      |det J_q|, G_q = w_q adj adj^T / |det J_q| and w_q |det J_q|;
//   3. v_j(q) = G_q grad phi_j(q) and u_j(q) = w_q |det J_q| phi_j(q) for the 27 x 27
//      (point, function) items;
//   4. the 378 entries i <= j: K_ij = sum_q grad phi_i(q) . v_j(q) (81 products) and
//      M_ij = sum_q phi_i(q) u_j(q) (27 products), each an exact-product compensated
//      sum, converted to double with one FP64 addition and scattered with FP64
//      reductions at the element's scatter ranks.
// The coefficient of a single stiffness (mass) operator is folded into G (u).
// Dirichlet condensation and the load vector follow kAssemble (FP64).
#include <vector>

#include "pxg_dfl.h"
#include "pxg_internal.h"

namespace pxg
{
namespace q2
{
constexpr int NT = 128;
constexpr int NQ = 27, N = 27, NP = N * (N + 1) / 2; // points, functions, pairs i <= j

// reference tables (filled by initQ2Tables): grad phi_j(q) and phi_j(q) as hi/lo pairs,
// phi_j(q) in FP64, the rule, and the pairs (i << 8 | j) in row-major order
__device__ float2 gDphi[NQ * N * 3];
__device__ float2 gPhi[NQ * N];
__device__ double gPhiD[NQ * N];
__device__ double gXi[NQ * 3];
__device__ double gW[NQ];
__device__ uint16_t gPairs[NP];

// shared-memory layout of a block (bytes)
constexpr size_t kDphi = 0;                                  // float2 [NQ][N][3]
constexpr size_t kPhi = kDphi + sizeof(float2) * NQ * N * 3; // float2 [NQ][N]
constexpr size_t kPhiD = kPhi + sizeof(float2) * NQ * N;     // double [NQ][N]
constexpr size_t kV = kPhiD + sizeof(double) * NQ * N;       // float2 [NQ][N][3]
constexpr size_t kU = kV + sizeof(float2) * NQ * N * 3;      // float2 [NQ][N]
constexpr size_t kG = kU + sizeof(float2) * NQ * N;          // float2 [NQ][6] G, then [NQ] mass weights
constexpr size_t kWJ = kG + sizeof(float2) * NQ * 7;         // double [NQ]: w_q |det J_q|
constexpr size_t kFq = kWJ + sizeof(double) * NQ;            // double [NQ]: load at the points
constexpr size_t kD = kFq + sizeof(double) * NQ;             // float2 [12][3]: edge differences
constexpr size_t kX = kD + sizeof(float2) * 36;              // double [8][3]
constexpr size_t kOrg = kX + sizeof(double) * 24;            // double [3] (+1)
constexpr size_t kBv = kOrg + sizeof(double) * 4;            // double [N]
constexpr size_t kDof = kBv + sizeof(double) * N;            // uint32 [N] (+1)
constexpr size_t kRp = kDof + sizeof(uint32_t) * 28;         // int32 [N] (+1)
constexpr size_t kCons = kRp + sizeof(int32_t) * 28;         // uint32 (+3)
constexpr size_t kSmem = kCons + 16;

// x-, y- and z-edges of the hexahedron as (from, to) vertex pairs whose other two
// lattice coordinates are (0,0), (1,0), (0,1), (1,1) in the order of the other axes
__constant__ int kEdges[3][4][2] = {{{0, 1}, {3, 2}, {4, 5}, {7, 6}},
                                    {{0, 3}, {1, 2}, {4, 7}, {5, 6}},
                                    {{0, 4}, {1, 5}, {3, 7}, {2, 6}}};

struct Acc
{
  float s, c;
};
// acc += a * b: exact high product (FMA TwoProd), TwoSum into the running sum, the
// errors and the low parts' products gathered in one float
__device__ __forceinline__ void mac(Acc & acc, dfl a, dfl b)
{
  float const p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  dfl const t = dflTwoSum(acc.s, p);
  acc.s = t.h;
  acc.c = __fadd_rn(acc.c, __fadd_rn(t.l, e));
}
__device__ __forceinline__ dfl ld(float2 const * p) { float2 const v = *p; return dfl{v.x, v.y}; }
__device__ __forceinline__ void st(float2 * p, dfl v) { *p = make_float2(v.h, v.l); }

// Dirichlet condensation of one entry (builder.hpp:76-124), out of line (FP64)
__device__ __noinline__ void condenseQ2(double * diag, double bcDiag, double * b, uint32_t dofi, uint32_t dofj,
                                        double bvi, double bvj, bool ci, bool cj, bool isDiag, double val)
{
  if (isDiag)
  {
    atomicAdd(diag, bcDiag);
    return;
  }
  if (!b)
    return;
  if (!ci)
  {
    double const t = val * bvj;
    if (t != 0.)
      atomicAdd(b + dofi, -t);
  }
  if (!cj)
  {
    double const t = val * bvi;
    if (t != 0.)
      atomicAdd(b + dofj, -t);
  }
}

__global__ void __launch_bounds__(NT) kAssembleQ2(AsmArgs a)
{
  extern __shared__ uint4 dynShared[];
  char * const sm = reinterpret_cast<char *>(dynShared);
  float2 * const tDphi = reinterpret_cast<float2 *>(sm + kDphi);
  float2 * const tPhi = reinterpret_cast<float2 *>(sm + kPhi);
  double * const tPhiD = reinterpret_cast<double *>(sm + kPhiD);
  float2 * const sV = reinterpret_cast<float2 *>(sm + kV);
  float2 * const sU = reinterpret_cast<float2 *>(sm + kU);
  float2 * const sG = reinterpret_cast<float2 *>(sm + kG);
  double * const sWJ = reinterpret_cast<double *>(sm + kWJ);
  double * const sFq = reinterpret_cast<double *>(sm + kFq);
  float2 * const sD = reinterpret_cast<float2 *>(sm + kD);
  double * const sX = reinterpret_cast<double *>(sm + kX);
  double * const sOrg = reinterpret_cast<double *>(sm + kOrg);
  double * const sBv = reinterpret_cast<double *>(sm + kBv);
  uint32_t * const sDof = reinterpret_cast<uint32_t *>(sm + kDof);
  int32_t * const sRp = reinterpret_cast<int32_t *>(sm + kRp);
  uint32_t * const sCons = reinterpret_cast<uint32_t *>(sm + kCons);
  int const t = threadIdx.x;

  for (int k = t; k < NQ * N * 3; k += NT)
    tDphi[k] = gDphi[k];
  for (int k = t; k < NQ * N; k += NT)
  {
    tPhi[k] = gPhi[k];
    tPhiD[k] = gPhiD[k];
  }

  LhsDev const & op0 = a.op[0];
  LhsDev const & op1 = a.op[1];
  bool const k0 = op0.on && op0.stiff, k1 = op1.on && op1.stiff;
  bool const m0 = op0.on && op0.mass, m1 = op1.on && op1.mass;
  bool const needK = k0 || k1, needM = m0 || m1;
  bool const kE = usesCoef(op0) || usesCoef(op1);
  bool const foldK = k0 != k1, foldM = m0 != m1;
  bool const anyBcOp = (op0.on && op0.bc) || (op1.on && op1.bc);
  bool const lhs = op0.on || op1.on;

  for (int64_t i0 = blockIdx.x; i0 < a.nelem; i0 += gridDim.x)
  {
    int64_t const e = elemOf(a, i0);
    __syncthreads(); // the previous element's reads of the shared state are done
    // ---- 0. node data
    if (t < N)
    {
      uint32_t const dof = a.emap[e * N + t];
      sDof[t] = dof;
      bool const c = a.bcMask && a.bcMask[dof];
      sBv[t] = (c && a.bcVal) ? a.bcVal[dof] : 0.;
      if (lhs)
        sRp[t] = a.rowPtr[dof];
      uint32_t const cons = __ballot_sync((1u << N) - 1u, c); // the N = 27 lanes of warp 0
      if (t == 0)
        *sCons = cons;
    }
    else if (t >= 32 && t < 32 + 24)
    {
      int const v = (t - 32) / 3, d = (t - 32) % 3;
      sX[3 * v + d] = a.xyz[3 * (int64_t)a.conn[e * 8 + v] + d];
    }
    __syncthreads();
    // ---- 1. edge differences, origin
    if (t < 36)
    {
      int const c = t / 12, k = (t / 3) % 4, d = t % 3;
      st(sD + t, toDfl(sX[3 * kEdges[c][k][1] + d] - sX[3 * kEdges[c][k][0] + d]));
    }
    else if (t >= 64 && t < 67)
    {
      int const d = t - 64;
      sOrg[d] = .125 * (sX[d] + sX[3 + d] + sX[6 + d] + sX[9 + d] + sX[12 + d] + sX[15 + d] + sX[18 + d] +
                        sX[21 + d]);
    }
    __syncthreads();
    uint32_t const cons = *sCons;
    // ---- 2. geometry at Gauss point q = t
    if (t < NQ)
    {
      double const xi[3] = {gXi[3 * t], gXi[3 * t + 1], gXi[3 * t + 2]};
      dfl f[3][2]; // (1 - xi_d) / 2, (1 + xi_d) / 2
#pragma unroll
      for (int d = 0; d < 3; ++d)
      {
        f[d][0] = toDfl(0.5 * (1. - xi[d]));
        f[d][1] = toDfl(0.5 * (1. + xi[d]));
      }
      dfl J[3][3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
      {
        int const o1 = c == 0 ? 1 : 0, o2 = c == 2 ? 1 : 2; // the other two axes, in order
        dfl w[4];
        w[0] = f[o1][0] * f[o2][0];
        w[1] = f[o1][1] * f[o2][0];
        w[2] = f[o1][0] * f[o2][1];
        w[3] = f[o1][1] * f[o2][1];
#pragma unroll
        for (int r = 0; r < 3; ++r)
        {
          dfl const s = dot2(ld(sD + 12 * c + 0 + r), w[0], ld(sD + 12 * c + 3 + r), w[1]) +
                        dot2(ld(sD + 12 * c + 6 + r), w[2], ld(sD + 12 * c + 9 + r), w[3]);
          J[r][c] = dfl{0.5f * s.h, 0.5f * s.l};
        }
      }
      dfl A[3][3];
      A[0][0] = dot2(J[1][1], J[2][2], -J[1][2], J[2][1]);
      A[0][1] = dot2(J[0][2], J[2][1], -J[0][1], J[2][2]);
      A[0][2] = dot2(J[0][1], J[1][2], -J[0][2], J[1][1]);
      A[1][0] = dot2(J[1][2], J[2][0], -J[1][0], J[2][2]);
      A[1][1] = dot2(J[0][0], J[2][2], -J[0][2], J[2][0]);
      A[1][2] = dot2(J[0][2], J[1][0], -J[0][0], J[1][2]);
      A[2][0] = dot2(J[1][0], J[2][1], -J[1][1], J[2][0]);
      A[2][1] = dot2(J[0][1], J[2][0], -J[0][0], J[2][1]);
      A[2][2] = dot2(J[0][0], J[1][1], -J[0][1], J[1][0]);
      dfl const adet = fabs(dot3(J[0][0], A[0][0], J[0][1], A[1][0], J[0][2], A[2][0]));
      dfl const wq = toDfl(gW[t]);
      dfl const wj = wq * adet;
      double const kfac = (kE && a.kE) ? a.kE[e] : 1.0;
      double const ksF = foldK ? (k0 ? (op0.stiff == 2 ? op0.sc * kfac : op0.sc)
                                     : (op1.stiff == 2 ? op1.sc * kfac : op1.sc))
                               : 1.0;
      double const msF = foldM ? massCoef(m0 ? op0 : op1, kfac) : 1.0;
      dfl const s = (toDfl(ksF) * wq) * rcp(adet);
      st(sG + 6 * t + 0, s * dot3(A[0][0], A[0][0], A[0][1], A[0][1], A[0][2], A[0][2]));
      st(sG + 6 * t + 1, s * dot3(A[1][0], A[1][0], A[1][1], A[1][1], A[1][2], A[1][2]));
      st(sG + 6 * t + 2, s * dot3(A[2][0], A[2][0], A[2][1], A[2][1], A[2][2], A[2][2]));
      st(sG + 6 * t + 3, s * dot3(A[0][0], A[1][0], A[0][1], A[1][1], A[0][2], A[1][2]));
      st(sG + 6 * t + 4, s * dot3(A[0][0], A[2][0], A[0][1], A[2][1], A[0][2], A[2][2]));
      st(sG + 6 * t + 5, s * dot3(A[1][0], A[2][0], A[1][1], A[2][1], A[1][2], A[2][2]));
      st(sG + 6 * NQ + t, toDfl(msF) * wj); // the mass weight, after the six G entries of every point
      sWJ[t] = toDouble(wj);
      if (a.b && a.rkind == 1)
      {
        double xq[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
          xq[r] = sOrg[r] + toDouble(dot3(J[r][0], toDfl(xi[0]), J[r][1], toDfl(xi[1]), J[r][2], toDfl(xi[2])));
        sFq[t] = evalFn(a.fn, a.rc, xq[0], xq[1], xq[2]);
      }
      else if (a.b && a.rkind == 2)
      {
        double v = 0.;
        for (int n = 0; n < N; ++n)
          v += tPhiD[t * N + n] * a.field[sDof[n]];
        sFq[t] = a.rc * v;
      }
    }
    __syncthreads();
    // ---- 3. v_j(q) = G_q grad phi_j(q), u_j(q) = (w |det J|)_q phi_j(q); load vector
    if (lhs)
      for (int k = t; k < NQ * N; k += NT)
      {
        int const q = k / N;
        float2 const * g = sG + 6 * q;
        dfl const d0 = ld(tDphi + 3 * k), d1 = ld(tDphi + 3 * k + 1), d2 = ld(tDphi + 3 * k + 2);
        if (needK)
        {
          dfl const G0 = ld(g), G1 = ld(g + 1), G2 = ld(g + 2), G3 = ld(g + 3), G4 = ld(g + 4), G5 = ld(g + 5);
          st(sV + 3 * k + 0, dot3(G0, d0, G3, d1, G4, d2));
          st(sV + 3 * k + 1, dot3(G3, d0, G1, d1, G5, d2));
          st(sV + 3 * k + 2, dot3(G4, d0, G5, d1, G2, d2));
        }
        if (needM)
          st(sU + k, ld(sG + 6 * NQ + q) * ld(tPhi + k));
      }
    if (a.b && a.rkind && t < N && !(a.rbc && ((cons >> t) & 1u)))
    {
      double fe = 0.;
      for (int q = 0; q < NQ; ++q)
        fe += sWJ[q] * tPhiD[q * N + t] * sFq[q];
      atomicAdd(a.b + sDof[t], fe);
    }
    if (a.b && anyBcOp && t < N && ((cons >> t) & 1u) && sBv[t] != 0.)
    {
      // Dirichlet values at the constrained DOFs, once per operator with BCs (buildLhs)
      for (int m = 0; m < 2; ++m)
        if (a.op[m].on && a.op[m].bc)
          atomicAdd(a.b + sDof[t], sBv[t]);
    }
    if (!lhs)
      continue;
    __syncthreads();
    // ---- 4. entries
    uint16_t const * rk = a.rank + e * (int64_t)(N * N);
    double const kd0 = k0 ? (op0.stiff == 2 ? op0.sc * ((kE && a.kE) ? a.kE[e] : 1.0) : op0.sc) : 0.;
    double const kd1 = k1 ? (op1.stiff == 2 ? op1.sc * ((kE && a.kE) ? a.kE[e] : 1.0) : op1.sc) : 0.;
    double const md0 = m0 ? massCoef(op0, (kE && a.kE) ? a.kE[e] : 1.0) : 0.;
    double const md1 = m1 ? massCoef(op1, (kE && a.kE) ? a.kE[e] : 1.0) : 0.;
    for (int p = t; p < NP; p += NT)
    {
      uint16_t const pr = gPairs[p];
      int const i = pr >> 8, j = pr & 0xff;
      dfl kv = dfl{0.f, 0.f}, mv = dfl{0.f, 0.f};
      if (needK)
      {
        Acc acc{0.f, 0.f};
#pragma unroll 3
        for (int q = 0; q < NQ; ++q)
        {
          float2 const * di = tDphi + 3 * (q * N + i);
          float2 const * vj = sV + 3 * (q * N + j);
          mac(acc, ld(di), ld(vj));
          mac(acc, ld(di + 1), ld(vj + 1));
          mac(acc, ld(di + 2), ld(vj + 2));
        }
        kv = dflFastTwoSum(acc.s, acc.c);
      }
      if (needM)
      {
        Acc acc{0.f, 0.f};
#pragma unroll 9
        for (int q = 0; q < NQ; ++q)
          mac(acc, ld(tPhi + q * N + i), ld(sU + q * N + j));
        mv = dflFastTwoSum(acc.s, acc.c);
      }
      int32_t const pij = sRp[i] + rk[i * N + j];
      int32_t const pji = sRp[j] + rk[j * N + i];
      bool const ci = (cons >> i) & 1u, cj = (cons >> j) & 1u;
#pragma unroll
      for (int m = 0; m < 2; ++m)
      {
        LhsDev const & op = a.op[m];
        if (!op.on)
          continue;
        dfl v;
        if (op.stiff)
        {
          v = foldK ? kv : toDfl(m ? kd1 : kd0) * kv;
          if (op.mass)
            v = v + (foldM ? mv : toDfl(m ? md1 : md0) * mv);
        }
        else
          v = foldM ? mv : toDfl(m ? md1 : md0) * mv;
        double const val = toDouble(v);
        if (op.bc && (ci || cj))
        {
          condenseQ2(op.vals + pij, a.bcDiag, a.b, sDof[i], sDof[j], sBv[i], sBv[j], ci, cj, i == j, val);
          continue;
        }
        atomicAdd(op.vals + pij, val);
        if (i != j)
          atomicAdd(op.vals + pji, val);
      }
    }
  }
}
} // namespace q2

pxg_status initQ2Tables(pxg_ctx * c)
{
  using namespace q2;
  std::vector<double> xi, w;
  hostRule(Q2HEX, xi, w);
  if ((int)w.size() != NQ)
    return fail(c, PXG_ERR_UNSUPPORTED, "Q2 rule: %d points", (int)w.size());
  std::vector<double> phi(NQ * N), dphi(NQ * N * 3);
  for (int q = 0; q < NQ; ++q)
    hostShape(Q2HEX, &xi[3 * q], &phi[q * N], &dphi[q * N * 3]);
  auto split = [](double x) {
    float const h = (float)x;
    return make_float2(h, (float)(x - (double)h));
  };
  std::vector<float2> dphiD(dphi.size()), phiD(phi.size());
  for (size_t k = 0; k < dphi.size(); ++k)
    dphiD[k] = split(dphi[k]);
  for (size_t k = 0; k < phi.size(); ++k)
    phiD[k] = split(phi[k]);
  std::vector<uint16_t> pairs;
  for (int i = 0; i < N; ++i)
    for (int j = i; j < N; ++j)
      pairs.push_back((uint16_t)(i << 8 | j));
  PXG_CUDA(c, cudaMemcpyToSymbol(gDphi, dphiD.data(), dphiD.size() * sizeof(float2)));
  PXG_CUDA(c, cudaMemcpyToSymbol(gPhi, phiD.data(), phiD.size() * sizeof(float2)));
  PXG_CUDA(c, cudaMemcpyToSymbol(gPhiD, phi.data(), phi.size() * sizeof(double)));
  PXG_CUDA(c, cudaMemcpyToSymbol(gXi, xi.data(), xi.size() * sizeof(double)));
  PXG_CUDA(c, cudaMemcpyToSymbol(gW, w.data(), w.size() * sizeof(double)));
  PXG_CUDA(c, cudaMemcpyToSymbol(gPairs, pairs.data(), pairs.size() * sizeof(uint16_t)));
  return initQ2F64Tables(c);
}

void launchAssembleQ2(AsmArgs const & a, cudaStream_t s, int sms)
{
  using namespace q2;
  static_assert(kSmem <= 227 * 1024, "shared memory");
  cudaFuncSetAttribute(kAssembleQ2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
  int64_t const blocks = a.nelem < (int64_t)sms * 4 ? a.nelem : (int64_t)sms * 4;
  if (blocks > 0)
    kAssembleQ2<<<(unsigned)blocks, NT, kSmem, s>>>(a);
}

} // namespace pxg
