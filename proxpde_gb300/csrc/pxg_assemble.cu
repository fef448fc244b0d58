// Element kernels of the GB300 assembly engine.
//
// One thread per element computes, in FP64, what proxpde's element loop computes per
// element (include/builder.hpp:53-153): CurFE geometry (include/curfe.hpp:50-103),
// the stiffness / mass matrices (include/assembly_lhs.hpp:52-65, 93-109, 207-221) and
// the load vector (include/assembly_rhs.hpp:61-88, 130-159), applies the Dirichlet
// condensation (builder.hpp:76-124), and adds the result into CSR values and the
// load vector with FP64 reductions (red.global.add.f64) at positions given by the
// per-element scatter map.  The same arithmetic, rearranged:
//   - J^+ = (J^T J)^-1 J^T and sqrt(det(J^T J)) are, for square J, J^-1 and |det J|;
//     they are formed from the adjugate: J^-1 J^-T = adj adj^T / det^2.
//   - Stiffness entries use the symmetric geometric factor G_q = w_q adj adj^T/|det|:
//     K_ij = sum_q dphiRef_i(q)^T G_q dphiRef_j(q); only j >= i is computed and both
//     (i,j) and (j,i) are written.
//   - On tetrahedra (affine map) G is constant and K_ij = sum_ab G_ab T_ab(ij) with
//     the reference tensors T_ab(ij) = sum_q w_q dphiRef_ia(q) dphiRef_jb(q), which
//     are computed once from the same quadrature rule.
// Round-off differs from the reference's Eigen evaluation order; values agree to
// ~1e-15 relative.
#include <cub/cub.cuh>

#include <cmath>
#include <type_traits>
#include <vector>

#include "pxg_dfl.h"
#include "pxg_internal.h"

namespace pxg
{

// ------------------------------------------------------------ constant tables
__constant__ double cP1phi[4 * 4], cP1dphi[4 * 3], cP1w[4], cP1xi[4 * 3], cP1T[6 * 16], cP1M[16];
__constant__ double cP2phi[11 * 10], cP2dphi[11 * 10 * 3], cP2w[11], cP2xi[11 * 3], cP2T[6 * 100],
    cP2M[100];
__constant__ double cQ1phi[8 * 8], cQ1dphi[8 * 8 * 3], cQ1w[8], cQ1xi[8 * 3];
__constant__ double cQ2phi[27 * 27], cQ2dphi[27 * 27 * 3], cQ2w[27], cQ2xi[27 * 3];
// the affine elements' reference tensors as hi/lo float pairs (kAssembleTet)
__constant__ float2 cP1Td[6 * 16], cP1Md[16], cP2Td[6 * 100], cP2Md[100];
__constant__ double cP1I[4], cP2I[10]; // sum_q w_q phi_i(q): the load vector of f = 1
__constant__ double cP1Ws;             // sum_q w_q of the Tet4 rule (the reference volume)

template <int T>
__device__ __forceinline__ double PHI(int q, int i)
{
  if constexpr (T == P1TET)
    return cP1phi[q * 4 + i];
  else if constexpr (T == P2TET)
    return cP2phi[q * 10 + i];
  else if constexpr (T == Q1HEX)
    return cQ1phi[q * 8 + i];
  else
    return cQ2phi[q * 27 + i];
}
template <int T>
__device__ __forceinline__ double DPHI(int q, int i, int d)
{
  if constexpr (T == P1TET)
    return cP1dphi[i * 3 + d];
  else if constexpr (T == P2TET)
    return cP2dphi[(q * 10 + i) * 3 + d];
  else if constexpr (T == Q1HEX)
    return cQ1dphi[(q * 8 + i) * 3 + d];
  else
    return cQ2dphi[(q * 27 + i) * 3 + d];
}
template <int T>
__device__ __forceinline__ double WQ(int q)
{
  if constexpr (T == P1TET)
    return cP1w[q];
  else if constexpr (T == P2TET)
    return cP2w[q];
  else if constexpr (T == Q1HEX)
    return cQ1w[q];
  else
    return cQ2w[q];
}
template <int T>
__device__ __forceinline__ double XI(int q, int d)
{
  if constexpr (T == P1TET)
    return cP1xi[q * 3 + d];
  else if constexpr (T == P2TET)
    return cP2xi[q * 3 + d];
  else if constexpr (T == Q1HEX)
    return cQ1xi[q * 3 + d];
  else
    return cQ2xi[q * 3 + d];
}
template <int T>
__device__ __forceinline__ double TT(int c, int i, int j)
{
  if constexpr (T == P1TET)
    return cP1T[(c * 4 + i) * 4 + j];
  else
    return cP2T[(c * 10 + i) * 10 + j];
}
template <int T>
__device__ __forceinline__ double MHAT(int i, int j)
{
  if constexpr (T == P1TET)
    return cP1M[i * 4 + j];
  else
    return cP2M[i * 10 + j];
}

// ------------------------------------------------- host reference elements
// Quadrature rules and shape functions of proxpde (src/qr.cpp:27, 38, 199-320;
// src/reffe.cpp:246-253, 374-383, 510-1003), restated for the engine's tables.
namespace
{
constexpr double kSqrt13rd = 0.5773502691896258; // src/qr.cpp:27
constexpr double kSqrt35th = 0.774596669241483;  // src/qr.cpp:38

void ruleHost(int t, std::vector<double> & xi, std::vector<double> & w)
{
  xi.clear();
  w.clear();
  if (t == P1TET)
  {
    double const a = 0.1381966011250105, b = 0.5854101966249685;
    xi = {a, a, a, b, a, a, a, b, a, a, a, b};
    w.assign(4, .25 / 6);
  }
  else if (t == P2TET)
  {
    double const c1 = 0.0714285714285714, c2 = 0.7857142857142857;
    double const d1 = 0.399403576166799, d2 = 0.100596423833201;
    xi = {0.25, 0.25, 0.25, c1, c1, c1, c2, c1, c1, c1, c2, c1, c1, c1, c2, d1, d1,
          d2,   d1,   d2,   d1, d2, d1, d1, d1, d2, d2, d2, d1, d2, d2, d2, d1};
    double const w0 = -0.0131555555555556, w1 = 0.0076222222222222, w2 = 0.024888888888889;
    w = {w0, w1, w1, w1, w1, w2, w2, w2, w2, w2, w2};
  }
  else if (t == Q1HEX)
  {
    for (int k = 0; k < 2; ++k)
      for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i)
        {
          xi.push_back(i ? kSqrt13rd : -kSqrt13rd);
          xi.push_back(j ? kSqrt13rd : -kSqrt13rd);
          xi.push_back(k ? kSqrt13rd : -kSqrt13rd);
          w.push_back(1.0);
        }
  }
  else
  {
    double const x[3] = {-kSqrt35th, 0.0, kSqrt35th};
    double const w1[3] = {5., 8., 5.};
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i)
        {
          xi.push_back(x[i]);
          xi.push_back(x[j]);
          xi.push_back(x[k]);
          w.push_back((w1[i] * w1[j] * w1[k]) / 729.);
        }
  }
}

double f1(int a, double x) { return a == 0 ? 0.5 * (1. - x) : 0.5 * (1. + x); }
double g1(int a, double) { return a == 0 ? -0.5 : 0.5; }
double f2(int a, double x) { return a == 0 ? 0.5 * x * (x - 1.) : (a == 1 ? 0.5 * x * (x + 1.) : 1. - x * x); }
double g2(int a, double x) { return a == 0 ? x - 0.5 : (a == 1 ? x + 0.5 : -2. * x); }

// 1D factor index per axis for Q1/Q2 nodes (src/reffe.cpp:684-1003 ordering)
constexpr int kQ1idx[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                              {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
constexpr int kQ2idx[27][3] = {
    {0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1},
    {0, 1, 1}, {2, 0, 0}, {1, 2, 0}, {2, 1, 0}, {0, 2, 0}, {0, 0, 2}, {1, 0, 2},
    {1, 1, 2}, {0, 1, 2}, {2, 0, 1}, {1, 2, 1}, {2, 1, 1}, {0, 2, 1}, {2, 2, 0},
    {0, 2, 2}, {2, 0, 2}, {1, 2, 2}, {2, 1, 2}, {2, 2, 1}, {2, 2, 2}};

void shapeHost(int t, double const * p, double * phi, double * dphi)
{
  double const x = p[0], y = p[1], z = p[2];
  if (t == P1TET || t == P2TET)
  {
    double const l[4] = {1. - x - y - z, x, y, z};
    double const dl[4][3] = {{-1., -1., -1.}, {1., 0., 0.}, {0., 1., 0.}, {0., 0., 1.}};
    if (t == P1TET)
    {
      for (int i = 0; i < 4; ++i)
      {
        phi[i] = l[i];
        for (int d = 0; d < 3; ++d)
          dphi[3 * i + d] = dl[i][d];
      }
      return;
    }
    for (int i = 0; i < 4; ++i)
    {
      phi[i] = l[i] * (2. * l[i] - 1.);
      for (int d = 0; d < 3; ++d)
        dphi[3 * i + d] = (4. * l[i] - 1.) * dl[i][d];
    }
    for (int e = 0; e < 6; ++e)
    {
      int const a = tetEdgeV(e, 0), b = tetEdgeV(e, 1);
      phi[4 + e] = 4. * l[a] * l[b];
      for (int d = 0; d < 3; ++d)
        dphi[3 * (4 + e) + d] = 4. * (l[a] * dl[b][d] + dl[a][d] * l[b]);
    }
    return;
  }
  int const n = (t == Q1HEX) ? 8 : 27;
  for (int i = 0; i < n; ++i)
  {
    int const * ix = (t == Q1HEX) ? kQ1idx[i] : kQ2idx[i];
    double fx, fy, fz, gx, gy, gz;
    if (t == Q1HEX)
    {
      fx = f1(ix[0], x), fy = f1(ix[1], y), fz = f1(ix[2], z);
      gx = g1(ix[0], x), gy = g1(ix[1], y), gz = g1(ix[2], z);
    }
    else
    {
      fx = f2(ix[0], x), fy = f2(ix[1], y), fz = f2(ix[2], z);
      gx = g2(ix[0], x), gy = g2(ix[1], y), gz = g2(ix[2], z);
    }
    phi[i] = fx * fy * fz;
    dphi[3 * i + 0] = gx * fy * fz;
    dphi[3 * i + 1] = fx * gy * fz;
    dphi[3 * i + 2] = fx * fy * gz;
  }
}

int gTablesDone[64] = {0};
} // namespace

// the host restatements, for the tables of other translation units
void hostRule(int t, std::vector<double> & xi, std::vector<double> & w) { ruleHost(t, xi, w); }
void hostShape(int t, double const * p, double * phi, double * dphi) { shapeHost(t, p, phi, dphi); }

pxg_status initTables(pxg_ctx * c)
{
  if (c->device >= 0 && c->device < 64 && gTablesDone[c->device])
    return PXG_OK;
  for (int t = 0; t < 4; ++t)
  {
    std::vector<double> xi, w;
    ruleHost(t, xi, w);
    int const nq = (int)w.size(), N = numDofs(t);
    std::vector<double> phi(nq * N), dphi(nq * N * 3);
    for (int q = 0; q < nq; ++q)
      shapeHost(t, &xi[3 * q], &phi[q * N], &dphi[q * N * 3]);
    if (t == P1TET || t == P2TET)
    {
      // reference tensors of the affine elements
      std::vector<double> T(6 * N * N, 0.), M(N * N, 0.);
      int const pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
      for (int q = 0; q < nq; ++q)
        for (int i = 0; i < N; ++i)
          for (int j = 0; j < N; ++j)
          {
            double const * di = &dphi[(q * N + i) * 3];
            double const * dj = &dphi[(q * N + j) * 3];
            for (int k = 0; k < 6; ++k)
            {
              double v = w[q] * di[pa[k]] * dj[pb[k]];
              if (k >= 3)
                v += w[q] * di[pb[k]] * dj[pa[k]];
              T[(k * N + i) * N + j] += v;
            }
            M[i * N + j] += w[q] * phi[q * N + i] * phi[q * N + j];
          }
      // the same as hi/lo float pairs, and sum_q w_q phi_i(q), for kAssembleTet
      std::vector<float2> Td(T.size()), Md(M.size());
      auto split = [](double x) { float const h = (float)x; return make_float2(h, (float)(x - (double)h)); };
      for (size_t k = 0; k < T.size(); ++k)
        Td[k] = split(T[k]);
      for (size_t k = 0; k < M.size(); ++k)
        Md[k] = split(M[k]);
      std::vector<double> I(N, 0.);
      for (int q = 0; q < nq; ++q)
        for (int i = 0; i < N; ++i)
          I[i] += w[q] * phi[q * N + i];
      if (t == P1TET)
      {
        PXG_CUDA(c, cudaMemcpyToSymbol(cP1Td, Td.data(), Td.size() * sizeof(float2)));
        PXG_CUDA(c, cudaMemcpyToSymbol(cP1Md, Md.data(), Md.size() * sizeof(float2)));
        PXG_CUDA(c, cudaMemcpyToSymbol(cP1I, I.data(), I.size() * 8));
        double ws = 0.;
        for (int q = 0; q < nq; ++q)
          ws += w[q];
        PXG_CUDA(c, cudaMemcpyToSymbol(cP1Ws, &ws, 8));
      }
      else
      {
        PXG_CUDA(c, cudaMemcpyToSymbol(cP2Td, Td.data(), Td.size() * sizeof(float2)));
        PXG_CUDA(c, cudaMemcpyToSymbol(cP2Md, Md.data(), Md.size() * sizeof(float2)));
        PXG_CUDA(c, cudaMemcpyToSymbol(cP2I, I.data(), I.size() * 8));
      }
      if (t == P1TET)
      {
        std::vector<double> d1(4 * 3);
        for (int i = 0; i < 12; ++i)
          d1[i] = dphi[i]; // constant gradients (q = 0)
        PXG_CUDA(c, cudaMemcpyToSymbol(cP1phi, phi.data(), phi.size() * 8));
        PXG_CUDA(c, cudaMemcpyToSymbol(cP1dphi, d1.data(), d1.size() * 8));
        PXG_CUDA(c, cudaMemcpyToSymbol(cP1w, w.data(), w.size() * 8));
        PXG_CUDA(c, cudaMemcpyToSymbol(cP1xi, xi.data(), xi.size() * 8));
        PXG_CUDA(c, cudaMemcpyToSymbol(cP1T, T.data(), T.size() * 8));
        PXG_CUDA(c, cudaMemcpyToSymbol(cP1M, M.data(), M.size() * 8));
      }
      else
      {
        PXG_CUDA(c, cudaMemcpyToSymbol(cP2phi, phi.data(), phi.size() * 8));
        PXG_CUDA(c, cudaMemcpyToSymbol(cP2dphi, dphi.data(), dphi.size() * 8));
        PXG_CUDA(c, cudaMemcpyToSymbol(cP2w, w.data(), w.size() * 8));
        PXG_CUDA(c, cudaMemcpyToSymbol(cP2xi, xi.data(), xi.size() * 8));
        PXG_CUDA(c, cudaMemcpyToSymbol(cP2T, T.data(), T.size() * 8));
        PXG_CUDA(c, cudaMemcpyToSymbol(cP2M, M.data(), M.size() * 8));
      }
    }
    else if (t == Q1HEX)
    {
      PXG_CUDA(c, cudaMemcpyToSymbol(cQ1phi, phi.data(), phi.size() * 8));
      PXG_CUDA(c, cudaMemcpyToSymbol(cQ1dphi, dphi.data(), dphi.size() * 8));
      PXG_CUDA(c, cudaMemcpyToSymbol(cQ1w, w.data(), w.size() * 8));
      PXG_CUDA(c, cudaMemcpyToSymbol(cQ1xi, xi.data(), xi.size() * 8));
    }
    else
    {
      PXG_CUDA(c, cudaMemcpyToSymbol(cQ2phi, phi.data(), phi.size() * 8));
      PXG_CUDA(c, cudaMemcpyToSymbol(cQ2dphi, dphi.data(), dphi.size() * 8));
      PXG_CUDA(c, cudaMemcpyToSymbol(cQ2w, w.data(), w.size() * 8));
      PXG_CUDA(c, cudaMemcpyToSymbol(cQ2xi, xi.data(), xi.size() * 8));
    }
  }
  pxg_status const q2 = initQ2Tables(c);
  if (q2 != PXG_OK)
    return q2;
  if (c->device >= 0 && c->device < 64)
    gTablesDone[c->device] = 1;
  return PXG_OK;
}

// ------------------------------------------------------------------ kernels
// adjugate and determinant of a 3x3 matrix
__device__ __forceinline__ double adj3(double const (&J)[3][3], double (&A)[3][3])
{
  A[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  A[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
  A[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
  A[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  A[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
  A[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
  A[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  A[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
  A[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
  return J[0][0] * A[0][0] + J[0][1] * A[1][0] + J[0][2] * A[2][0];
}

// G = s * A A^T (symmetric, packed 00 11 22 01 02 12)
__device__ __forceinline__ void gram(double const (&A)[3][3], double s, double * G)
{
  G[0] = s * (A[0][0] * A[0][0] + A[0][1] * A[0][1] + A[0][2] * A[0][2]);
  G[1] = s * (A[1][0] * A[1][0] + A[1][1] * A[1][1] + A[1][2] * A[1][2]);
  G[2] = s * (A[2][0] * A[2][0] + A[2][1] * A[2][1] + A[2][2] * A[2][2]);
  G[3] = s * (A[0][0] * A[1][0] + A[0][1] * A[1][1] + A[0][2] * A[1][2]);
  G[4] = s * (A[0][0] * A[2][0] + A[0][1] * A[2][1] + A[0][2] * A[2][2]);
  G[5] = s * (A[1][0] * A[2][0] + A[1][1] * A[2][1] + A[1][2] * A[2][2]);
}

__device__ __forceinline__ void red(double * p, double v) { atomicAdd(p, v); }

template <int T, int NT>
__global__ void __launch_bounds__(NT) kAssemble(AsmArgs a)
{
  constexpr int NV = Elem<T>::NV, N = Elem<T>::N, NQ = Elem<T>::NQ;
  constexpr bool HEX = Elem<T>::hex;
  int64_t const i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i0 >= a.nelem)
    return;
  int64_t const e = elemOf(a, i0);

  double X[NV][3];
#pragma unroll
  for (int v = 0; v < NV; ++v)
  {
    uint32_t const id = a.conn[e * NV + v];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      X[v][d] = a.xyz[3 * (int64_t)id + d];
  }
  uint32_t dof[N];
#pragma unroll
  for (int i = 0; i < N; ++i)
    dof[i] = a.emap[e * N + i];
  uint32_t cons = 0;
  if (a.bcMask)
  {
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (a.bcMask[dof[i]])
        cons |= 1u << i;
  }
  double const kfac = a.kE ? a.kE[e] : 1.0;
  bool const needK = (a.op[0].on && a.op[0].stiff) || (a.op[1].on && a.op[1].stiff);
  bool const needM = (a.op[0].on && a.op[0].mass) || (a.op[1].on && a.op[1].mass);

  // --- geometry (CurFE::reinit)
  double G[HEX ? NQ : 1][6];
  double jxw[NQ];
  double fq[NQ];
  double adet = 0.;
  if constexpr (!HEX)
  {
    double J[3][3], A[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int cc = 0; cc < 3; ++cc)
        J[r][cc] = X[cc + 1][r] - X[0][r];
    double const det = adj3(J, A);
    adet = fabs(det);
    gram(A, 1.0 / adet, G[0]);
#pragma unroll
    for (int q = 0; q < NQ; ++q)
      jxw[q] = adet * WQ<T>(q);
    if (a.rkind == 1)
    {
#pragma unroll
      for (int q = 0; q < NQ; ++q)
      {
        double xq[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
          xq[r] = X[0][r] + (J[r][0] * XI<T>(q, 0) + J[r][1] * XI<T>(q, 1) + J[r][2] * XI<T>(q, 2));
        fq[q] = evalFn(a.fn, a.rc, xq[0], xq[1], xq[2]);
      }
    }
  }
  else
  {
    double P[N][3];
    mappingPoints<T>(X, P);
    double o[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      o[d] = .125 * (X[0][d] + X[1][d] + X[2][d] + X[3][d] + X[4][d] + X[5][d] + X[6][d] + X[7][d]);
#pragma unroll
    for (int q = 0; q < NQ; ++q)
    {
      double J[3][3] = {{0., 0., 0.}, {0., 0., 0.}, {0., 0., 0.}}, A[3][3];
#pragma unroll
      for (int n = 0; n < N; ++n)
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int cc = 0; cc < 3; ++cc)
            J[r][cc] += P[n][r] * DPHI<T>(q, n, cc);
      double const det = adj3(J, A);
      double const ad = fabs(det);
      gram(A, WQ<T>(q) / ad, G[q]);
      jxw[q] = WQ<T>(q) * ad;
      if (a.rkind == 1)
      {
        double xq[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
          xq[r] = o[r] + (J[r][0] * XI<T>(q, 0) + J[r][1] * XI<T>(q, 1) + J[r][2] * XI<T>(q, 2));
        fq[q] = evalFn(a.fn, a.rc, xq[0], xq[1], xq[2]);
      }
    }
  }
  if (a.rkind == 3)
  {
    // values of f at the quadrature points, evaluated by the caller (pxg_get_qpoints)
#pragma unroll
    for (int q = 0; q < NQ; ++q)
      fq[q] = a.rc * a.field[e * NQ + q];
  }
  if (a.rkind == 2)
  {
    double loc[N];
#pragma unroll
    for (int n = 0; n < N; ++n)
      loc[n] = a.field[dof[n]];
#pragma unroll
    for (int q = 0; q < NQ; ++q)
    {
      double s = 0.;
#pragma unroll
      for (int n = 0; n < N; ++n)
        s += PHI<T>(q, n) * loc[n];
      fq[q] = a.rc * s;
    }
  }

  // --- local matrices row by row, scattered as they are produced
  bool const anyBc = cons && ((a.op[0].on && a.op[0].bc) || (a.op[1].on && a.op[1].bc));
  double lift[2][N];
  if (anyBc)
  {
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
      for (int i = 0; i < N; ++i)
        lift[m][i] = 0.;
  }
  int64_t const NN = (int64_t)N * N;
  uint16_t const * rk = a.rank + e * NN;
#pragma unroll 1
  for (int i = 0; i < N; ++i)
  {
    int32_t const rpi = a.rowPtr[dof[i]];
    double v[HEX ? NQ : 1][3];
    if constexpr (HEX)
    {
      if (needK)
      {
#pragma unroll
        for (int q = 0; q < NQ; ++q)
        {
          double const d0 = DPHI<T>(q, i, 0), d1 = DPHI<T>(q, i, 1), d2 = DPHI<T>(q, i, 2);
          v[q][0] = G[q][0] * d0 + G[q][3] * d1 + G[q][4] * d2;
          v[q][1] = G[q][3] * d0 + G[q][1] * d1 + G[q][5] * d2;
          v[q][2] = G[q][4] * d0 + G[q][5] * d1 + G[q][2] * d2;
        }
      }
    }
#pragma unroll 1
    for (int j = i; j < N; ++j)
    {
      double kv = 0., mv = 0.;
      if constexpr (HEX)
      {
        if (needK)
        {
#pragma unroll
          for (int q = 0; q < NQ; ++q)
            kv += v[q][0] * DPHI<T>(q, j, 0) + v[q][1] * DPHI<T>(q, j, 1) + v[q][2] * DPHI<T>(q, j, 2);
        }
        if (needM)
        {
#pragma unroll
          for (int q = 0; q < NQ; ++q)
            mv += jxw[q] * (PHI<T>(q, i) * PHI<T>(q, j));
        }
      }
      else
      {
        if (needK)
        {
#pragma unroll
          for (int k = 0; k < 6; ++k)
            kv += G[0][k] * TT<T>(k, i, j);
        }
        if (needM)
          mv = adet * MHAT<T>(i, j);
      }
      int32_t const pij = rpi + rk[i * N + j];
      int32_t const pji = a.rowPtr[dof[j]] + rk[j * N + i];
#pragma unroll
      for (int m = 0; m < 2; ++m)
      {
        LhsDev const & op = a.op[m];
        if (!op.on)
          continue;
        double val = 0.;
        if (op.stiff)
          val += (op.stiff == 2 ? op.sc * kfac : op.sc) * kv;
        if (op.mass)
          val += massCoef(op, kfac) * mv;
        if (op.bc && cons)
        {
          bool const ci = (cons >> i) & 1u, cj = (cons >> j) & 1u;
          if (ci || cj)
          {
            if (i == j)
              red(op.vals + pij, a.bcDiag);
            else
            {
              if (!ci)
                lift[m][i] -= val * a.bcVal[dof[j]];
              if (!cj)
                lift[m][j] -= val * a.bcVal[dof[i]];
            }
            continue;
          }
        }
        red(op.vals + pij, val);
        if (j != i)
          red(op.vals + pji, val);
      }
    }
  }
  if (a.b)
  {
    // BC lifts of the lhs ops (buildLhs: b += C(-Ke h), and h at constrained DOFs)
    if (anyBc)
    {
#pragma unroll
      for (int m = 0; m < 2; ++m)
      {
        if (!a.op[m].on || !a.op[m].bc)
          continue;
#pragma unroll 1
        for (int i = 0; i < N; ++i)
        {
          double const add = ((cons >> i) & 1u) ? a.bcVal[dof[i]] : lift[m][i];
          if (add != 0.)
            red(a.b + dof[i], add);
        }
      }
    }
    // load vector (buildRhs: b += C Fe)
    if (a.rkind)
    {
#pragma unroll 1
      for (int i = 0; i < N; ++i)
      {
        if (a.rbc && ((cons >> i) & 1u))
          continue;
        double fe = 0.;
#pragma unroll
        for (int q = 0; q < NQ; ++q)
          fe += jxw[q] * PHI<T>(q, i) * fq[q];
        red(a.b + dof[i], fe);
      }
    }
  }
}

// ------------------------------------------- tetrahedra in double-float arithmetic
// kAssembleTet: the P1/P2 element loop of kAssemble with the geometry and the entries
// on the FP32 pipes (double-float, pxg_dfl.h).  At 1/64 of the FP32 rate, the FP64
// pipe bounds the FP64 form of this loop (ncu, P2 32^3: FP64 pipe 82 % busy, issue
// 12 %).  Per element: J from the vertex differences (FP64 subtractions, exact
// conversions), adj(J), |det J| and G = adj adj^T / |det J| in double-float; an entry
// is the six-term product of G with the reference tensor (its hi/lo float pairs in
// constant memory, errors gathered in one float), the mass entry |det J| Mhat_ij.  A
// single stiffness (mass) operator's coefficient is folded into G (|det J|) once per
// element.  The values are converted to double with one FP64 addition each; BC
// condensation and the load vector follow kAssemble in FP64.

template <int T>
__device__ __forceinline__ dfl TTd(int c, int i, int j)
{
  float2 const v = T == P1TET ? cP1Td[(c * 4 + i) * 4 + j] : cP2Td[(c * 10 + i) * 10 + j];
  return dfl{v.x, v.y};
}
template <int T>
__device__ __forceinline__ dfl MHATd(int i, int j)
{
  float2 const v = T == P1TET ? cP1Md[i * 4 + j] : cP2Md[i * 10 + j];
  return dfl{v.x, v.y};
}
template <int T>
__device__ __forceinline__ double PINT(int i)
{
  return T == P1TET ? cP1I[i] : cP2I[i];
}

// sum_k g_k t_k over six double-float pairs: exact high products (FMA TwoProd), their
// sum by TwoSum, every term of order 2^-24 gathered in one float, one renormalisation
__device__ __forceinline__ dfl dot6(dfl const (&g)[6], dfl const (&t)[6])
{
  float p[6], lo = 0.f;
#pragma unroll
  for (int k = 0; k < 6; ++k)
  {
    p[k] = __fmul_rn(g[k].h, t[k].h);
    float e = __fmaf_rn(g[k].h, t[k].h, -p[k]);
    e = __fmaf_rn(g[k].h, t[k].l, e);
    e = __fmaf_rn(g[k].l, t[k].h, e);
    lo = __fadd_rn(lo, e);
  }
  float s = p[0];
#pragma unroll
  for (int k = 1; k < 6; ++k)
  {
    dfl const r = dflTwoSum(s, p[k]);
    s = r.h;
    lo = __fadd_rn(lo, r.l);
  }
  return dflFastTwoSum(s, lo);
}

// v[i] for a run-time i by a chain of selects: v stays in registers
template <typename V, int N>
__device__ __forceinline__ V pickN(V const (&v)[N], int i)
{
  V r = v[0];
#pragma unroll
  for (int n = 1; n < N; ++n)
    r = i == n ? v[n] : r;
  return r;
}

// Dirichlet condensation of one entry (builder.hpp:76-124): a constrained diagonal
// takes bcDiag, a free row the lift -K_ij h_j, added to b at once.  Out of line: its
// FP64 code would otherwise be predicated into every entry.
__device__ __noinline__ void condenseTet(double * diag, double bcDiag, double * b, uint32_t dofi, uint32_t dofj,
                                         double const * bcVal, bool ci, bool cj, bool isDiag, double val)
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
    double const t = val * bcVal[dofj];
    if (t != 0.)
      atomicAdd(b + dofi, -t);
  }
  if (!cj)
  {
    double const t = val * bcVal[dofi];
    if (t != 0.)
      atomicAdd(b + dofj, -t);
  }
}

template <int T, int NT>
__global__ void __launch_bounds__(NT) kAssembleTet(AsmArgs a)
{
  constexpr int N = Elem<T>::N, NQ = Elem<T>::NQ;
  int64_t const i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i0 >= a.nelem)
    return;
  int64_t const e = elemOf(a, i0);

  double X[4][3];
#pragma unroll
  for (int v = 0; v < 4; ++v)
  {
    uint32_t const id = a.conn[e * 4 + v];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      X[v][d] = a.xyz[3 * (int64_t)id + d];
  }
  uint32_t dof[N];
#pragma unroll
  for (int i = 0; i < N; ++i)
    dof[i] = a.emap[e * N + i];
  uint32_t cons = 0;
  if (a.bcMask)
  {
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (a.bcMask[dof[i]])
        cons |= 1u << i;
  }
  LhsDev const & op0 = a.op[0];
  LhsDev const & op1 = a.op[1];
  bool const k0 = op0.on && op0.stiff, k1 = op1.on && op1.stiff;
  bool const m0 = op0.on && op0.mass, m1 = op1.on && op1.mass;
  bool const needK = k0 || k1, needM = m0 || m1;
  bool const kE = usesCoef(op0) || usesCoef(op1);
  double const kfac = (kE && a.kE) ? a.kE[e] : 1.0;

  // --- geometry in double-float: J columns = vertex differences
  dfl J[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int cc = 0; cc < 3; ++cc)
      J[r][cc] = toDfl(X[cc + 1][r] - X[0][r]);
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
  dfl const det = dot3(J[0][0], A[0][0], J[0][1], A[1][0], J[0][2], A[2][0]);
  dfl const adet = fabs(det);
  // operator coefficients: a single stiffness (mass) operator's is folded into G (|det J|)
  bool const foldK = k0 != k1, foldM = m0 != m1;
  double const ks0 = k0 ? (op0.stiff == 2 ? op0.sc * kfac : op0.sc) : 0.;
  double const ks1 = k1 ? (op1.stiff == 2 ? op1.sc * kfac : op1.sc) : 0.;
  double const ms0 = m0 ? massCoef(op0, kfac) : 0., ms1 = m1 ? massCoef(op1, kfac) : 0.;
  dfl G[6];
  {
    dfl const s = fromDouble<dfl>(foldK ? (k0 ? ks0 : ks1) : 1.0) * rcp(adet);
    G[0] = s * dot3(A[0][0], A[0][0], A[0][1], A[0][1], A[0][2], A[0][2]);
    G[1] = s * dot3(A[1][0], A[1][0], A[1][1], A[1][1], A[1][2], A[1][2]);
    G[2] = s * dot3(A[2][0], A[2][0], A[2][1], A[2][1], A[2][2], A[2][2]);
    G[3] = s * dot3(A[0][0], A[1][0], A[0][1], A[1][1], A[0][2], A[1][2]);
    G[4] = s * dot3(A[0][0], A[2][0], A[0][1], A[2][1], A[0][2], A[2][2]);
    G[5] = s * dot3(A[1][0], A[2][0], A[1][1], A[2][1], A[1][2], A[2][2]);
  }
  dfl const am = foldM ? fromDouble<dfl>(m0 ? ms0 : ms1) * adet : adet;
  dfl const kd0 = fromDouble<dfl>(ks0), kd1 = fromDouble<dfl>(ks1);
  dfl const md0 = fromDouble<dfl>(ms0), md1 = fromDouble<dfl>(ms1);

  // --- entries.  The element's DOFs and row pointers are read with select chains
  // (pickN): a run-time index into a register array moves it to local memory, and every
  // entry then waited on a local load and on the dependent rowPtr load.  P1's ten
  // entries are unrolled.
  int32_t rpn[N];
#pragma unroll
  for (int n = 0; n < N; ++n)
    rpn[n] = a.rowPtr[dof[n]];
  bool const anyBc = cons && ((op0.on && op0.bc) || (op1.on && op1.bc));
  uint16_t const * rk = a.rank + e * (int64_t)(N * N);
  constexpr int kRowUnroll = N <= 4 ? N : 1; // P1: the 10 entries fully unrolled
  // P1 with the usual operator pair, a stiffness-only operator and then a mass-only one
  // (both coefficients folded above), in a warp none of whose elements has a Dirichlet
  // node under an operator with BCs: a loop without the per-entry operator branches
  // (96^3 x 6: 0.78 -> 0.75 ms; for P2 the same loop measured 2 % slower, so P2 keeps
  // the general one).  The vote runs over the active lanes: the last block's spare
  // threads have returned.
  bool fastDone = false;
  bool const kmPair = op0.on && op0.stiff && !op0.mass && op1.on && !op1.stiff && op1.mass;
  if constexpr (T == P1TET)
    fastDone = kmPair && !__any_sync(__activemask(), anyBc);
  if (fastDone)
  {
#pragma unroll kRowUnroll
    for (int i = 0; i < N; ++i)
    {
      int32_t const rpi = pickN(rpn, i);
#pragma unroll 1
      for (int j = i; j < N; ++j)
      {
        dfl t[6];
#pragma unroll
        for (int k = 0; k < 6; ++k)
          t[k] = TTd<T>(k, i, j);
        double const valK = toDouble(dot6(G, t));
        double const valM = toDouble(am * MHATd<T>(i, j));
        int32_t const pij = rpi + rk[i * N + j];
        red(op0.vals + pij, valK);
        red(op1.vals + pij, valM);
        if (j != i)
        {
          int32_t const pji = pickN(rpn, j) + rk[j * N + i];
          red(op0.vals + pji, valK);
          red(op1.vals + pji, valM);
        }
      }
    }
  }
  else
  {
#pragma unroll kRowUnroll
    for (int i = 0; i < N; ++i)
    {
      uint32_t const dofi = pickN(dof, i);
      int32_t const rpi = pickN(rpn, i);
      bool const ci = (cons >> i) & 1u;
#pragma unroll 1
      for (int j = i; j < N; ++j)
      {
        dfl kv = dfl{0.f, 0.f}, mv = dfl{0.f, 0.f};
        if (needK)
        {
          dfl t[6];
#pragma unroll
          for (int k = 0; k < 6; ++k)
            t[k] = TTd<T>(k, i, j);
          kv = dot6(G, t);
        }
        if (needM)
          mv = am * MHATd<T>(i, j);
        int32_t const pij = rpi + rk[i * N + j];
        int32_t const pji = pickN(rpn, j) + rk[j * N + i];
        bool const cj = (cons >> j) & 1u;
#pragma unroll
        for (int m = 0; m < 2; ++m)
        {
          LhsDev const & op = a.op[m];
          if (!op.on)
            continue;
          dfl v;
          if (op.stiff)
          {
            v = foldK ? kv : (m ? kd1 : kd0) * kv;
            if (op.mass)
              v = v + (foldM ? mv : (m ? md1 : md0) * mv);
          }
          else
            v = foldM ? mv : (m ? md1 : md0) * mv;
          double const val = toDouble(v);
          if (anyBc && op.bc && (ci || cj))
          {
            condenseTet(op.vals + pij, a.bcDiag, a.b, dofi, pickN(dof, j), a.bcVal, ci, cj, i == j, val);
            continue;
          }
          red(op.vals + pij, val);
          if (j != i)
            red(op.vals + pji, val);
        }
      }
    }
  }
  if (!a.b)
    return;
  // Dirichlet values at the constrained DOFs, once per operator with BCs (buildLhs)
  if (anyBc)
  {
#pragma unroll
    for (int m = 0; m < 2; ++m)
    {
      if (!a.op[m].on || !a.op[m].bc)
        continue;
#pragma unroll
      for (int n = 0; n < N; ++n)
        if ((cons >> n) & 1u)
        {
          double const h = a.bcVal[dof[n]];
          if (h != 0.)
            red(a.b + dof[n], h);
        }
    }
  }
  if (!a.rkind)
    return;
  // load vector (buildRhs: b += C Fe), in FP64
  double const adetD = toDouble(adet);
  if (a.rkind == 1 && a.fn == PXG_FN_CONST)
  {
    // f = c: Fe_i = c |det J| sum_q w_q phi_i(q)
    double const f = evalFn(a.fn, a.rc, 0., 0., 0.) * adetD;
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (!(a.rbc && ((cons >> i) & 1u)))
        red(a.b + dof[i], f * PINT<T>(i));
    return;
  }
  double fq[NQ];
  if (a.rkind == 1)
  {
    // the vertices again (cache hits): keeping them in registers through the entry
    // loop cost 24 registers per thread
#pragma unroll
    for (int v = 0; v < 4; ++v)
    {
      uint32_t const id = a.conn[e * 4 + v];
#pragma unroll
      for (int d = 0; d < 3; ++d)
        X[v][d] = a.xyz[3 * (int64_t)id + d];
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q)
    {
      double xq[3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
        xq[r] = X[0][r] + ((X[1][r] - X[0][r]) * XI<T>(q, 0) + (X[2][r] - X[0][r]) * XI<T>(q, 1) +
                           (X[3][r] - X[0][r]) * XI<T>(q, 2));
      fq[q] = evalFn(a.fn, a.rc, xq[0], xq[1], xq[2]);
    }
  }
  else
  {
    double loc[N];
#pragma unroll
    for (int n = 0; n < N; ++n)
      loc[n] = a.field[dof[n]];
#pragma unroll
    for (int q = 0; q < NQ; ++q)
    {
      double s = 0.;
#pragma unroll
      for (int n = 0; n < N; ++n)
        s += PHI<T>(q, n) * loc[n];
      fq[q] = a.rc * s;
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i)
  {
    if (a.rbc && ((cons >> i) & 1u))
      continue;
    double fe = 0.;
#pragma unroll
    for (int q = 0; q < NQ; ++q)
      fe += (adetD * WQ<T>(q)) * PHI<T>(q, i) * fq[q];
    red(a.b + dof[i], fe);
  }
}

// ------------------------------------------------- tetrahedra in FP64 arithmetic
// kAssembleTet64 (the default for P1/P2) in IEEE binary64 throughout.  Per element:
// J from the vertex differences, adj(J), |det J|, G = adj adj^T / |det J| (with a
// single stiffness operator's coefficient folded in).  P1 reads its entries from G
// directly; P2 with the usual stiffness + mass pair uses the barycentric form below,
// and otherwise the six-term products of G with the reference tensor (FP64 constant
// memory).  A mass entry is |det J| Mhat_ij (a single mass operator's coefficient
// folded into |det J|).  P2 tetrahedron: src/reffe.cpp:542-642, vertices then the
// edges 01 12 20 03 13 23.

// P2 in barycentric form.  With lambda_0 = 1 - x - y - z, lambda_1..3 = x, y, z, the
// vertex and edge functions are phi_i = lambda_i (2 lambda_i - 1) and
// phi_(ab) = 4 lambda_a lambda_b, whose gradients are linear in the lambdas, so with
// s_kl = k |T| grad lambda_k . grad lambda_l and the exact moments
// (1/|T|) int lambda_k lambda_l = (1 + delta_kl) / 20 the stiffness entries are short
// integer combinations of s' = s / 5:
//   vertex-vertex        K_ii = 3 s'_ii,  K_ij = -s'_ij
//   vertex i, edge (ab)  i = a: 3 s'_ib - s'_ii;  i not in (ab): -(s'_ia + s'_ib)
//   edge-edge            the same edge: 8 (s'_aa + s'_bb + s'_ab); sharing vertex v with
//                        other ends p, q: 4 (s'_vv + s'_vq + s'_pv + 2 s'_pq); disjoint
//                        (ab), (cd): 4 (s'_ac + s'_ad + s'_bc + s'_bd)
// The gradients of the lambdas sum to zero, so every row of s sums to zero and so does
// all of s.  With E_ab = s'_aa + s'_bb + s'_ab and r the vertex outside v, p, q the
// edge-edge entries become 8 E_ab, 4 (2 s'_pq - s'_vr) (six distinct values over the
// twelve pairs: the pairs sharing r with the same p, q give the same) and
// -4 (E_ab + s'_ab): 36 FP64 operations for the 21 entries instead of 78.
// The reference's 11-point rule integrates these degree-2 integrands exactly, so the
// values agree with its per-quadrature-point sums to round-off (64 FP64 operations per
// element for the 55 entries, instead of 177 for the reference-tensor products without
// their zero terms).
// exact negation: the sign bit flipped on the integer pipe
__device__ __forceinline__ double negx(double x)
{
  return __hiloint2double(__double2hiint(x) ^ (int)0x80000000, __double2loint(x));
}
template <int I, int J>
__device__ __forceinline__ double p2Stiff(double const (&s)[4][4], double const (&E)[6])
{
  if constexpr (J < 4)
    return I == J ? 3.0 * s[I][I] : negx(s[I][J]);
  else
  {
    constexpr int c = p2EdgeEnd(J, 0), d = p2EdgeEnd(J, 1);
    if constexpr (I < 4)
    {
      if constexpr (I == c)
        return fma(3.0, s[I][d], -s[I][I]);
      else if constexpr (I == d)
        return fma(3.0, s[I][c], -s[I][I]);
      else
        return -s[I][c] - s[I][d];
    }
    else
    {
      constexpr int a = p2EdgeEnd(I, 0), b = p2EdgeEnd(I, 1);
      if constexpr (I == J)
        return 8.0 * E[I - 4];
      else if constexpr (a == c || a == d || b == c || b == d)
      {
        constexpr int v = (a == c || a == d) ? a : b, p = v == a ? b : a, q = c == v ? d : c;
        constexpr int r = 6 - v - p - q;
        return 4.0 * fma(2.0, s[p < q ? p : q][p < q ? q : p], -s[v < r ? v : r][v < r ? r : v]);
      }
      else
        return -4.0 * (E[I - 4] + s[a][b]);
    }
  }
}
// a representative entry of each P2 mass class
__host__ __device__ constexpr int p2MassRepI(int c) { return c < 4 ? 0 : 4; }
__host__ __device__ constexpr int p2MassRepJ(int c)
{
  return c == 0 ? 0 : c == 1 ? 1 : c == 2 ? 4 : c == 3 ? 5 : c == 4 ? 4 : c == 5 ? 5 : 9;
}
// f(I, J) for the 55 pairs I <= J of the P2 element, as compile-time constants
template <int I, int J, class F>
__device__ __forceinline__ void p2ForPairs(F && f)
{
  f(std::integral_constant<int, I>{}, std::integral_constant<int, J>{});
  if constexpr (J + 1 < 10)
    p2ForPairs<I, J + 1>(f);
  else if constexpr (I + 1 < 10)
    p2ForPairs<I + 1, I + 1>(f);
}

template <int T, int NT>
__global__ void __launch_bounds__(NT) kAssembleTet64(AsmArgs a)
{
  constexpr int N = Elem<T>::N, NQ = Elem<T>::NQ;
  int64_t const i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i0 >= a.nelem)
    return;
  int64_t const e = elemOf(a, i0);

  double X[4][3];
#pragma unroll
  for (int v = 0; v < 4; ++v)
  {
    uint32_t const id = a.conn[e * 4 + v];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      X[v][d] = a.xyz[3 * (int64_t)id + d];
  }
  uint32_t dof[N];
#pragma unroll
  for (int i = 0; i < N; ++i)
    dof[i] = a.emap[e * N + i];
  uint32_t cons = 0;
  if (a.bcMask)
  {
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (a.bcMask[dof[i]])
        cons |= 1u << i;
  }
  LhsDev const & op0 = a.op[0];
  LhsDev const & op1 = a.op[1];
  bool const k0 = op0.on && op0.stiff, k1 = op1.on && op1.stiff;
  bool const m0 = op0.on && op0.mass, m1 = op1.on && op1.mass;
  bool const needK = k0 || k1, needM = m0 || m1;
  bool const kE = usesCoef(op0) || usesCoef(op1);
  double const kfac = (kE && a.kE) ? a.kE[e] : 1.0;

  double J[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int cc = 0; cc < 3; ++cc)
      J[r][cc] = X[cc + 1][r] - X[0][r];
  double A[3][3];
  double const adet = fabs(adj3(J, A));
  bool const foldK = k0 != k1, foldM = m0 != m1;
  double const ks0 = k0 ? (op0.stiff == 2 ? op0.sc * kfac : op0.sc) : 0.;
  double const ks1 = k1 ? (op1.stiff == 2 ? op1.sc * kfac : op1.sc) : 0.;
  double const ms0 = m0 ? massCoef(op0, kfac) : 0., ms1 = m1 ? massCoef(op1, kfac) : 0.;
  // 1/|det J|: hardware estimate and one third-order Newton step (y (1 + e + e^2),
  // e = 1 - x y), instead of a full-precision division with its special cases
  double ra;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(ra) : "d"(adet));
  {
    double const e = fma(-adet, ra, 1.0);
    ra = fma(ra, fma(e, e, e), ra);
  }
  bool const anyBc = cons && ((op0.on && op0.bc) || (op1.on && op1.bc));
  bool const kmPair = op0.on && op0.stiff && !op0.mass && op1.on && !op1.stiff && op1.mass;
  // the usual operator pair (stiffness-only, then mass-only, both folded) in a warp
  // without constrained entries: a loop without per-entry operator branches
  bool const fast = kmPair && !__any_sync(__activemask(), anyBc);
  double G[6];
  {
    double gs = (foldK ? (k0 ? ks0 : ks1) : 1.0) * ra;
    if constexpr (T == P1TET)
      gs *= cP1Ws;
    else if (fast)
      gs *= 1.0 / 30.0; // s'_(a+1)(b+1) = G_ab of the barycentric form
    gram(A, gs, G);
  }
  double const am = foldM ? (m0 ? ms0 : ms1) * adet : adet;
  // P1: grad phi_i |det J| are the adjugate rows (i = 1..3) and minus their sum (i = 0),
  // so K_ij = k / (6 |det J|) A_i . A_j reads the Gram entries of the adjugate directly:
  // K_(a+1)(b+1) = G_ab, K_0(b+1) = -sum_a G_ab, K_00 = sum_ab G_ab, with G carrying
  // the sum of the Tet4 weights (the reference volume 1/6)
  double K1[4][4];
  if constexpr (T == P1TET)
  {
    double const Gs[3][3] = {{G[0], G[3], G[4]}, {G[3], G[1], G[5]}, {G[4], G[5], G[2]}};
    double cs[3];
#pragma unroll
    for (int b = 0; b < 3; ++b)
    {
      cs[b] = Gs[0][b] + (Gs[1][b] + Gs[2][b]);
      K1[0][b + 1] = -cs[b];
#pragma unroll
      for (int a = 0; a < 3; ++a)
        K1[a + 1][b + 1] = Gs[a][b];
    }
    K1[0][0] = cs[0] + (cs[1] + cs[2]);
  }

  // the warp-group scatter of P2 finds its positions in its own map
  bool const grouped = T == P2TET && fast && a.grpOff;
  int32_t rpn[N];
#pragma unroll
  for (int n = 0; n < N; ++n)
    rpn[n] = grouped ? 0 : a.rowPtr[dof[n]];
  uint16_t const * rk = a.rank + e * (int64_t)(N * N);
  constexpr int kRowUnroll = N <= 4 ? N : 1;
  if constexpr (T == P2TET)
  {
    if (fast)
    {
      // the 55 entries unrolled in the barycentric form (the adjugate rows are the
      // gradients of lambda_1..3 times det J, lambda_0's is minus their sum) and the
      // mass from its seven distinct values
      double s[4][4];
      s[1][1] = G[0];
      s[2][2] = G[1];
      s[3][3] = G[2];
      s[1][2] = s[2][1] = G[3];
      s[1][3] = s[3][1] = G[4];
      s[2][3] = s[3][2] = G[5];
      double const c1 = G[0] + (G[3] + G[4]), c2 = G[3] + (G[1] + G[5]), c3 = G[4] + (G[5] + G[2]);
      s[0][1] = s[1][0] = negx(c1);
      s[0][2] = s[2][0] = negx(c2);
      s[0][3] = s[3][0] = negx(c3);
      s[0][0] = c1 + (c2 + c3);
      double E[6]; // E_ab = s'_aa + s'_bb + s'_ab of the six edges
#pragma unroll
      for (int n = 0; n < 6; ++n)
        E[n] = (s[p2EdgeEnd(4 + n, 0)][p2EdgeEnd(4 + n, 0)] + s[p2EdgeEnd(4 + n, 1)][p2EdgeEnd(4 + n, 1)]) +
               s[p2EdgeEnd(4 + n, 0)][p2EdgeEnd(4 + n, 1)];
      double mc[7];
#pragma unroll
      for (int c = 0; c < 7; ++c)
        mc[c] = am * MHAT<T>(p2MassRepI(c), p2MassRepJ(c));
      if (!grouped)
        pdlWait(); // the writes start here (the grouped path waits before its flush)
      if (a.grpOff)
      {
        // warp-group scatter: the lane's values and the group's contribution codes to
        // shared memory, then one reduction per distinct position of the warp's 32
        // elements, in ascending order
        extern __shared__ double gsm[];
        int const lane = threadIdx.x & 31;
        unsigned char * const wbase = reinterpret_cast<unsigned char *>(gsm) + (threadIdx.x >> 5) * kP2GroupSmemPerWarp;
        double * const sw = reinterpret_cast<double *>(wbase);
        uint16_t * const si = reinterpret_cast<uint16_t *>(wbase + kP2GroupValues * 32 * sizeof(double));
        // value v of lane l at v * 32 + (l ^ (v & 15)): the flush reads, in one
        // instruction, values of the same few elements (lanes) for different entries,
        // which this swizzle spreads over the banks
        auto swAt = [sw](uint32_t v, uint32_t l) -> double & { return sw[v * 32 + (l ^ (v & 15u))]; };
        p2ForPairs<0, 0>([&](auto I, auto J) {
          constexpr int i = decltype(I)::value, j = decltype(J)::value;
          swAt(p2UpperIdx(i, j), lane) = p2Stiff<i, j>(s, E);
        });
#pragma unroll
        for (int c = 0; c < 7; ++c)
          swAt(55 + c, lane) = mc[c];
        unsigned const mask = __activemask();
        int const W = __popc(mask); // the active lanes are 0 .. W - 1
        int64_t const g = e >> 5;
        int const nItems = W * 100;
        int32_t const dEnd = a.grpOff[g + 1];
        constexpr int U = 4;
        // the map of the next batch of positions is loaded while this one is summed and
        // reduced; the first batch's loads are issued before the codes are staged
        int32_t npos[U];
        int nb0[U], nb1[U];
        auto loadBatch = [&](int32_t d0) {
#pragma unroll
          for (int u = 0; u < U; ++u)
          {
            int32_t const d = d0 + u * W + lane;
            npos[u] = d < dEnd ? a.grpPos[d] : 0;
            nb0[u] = d < dEnd ? a.grpBeg[d] : 0;
            nb1[u] = d + 1 < dEnd ? a.grpBeg[d + 1] : nItems;
          }
        };
        loadBatch(a.grpOff[g]);
        // the group's codes: W * 100 of them, 16 bytes (8 codes) per load; the map pads
        // the last group's codes to a multiple of 8
        uint4 const * const gi = reinterpret_cast<uint4 const *>(a.grpItem + g * kP2GroupItems);
        // every load of a batch in flight before the first store: at most 13 per lane
        // for any warp width (ceil(12.5 W) / W < 13.5), in two batches of seven
        int const n8 = (nItems + 7) / 8;
        uint4 * const si4 = reinterpret_cast<uint4 *>(si);
        static_assert(kP2GroupItems / 8 <= 32 * 14, "code staging batches");
#pragma unroll
        for (int h = 0; h < 2; ++h)
        {
          uint4 tmp[7];
#pragma unroll
          for (int r = 0; r < 7; ++r)
          {
            int const k = lane + (7 * h + r) * W;
            if (k < n8)
              tmp[r] = gi[k];
          }
#pragma unroll
          for (int r = 0; r < 7; ++r)
          {
            int const k = lane + (7 * h + r) * W;
            if (k < n8)
              si4[k] = tmp[r];
          }
        }
        __syncwarp(mask);
        pdlWait(); // the writes start here
        for (int32_t d0 = a.grpOff[g]; d0 < dEnd; d0 += U * W)
        {
          int32_t pos[U];
          int b0[U], b1[U];
#pragma unroll
          for (int u = 0; u < U; ++u)
            pos[u] = npos[u], b0[u] = nb0[u], b1[u] = nb1[u];
          loadBatch(d0 + U * W);
#pragma unroll
          for (int u = 0; u < U; ++u)
          {
            if (d0 + u * W + lane >= dEnd)
              break;
            // the position's contributions in element order: no addition for the
            // first (the FP64 pipe is the scarce one)
            // a position with few contributions: one reduction each (the L2 atomic unit
            // has room, the FP64 pipe has not); more: sum them here, reduce once
            if (b1[u] - b0[u] <= a.grpRedMax)
            {
              for (int k = b0[u]; k < b1[u]; ++k)
              {
                uint32_t const code = si[k];
                red(op0.vals + pos[u], swAt((code >> 5) & 63u, code & 31u));
                red(op1.vals + pos[u], swAt(55 + (code >> 11), code & 31u));
              }
              continue;
            }
            uint32_t code = si[b0[u]];
            double kk = swAt((code >> 5) & 63u, code & 31u);
            double mm = swAt(55 + (code >> 11), code & 31u);
            for (int k = b0[u] + 1; k < b1[u]; ++k)
            {
              code = si[k];
              kk += swAt((code >> 5) & 63u, code & 31u);
              mm += swAt(55 + (code >> 11), code & 31u);
            }
            red(op0.vals + pos[u], kk);
            red(op1.vals + pos[u], mm);
          }
        }
        goto entriesDone;
      }
      p2ForPairs<0, 0>([&](auto I, auto J) {
        constexpr int i = decltype(I)::value, j = decltype(J)::value;
        double const kv = p2Stiff<i, j>(s, E);
        double const mv = mc[p2MassClass(i, j)];
        int32_t const pij = rpn[i] + rk[i * N + j];
        red(op0.vals + pij, kv);
        red(op1.vals + pij, mv);
        if constexpr (j != i)
        {
          int32_t const pji = rpn[j] + rk[j * N + i];
          red(op0.vals + pji, kv);
          red(op1.vals + pji, mv);
        }
      });
      goto entriesDone;
    }
  }
  pdlWait(); // the writes start here
#pragma unroll kRowUnroll
  for (int i = 0; i < N; ++i)
  {
    uint32_t const dofi = pickN(dof, i);
    int32_t const rpi = pickN(rpn, i);
    bool const ci = (cons >> i) & 1u;
#pragma unroll kRowUnroll
    for (int j = i; j < N; ++j)
    {
      double kv = 0., mv = 0.;
      if (needK)
      {
        if constexpr (T == P1TET)
          kv = K1[i][j];
        else
        {
          kv = G[0] * TT<T>(0, i, j);
#pragma unroll
          for (int k = 1; k < 6; ++k)
            kv = fma(G[k], TT<T>(k, i, j), kv);
        }
      }
      if (needM)
        mv = am * MHAT<T>(i, j);
      int32_t const pij = rpi + rk[i * N + j];
      int32_t const pji = pickN(rpn, j) + rk[j * N + i];
      if (fast)
      {
        red(op0.vals + pij, kv);
        red(op1.vals + pij, mv);
        if (j != i)
        {
          red(op0.vals + pji, kv);
          red(op1.vals + pji, mv);
        }
        continue;
      }
      bool const cj = (cons >> j) & 1u;
#pragma unroll
      for (int m = 0; m < 2; ++m)
      {
        LhsDev const & op = a.op[m];
        if (!op.on)
          continue;
        double v;
        if (op.stiff)
        {
          v = foldK ? kv : (m ? ks1 : ks0) * kv;
          if (op.mass)
            v = foldM ? v + mv : fma(m ? ms1 : ms0, mv, v);
        }
        else
          v = foldM ? mv : (m ? ms1 : ms0) * mv;
        if (anyBc && op.bc && (ci || cj))
        {
          condenseTet(op.vals + pij, a.bcDiag, a.b, dofi, pickN(dof, j), a.bcVal, ci, cj, i == j, v);
          continue;
        }
        red(op.vals + pij, v);
        if (j != i)
          red(op.vals + pji, v);
      }
    }
  }
entriesDone:
  if (!a.b)
    return;
  if (anyBc)
  {
#pragma unroll
    for (int m = 0; m < 2; ++m)
    {
      if (!a.op[m].on || !a.op[m].bc)
        continue;
#pragma unroll
      for (int n = 0; n < N; ++n)
        if ((cons >> n) & 1u)
        {
          double const h = a.bcVal[dof[n]];
          if (h != 0.)
            red(a.b + dof[n], h);
        }
    }
  }
  if (!a.rkind)
    return;
  if (a.rkind == 1 && a.fn == PXG_FN_CONST)
  {
    double const f = evalFn(a.fn, a.rc, 0., 0., 0.) * adet;
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (!(a.rbc && ((cons >> i) & 1u)))
        red(a.b + dof[i], f * PINT<T>(i));
    return;
  }
  double fq[NQ];
  if (a.rkind == 1)
  {
#pragma unroll
    for (int q = 0; q < NQ; ++q)
    {
      double xq[3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
        xq[r] = X[0][r] + (J[r][0] * XI<T>(q, 0) + J[r][1] * XI<T>(q, 1) + J[r][2] * XI<T>(q, 2));
      fq[q] = evalFn(a.fn, a.rc, xq[0], xq[1], xq[2]);
    }
  }
  else
  {
    double loc[N];
#pragma unroll
    for (int n = 0; n < N; ++n)
      loc[n] = a.field[dof[n]];
#pragma unroll
    for (int q = 0; q < NQ; ++q)
    {
      double s = 0.;
#pragma unroll
      for (int n = 0; n < N; ++n)
        s += PHI<T>(q, n) * loc[n];
      fq[q] = a.rc * s;
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i)
  {
    if (a.rbc && ((cons >> i) & 1u))
      continue;
    double fe = 0.;
#pragma unroll
    for (int q = 0; q < NQ; ++q)
      fe += (adet * WQ<T>(q)) * PHI<T>(q, i) * fq[q];
    red(a.b + dof[i], fe);
  }
}

// CurFE::qpoint (include/curfe.hpp:80) of every element and quadrature point:
// origin + J(xi_q) xi_q, J from the mapping points as in kAssemble; origin = the first
// vertex (tetrahedra, include/geo.hpp:583-588) or the vertex average (hexahedra,
// geo.hpp:721-728).  One thread per element; out[(e * NQ + q) * 3 + d].
template <int T>
__global__ void __launch_bounds__(128) kQpoints(int64_t nelem, double const * __restrict__ xyz,
                                                uint32_t const * __restrict__ conn, double * __restrict__ out)
{
  constexpr int NV = Elem<T>::NV, N = Elem<T>::N, NQ = Elem<T>::NQ;
  int64_t const e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= nelem)
    return;
  double X[NV][3];
#pragma unroll
  for (int v = 0; v < NV; ++v)
  {
    uint32_t const id = conn[e * NV + v];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      X[v][d] = xyz[3 * (int64_t)id + d];
  }
  double * o = out + e * NQ * 3;
  if constexpr (!Elem<T>::hex)
  {
#pragma unroll 1
    for (int q = 0; q < NQ; ++q)
#pragma unroll
      for (int r = 0; r < 3; ++r)
        o[3 * q + r] = X[0][r] + ((X[1][r] - X[0][r]) * XI<T>(q, 0) + (X[2][r] - X[0][r]) * XI<T>(q, 1) +
                                  (X[3][r] - X[0][r]) * XI<T>(q, 2));
  }
  else
  {
    double P[N][3];
    mappingPoints<T>(X, P);
    double org[3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      org[d] = .125 * (X[0][d] + X[1][d] + X[2][d] + X[3][d] + X[4][d] + X[5][d] + X[6][d] + X[7][d]);
#pragma unroll 1
    for (int q = 0; q < NQ; ++q)
    {
      double J[3][3] = {{0., 0., 0.}, {0., 0., 0.}, {0., 0., 0.}};
#pragma unroll
      for (int n = 0; n < N; ++n)
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int cc = 0; cc < 3; ++cc)
            J[r][cc] += P[n][r] * DPHI<T>(q, n, cc);
#pragma unroll
      for (int r = 0; r < 3; ++r)
        o[3 * q + r] = org[r] + (J[r][0] * XI<T>(q, 0) + J[r][1] * XI<T>(q, 1) + J[r][2] * XI<T>(q, 2));
    }
  }
}

// ------------------------------------------- near-zero entries in the reference order
// closeMatrix's prune(1., 1e-16) (include/builder.hpp:369) decides on absolute values,
// so an entry that is mathematically zero is kept or dropped by the round-off of its
// evaluation: on a jittered P2 mesh the reference's CurFE form leaves 1e-16 residues
// where the engine's reference-tensor form gives exact zeros.  For the entries whose
// value lies within the engine's round-off of the threshold (|v| <= 1e-16 + 64 eps
// max|row|), the value is recomputed in the reference's evaluation order: per element,
// CurFE::reinit (include/curfe.hpp:50-103: J from the mapping points, J^T J, its
// cofactor inverse, sqrt(det), J^+, dphi = dphiRef J^+) and the stiffness / mass sums
// over the quadrature points (include/assembly_lhs.hpp:52-65, 207-221) with the
// Dirichlet condensation of builder.hpp:76-124; over elements, the triplets' sum in
// emission order (setFromTriplets: the first contribution, then each later one added).
// Every operation is a separately rounded IEEE operation (the intrinsics below are
// never contracted into FMAs), in the order the reference's expressions give.
__device__ __forceinline__ double dA(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dS(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dM(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dD(double a, double b) { return __ddiv_rn(a, b); }

struct RefOp
{
  int stiff, mass, bc;
  double sc, mc;
};
struct RepairArgs
{
  double const * xyz;
  uint32_t const * conn;
  uint32_t const * emap;
  int32_t const * rowPtr;
  int32_t const * colIdx;
  double const * kE;
  uint8_t const * bcMask;
  double bcDiag;
  int32_t const * dofElemPtr;
  uint32_t const * dofElem;
  RefOp ops[8];
  int nops;
  int64_t const * flagged; // positions in the structural pattern
  int32_t const * flaggedRow;
  int64_t nflagged;
  double * vals; // values on the structural pattern, the flagged ones overwritten
};

// the element's local entry (i, j) of one operator, before any condensation
template <int T>
__device__ double refElemEntry(RepairArgs const & a, int64_t e, int i, int j, RefOp const & op)
{
  constexpr int NV = Elem<T>::NV, N = Elem<T>::N, NQ = Elem<T>::NQ;
  double X[NV][3];
  for (int v = 0; v < NV; ++v)
  {
    uint32_t const id = a.conn[e * NV + v];
    for (int d = 0; d < 3; ++d)
      X[v][d] = a.xyz[3 * (int64_t)id + d];
  }
  double P[N][3];
  mappingPoints<T>(X, P);
  double const kfac = a.kE ? a.kE[e] : 1.0;
  double jxw[NQ], Di[NQ][3], Dj[NQ][3];
  for (int q = 0; q < NQ; ++q)
  {
    double J[3][3];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c)
        J[r][c] = 0.;
    for (int n = 0; n < N; ++n)
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
          J[r][c] = dA(J[r][c], dM(P[n][r], DPHI<T>(q, n, c)));
    double A[3][3];
    for (int x = 0; x < 3; ++x)
      for (int y = 0; y < 3; ++y)
        A[x][y] = dA(dA(dM(J[0][x], J[0][y]), dM(J[1][x], J[1][y])), dM(J[2][x], J[2][y]));
    double const c00 = dS(dM(A[1][1], A[2][2]), dM(A[1][2], A[2][1]));
    double const c01 = dS(dM(A[1][2], A[2][0]), dM(A[1][0], A[2][2]));
    double const c02 = dS(dM(A[1][0], A[2][1]), dM(A[1][1], A[2][0]));
    double const det = dA(dA(dM(A[0][0], c00), dM(A[0][1], c01)), dM(A[0][2], c02));
    double Ai[3][3];
    Ai[0][0] = dD(c00, det);
    Ai[1][0] = dD(c01, det);
    Ai[2][0] = dD(c02, det);
    Ai[0][1] = dD(dS(dM(A[0][2], A[2][1]), dM(A[0][1], A[2][2])), det);
    Ai[1][1] = dD(dS(dM(A[0][0], A[2][2]), dM(A[0][2], A[2][0])), det);
    Ai[2][1] = dD(dS(dM(A[0][1], A[2][0]), dM(A[0][0], A[2][1])), det);
    Ai[0][2] = dD(dS(dM(A[0][1], A[1][2]), dM(A[0][2], A[1][1])), det);
    Ai[1][2] = dD(dS(dM(A[0][2], A[1][0]), dM(A[0][0], A[1][2])), det);
    Ai[2][2] = dD(dS(dM(A[0][0], A[1][1]), dM(A[0][1], A[1][0])), det);
    double Jp[3][3];
    for (int x = 0; x < 3; ++x)
      for (int c = 0; c < 3; ++c)
        Jp[x][c] = dA(dA(dM(Ai[x][0], J[c][0]), dM(Ai[x][1], J[c][1])), dM(Ai[x][2], J[c][2]));
    jxw[q] = dM(__dsqrt_rn(det), WQ<T>(q));
    for (int c = 0; c < 3; ++c)
    {
      Di[q][c] = dA(dA(dM(DPHI<T>(q, i, 0), Jp[0][c]), dM(DPHI<T>(q, i, 1), Jp[1][c])), dM(DPHI<T>(q, i, 2), Jp[2][c]));
      Dj[q][c] = dA(dA(dM(DPHI<T>(q, j, 0), Jp[0][c]), dM(DPHI<T>(q, j, 1), Jp[1][c])), dM(DPHI<T>(q, j, 2), Jp[2][c]));
    }
  }
  double ke = 0.;
  if (op.stiff)
  {
    double const c = op.stiff == 1 ? op.sc : dM(1.0, dM(op.sc, kfac));
    for (int q = 0; q < NQ; ++q)
    {
      double const sq = dM(c, jxw[q]);
      double const a0 = dM(sq, Di[q][0]), a1 = dM(sq, Di[q][1]), a2 = dM(sq, Di[q][2]);
      ke = dA(ke, dA(dA(dM(a0, Dj[q][0]), dM(a1, Dj[q][1])), dM(a2, Dj[q][2])));
    }
  }
  if (op.mass)
  {
    double const c = op.mass == 1 ? op.mc : dM(1.0, dM(op.mc, kfac));
    for (int q = 0; q < NQ; ++q)
    {
      double const sq = dM(c, jxw[q]);
      ke = dA(ke, dM(dM(sq, PHI<T>(q, i)), PHI<T>(q, j)));
    }
  }
  return ke;
}

// one thread per flagged entry: the sum of the element contributions in emission order
// (operators in call order, elements in ascending order)
template <int T>
__global__ void __launch_bounds__(128) kRepairEntries(RepairArgs a)
{
  constexpr int N = Elem<T>::N;
  int64_t const k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= a.nflagged)
    return;
  int64_t const p = a.flagged[k];
  int32_t const r = a.flaggedRow[k];
  int32_t const col = a.colIdx[p];
  bool const consR = a.bcMask && a.bcMask[r], consC = a.bcMask && a.bcMask[col];
  double v = 0.;
  bool first = true;
  for (int o = 0; o < a.nops; ++o)
  {
    RefOp const op = a.ops[o];
    for (int32_t t = a.dofElemPtr[r]; t < a.dofElemPtr[r + 1]; ++t)
    {
      int64_t const e = a.dofElem[t];
      int i = -1, j = -1;
      for (int n = 0; n < N; ++n)
      {
        uint32_t const d = a.emap[e * N + n];
        if ((int32_t)d == r)
          i = n;
        if ((int32_t)d == col)
          j = n;
      }
      if (i < 0 || j < 0)
        continue;
      double ke;
      if (op.bc && (consR || consC))
        ke = (r == col && consR) ? a.bcDiag : 0.;
      else
        ke = refElemEntry<T>(a, e, i, j, op);
      v = first ? ke : dA(v, ke);
      first = false;
    }
  }
  a.vals[p] = v;
}

// entries within the engine's round-off of the prune threshold: |v| <= 1e-16 +
// 64 eps max|row|.  count != nullptr: count them; else write their positions and rows
__global__ void kFlagNearZero(int32_t const * __restrict__ rowPtr, double const * __restrict__ vals, int64_t n,
                              unsigned long long * count, int64_t * pos, int32_t * row, int64_t cap)
{
  int64_t const r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n)
    return;
  double mx = 0.;
  for (int32_t p = rowPtr[r]; p < rowPtr[r + 1]; ++p)
    mx = fmax(mx, fabs(vals[p]));
  double const tau = 1e-16 + 64. * 2.220446049250313e-16 * mx;
  for (int32_t p = rowPtr[r]; p < rowPtr[r + 1]; ++p)
    if (fabs(vals[p]) <= tau)
    {
      unsigned long long const k = atomicAdd(count, 1ull);
      if (pos && (int64_t)k < cap)
      {
        pos[k] = p;
        row[k] = (int32_t)r;
      }
    }
}

// element lists per DOF: counts, then the fill, then each list sorted ascending
__global__ void kDofElemCount(uint32_t const * __restrict__ emap, int64_t nelem, int N, int32_t * cnt)
{
  int64_t const t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nelem * N)
    return;
  atomicAdd(cnt + emap[t], 1);
}
__global__ void kDofElemFill(uint32_t const * __restrict__ emap, int64_t nelem, int N, int32_t * cursor,
                             uint32_t * list)
{
  int64_t const t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nelem * N)
    return;
  int32_t const at = atomicAdd(cursor + emap[t], 1);
  list[at] = (uint32_t)(t / N);
}
__global__ void kDofElemSort(int32_t const * __restrict__ ptr, int64_t ndof, uint32_t * list)
{
  int64_t const d = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (d >= ndof)
    return;
  for (int32_t a = ptr[d] + 1; a < ptr[d + 1]; ++a)
  {
    uint32_t const v = list[a];
    int32_t b = a - 1;
    while (b >= ptr[d] && list[b] > v)
    {
      list[b + 1] = list[b];
      --b;
    }
    list[b + 1] = v;
  }
}

template <int T>
__global__ void kInterpolate(int64_t nelem, double const * __restrict__ xyz, uint32_t const * __restrict__ conn,
                             uint32_t const * __restrict__ emap, int fn, double c, double * __restrict__ v)
{
  constexpr int NV = Elem<T>::NV, N = Elem<T>::N;
  int64_t const e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= nelem)
    return;
  double X[NV][3], P[N][3];
#pragma unroll
  for (int k = 0; k < NV; ++k)
  {
    uint32_t const id = conn[e * NV + k];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      X[k][d] = xyz[3 * (int64_t)id + d];
  }
  mappingPoints<T>(X, P);
#pragma unroll 1
  for (int i = 0; i < N; ++i)
    v[emap[e * N + i]] = evalFn(fn, c, P[i][0], P[i][1], P[i][2]);
}

// prune(1., 1e-16): an entry is dropped when |v| <= 1e-16 (Eigen's isMuchSmallerThan)
__device__ __forceinline__ bool pruned(double v) { return fabs(v) <= 1e-16; }

// Streams the value array once: 16-byte loads, four per thread in flight (about 20 MB
// over the grid, enough to keep HBM busy), evict-first because the values are not
// reused by the count. A value array that starts 8 bytes off a 16-byte boundary has
// its first entry counted alone, and an odd remainder its last.
__global__ void kPruneCount(double const * __restrict__ vals, int64_t n, unsigned long long * out)
{
  unsigned long long cnt = 0;
  int64_t const head = (n > 0 && (reinterpret_cast<uintptr_t>(vals) & 15) != 0) ? 1 : 0;
  int64_t const n2 = (n - head) / 2;
  int64_t const t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t const stride = (int64_t)gridDim.x * blockDim.x;
  if (t == 0)
  {
    if (head)
      cnt += pruned(vals[0]) ? 1ull : 0ull;
    if ((n - head) & 1)
      cnt += pruned(vals[n - 1]) ? 1ull : 0ull;
  }
  double2 const * v2 = reinterpret_cast<double2 const *>(vals + head);
  int64_t k = t;
  for (; k + 3 * stride < n2; k += 4 * stride)
  {
    double2 const a = __ldcs(v2 + k), b = __ldcs(v2 + k + stride);
    double2 const c = __ldcs(v2 + k + 2 * stride), d = __ldcs(v2 + k + 3 * stride);
    cnt += (pruned(a.x) ? 1ull : 0ull) + (pruned(a.y) ? 1ull : 0ull) + (pruned(b.x) ? 1ull : 0ull) +
           (pruned(b.y) ? 1ull : 0ull) + (pruned(c.x) ? 1ull : 0ull) + (pruned(c.y) ? 1ull : 0ull) +
           (pruned(d.x) ? 1ull : 0ull) + (pruned(d.y) ? 1ull : 0ull);
  }
  for (; k < n2; k += stride)
  {
    double2 const a = __ldcs(v2 + k);
    cnt += (pruned(a.x) ? 1ull : 0ull) + (pruned(a.y) ? 1ull : 0ull);
  }
  using WR = cub::WarpReduce<unsigned long long>;
  __shared__ typename WR::TempStorage ts[8];
  unsigned long long const s = WR(ts[threadIdx.x / 32]).Sum(cnt);
  if ((threadIdx.x & 31) == 0 && s)
    atomicAdd(out, s);
}

__global__ void kRowKept(int32_t const * __restrict__ rowPtr, double const * __restrict__ vals, int64_t nrows,
                         int32_t * __restrict__ kept)
{
  int64_t const r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nrows)
    return;
  int32_t k = 0;
  for (int32_t p = rowPtr[r]; p < rowPtr[r + 1]; ++p)
    k += pruned(vals[p]) ? 0 : 1;
  kept[r] = k;
}

__global__ void kCompact(int32_t const * __restrict__ rowPtr, int32_t const * __restrict__ col,
                         double const * __restrict__ vals, int64_t nrows, int32_t const * __restrict__ newPtr,
                         int32_t * __restrict__ colOut, double * __restrict__ valOut)
{
  int64_t const r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= nrows)
    return;
  int32_t o = newPtr[r];
  for (int32_t p = rowPtr[r]; p < rowPtr[r + 1]; ++p)
    if (!pruned(vals[p]))
    {
      colOut[o] = col[p];
      valOut[o] = vals[p];
      ++o;
    }
}

// Adjoint gradient g_e = -(C u)_e^T K_e (C lambda)_e for any element type (the
// stiffness entries are those of kAssemble with the coefficient k_e).
template <int T>
__global__ void __launch_bounds__(128) kAdjointGrad(AdjArgs a)
{
  constexpr int NV = Elem<T>::NV, N = Elem<T>::N, NQ = Elem<T>::NQ;
  constexpr bool HEX = Elem<T>::hex;
  int64_t const e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= a.nelem)
    return;
  double X[NV][3];
#pragma unroll
  for (int v = 0; v < NV; ++v)
  {
    uint32_t const id = a.conn[e * NV + v];
#pragma unroll
    for (int d = 0; d < 3; ++d)
      X[v][d] = a.xyz[3 * (int64_t)id + d];
  }
  double ue[N], le[N];
#pragma unroll
  for (int i = 0; i < N; ++i)
  {
    uint32_t const d = a.emap[e * N + i];
    bool const c = a.bcMask && a.bcMask[d];
    ue[i] = c ? 0. : a.u[d];
    le[i] = c ? 0. : a.lam[d];
  }
  if constexpr (T == P1TET)
  {
    // constant gradients: u^T K0_e lambda = |det J| / 6 (J^-T grad^ u) . (J^-T grad^ lambda)
    // = (A^T grad^ u) . (A^T grad^ lambda) / (6 |det J|), A = adj(J), grad^ u = the
    // vertex differences u_1 - u_0, u_2 - u_0, u_3 - u_0 (about 60 FP64 operations
    // instead of the element matrix and its contraction)
    double J[3][3], A[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int cc = 0; cc < 3; ++cc)
        J[r][cc] = X[cc + 1][r] - X[0][r];
    double const det = adj3(J, A);
    double const du[3] = {ue[1] - ue[0], ue[2] - ue[0], ue[3] - ue[0]};
    double const dl[3] = {le[1] - le[0], le[2] - le[0], le[3] - le[0]};
    double gu[3], gl[3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
    {
      gu[c] = A[0][c] * du[0] + A[1][c] * du[1] + A[2][c] * du[2];
      gl[c] = A[0][c] * dl[0] + A[1][c] * dl[1] + A[2][c] * dl[2];
    }
    double const s = (gu[0] * gl[0] + gu[1] * gl[1] + gu[2] * gl[2]) / (6.0 * fabs(det));
    a.g[e] = -(a.kE[e] * s);
    return;
  }
  double G[HEX ? NQ : 1][6];
  if constexpr (!HEX)
  {
    double J[3][3], A[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int cc = 0; cc < 3; ++cc)
        J[r][cc] = X[cc + 1][r] - X[0][r];
    double const det = adj3(J, A);
    gram(A, 1.0 / fabs(det), G[0]);
  }
  else
  {
    double P[N][3];
    mappingPoints<T>(X, P);
#pragma unroll
    for (int q = 0; q < NQ; ++q)
    {
      double J[3][3] = {{0., 0., 0.}, {0., 0., 0.}, {0., 0., 0.}}, A[3][3];
#pragma unroll
      for (int n = 0; n < N; ++n)
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int cc = 0; cc < 3; ++cc)
            J[r][cc] += P[n][r] * DPHI<T>(q, n, cc);
      double const det = adj3(J, A);
      gram(A, WQ<T>(q) / fabs(det), G[q]);
    }
  }
  double s = 0.;
#pragma unroll 1
  for (int i = 0; i < N; ++i)
  {
#pragma unroll 1
    for (int j = i; j < N; ++j)
    {
      double kv = 0.;
      if constexpr (HEX)
      {
#pragma unroll
        for (int q = 0; q < NQ; ++q)
        {
          double const d0 = DPHI<T>(q, i, 0), d1 = DPHI<T>(q, i, 1), d2 = DPHI<T>(q, i, 2);
          double const v0 = G[q][0] * d0 + G[q][3] * d1 + G[q][4] * d2;
          double const v1 = G[q][3] * d0 + G[q][1] * d1 + G[q][5] * d2;
          double const v2 = G[q][4] * d0 + G[q][5] * d1 + G[q][2] * d2;
          kv += v0 * DPHI<T>(q, j, 0) + v1 * DPHI<T>(q, j, 1) + v2 * DPHI<T>(q, j, 2);
        }
      }
      else
      {
#pragma unroll
        for (int k = 0; k < 6; ++k)
          kv += G[0][k] * TT<T>(k, i, j);
      }
      s += kv * ((i == j) ? ue[i] * le[i] : ue[i] * le[j] + ue[j] * le[i]);
    }
  }
  a.g[e] = -(a.kE[e] * s);
}

pxg_status launchAdjointGrad(pxg_ctx * c, double const * u, double const * lam, double * g, cudaStream_t s)
{
  AdjArgs a{c->nelem, c->xyz.p, c->conn.p, c->emap.p, c->kE.p, c->nbc ? c->bcMask.p : nullptr, u, lam, g};
  unsigned const blocks = (unsigned)((c->nelem + 127) / 128);
  switch (c->etype)
  {
  case P1TET:
    kAdjointGrad<P1TET><<<blocks, 128, 0, s>>>(a);
    break;
  case P2TET:
    kAdjointGrad<P2TET><<<blocks, 128, 0, s>>>(a);
    break;
  case Q1HEX:
    if (c->q1Generic)
      kAdjointGrad<Q1HEX><<<blocks, 128, 0, s>>>(a);
    else
      launchAdjointGradQ1(a, s, c->arith == PXG_ARITH_FP64);
    break;
  case Q2HEX:
    kAdjointGrad<Q2HEX><<<blocks, 128, 0, s>>>(a);
    break;
  }
  PXG_CUDA(c, cudaGetLastError());
  return PXG_OK;
}

} // namespace pxg

using namespace pxg;

namespace
{
// Threads per block: 64, 128 or 256 for the tetrahedra (autotuner candidates), 128
// for the hexahedra of the generic kernel.
template <int T>
void launchAssembleTet(AsmArgs const & a, cudaStream_t s, int threads)
{
  auto go = [&](auto kern, int nt) {
    unsigned const blocks = (unsigned)((a.nelem + nt - 1) / nt);
    kern<<<blocks, nt, 0, s>>>(a);
  };
  if (threads == 64)
    return go(kAssembleTet<T, 64>, 64);
  if (threads == 256)
    return go(kAssembleTet<T, 256>, 256);
  go(kAssembleTet<T, 128>, 128);
}

template <int T>
void launchAssembleTet64(AsmArgs const & a, cudaStream_t s, int threads)
{
  auto go = [&](auto kern, int nt) {
    unsigned const blocks = (unsigned)((a.nelem + nt - 1) / nt);
    size_t smem = 0;
    if (T == P2TET && a.grpOff)
    {
      // the warp-group scatter's values and codes
      smem = (size_t)(nt / 32) * kP2GroupSmemPerWarp;
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
    if (blocks > 0)
      launchElemKernel(kern, blocks, nt, smem, s, a);
  };
  if (threads == 64)
    return go(kAssembleTet64<T, 64>, 64);
  if (threads == 256)
    return go(kAssembleTet64<T, 256>, 256);
  go(kAssembleTet64<T, 128>, 128);
}

template <int T>
void launchAssemble(AsmArgs const & a, cudaStream_t s, int threads)
{
  auto go = [&](auto kern, int nt) {
    unsigned const blocks = (unsigned)((a.nelem + nt - 1) / nt);
    kern<<<blocks, nt, 0, s>>>(a);
  };
  if constexpr (T == P1TET || T == P2TET)
  {
    if (threads == 64)
      return go(kAssemble<T, 64>, 64);
    if (threads == 256)
      return go(kAssemble<T, 256>, 256);
  }
  go(kAssemble<T, 128>, 128);
}

} // namespace

// Remember what pxg_assemble adds into a value array (its recipe), for the
// reference-order recomputation of its near-zero entries at pxg_close_matrix.
void recordRecipe(pxg_ctx * c, double const * vals, pxg_lhs_op const & o, bool accumulate)
{
  auto & rs = c->recipes;
  size_t k = 0;
  while (k < rs.size() && rs[k].vals != vals)
    ++k;
  if (k == rs.size())
  {
    if (rs.size() >= 16)
      rs.erase(rs.begin());
    rs.push_back(pxg_ctx::Recipe{});
    k = rs.size() - 1;
    rs[k].vals = vals;
  }
  pxg_ctx::Recipe & R = rs[k];
  if (!accumulate)
  {
    R.ops.clear();
    R.valid = true;
    R.meshVer = c->meshVer, R.coefVer = c->coefVer, R.bcVer = c->bcVer;
  }
  else if (R.meshVer != c->meshVer || R.coefVer != c->coefVer || R.bcVer != c->bcVer)
    R.valid = false; // calls on different data: the sum cannot be recomputed
  if (R.ops.size() >= 8)
    R.valid = false;
  else
    R.ops.push_back(pxg_ctx::LhsRec{o.stiffness, o.mass, o.apply_bc, o.stiff_coef, o.mass_coef});
}

namespace pxg
{
// zero the outputs of an assembly (z0, z1: n values; zb: nb), letting the element kernel
// that follows start at once as its programmatic dependent (pdlWait)
__global__ void __launch_bounds__(256) kZeroOutputs(double * z0, double * z1, int64_t n, double * zb, int64_t nb)
{
  asm volatile("griddepcontrol.launch_dependents;");
  int64_t const nthr = (int64_t)gridDim.x * blockDim.x, t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int64_t k = t; k < n; k += nthr)
  {
    if (z0)
      z0[k] = 0.;
    if (z1)
      z1[k] = 0.;
  }
  for (int64_t k = t; k < nb; k += nthr)
    zb[k] = 0.;
}
} // namespace pxg

// the element lists of every DOF, ascending (built once per DOF map)
pxg_status ensureDofElem(pxg_ctx * c)
{
  if (c->dofElemPtr.p)
    return PXG_OK;
  int64_t const n = c->ndof, m = c->nelem * c->N;
  DevBuf<int32_t> cnt, cursor;
  PXG_CUDA(c, cnt.alloc(n + 1));
  PXG_CUDA(c, cudaMemset(cnt.p, 0, (n + 1) * 4));
  unsigned const bm = (unsigned)((m + 255) / 256), bn = (unsigned)((n + 255) / 256);
  kDofElemCount<<<bm, 256>>>(c->emap.p, c->nelem, c->N, cnt.p);
  PXG_CUDA(c, c->dofElemPtr.alloc(n + 1));
  size_t tb = 0;
  PXG_CUDA(c, cub::DeviceScan::ExclusiveSum(nullptr, tb, cnt.p, c->dofElemPtr.p, n + 1));
  DevBuf<unsigned char> tmp;
  PXG_CUDA(c, tmp.alloc(tb));
  PXG_CUDA(c, cub::DeviceScan::ExclusiveSum(tmp.p, tb, cnt.p, c->dofElemPtr.p, n + 1));
  PXG_CUDA(c, cursor.alloc(n + 1));
  PXG_CUDA(c, cudaMemcpy(cursor.p, c->dofElemPtr.p, (n + 1) * 4, cudaMemcpyDeviceToDevice));
  PXG_CUDA(c, c->dofElem.alloc(m));
  kDofElemFill<<<bm, 256>>>(c->emap.p, c->nelem, c->N, cursor.p, c->dofElem.p);
  kDofElemSort<<<bn, 256>>>(c->dofElemPtr.p, n, c->dofElem.p);
  PXG_CUDA(c, cudaGetLastError());
  PXG_CUDA(c, cudaDeviceSynchronize());
  return PXG_OK;
}

// Builder::closeMatrix's prune(1., 1e-16) and compaction of a structural CSR (row
// pointers rowPtr[n + 1], columns colIdx) with values vals: kept entries per row, their
// exclusive scan (the new row pointers), the compaction, and the kept count read back
// (the stream is synchronised).  Scratch is allocated per call on c's device.
namespace pxg
{
pxg_status closeCsr(pxg_ctx * c, int32_t const * rowPtr, int32_t const * colIdx, int64_t n, double const * vals,
                    int32_t * rp, int32_t * ci, double * vout, int64_t * nnzOut, cudaStream_t s)
{
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  DevBuf<int32_t> kept;
  PXG_CUDA(c, kept.alloc(n + 1));
  unsigned const blocks = (unsigned)((n + 255) / 256);
  kRowKept<<<blocks, 256, 0, s>>>(rowPtr, vals, n, kept.p);
  PXG_CUDA(c, cudaMemsetAsync(kept.p + n, 0, 4, s));
  size_t tb = 0;
  PXG_CUDA(c, cub::DeviceScan::ExclusiveSum(nullptr, tb, kept.p, rp, n + 1, s));
  DevBuf<unsigned char> tmp;
  PXG_CUDA(c, tmp.alloc(tb));
  PXG_CUDA(c, cub::DeviceScan::ExclusiveSum(tmp.p, tb, kept.p, rp, n + 1, s));
  kCompact<<<blocks, 256, 0, s>>>(rowPtr, colIdx, vals, n, rp, ci, vout);
  PXG_CUDA(c, cudaGetLastError());
  int32_t tot = 0;
  PXG_CUDA(c, cudaMemcpyAsync(&tot, rp + n, 4, cudaMemcpyDeviceToHost, s));
  PXG_CUDA(c, cudaStreamSynchronize(s));
  *nnzOut = tot;
  return PXG_OK;
}
} // namespace pxg

namespace
{
// Candidate thread counts of the autotuner for an element type (0-terminated)
void threadCandidates(pxg_ctx const * c, int (&out)[4])
{
  out[0] = out[1] = out[2] = out[3] = 0;
  bool const fp64 = c->arith == PXG_ARITH_FP64;
  if (c->etype == P1TET || c->etype == P2TET)
    out[0] = 64, out[1] = 128, out[2] = 256;
  else if (c->etype == Q1HEX && !c->q1Generic && !c->q1Thread && (c->q1Group || !fp64))
    out[0] = 256, out[1] = 512;
  else if (c->etype == Q1HEX && !c->q1Generic && !c->q1Thread)
    out[0] = 64, out[1] = 128;
  else
    out[0] = 128;
}
} // namespace

extern "C"
{

pxg_status pxg_assemble(pxg_ctx * c, pxg_lhs_op const * op0, double * vals0, pxg_lhs_op const * op1,
                        double * vals1, pxg_rhs_op const * rhs, double * b, unsigned flags, void * stream)
{
  if (!c)
    return PXG_ERR_INVALID_ARG;
  if (!c->rowPtr.p)
    return fail(c, PXG_ERR_INVALID_ARG, "build the pattern first");
  cudaStream_t const s = (cudaStream_t)stream;
  AsmArgs a{};
  a.nelem = c->nelem;
  a.xyz = c->xyz.p;
  a.conn = c->conn.p;
  a.emap = c->emap.p;
  a.rowPtr = c->rowPtr.p;
  a.rank = c->rank.p;
  a.kE = c->hasCoef ? c->kE.p : nullptr;
  a.bcMask = c->nbc ? c->bcMask.p : nullptr;
  a.bcVal = c->nbc ? c->bcVal.p : nullptr;
  a.bcDiag = c->bcDiag;
  pxg_lhs_op const * ops[2] = {op0, op1};
  double * outs[2] = {vals0, vals1};
  bool any = false;
  for (int m = 0; m < 2; ++m)
  {
    if (!ops[m])
      continue;
    pxg_lhs_op const & o = *ops[m];
    if (o.stiffness < 0 || o.stiffness > 2 || o.mass < 0 || o.mass > 2)
      return fail(c, PXG_ERR_INVALID_ARG, "lhs op %d: bad stiffness/mass kind", m);
    if (!outs[m])
      return fail(c, PXG_ERR_INVALID_ARG, "lhs op %d has no output array", m);
    if ((o.stiffness == 2 || o.mass == 2) && !c->hasCoef)
      return fail(c, PXG_ERR_INVALID_ARG, "lhs op %d needs the per-element coefficient (pxg_set_coef)", m);
    a.op[m] = LhsDev{1, o.stiffness, o.mass, o.apply_bc, o.stiff_coef, o.mass_coef, outs[m]};
    any = true;
  }
  if (rhs && rhs->kind)
  {
    if (rhs->kind < 0 || rhs->kind > 3)
      return fail(c, PXG_ERR_INVALID_ARG, "rhs kind %d", rhs->kind);
    if (rhs->kind == 3 && !rhs->field)
      return fail(c, PXG_ERR_INVALID_ARG, "rhs kind 3 needs the values at the quadrature points");
    if (rhs->kind == 1 && (rhs->fn < 0 || rhs->fn > PXG_FN_COORD_Z))
      return fail(c, PXG_ERR_INVALID_ARG, "unknown analytic function %d", rhs->fn);
    if (rhs->kind == 2 && !rhs->field)
      return fail(c, PXG_ERR_INVALID_ARG, "projection needs a field");
    if (!b)
      return fail(c, PXG_ERR_INVALID_ARG, "rhs op has no output vector");
    a.rkind = rhs->kind;
    a.fn = rhs->fn;
    a.rc = rhs->coef;
    a.field = rhs->field;
    a.rbc = rhs->apply_bc;
    any = true;
  }
  a.b = b;
  if (!any)
    return PXG_OK;
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  for (int m = 0; m < 2; ++m)
    if (a.op[m].on)
      recordRecipe(c, outs[m], *ops[m], (flags & PXG_ACCUMULATE) != 0);
  if (!(flags & PXG_ACCUMULATE))
  {
    // the default FP64 element kernels in element order, outside a stream capture: a
    // zeroing kernel that the element kernel overlaps (its blocks compute while the
    // outputs are zeroed, and wait before they write); otherwise memsets.  Measured
    // against the memsets: P1 16^3 x 6 0.033 -> 0.025 ms (one launch fewer), Q1 128^3
    // 5.14 -> 5.13 ms, Q2 48^3 equal; P2 64^3 x 6 1.41 -> 1.43 ms, so P2 keeps memsets
    bool const fp64 = c->arith == PXG_ARITH_FP64;
    bool const pdlOk = fp64 && c->zeroOverlap && c->scatter == PXG_SCATTER_REDUCE &&
                       ((c->etype == Q1HEX && !c->q1Generic && !c->q1Thread && !c->q1Group) ||
                        (c->etype == P1TET && !c->tetGeneric) || (c->etype == Q2HEX && !c->q2Generic));
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (pdlOk)
      PXG_CUDA(c, cudaStreamIsCapturing(s, &cs));
    if (pdlOk && cs == cudaStreamCaptureStatusNone)
    {
      kZeroOutputs<<<(unsigned)(2 * c->sms), 256, 0, s>>>(a.op[0].on ? a.op[0].vals : nullptr,
                                                          a.op[1].on ? a.op[1].vals : nullptr, c->nnz, b,
                                                          b ? c->ndof : 0);
      PXG_CUDA(c, cudaGetLastError());
      a.pdl = 1;
    }
    else
    {
      for (int m = 0; m < 2; ++m)
        if (a.op[m].on)
          PXG_CUDA(c, cudaMemsetAsync(a.op[m].vals, 0, (size_t)c->nnz * 8, s));
      if (b)
        PXG_CUDA(c, cudaMemsetAsync(b, 0, (size_t)c->ndof * 8, s));
    }
  }
  // rhs kind 3 (values at the quadrature points) runs in the per-quadrature-point FP64
  // kernel, after the element kernel has done the matrices and their BC lifts
  auto launchValuesLoad = [&](AsmArgs const & la) {
    AsmArgs l2 = la;
    l2.op[0].on = l2.op[1].on = 0;
    switch (c->etype)
    {
    case P1TET:
      launchAssemble<P1TET>(l2, s, 0);
      break;
    case P2TET:
      launchAssemble<P2TET>(l2, s, 0);
      break;
    case Q1HEX:
      launchAssemble<Q1HEX>(l2, s, 0);
      break;
    case Q2HEX:
      launchAssemble<Q2HEX>(l2, s, 0);
      break;
    }
  };
  auto launchElem = [&](AsmArgs const & la) {
    bool const fp64 = c->arith == PXG_ARITH_FP64;
    switch (c->etype)
    {
    case P1TET:
      if (c->tetGeneric)
        launchAssemble<P1TET>(la, s, c->threads);
      else if (fp64)
        launchAssembleTet64<P1TET>(la, s, c->threads);
      else
        launchAssembleTet<P1TET>(la, s, c->threads);
      break;
    case P2TET:
      if (c->tetGeneric)
        launchAssemble<P2TET>(la, s, c->threads);
      else if (fp64)
      {
        AsmArgs lg = la;
        if (!la.perm && c->groups.built && c->groupScatter)
        {
          lg.grpOff = c->groups.off.p;
          lg.grpPos = c->groups.pos.p;
          lg.grpBeg = c->groups.beg.p;
          lg.grpItem = c->groups.item.p;
          lg.grpRedMax = c->groupRedMax;
        }
        // the warp-group scatter's shared memory favours small blocks (64 threads: ten
        // warps per SM), so that is its default
        launchAssembleTet64<P2TET>(lg, s, c->threads ? c->threads : (lg.grpOff ? 64 : 128));
      }
      else
        launchAssembleTet<P2TET>(la, s, c->threads);
      break;
    case Q1HEX:
      if (c->q1Generic)
        launchAssemble<Q1HEX>(la, s, c->threads);
      else if (c->q1Thread || c->q1Group || !fp64)
        launchAssembleQ1(la, s, fp64, c->q1Thread, c->threads);
      else
        launchAssembleQ1F64(la, s, c->threads);
      break;
    case Q2HEX:
      if (c->q2Generic)
        launchAssemble<Q2HEX>(la, s, c->threads);
      else if (fp64)
        launchAssembleQ2F64(la, s);
      else
        launchAssembleQ2(la, s, c->sms);
      break;
    }
  };
  auto launch = [&](AsmArgs const & la) {
    if (la.rkind != 3)
      return launchElem(la);
    if (la.op[0].on || la.op[1].on)
    {
      AsmArgs l1 = la;
      l1.rkind = 0;
      launchElem(l1);
    }
    launchValuesLoad(la);
  };
  // the warp-group scatter map of the P2 FP64 kernel, on first use outside a capture
  // (inside one, the kernel adds its entries one by one)
  if (c->etype == P2TET && c->arith == PXG_ARITH_FP64 && c->scatter == PXG_SCATTER_REDUCE && c->groupScatter &&
      !c->tetGeneric && !c->groups.built && (a.op[0].on || a.op[1].on))
  {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    PXG_CUDA(c, cudaStreamIsCapturing(s, &cs));
    if (cs == cudaStreamCaptureStatusNone && buildScatterGroups(c) != PXG_OK)
    {
      // no room for the map (its build holds ~2.7 KB per element for a moment): this
      // context adds its entries one by one, the same sums in another order
      cudaGetLastError();
      c->groups.reset();
      c->groupScatter = false;
      c->err.clear();
    }
  }
  if (c->scatter == PXG_SCATTER_COLOUR)
  {
    if (!c->colour.built)
    {
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      PXG_CUDA(c, cudaStreamIsCapturing(s, &cs));
      if (cs != cudaStreamCaptureStatusNone)
        return fail(c, PXG_ERR_INVALID_ARG, "the colour-ordered scatter needs its colouring before a stream capture");
      if ((st = buildColouring(c)) != PXG_OK)
        return st;
    }
    // one launch per colour class, in colour order
    for (int k = 0; k < c->colour.ncol; ++k)
    {
      AsmArgs la = a;
      la.perm = c->colour.perm.p;
      la.permBase = c->colour.start[k];
      la.nelem = c->colour.start[k + 1] - c->colour.start[k];
      if (la.nelem > 0)
        launch(la);
    }
  }
  else
    launch(a);
  PXG_CUDA(c, cudaGetLastError());
  return PXG_OK;
}

pxg_status pxg_set_scatter(pxg_ctx * c, int scatter, int threads)
{
  if (!c || (scatter != PXG_SCATTER_REDUCE && scatter != PXG_SCATTER_COLOUR))
    return PXG_ERR_INVALID_ARG;
  if (c->etype < 0)
    return fail(c, PXG_ERR_INVALID_ARG, "set the mesh first");
  if (threads)
  {
    int cand[4];
    threadCandidates(c, cand);
    bool ok = false;
    for (int t : cand)
      ok = ok || (t && t == threads);
    if (!ok)
      return fail(c, PXG_ERR_INVALID_ARG, "%d threads per block is not a variant of this element kernel", threads);
  }
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  if (scatter == PXG_SCATTER_COLOUR && (st = buildColouring(c)) != PXG_OK)
    return st;
  c->scatter = scatter;
  c->threads = threads;
  return PXG_OK;
}

pxg_status pxg_set_arithmetic(pxg_ctx * c, int arith)
{
  if (!c)
    return PXG_ERR_INVALID_ARG;
  if (arith != PXG_ARITH_FP64 && arith != PXG_ARITH_DFL)
    return fail(c, PXG_ERR_INVALID_ARG, "arithmetic %d", arith);
  c->arith = arith;
  c->threads = 0;
  return PXG_OK;
}

pxg_status pxg_colouring(pxg_ctx * c, int * ncolours, uint32_t * order, int64_t * offsets)
{
  if (!c || !ncolours)
    return PXG_ERR_INVALID_ARG;
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  if ((st = buildColouring(c)) != PXG_OK)
    return st;
  *ncolours = c->colour.ncol;
  if (order)
    PXG_CUDA(c, cudaMemcpy(order, c->colour.perm.p, (size_t)c->nelem * 4, cudaMemcpyDeviceToHost));
  if (offsets)
    for (int k = 0; k <= c->colour.ncol; ++k)
      offsets[k] = c->colour.start[k];
  return PXG_OK;
}

pxg_status pxg_autotune(pxg_ctx * c, pxg_lhs_op const * op0, pxg_lhs_op const * op1, pxg_rhs_op const * rhs,
                        pxg_tune_report * rep)
{
  if (!c || !rep)
    return PXG_ERR_INVALID_ARG;
  if (!c->rowPtr.p)
    return fail(c, PXG_ERR_INVALID_ARG, "build the pattern first");
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  // scratch outputs
  DevBuf<double> v0, v1, bb;
  if (op0)
    PXG_CUDA(c, v0.alloc(c->nnz));
  if (op1)
    PXG_CUDA(c, v1.alloc(c->nnz));
  if (rhs && rhs->kind)
    PXG_CUDA(c, bb.alloc(c->ndof));
  int cand[4];
  threadCandidates(c, cand);
  bool const colourOk = buildColouring(c) == PXG_OK;
  int const keepScatter = c->scatter, keepThreads = c->threads;
  cudaStream_t s = nullptr;
  PXG_CUDA(c, cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  PXG_CUDA(c, cudaEventCreate(&e0));
  PXG_CUDA(c, cudaEventCreate(&e1));
  *rep = pxg_tune_report{};
  rep->ncolours = colourOk ? c->colour.ncol : 0;
  double best = 1e300;
  int bestT = keepThreads, bestS = keepScatter;
  st = PXG_OK;
  for (int sc = 0; sc < 2 && st == PXG_OK; ++sc)
  {
    if (sc == PXG_SCATTER_COLOUR && !colourOk)
      continue;
    for (int t : cand)
    {
      if (!t || rep->ncand >= 16 || st != PXG_OK)
        break;
      c->scatter = sc;
      c->threads = t;
      auto run = [&] { return pxg_assemble(c, op0, v0.p, op1, v1.p, rhs, bb.p, 0u, s); };
      if ((st = run()) != PXG_OK) // warm-up
        break;
      constexpr int kReps = 3;
      cudaEventRecord(e0, s);
      for (int r = 0; r < kReps && st == PXG_OK; ++r)
        st = run();
      cudaEventRecord(e1, s);
      if (cudaEventSynchronize(e1) != cudaSuccess)
        st = cudaFail(c, cudaGetLastError(), "autotune");
      if (st != PXG_OK)
        break;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      double const per = ms / kReps;
      rep->cand_threads[rep->ncand] = t;
      rep->cand_scatter[rep->ncand] = sc;
      rep->cand_ms[rep->ncand] = per;
      ++rep->ncand;
      if (per < best)
      {
        best = per;
        bestT = t;
        bestS = sc;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  c->scatter = st == PXG_OK ? bestS : keepScatter;
  c->threads = st == PXG_OK ? bestT : keepThreads;
  rep->threads = c->threads;
  rep->scatter = c->scatter;
  return st;
}

pxg_status pxg_prune_count(pxg_ctx * c, double const * vals, int64_t * pruned, void * stream)
{
  if (!c || !vals || !pruned)
    return PXG_ERR_INVALID_ARG;
  if (!c->rowPtr.p)
    return fail(c, PXG_ERR_INVALID_ARG, "no pattern built");
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  cudaStream_t const s = (cudaStream_t)stream;
  PXG_CUDA(c, cudaMemsetAsync(c->counter.p, 0, 8, s));
  kPruneCount<<<152 * 8, 256, 0, s>>>(vals, c->nnz, c->counter.p);
  PXG_CUDA(c, cudaGetLastError());
  unsigned long long h = 0;
  PXG_CUDA(c, cudaMemcpyAsync(&h, c->counter.p, 8, cudaMemcpyDeviceToHost, s));
  PXG_CUDA(c, cudaStreamSynchronize(s));
  *pruned = (int64_t)h;
  return PXG_OK;
}

pxg_status pxg_prune_count_device(pxg_ctx * c, double const * vals, int64_t * pruned_dev, void * stream)
{
  if (!c || !vals || !pruned_dev)
    return PXG_ERR_INVALID_ARG;
  if (!c->rowPtr.p)
    return fail(c, PXG_ERR_INVALID_ARG, "no pattern built");
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  cudaStream_t const s = (cudaStream_t)stream;
  auto * cnt = reinterpret_cast<unsigned long long *>(pruned_dev);
  PXG_CUDA(c, cudaMemsetAsync(cnt, 0, 8, s));
  kPruneCount<<<152 * 8, 256, 0, s>>>(vals, c->nnz, cnt);
  PXG_CUDA(c, cudaGetLastError());
  return PXG_OK;
}

pxg_status pxg_close_matrix(pxg_ctx * c, double const * vals, int32_t * rp, int32_t * ci, double * vout,
                            int64_t * nnzOut, void * stream)
{
  if (!c || !vals || !rp || !ci || !vout || !nnzOut)
    return PXG_ERR_INVALID_ARG;
  if (!c->rowPtr.p)
    return fail(c, PXG_ERR_INVALID_ARG, "no pattern built");
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  cudaStream_t const s = (cudaStream_t)stream;
  // an array this context assembled, on unchanged data: its near-zero entries are
  // recomputed in the reference's evaluation order before the prune
  pxg_ctx::Recipe const * R = nullptr;
  for (auto const & r: c->recipes)
    if (r.vals == vals && r.valid && r.meshVer == c->meshVer && r.coefVer == c->coefVer && r.bcVer == c->bcVer)
      R = &r;
  if (!R)
    return closeCsr(c, c->rowPtr.p, c->colIdx.p, c->ndof, vals, rp, ci, vout, nnzOut, s);
  int64_t const n = c->ndof;
  unsigned const bn = (unsigned)((n + 127) / 128);
  PXG_CUDA(c, cudaMemsetAsync(c->counter.p, 0, 8, s));
  kFlagNearZero<<<bn, 128, 0, s>>>(c->rowPtr.p, vals, n, c->counter.p, nullptr, nullptr, 0);
  unsigned long long nf = 0;
  PXG_CUDA(c, cudaMemcpyAsync(&nf, c->counter.p, 8, cudaMemcpyDeviceToHost, s));
  PXG_CUDA(c, cudaStreamSynchronize(s));
  if (nf == 0)
    return closeCsr(c, c->rowPtr.p, c->colIdx.p, n, vals, rp, ci, vout, nnzOut, s);
  if ((st = ensureDofElem(c)) != PXG_OK)
    return st;
  DevBuf<double> fixed;
  DevBuf<int64_t> pos;
  DevBuf<int32_t> row;
  PXG_CUDA(c, fixed.alloc(c->nnz));
  PXG_CUDA(c, pos.alloc(nf));
  PXG_CUDA(c, row.alloc(nf));
  PXG_CUDA(c, cudaMemcpyAsync(fixed.p, vals, c->nnz * 8, cudaMemcpyDeviceToDevice, s));
  PXG_CUDA(c, cudaMemsetAsync(c->counter.p, 0, 8, s));
  kFlagNearZero<<<bn, 128, 0, s>>>(c->rowPtr.p, vals, n, c->counter.p, pos.p, row.p, (int64_t)nf);
  RepairArgs ra{};
  ra.xyz = c->xyz.p;
  ra.conn = c->conn.p;
  ra.emap = c->emap.p;
  ra.rowPtr = c->rowPtr.p;
  ra.colIdx = c->colIdx.p;
  ra.kE = c->hasCoef ? c->kE.p : nullptr;
  ra.bcMask = c->nbc ? c->bcMask.p : nullptr;
  ra.bcDiag = c->bcDiag;
  ra.dofElemPtr = c->dofElemPtr.p;
  ra.dofElem = c->dofElem.p;
  ra.nops = (int)R->ops.size();
  for (int o = 0; o < ra.nops; ++o)
    ra.ops[o] = RefOp{R->ops[o].stiff, R->ops[o].mass, R->ops[o].bc, R->ops[o].sc, R->ops[o].mc};
  ra.flagged = pos.p;
  ra.flaggedRow = row.p;
  ra.nflagged = (int64_t)nf;
  ra.vals = fixed.p;
  unsigned const bf = (unsigned)((nf + 127) / 128);
  switch (c->etype)
  {
  case P1TET:
    kRepairEntries<P1TET><<<bf, 128, 0, s>>>(ra);
    break;
  case P2TET:
    kRepairEntries<P2TET><<<bf, 128, 0, s>>>(ra);
    break;
  case Q1HEX:
    kRepairEntries<Q1HEX><<<bf, 128, 0, s>>>(ra);
    break;
  case Q2HEX:
    kRepairEntries<Q2HEX><<<bf, 128, 0, s>>>(ra);
    break;
  }
  PXG_CUDA(c, cudaGetLastError());
  return closeCsr(c, c->rowPtr.p, c->colIdx.p, n, fixed.p, rp, ci, vout, nnzOut, s);
}

pxg_status pxg_get_qpoints(pxg_ctx * c, double * qpts, int mem, void * stream)
{
  if (!c || !qpts)
    return PXG_ERR_INVALID_ARG;
  if (c->etype < 0)
    return fail(c, PXG_ERR_INVALID_ARG, "set the mesh first");
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  cudaStream_t const s = (cudaStream_t)stream;
  size_t const count = (size_t)c->nelem * numQpts(c->etype) * 3;
  DevBuf<double> tmp;
  double * out = qpts;
  if (mem == PXG_MEM_HOST)
  {
    PXG_CUDA(c, tmp.alloc(count));
    out = tmp.p;
  }
  unsigned const blocks = (unsigned)((c->nelem + 127) / 128);
  switch (c->etype)
  {
  case P1TET:
    kQpoints<P1TET><<<blocks, 128, 0, s>>>(c->nelem, c->xyz.p, c->conn.p, out);
    break;
  case P2TET:
    kQpoints<P2TET><<<blocks, 128, 0, s>>>(c->nelem, c->xyz.p, c->conn.p, out);
    break;
  case Q1HEX:
    kQpoints<Q1HEX><<<blocks, 128, 0, s>>>(c->nelem, c->xyz.p, c->conn.p, out);
    break;
  case Q2HEX:
    kQpoints<Q2HEX><<<blocks, 128, 0, s>>>(c->nelem, c->xyz.p, c->conn.p, out);
    break;
  }
  PXG_CUDA(c, cudaGetLastError());
  if (mem == PXG_MEM_HOST)
  {
    PXG_CUDA(c, cudaMemcpyAsync(qpts, out, count * 8, cudaMemcpyDeviceToHost, s));
    PXG_CUDA(c, cudaStreamSynchronize(s));
  }
  return PXG_OK;
}

pxg_status pxg_interpolate(pxg_ctx * c, int fn, double coef, double * v, void * stream)
{
  if (!c || !v)
    return PXG_ERR_INVALID_ARG;
  if (!c->emap.p)
    return fail(c, PXG_ERR_INVALID_ARG, "no DOF map");
  if (fn < 0 || fn > PXG_FN_COORD_Z)
    return fail(c, PXG_ERR_INVALID_ARG, "unknown analytic function %d", fn);
  pxg_status st = ensureDevice(c);
  if (st != PXG_OK)
    return st;
  cudaStream_t const s = (cudaStream_t)stream;
  unsigned const blocks = (unsigned)((c->nelem + 127) / 128);
  switch (c->etype)
  {
  case P1TET:
    kInterpolate<P1TET><<<blocks, 128, 0, s>>>(c->nelem, c->xyz.p, c->conn.p, c->emap.p, fn, coef, v);
    break;
  case P2TET:
    kInterpolate<P2TET><<<blocks, 128, 0, s>>>(c->nelem, c->xyz.p, c->conn.p, c->emap.p, fn, coef, v);
    break;
  case Q1HEX:
    kInterpolate<Q1HEX><<<blocks, 128, 0, s>>>(c->nelem, c->xyz.p, c->conn.p, c->emap.p, fn, coef, v);
    break;
  case Q2HEX:
    kInterpolate<Q2HEX><<<blocks, 128, 0, s>>>(c->nelem, c->xyz.p, c->conn.p, c->emap.p, fn, coef, v);
    break;
  }
  PXG_CUDA(c, cudaGetLastError());
  return PXG_OK;
}

} // extern "C"
