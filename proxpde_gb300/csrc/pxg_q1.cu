// Q1 hexahedron element kernel with the 2x2x2 Gauss rule, written for GB300's FP64
// rate (about 1.2 TFLOP/s, 1/64 of FP32).  It computes the element matrices of
// proxpde's CurFE + AssemblyStiffness(FE) + AssemblyMass + AssemblyRhsAnalytic
// (include/curfe.hpp:50-103, include/assembly_lhs.hpp:52-109, 207-221,
// include/assembly_rhs.hpp:61-88) in two steps that cut the FP64 work:
//  1. the tensor-product structure of Q1 on the 2x2x2 rule (below) needs about
//     2,000 arithmetic operations per element instead of about 4,100;
//  2. those operations run in double-float arithmetic (pxg_dfl.h) on the FP32 pipe
//     (T = dfl); the FP64 pipe keeps the edge differences, the element-origin
//     sincospi and the final hi + lo sums.  T = double gives the plain FP64 kernel.
//
// Notation: a node or a quadrature point is a triple (x, y, z) in {0,1}^3.
//   1D factors at the Gauss points xi = -g, +g (g = 0.5773502691896258, src/qr.cpp:27):
//   l_a(q) = 0.5 (1 -+ xi_q)  ->  l_a(q) = A if a == q else B,  A = (1+g)/2, B = (1-g)/2
//   l'_a = -1/2 (a = 0), +1/2 (a = 1).
//   grad phi_n(q) = ( l'_nx l_ny(qy) l_nz(qz),  l_nx(qx) l'_ny l_nz(qz),  l_nx(qx) l_ny(qy) l'_nz ).
// Jacobian: column x of J depends on (qy, qz) only; it is the bilinear interpolation
//   of the x-edge differences X(1,y,z) - X(0,y,z) (times 1/2); likewise for y and z.
// Stiffness: with G_q = adj(J_q) adj(J_q)^T / (4 |det J_q|) (the 1/4 is l' l'),
//   K_ij = sum_q sum_ab G_q,ab d_a(i,q) d_b(j,q) splits into per-axis contractions:
//   diagonal terms S_x[c(iy,jy)][c(iz,jz)] = sum_q G_q,xx W_c(qy) W_c'(qz) and cross
//   terms U_xy[jx][iy][c(iz,jz)] = sum_q G_q,xy l_jx(qx) l_iy(qy) W_c(qz) etc., where
//   W_c(q) = l_i(q) l_j(q) depends only on the class c of (i, j): 00, 11 or mixed.
// Mass: M_ij = sum_q |det J_q| W(ix,jx;qx) W(iy,jy;qy) W(iz,jz;qz) -> a 3x3x3 table.
// Load: f at qpoint = origin + J_q xi_q (the reference's CurFE::qpoint); for small
//   offsets sin(pi(o + d)) = sin(pi o) cos(pi d) + cos(pi o) sin(pi d) with short
//   series for the offset part, else sinpi directly.
#include <type_traits>

#include "pxg_dfl.h"
#include "pxg_internal.h"

namespace pxg
{

namespace q1
{
constexpr double g = 0.5773502691896258;
constexpr double A = 0.5 * (1. + g);
constexpr double B = 0.5 * (1. - g);
constexpr double AA = A * A, BB = B * B, AB = A * B;
constexpr double PI = 3.141592653589793;

// node <-> (x, y, z) of proxpde's Q1 hexahedron (src/reffe.cpp:684-759)
__host__ __device__ constexpr int nx(int n) { return (n == 1 || n == 2 || n == 5 || n == 6) ? 1 : 0; }
__host__ __device__ constexpr int ny(int n) { return (n == 2 || n == 3 || n == 6 || n == 7) ? 1 : 0; }
__host__ __device__ constexpr int nz(int n) { return n >= 4 ? 1 : 0; }
__host__ __device__ constexpr int node(int x, int y, int z)
{
  return z * 4 + (y ? (x ? 2 : 3) : (x ? 1 : 0));
}
// class of a pair of 1D indices: 0 = (0,0), 1 = (1,1), 2 = mixed
__host__ __device__ constexpr int cls(int a, int b) { return a == b ? a : 2; }
// l_a(q)
__host__ __device__ constexpr double L(int a, int q) { return a == q ? A : B; }

// Unroll factor of the outer loops: the FP64 variant unrolls everything; the
// double-float variant keeps loops, because its fully unrolled code (~27k
// instructions per element) does not fit the instruction cache (ncu: most stalls
// were "no instruction").
template <typename T>
constexpr int kFull(int n)
{
  return std::is_same_v<T, double> ? n : 1;
}

// 2-point contraction of a pair (v0 at q = 0, v1 at q = 1) with l_a
template <typename T>
__device__ __forceinline__ T cL(int a, T v0, T v1)
{
  return a == 0 ? cst<T>(A) * v0 + cst<T>(B) * v1 : cst<T>(B) * v0 + cst<T>(A) * v1;
}
// ... with W_c = l_i l_j of class c
template <typename T>
__device__ __forceinline__ T cW(int c, T v0, T v1)
{
  return c == 2 ? cst<T>(AB) * (v0 + v1)
                : (c == 0 ? cst<T>(AA) * v0 + cst<T>(BB) * v1 : cst<T>(BB) * v0 + cst<T>(AA) * v1);
}
// k += sign * v, sign = l'_a l'_b / (1/4) = +1 if a == b else -1
template <typename T>
__device__ __forceinline__ void addSgn(T & k, int a, int b, T v)
{
  if (a == b)
    k = k + v;
  else
    k = k - v;
}

// sin(pi x) near a point whose sincospi is known: x = o + d
__device__ __forceinline__ double sinpiNear(double so, double co, double o, double d)
{
  double const u = PI * d;
  if (fabs(u) < 0.05)
  {
    double const u2 = u * u;
    // sin u = u (1 - u^2/6 + u^4/120 - u^6/5040), cos u = 1 - u^2/2 + u^4/24 - u^6/720 + u^8/40320
    double const s = u * fma(u2, fma(u2, fma(u2, -1.0 / 5040.0, 1.0 / 120.0), -1.0 / 6.0), 1.0);
    double const c = fma(u2, fma(u2, fma(u2, fma(u2, 1.0 / 40320.0, -1.0 / 720.0), 1.0 / 24.0), -0.5), 1.0);
    return fma(so, c, co * s);
  }
  return sinpi(o + d);
}
// The same in double-float.  For |u| < 0.05 the terms u^4/120 (< 6e-8) and beyond,
// and u^4/24 (< 3e-7) and beyond, are needed to 1e-14 absolute only, which float
// arithmetic gives; u^2/6 and u^2/2 are kept in double-float.
__device__ __forceinline__ dfl sinpiNear(dfl so, dfl co, double o, dfl d)
{
  dfl const u = cst<dfl>(PI) * d;
  if (fabsf(u.h) < 0.05f)
  {
    dfl const u2 = u * u;
    float const v = u2.h;
    float const hs = v * v * (1.f / 120.f - v * (1.f / 5040.f));
    float const hc = v * v * (1.f / 24.f - v * (1.f / 720.f - v * (1.f / 40320.f)));
    dfl const es = dfl{hs, 0.f} - u2 * cst<dfl>(1.0 / 6.0); // sin u = u (1 + es)
    dfl const c = (cst<dfl>(1.0) - dfl{0.5f * u2.h, 0.5f * u2.l}) + dfl{hc, 0.f};
    dfl const s = u + u * es;
    return so * c + co * s;
  }
  return toDfl(sinpi(o + toDouble(d)));
}

// Per-element geometry at the 8 Gauss points: G[0..5][q] = xx yy zz xy xz yz entries
// of adj(J) adj(J)^T / (4 |det J|), ad[q] = |det J_q|, off[q] = J_q xi_q.
template <typename T>
struct Q1Geo
{
  T G[6][8];
  T ad[8];
  T off[8][3];
};

template <typename T>
__device__ __forceinline__ void q1Geometry(double const (&X)[8][3], Q1Geo<T> & geo)
{
  // Jacobian columns: Jc[axis][p][t][r] with p, t the quadrature coordinates of the
  // two other axes in increasing order and r the physical coordinate; column `axis`
  // of J is the bilinear interpolation of half the edge differences along it.  The
  // differences are taken in FP64, then converted.
  T Jc[3][2][2][3];
  constexpr int RU = kFull<T>(3), QU = kFull<T>(8);
#pragma unroll RU
  for (int r = 0; r < 3; ++r)
  {
    T dd[3][2][2];
#pragma unroll
    for (int s = 0; s < 2; ++s)
#pragma unroll
      for (int t = 0; t < 2; ++t)
      {
        dd[0][s][t] = fromDouble<T>(X[node(1, s, t)][r] - X[node(0, s, t)][r]); // along x, at (y, z)
        dd[1][s][t] = fromDouble<T>(X[node(s, 1, t)][r] - X[node(s, 0, t)][r]); // along y, at (x, z)
        dd[2][s][t] = fromDouble<T>(X[node(s, t, 1)][r] - X[node(s, t, 0)][r]); // along z, at (x, y)
      }
#pragma unroll
    for (int ax = 0; ax < 3; ++ax)
    {
      T h[2][2];
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int t = 0; t < 2; ++t)
          h[p][t] = cst<T>(0.5 * L(0, p)) * dd[ax][0][t] + cst<T>(0.5 * L(1, p)) * dd[ax][1][t];
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int t = 0; t < 2; ++t)
          Jc[ax][p][t][r] = cst<T>(L(0, t)) * h[p][0] + cst<T>(L(1, t)) * h[p][1];
    }
  }
#pragma unroll QU
  for (int q = 0; q < 8; ++q)
  {
    int const qx = q & 1, qy = (q >> 1) & 1, qz = q >> 2;
    T J[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
    {
      J[r][0] = Jc[0][qy][qz][r];
      J[r][1] = Jc[1][qx][qz][r];
      J[r][2] = Jc[2][qx][qy][r];
    }
    T C[3][3]; // adj(J) = J^-1 det J
    C[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    C[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    C[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    C[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    C[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
    C[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
    C[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    C[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
    C[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    T const det = J[0][0] * C[0][0] + J[0][1] * C[1][0] + J[0][2] * C[2][0];
    T const adet = fabs(det);
    geo.ad[q] = adet;
    T const s = cst<T>(0.25) * rcp(adet);
    geo.G[0][q] = s * (C[0][0] * C[0][0] + C[0][1] * C[0][1] + C[0][2] * C[0][2]);
    geo.G[1][q] = s * (C[1][0] * C[1][0] + C[1][1] * C[1][1] + C[1][2] * C[1][2]);
    geo.G[2][q] = s * (C[2][0] * C[2][0] + C[2][1] * C[2][1] + C[2][2] * C[2][2]);
    geo.G[3][q] = s * (C[0][0] * C[1][0] + C[0][1] * C[1][1] + C[0][2] * C[1][2]);
    geo.G[4][q] = s * (C[0][0] * C[2][0] + C[0][1] * C[2][1] + C[0][2] * C[2][2]);
    geo.G[5][q] = s * (C[1][0] * C[2][0] + C[1][1] * C[2][1] + C[1][2] * C[2][2]);
    T const xq = cst<T>(qx ? g : -g), yq = cst<T>(qy ? g : -g), zq = cst<T>(qz ? g : -g);
#pragma unroll
    for (int r = 0; r < 3; ++r)
      geo.off[q][r] = J[r][0] * xq + J[r][1] * yq + J[r][2] * zq;
  }
}

// Element stiffness with unit coefficient (upper triangle j >= i of Kl).
template <typename T>
__device__ __forceinline__ void q1Stiffness(Q1Geo<T> const & geo, T (&Kl)[8][8])
{
  // diagonal-direction tables S_a[c1][c2] (c1, c2 = classes of the two other axes)
  constexpr int AU = kFull<T>(3), IU = kFull<T>(8);
  T S[3][3][3];
#pragma unroll AU
  for (int ax = 0; ax < 3; ++ax)
  {
    // sum over the derivative axis, then contract the two others with W
    T H[2][2]; // [p][t] over the remaining axes in increasing order
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
      for (int t = 0; t < 2; ++t)
      {
        int q0, q1; // quadrature points are numbered x fastest: q = qx + 2 qy + 4 qz
        if (ax == 0)
          q0 = 2 * p + 4 * t, q1 = 1 + 2 * p + 4 * t;
        else if (ax == 1)
          q0 = p + 4 * t, q1 = p + 2 + 4 * t;
        else
          q0 = p + 2 * t, q1 = p + 2 * t + 4;
        H[p][t] = geo.G[ax][q0] + geo.G[ax][q1];
      }
    T R[2][3];
#pragma unroll
    for (int p = 0; p < 2; ++p)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        R[p][c] = cW<T>(c, H[p][0], H[p][1]);
#pragma unroll
    for (int c1 = 0; c1 < 3; ++c1)
#pragma unroll
      for (int c2 = 0; c2 < 3; ++c2)
        S[ax][c1][c2] = cW<T>(c1, R[0][c2], R[1][c2]);
  }
  // cross tables, generic in the axis pair (a < b), third axis t:
  //   U_ab[first index][second index][class], entries sum_q G_ab l(qa) l(qb) W(qt)
  T U[3][2][2][3]; // pair 0 = xy, 1 = xz, 2 = yz
#pragma unroll AU
  for (int pr = 0; pr < 3; ++pr)
  {
    int const axA = pr == 2 ? 1 : 0, axB = pr == 0 ? 1 : 2;
    int const axT = 3 - axA - axB;
    auto qidx = [&](int va, int vb, int vt) {
      int c[3];
      c[axA] = va, c[axB] = vb, c[axT] = vt;
      return c[0] + 2 * c[1] + 4 * c[2];
    };
    T V[2][2][3]; // [qa][qb][class of the third axis]
#pragma unroll
    for (int qa = 0; qa < 2; ++qa)
#pragma unroll
      for (int qb = 0; qb < 2; ++qb)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          V[qa][qb][c] = cW<T>(c, geo.G[3 + pr][qidx(qa, qb, 0)], geo.G[3 + pr][qidx(qa, qb, 1)]);
    T Y[2][2][3]; // [qa][b][c]
#pragma unroll
    for (int qa = 0; qa < 2; ++qa)
#pragma unroll
      for (int bb = 0; bb < 2; ++bb)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          Y[qa][bb][c] = cL<T>(bb, V[qa][0][c], V[qa][1][c]);
#pragma unroll
    for (int aa = 0; aa < 2; ++aa)
#pragma unroll
      for (int bb = 0; bb < 2; ++bb)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          U[pr][aa][bb][c] = cL<T>(aa, Y[0][bb][c], Y[1][bb][c]);
  }
#pragma unroll IU
  for (int i = 0; i < 8; ++i)
#pragma unroll IU
    for (int j = i; j < 8; ++j)
    {
      int const ix = nx(i), iy = ny(i), iz = nz(i), jx = nx(j), jy = ny(j), jz = nz(j);
      int const cx = cls(ix, jx), cy = cls(iy, jy), cz = cls(iz, jz);
      T k = (ix == jx) ? S[0][cy][cz] : -S[0][cy][cz];
      addSgn(k, iy, jy, S[1][cx][cz]);
      addSgn(k, iz, jz, S[2][cx][cy]);
      // D_i,x D_j,y G_xy + D_i,y D_j,x G_yx (third axis z)
      addSgn(k, ix, jy, U[0][jx][iy][cz]);
      addSgn(k, iy, jx, U[0][ix][jy][cz]);
      // x, z (third axis y)
      addSgn(k, ix, jz, U[1][jx][iz][cy]);
      addSgn(k, iz, jx, U[1][ix][jz][cy]);
      // y, z (third axis x)
      addSgn(k, iy, jz, U[2][jy][iz][cx]);
      addSgn(k, iz, jy, U[2][iy][jz][cx]);
      Kl[i][j] = k;
    }
}

// mass table Mt[cx][cy][cz] (unit coefficient)
template <typename T>
__device__ __forceinline__ void q1Mass(T const (&ad)[8], T (&Mt)[3][3][3])
{
  T Vm[2][2][3]; // [qx][qy][cz]
#pragma unroll
  for (int qx = 0; qx < 2; ++qx)
#pragma unroll
    for (int qy = 0; qy < 2; ++qy)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        Vm[qx][qy][c] = cW<T>(c, ad[qx + 2 * qy], ad[qx + 2 * qy + 4]);
  T Ym[2][3][3]; // [qx][cy][cz]
#pragma unroll
  for (int qx = 0; qx < 2; ++qx)
#pragma unroll
    for (int cy = 0; cy < 3; ++cy)
#pragma unroll
      for (int cz = 0; cz < 3; ++cz)
        Ym[qx][cy][cz] = cW<T>(cy, Vm[qx][0][cz], Vm[qx][1][cz]);
#pragma unroll
  for (int cx = 0; cx < 3; ++cx)
#pragma unroll
    for (int cy = 0; cy < 3; ++cy)
#pragma unroll
      for (int cz = 0; cz < 3; ++cz)
        Mt[cx][cy][cz] = cW<T>(cx, Ym[0][cy][cz], Ym[1][cy][cz]);
}

__device__ __forceinline__ void loadVerts(uint32_t const * conn, double const * xyz, int64_t e, double (&X)[8][3])
{
  uint4 const c0 = reinterpret_cast<uint4 const *>(conn)[2 * e];
  uint4 const c1 = reinterpret_cast<uint4 const *>(conn)[2 * e + 1];
  uint32_t const v[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int d = 0; d < 3; ++d)
      X[n][d] = xyz[3 * (int64_t)v[n] + d];
}

__device__ __forceinline__ void loadDofs(uint32_t const * emap, int64_t e, uint32_t (&dof)[8])
{
  uint4 const d0 = reinterpret_cast<uint4 const *>(emap)[2 * e];
  uint4 const d1 = reinterpret_cast<uint4 const *>(emap)[2 * e + 1];
  dof[0] = d0.x, dof[1] = d0.y, dof[2] = d0.z, dof[3] = d0.w;
  dof[4] = d1.x, dof[5] = d1.y, dof[6] = d1.z, dof[7] = d1.w;
}
} // namespace q1

template <typename T>
__global__ void __launch_bounds__(128) kAssembleQ1(AsmArgs a)
{
  using namespace q1;
  int64_t const e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= a.nelem)
    return;

  double X[8][3];
  uint32_t dof[8];
  loadVerts(a.conn, a.xyz, e, X);
  loadDofs(a.emap, e, dof);
  uint32_t cons = 0;
  if (a.bcMask)
  {
#pragma unroll
    for (int i = 0; i < 8; ++i)
      if (a.bcMask[dof[i]])
        cons |= 1u << i;
  }
  double const kfac = a.kE ? a.kE[e] : 1.0;
  bool const needK = (a.op[0].on && a.op[0].stiff) || (a.op[1].on && a.op[1].stiff);
  bool const needM = (a.op[0].on && a.op[0].mass) || (a.op[1].on && a.op[1].mass);

  Q1Geo<T> geo;
  q1Geometry<T>(X, geo);
  T Kl[8][8];
  if (needK)
    q1Stiffness<T>(geo, Kl);
  T Mt[3][3][3];
  if (needM)
    q1Mass<T>(geo.ad, Mt);

  // ---- scatter the matrices (with the Dirichlet condensation, builder.hpp:76-124)
  bool const anyBc = cons && ((a.op[0].on && a.op[0].bc) || (a.op[1].on && a.op[1].bc));
  double lift[2][8];
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int i = 0; i < 8; ++i)
      lift[m][i] = 0.;
  uint16_t const * rk = a.rank + e * 64;
  int32_t rp[8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
    rp[i] = a.rowPtr[dof[i]];
#pragma unroll
  for (int m = 0; m < 2; ++m)
  {
    LhsDev const op = a.op[m];
    if (!op.on)
      continue;
    T const ks = fromDouble<T>(op.stiff ? (op.stiff == 2 ? op.sc * kfac : op.sc) : 0.);
    T const ms = fromDouble<T>(op.mass ? op.mc : 0.);
    constexpr int IU = kFull<T>(8);
#pragma unroll IU
    for (int i = 0; i < 8; ++i)
#pragma unroll IU
      for (int j = i; j < 8; ++j)
      {
        T v = cst<T>(0.0);
        if (op.stiff)
          v = ks * Kl[i][j];
        if (op.mass)
          v = v + ms * Mt[cls(nx(i), nx(j))][cls(ny(i), ny(j))][cls(nz(i), nz(j))];
        double const val = toDouble(v);
        if (anyBc && op.bc)
        {
          bool const ci = (cons >> i) & 1u, cj = (cons >> j) & 1u;
          if (ci || cj)
          {
            if (i == j)
              atomicAdd(op.vals + rp[i] + rk[i * 8 + i], a.bcDiag);
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
        atomicAdd(op.vals + rp[i] + rk[i * 8 + j], val);
        if (j != i)
          atomicAdd(op.vals + rp[j] + rk[j * 8 + i], val);
      }
  }

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
      for (int i = 0; i < 8; ++i)
      {
        double const add = ((cons >> i) & 1u) ? a.bcVal[dof[i]] : lift[m][i];
        if (add != 0.)
          atomicAdd(a.b + dof[i], add);
      }
    }
  }
  if (a.rkind)
  {
    // r_q = |det J_q| f(qpoint_q), then Fe_i = sum_q r_q l_ix(qx) l_iy(qy) l_iz(qz)
    T rq[8];
    if (a.rkind == 1)
    {
      double o[3];
#pragma unroll
      for (int d = 0; d < 3; ++d)
        o[d] = .125 * (X[0][d] + X[1][d] + X[2][d] + X[3][d] + X[4][d] + X[5][d] + X[6][d] + X[7][d]);
      if (a.fn == PXG_FN_SIN3)
      {
        T so[3], co[3];
#pragma unroll
        for (int d = 0; d < 3; ++d)
        {
          double s, c;
          sincospi(o[d], &s, &c);
          so[d] = fromDouble<T>(s);
          co[d] = fromDouble<T>(c);
        }
        T const rc = fromDouble<T>(a.rc);
        constexpr int QU = kFull<T>(8);
#pragma unroll QU
        for (int q = 0; q < 8; ++q)
        {
          T const f = sinpiNear(so[0], co[0], o[0], geo.off[q][0]) * sinpiNear(so[1], co[1], o[1], geo.off[q][1]) *
                      sinpiNear(so[2], co[2], o[2], geo.off[q][2]);
          rq[q] = geo.ad[q] * (rc * f);
        }
      }
      else
      {
#pragma unroll
        for (int q = 0; q < 8; ++q)
          rq[q] = fromDouble<T>(toDouble(geo.ad[q]) * evalFn(a.fn, a.rc, o[0] + toDouble(geo.off[q][0]),
                                                              o[1] + toDouble(geo.off[q][1]),
                                                              o[2] + toDouble(geo.off[q][2])));
      }
    }
    else
    {
      // projection of a DOF field: f_q = coef * sum_n phi_n(q) field_n
      T loc[8];
#pragma unroll
      for (int n = 0; n < 8; ++n)
        loc[n] = fromDouble<T>(a.field[dof[n]]);
      T const rc = fromDouble<T>(a.rc);
#pragma unroll
      for (int q = 0; q < 8; ++q)
      {
        int const qx = q & 1, qy = (q >> 1) & 1, qz = q >> 2;
        T s = cst<T>(0.0);
#pragma unroll
        for (int n = 0; n < 8; ++n)
          s = s + cst<T>(L(nx(n), qx) * L(ny(n), qy) * L(nz(n), qz)) * loc[n];
        rq[q] = geo.ad[q] * (rc * s);
      }
    }
    T Ry[2][2][2]; // [qx][qy][iz]: contract z, then y, then x
#pragma unroll
    for (int qx = 0; qx < 2; ++qx)
#pragma unroll
      for (int qy = 0; qy < 2; ++qy)
#pragma unroll
        for (int iz = 0; iz < 2; ++iz)
          Ry[qx][qy][iz] = cL<T>(iz, rq[qx + 2 * qy], rq[qx + 2 * qy + 4]);
    T Rx[2][2][2]; // [qx][iy][iz]
#pragma unroll
    for (int qx = 0; qx < 2; ++qx)
#pragma unroll
      for (int iy = 0; iy < 2; ++iy)
#pragma unroll
        for (int iz = 0; iz < 2; ++iz)
          Rx[qx][iy][iz] = cL<T>(iy, Ry[qx][0][iz], Ry[qx][1][iz]);
#pragma unroll
    for (int i = 0; i < 8; ++i)
    {
      if (a.rbc && ((cons >> i) & 1u))
        continue;
      int const ix = nx(i), iy = ny(i), iz = nz(i);
      atomicAdd(a.b + dof[i], toDouble(cL<T>(ix, Rx[0][iy][iz], Rx[1][iy][iz])));
    }
  }
}

void launchAssembleQ1(AsmArgs const & a, cudaStream_t s, bool fp64)
{
  unsigned const blocks = (unsigned)((a.nelem + 127) / 128);
  if (fp64)
    kAssembleQ1<double><<<blocks, 128, 0, s>>>(a);
  else
    kAssembleQ1<dfl><<<blocks, 128, 0, s>>>(a);
}

// Adjoint gradient g_e = -(C u)_e^T K_e (C lambda)_e, K_e = k_e K0_e (Q1, 2x2x2 rule):
// the same element stiffness as kAssembleQ1, contracted with the two local vectors.
template <typename T>
__global__ void __launch_bounds__(128) kAdjointGradQ1(AdjArgs a)
{
  using namespace q1;
  int64_t const e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= a.nelem)
    return;
  double X[8][3];
  uint32_t dof[8];
  loadVerts(a.conn, a.xyz, e, X);
  loadDofs(a.emap, e, dof);
  T ue[8], le[8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
  {
    bool const c = a.bcMask && a.bcMask[dof[i]];
    ue[i] = fromDouble<T>(c ? 0. : a.u[dof[i]]);
    le[i] = fromDouble<T>(c ? 0. : a.lam[dof[i]]);
  }
  Q1Geo<T> geo;
  q1Geometry<T>(X, geo);
  T Kl[8][8];
  q1Stiffness<T>(geo, Kl);
  T s = cst<T>(0.0);
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = i; j < 8; ++j)
      s = s + Kl[i][j] * ((i == j) ? ue[i] * le[i] : ue[i] * le[j] + ue[j] * le[i]);
  a.g[e] = -(a.kE[e] * toDouble(s));
}

void launchAdjointGradQ1(AdjArgs const & a, cudaStream_t s, bool fp64)
{
  unsigned const blocks = (unsigned)((a.nelem + 127) / 128);
  if (fp64)
    kAdjointGradQ1<double><<<blocks, 128, 0, s>>>(a);
  else
    kAdjointGradQ1<dfl><<<blocks, 128, 0, s>>>(a);
}

} // namespace pxg
