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

// The direct paths of sinpiNear (offsets beyond the short series), out of line so
// that their FP64 code is not predicated into every call.
__device__ __noinline__ double sinpiFar(double o, double d) { return sinpi(o + d); }
__device__ __noinline__ dfl sinpiFar(double o, dfl d) { return toDfl(sinpi(o + toDouble(d))); }

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
  return sinpiFar(o, d);
}
// The same in double-float.  For |u| < 0.05 the terms u^4/120 (< 6e-8) and beyond,
// and u^4/24 (< 3e-7) and beyond, are needed to 1e-14 absolute only, which float
// arithmetic gives; u^2/6 and u^2/2 are kept in double-float.
__device__ __noinline__ dfl sinpiNear(dfl so, dfl co, double o, dfl d)
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
    return dot2(so, c, co, s);
  }
  return sinpiFar(o, d);
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
  int64_t const i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= a.nelem)
    return;
  int64_t const e = elemOf(a, i);

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
    T const ms = fromDouble<T>(op.mass ? massCoef(op, kfac) : 0.);
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

// =====================================================================================
// Eight lanes per element (the default Q1 kernel).
//
// With one thread per element, the dynamically indexed arrays of the tensor-product
// formulation (about 2 KB a thread) live in local memory. At full occupancy that is
// about 330 MB, beyond the 129 MB L2, and it streams through HBM (ncu: ~5 KB of DRAM
// traffic per element against ~1 KB of algorithmic traffic). Here a group of eight
// lanes takes one element and the element's shared state (1 KB) lives in shared
// memory. Lane l stands for the vertex and the Gauss point at lattice position
// (l & 1, (l >> 1) & 1, l >> 2); proxpde's number of that vertex is l ^ bit1(l).
//  A. lane = Gauss point q: the Jacobian by 2-point transforms across the lanes
//     (shuffles), then adj(J), |det J|, G_q and the offset J_q xi_q;
//  D. the load vector: f at the Gauss point, then the transposed transforms give the
//     node values;
//  B. lane = table job: the eight contractions over q of the tensor-product
//     formulation: S_x, S_y, S_z, U_xy, U_xz, U_yz and the mass tables Sa, Sb with
//     Mt[cx][cy][cz] = alpha_cx Sa[cy][cz] + beta_cx Sb[cy][cz], where
//     W_c(q) = alpha_c + beta_c (-1)^q; one code path with per-lane weights;
//  C. lane = matrix entries: the 36 pairs i <= j dealt round-robin; an entry is a
//     signed sum of nine table values (two more for the mass), scaled per operator
//     and scattered with FP64 reductions.
namespace q1g
{
using namespace q1;

// Threads per block (default; 512 is the autotuner's other candidate: the entry phase
// takes a warp of element slots at a time, so a block holds at least 32 elements).
// The phases end at block barriers: the warps of a block then run the same phase, and
// the SM's instruction cache holds the code of a few phases only (one per resident
// block).  Measured at 128^3 on an earlier form of the kernel (ms per launch): 128
// threads with warp-level syncs 3.11, 128 / 256 / 512 / 1024 threads with block
// barriers 3.03 / 2.77 / 3.09 / 3.40; 256 threads at 80 registers 2.99.
constexpr int kThreads = 256;
constexpr unsigned kFull = 0xffffffffu;
constexpr double kAlpha01 = 0.5 * (AA + BB), kBeta0 = 0.5 * (AA - BB);

__device__ __forceinline__ dfl shx(dfl v, int m)
{
  return dfl{__shfl_xor_sync(kFull, v.h, m), __shfl_xor_sync(kFull, v.l, m)};
}
__device__ __forceinline__ double shx(double v, int m) { return __shfl_xor_sync(kFull, v, m); }
__device__ __forceinline__ dfl shs(dfl v, int src)
{
  return dfl{__shfl_sync(kFull, v.h, src), __shfl_sync(kFull, v.l, src)};
}
__device__ __forceinline__ double shs(double v, int src) { return __shfl_sync(kFull, v, src); }
// v * (bit ? 1/2 : -1/2)
__device__ __forceinline__ dfl halfSgn(dfl v, int bit)
{
  float const s = bit ? 0.5f : -0.5f;
  return dfl{v.h * s, v.l * s};
}
__device__ __forceinline__ double halfSgn(double v, int bit) { return v * (bit ? 0.5 : -0.5); }
// n ? -v : v, n in {0, 1}
__device__ __forceinline__ dfl negIf(dfl v, uint32_t n)
{
  uint32_t const m = n << 31;
  return dfl{__uint_as_float(__float_as_uint(v.h) ^ m), __uint_as_float(__float_as_uint(v.l) ^ m)};
}
__device__ __forceinline__ double negIf(double v, uint32_t n) { return n ? -v : v; }
__device__ __forceinline__ dfl scl(dfl v, float s) { return dfl{v.h * s, v.l * s}; }
__device__ __forceinline__ double scl(double v, double s) { return v * s; }
// 2-point transform along the axis of lane mask m: at the lane with bit b,
// sum_n L(n, b) v(n) = A v(b) + B v(1 - b) (node values -> Gauss point, and back)
template <typename T>
__device__ __forceinline__ T lerp2(T v, int m)
{
  return dot2(cst<T>(A), v, cst<T>(B), shx(v, m));
}

// Out of line, like sinpiNear: a smaller instruction footprint for the phases of the
// group kernel (measured 0.8 % faster at 128^3).
// sin(pi o), cos(pi o): o = k/2 + r with |r| <= 1/4 (exact in FP64; adding 1.5 * 2^52
// rounds 2o to an integer), Taylor polynomials of sin and cos at x = pi r with the
// terms above 2^-24 in double-float and the rest in float, then the quadrant k mod 4.
__device__ __noinline__ void sinCosPiG(double o, dfl & s, dfl & c)
{
  constexpr double kRound = 6755399441055744.0;
  double const kk = fma(2.0, o, kRound);
  int const quad = __double2loint(kk) & 3;
  double const r = fma(-0.5, kk - kRound, o);
  dfl const x = toDfl(r) * cst<dfl>(PI);
  dfl const t = x * x;
  float const tf = t.h;
  // sin x / x = 1 - t/3! + t^2/5! - t^3/7! + t^4/9! - t^5/11! + t^6/13! - t^7/15!
  float const ps = tf * (-1.f / 39916800.f + tf * (1.f / 6227020800.f - tf * (1.f / 1307674368000.f)));
  dfl hs = cst<dfl>(1.0 / 362880.0) + dfl{ps, 0.f};
  hs = cst<dfl>(-1.0 / 5040.0) + t * hs;
  hs = cst<dfl>(1.0 / 120.0) + t * hs;
  hs = cst<dfl>(-1.0 / 6.0) + t * hs;
  hs = cst<dfl>(1.0) + t * hs;
  dfl const sr = x * hs;
  // cos x = 1 - t/2! + t^2/4! - t^3/6! + t^4/8! - t^5/10! + t^6/12! - t^7/14! + t^8/16!
  float const pc =
      tf * (-1.f / 3628800.f + tf * (1.f / 479001600.f + tf * (-1.f / 87178291200.f + tf * (1.f / 20922789888000.f))));
  dfl hc = cst<dfl>(1.0 / 40320.0) + dfl{pc, 0.f};
  hc = cst<dfl>(-1.0 / 720.0) + t * hc;
  hc = cst<dfl>(1.0 / 24.0) + t * hc;
  hc = cst<dfl>(-0.5) + t * hc;
  hc = cst<dfl>(1.0) + t * hc;
  dfl const sa = (quad & 1) ? hc : sr, ca = (quad & 1) ? sr : hc;
  s = negIf(sa, (quad >> 1) & 1);
  c = negIf(ca, ((quad + 1) >> 1) & 1);
}
__device__ __forceinline__ void sinCosPiG(double o, double & s, double & c) { sincospi(o, &s, &c); }

// Job t of phase B: G component, strides of the axes (u, v, w) in the Gauss point index
// (as log2), kind (0 = sum along u, 1 = alternating sum along u, 2 = l_a along u and v).
//   0 S_x: G_xx (x, y, z)   1 S_y: G_yy (y, x, z)   2 S_z: G_zz (z, x, y)
//   3 Sa: |det J| (x, y, z) 4 Sb: |det J| (x, y, z) 5 U_xy: G_xy (x, y, z)
//   6 U_xz: G_xz (x, z, y)  7 U_yz: G_yz (y, z, x)
constexpr uint64_t jobc(uint64_t cmp, uint64_t su, uint64_t sv, uint64_t sw, uint64_t kind)
{
  return cmp | su << 3 | sv << 5 | sw << 7 | kind << 9;
}
constexpr uint64_t kJobsLo = jobc(0, 0, 1, 2, 0) | jobc(1, 1, 0, 2, 0) << 16 | jobc(2, 2, 0, 1, 0) << 32 |
                             jobc(6, 0, 1, 2, 0) << 48;
constexpr uint64_t kJobsHi = jobc(6, 0, 1, 2, 1) | jobc(3, 0, 1, 2, 2) << 16 | jobc(4, 0, 2, 1, 2) << 32 |
                             jobc(5, 1, 2, 0, 2) << 48;

// Shared memory of a block of NT threads, NS = NT / 8 element slots (one per lane group):
//   tab   T[96][NS + 1]: the tables (phase B -> C), row job * 12 + row * 3 + class,
//         one column per slot; it aliases G, T[NS][kGStride] (phase A -> B), where a
//         slot holds G_xx, G_yy, G_zz, G_xy, G_xz, G_yz and |det J| at its 8 Gauss points
//   slotw uint32_t[NS][kSlotWords]: rowPtr of the nodes' DOFs, the DOFs, the 8 x 8
//         scatter ranks (uint16) and the mask of constrained nodes
//   bv    double[NS][kBvStride]: Dirichlet value of each node (0 when free), then k_e
//   desc  uint4[36][6]: the pair descriptors of phase C (a copy of kPairs32 / kPairs64)
// The slot strides are odd multiples of the access width, so that the lane-per-slot
// reads of phase C, and the group-per-slot accesses of the other phases, spread over
// the banks.
constexpr int kGStride = 57, kSlotWords = 49, kBvStride = 9;
constexpr int kSwRp = 0, kSwDof = 8, kSwRank = 16, kSwCons = 48;

template <int NT>
struct Smem
{
  static constexpr int NS = NT / 8, kRow = NS + 1;
  static constexpr size_t tabBytes = (size_t)(96 * kRow > NS * kGStride ? 96 * kRow : NS * kGStride) * 8;
  // the scratch of phases 0 and D (vertex and centroid coordinates, the centroid's sin
  // and cos) behind G in the table region, which the tables overwrite only in phase B
  static constexpr size_t scratchOff = (size_t)NS * kGStride * 8;
  // [NS][3] centroid coordinates, [NS][3] sin, [NS][3] cos, then [NS][8][3] vertex coordinates
  static_assert(scratchOff + (size_t)NS * (3 * 24 + 24 * 8) <= tabBytes, "phase D scratch overlaps the next region");
  static constexpr size_t slotOff = (tabBytes + 15) / 16 * 16;
  static constexpr size_t bvOff = slotOff + ((size_t)NS * kSlotWords * 4 + 15) / 16 * 16;
  static constexpr size_t descOff = (bvOff + (size_t)NS * kBvStride * 8 + 15) / 16 * 16;
  static constexpr size_t bytes = descOff + 36 * 6 * 16;
};
template <int NT>
constexpr size_t smemBytes()
{
  return Smem<NT>::bytes;
}

// The 36 pairs i <= j (row-major) as 24 words each, read by a whole warp at once:
//   [0..8]   byte offsets in a slot's column of tab of the nine stiffness terms (the
//            formulas of q1Stiffness), [9..17] their signs as floats +-1,
//   [18, 19] byte offsets of the two mass-table terms, [20] cx (the class of the pair
//            along x), [21] i | j << 3, [22] the byte offsets in the rank array of
//            entries (i, j) and (j, i), low and high half, [23] unused.
template <int NS>
struct PairTable
{
  alignas(16) uint32_t w[36 * 24];
};
template <int NS>
constexpr PairTable<NS> makePairTable()
{
  PairTable<NS> t{};
  constexpr uint32_t row = 8u * (NS + 1);
  int p = 0;
  for (int i = 0; i < 8; ++i)
    for (int j = i; j < 8; ++j, ++p)
    {
      int const li = i ^ ((i >> 1) & 1), lj = j ^ ((j >> 1) & 1);
      int const ix = li & 1, iy = (li >> 1) & 1, iz = li >> 2;
      int const jx = lj & 1, jy = (lj >> 1) & 1, jz = lj >> 2;
      int const cx = cls(ix, jx), cy = cls(iy, jy), cz = cls(iz, jz);
      uint32_t const off[9] = {(uint32_t)(0 * 12 + cy * 3 + cz),            (uint32_t)(1 * 12 + cx * 3 + cz),
                               (uint32_t)(2 * 12 + cx * 3 + cy),            (uint32_t)(5 * 12 + (2 * jx + iy) * 3 + cz),
                               (uint32_t)(5 * 12 + (2 * ix + jy) * 3 + cz), (uint32_t)(6 * 12 + (2 * jx + iz) * 3 + cy),
                               (uint32_t)(6 * 12 + (2 * ix + jz) * 3 + cy), (uint32_t)(7 * 12 + (2 * jy + iz) * 3 + cx),
                               (uint32_t)(7 * 12 + (2 * iy + jz) * 3 + cx)};
      bool const pos[9] = {ix == jx, iy == jy, iz == jz, ix == jy, iy == jx, ix == jz, iz == jx, iy == jz, iz == jy};
      uint32_t * w = t.w + 24 * p;
      for (int k = 0; k < 9; ++k)
      {
        w[k] = off[k] * row;
        w[9 + k] = pos[k] ? 0x3f800000u : 0xbf800000u;
      }
      w[18] = (uint32_t)(3 * 12 + cy * 3 + cz) * row;
      w[19] = (uint32_t)(4 * 12 + cy * 3 + cz) * row;
      w[20] = (uint32_t)cx;
      w[21] = (uint32_t)(i | j << 3);
      w[22] = (uint32_t)(2 * (i * 8 + j)) | (uint32_t)(2 * (j * 8 + i)) << 16;
      w[23] = 0;
    }
  return t;
}
__device__ PairTable<32> const kPairs32 = makePairTable<32>();
__device__ PairTable<64> const kPairs64 = makePairTable<64>();

// Dirichlet condensation of one entry (builder.hpp:76-124): a constrained diagonal
// takes bcDiag, a free row the lift -K_ij h_j.  Out of line: its FP64 code would
// otherwise be predicated into every entry.
__device__ __noinline__ void condenseEntry(double * diag, double bcDiag, double * b, uint32_t dofi, uint32_t dofj,
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

template <typename T>
__device__ __forceinline__ T pick3(T const (&v)[3], int d)
{
  return d == 0 ? v[0] : (d == 1 ? v[1] : v[2]);
}

template <typename T>
__device__ __forceinline__ T ldTab(char const * col, uint32_t off)
{
  return *reinterpret_cast<T const *>(col + off);
}

template <typename T, int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) kAssembleQ1Group(AsmArgs a)
{
  using S = Smem<NT>;
  constexpr int NS = S::NS, kRow = S::kRow, SW = NS / 32;
  static_assert(NS % 32 == 0, "phase C takes a warp of slots at a time");
  extern __shared__ uint4 dynShared[];
  char * const smem = reinterpret_cast<char *>(dynShared);
  T * const tab = reinterpret_cast<T *>(smem);
  uint32_t * const slotw = reinterpret_cast<uint32_t *>(smem + S::slotOff);
  double * const bvAll = reinterpret_cast<double *>(smem + S::bvOff);
  // phase D scratch behind G (the tables overwrite it only in phase B)
  double * const sOd = reinterpret_cast<double *>(smem + S::scratchOff); // [NS][3]
  T * const sSo = reinterpret_cast<T *>(sOd + 3 * NS);
  T * const sCo = sSo + 3 * NS;
  double * const sXv = reinterpret_cast<double *>(sCo + 3 * NS); // [NS][8][3]
  // the pair descriptors of phase C, copied once per block: shared-memory reads
  // wait less than the L1 hits of the global table
  uint4 * const sDesc = reinterpret_cast<uint4 *>(smem + S::descOff);
  {
    uint4 const * const src = reinterpret_cast<uint4 const *>(NS == 32 ? kPairs32.w : kPairs64.w);
    for (int k = threadIdx.x; k < 36 * 6; k += NT)
      sDesc[k] = src[k];
  }

  int const l = threadIdx.x & 7;
  int const g0 = threadIdx.x & 24; // first lane of the group in the warp
  int const slot = threadIdx.x >> 3;
  T * const G = tab + slot * kGStride; // G[c * 8 + q]
  uint32_t * const sw = slotw + slot * kSlotWords;
  double * const bv = bvAll + slot * kBvStride;
  int64_t const eg = (int64_t)blockIdx.x * NS + slot;
  bool const live = eg < a.nelem;
  int64_t const e = elemOf(a, live ? eg : a.nelem - 1); // a tail group recomputes the last element, writes nothing
  int const bx = l & 1, by = (l >> 1) & 1, bz = l >> 2;
  bool const lhs = a.op[0].on || a.op[1].on;

  // ---- node data: lane l = node l
  uint32_t const dofl = a.emap[8 * e + l];
  bool const cl = a.bcMask && a.bcMask[dofl];
  uint32_t const cons = (__ballot_sync(kFull, cl) >> g0) & 0xffu;
  double const bvl = (cl && a.bcVal) ? a.bcVal[dofl] : 0.;
  sw[kSwDof + l] = dofl;
  bv[l] = bvl;
  if (l == 0)
  {
    sw[kSwCons] = cons;
    // the element's coefficient for phase C, in the slot's spare ninth word of bv
    bool const needKE = usesCoef(a.op[0]) || usesCoef(a.op[1]);
    bv[8] = (needKE && a.kE) ? a.kE[e] : 1.0;
  }
  if (lhs)
  {
    sw[kSwRp + l] = a.rowPtr[dofl];
    uint4 const r = reinterpret_cast<uint4 const *>(a.rank + 64 * e)[l];
    sw[kSwRank + 4 * l + 0] = r.x;
    sw[kSwRank + 4 * l + 1] = r.y;
    sw[kSwRank + 4 * l + 2] = r.z;
    sw[kSwRank + 4 * l + 3] = r.w;
  }

  // ---- vertex coordinates: lane l = lattice vertex l = node l ^ by, relative to vertex 0
  uint32_t const vtx = a.conn[8 * e + (l ^ by)];
  double X0[3];
  T Y[3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
  {
    double const x = a.xyz[3 * (int64_t)vtx + d];
    X0[d] = __shfl_sync(kFull, x, g0);
    Y[d] = fromDouble<T>(x - X0[d]);
    sXv[(8 * slot + (l ^ by)) * 3 + d] = x; // node order, for the vertex average (phase D)
  }
  __syncthreads();

  // ---- A. geometry at Gauss point q = l
  T J[3][3];
  {
    T Dx[3], Lx[3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
    {
      T const p = shx(Y[r], 1);
      Dx[r] = halfSgn(Y[r] - p, bx);
      Lx[r] = dot2(cst<T>(A), Y[r], cst<T>(B), p);
    }
    T DxLy[3], LxDy[3], LxLy[3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
    {
      T const pd = shx(Dx[r], 2), pl = shx(Lx[r], 2);
      DxLy[r] = dot2(cst<T>(A), Dx[r], cst<T>(B), pd);
      LxDy[r] = halfSgn(Lx[r] - pl, by);
      LxLy[r] = dot2(cst<T>(A), Lx[r], cst<T>(B), pl);
    }
#pragma unroll
    for (int r = 0; r < 3; ++r)
    {
      T const p1 = shx(DxLy[r], 4), p2 = shx(LxDy[r], 4), p3 = shx(LxLy[r], 4);
      J[r][0] = dot2(cst<T>(A), DxLy[r], cst<T>(B), p1);
      J[r][1] = dot2(cst<T>(A), LxDy[r], cst<T>(B), p2);
      J[r][2] = halfSgn(LxLy[r] - p3, bz);
    }
  }
  T adet, off[3];
  {
    T C[3][3]; // adj(J)
    C[0][0] = dot2(J[1][1], J[2][2], -J[1][2], J[2][1]);
    C[0][1] = dot2(J[0][2], J[2][1], -J[0][1], J[2][2]);
    C[0][2] = dot2(J[0][1], J[1][2], -J[0][2], J[1][1]);
    C[1][0] = dot2(J[1][2], J[2][0], -J[1][0], J[2][2]);
    C[1][1] = dot2(J[0][0], J[2][2], -J[0][2], J[2][0]);
    C[1][2] = dot2(J[0][2], J[1][0], -J[0][0], J[1][2]);
    C[2][0] = dot2(J[1][0], J[2][1], -J[1][1], J[2][0]);
    C[2][1] = dot2(J[0][1], J[2][0], -J[0][0], J[2][1]);
    C[2][2] = dot2(J[0][0], J[1][1], -J[0][1], J[1][0]);
    T const det = dot3(J[0][0], C[0][0], J[0][1], C[1][0], J[0][2], C[2][0]);
    adet = fabs(det);
    T const s = cst<T>(0.25) * rcp(adet);
    G[0 * 8 + l] = s * dot3(C[0][0], C[0][0], C[0][1], C[0][1], C[0][2], C[0][2]);
    G[1 * 8 + l] = s * dot3(C[1][0], C[1][0], C[1][1], C[1][1], C[1][2], C[1][2]);
    G[2 * 8 + l] = s * dot3(C[2][0], C[2][0], C[2][1], C[2][1], C[2][2], C[2][2]);
    G[3 * 8 + l] = s * dot3(C[0][0], C[1][0], C[0][1], C[1][1], C[0][2], C[1][2]);
    G[4 * 8 + l] = s * dot3(C[0][0], C[2][0], C[0][1], C[2][1], C[0][2], C[2][2]);
    G[5 * 8 + l] = s * dot3(C[1][0], C[2][0], C[1][1], C[2][1], C[1][2], C[2][2]);
    G[6 * 8 + l] = adet;
    T const xq = negIf(cst<T>(g), !bx), yq = negIf(cst<T>(g), !by), zq = negIf(cst<T>(g), !bz);
#pragma unroll
    for (int r = 0; r < 3; ++r)
      off[r] = dot3(J[r][0], xq, J[r][1], yq, J[r][2], zq);
  }

  // ---- D. load vector (and the Dirichlet rows' h, once per operator with bc)
  bool const anyBc = cons && ((a.op[0].on && a.op[0].bc) || (a.op[1].on && a.op[1].bc));
  if (a.b)
  {
    if (anyBc && live && cl && bvl != 0.)
    {
#pragma unroll
      for (int m = 0; m < 2; ++m)
        if (a.op[m].on && a.op[m].bc)
          atomicAdd(a.b + dofl, bvl);
    }
    if (a.rkind)
    {
      T rq;
      if (a.rkind == 1)
      {
        // the centroid (the vertex average, the hexahedron's origin) and, for the sin
        // load, sin and cos of pi times its coordinates: one thread per (element,
        // coordinate) of the block, through shared memory behind G
        if (threadIdx.x < 3 * NS)
        {
          double const * xv = sXv + 24 * (threadIdx.x / 3) + threadIdx.x % 3;
          double const od = 0.125 * (xv[0] + xv[3] + xv[6] + xv[9] + xv[12] + xv[15] + xv[18] + xv[21]);
          sOd[threadIdx.x] = od;
          if (a.fn == PXG_FN_SIN3)
          {
            T so, co;
            sinCosPiG(od, so, co);
            sSo[threadIdx.x] = so;
            sCo[threadIdx.x] = co;
          }
        }
        __syncthreads();
        if (a.fn == PXG_FN_SIN3)
        {
          T f = cst<T>(1.0);
#pragma unroll
          for (int d = 0; d < 3; ++d)
            f = f * sinpiNear(sSo[3 * slot + d], sCo[3 * slot + d], sOd[3 * slot + d], off[d]);
          rq = adet * (fromDouble<T>(a.rc) * f);
        }
        else
        {
          double x[3];
#pragma unroll
          for (int d = 0; d < 3; ++d)
            x[d] = sOd[3 * slot + d] + toDouble(off[d]);
          rq = fromDouble<T>(toDouble(adet) * evalFn(a.fn, a.rc, x[0], x[1], x[2]));
        }
      }
      else
      {
        // projection of a DOF field: node values -> Gauss point
        T v = fromDouble<T>(a.field[sw[kSwDof + (l ^ by)]]);
        v = lerp2(v, 1);
        v = lerp2(v, 2);
        v = lerp2(v, 4);
        rq = adet * (fromDouble<T>(a.rc) * v);
      }
      T F = lerp2(rq, 1);
      F = lerp2(F, 2);
      F = lerp2(F, 4);
      int const n = l ^ by;
      if (live && !(a.rbc && ((cons >> n) & 1u)))
        atomicAdd(a.b + sw[kSwDof + n], toDouble(F));
    }
  }
  if (!lhs)
    return; // uniform over the block: the kernel arguments

  // ---- B. tables: warp w takes job w / SW for the 32 slots 32 (w % SW) + lane, so that
  // the job is uniform over the warp (the sum jobs skip the U jobs' second transform
  // and fourth row)
  __syncthreads(); // G of every slot is written
  {
    int const job = (threadIdx.x >> 5) / SW;
    int const sB = 32 * ((threadIdx.x >> 5) % SW) + (threadIdx.x & 31);
    uint32_t const code = (uint32_t)((job < 4 ? kJobsLo : kJobsHi) >> (16 * (job & 3))) & 0x7ffu;
    int const cmp = code & 7, su = 1 << ((code >> 3) & 3), sv = 1 << ((code >> 5) & 3), sw3 = 1 << ((code >> 7) & 3);
    int const kind = code >> 9;
    T const * const Gs = tab + sB * kGStride;
    T F[2][2][2]; // [qw][qv][qu]
#pragma unroll
    for (int qw = 0; qw < 2; ++qw)
#pragma unroll
      for (int qv = 0; qv < 2; ++qv)
#pragma unroll
        for (int qu = 0; qu < 2; ++qu)
          F[qw][qv][qu] = Gs[cmp * 8 + qu * su + qv * sv + qw * sw3];
    __syncthreads(); // the tables overwrite G
    // constants of the class formulas, evaluated at compile time
    constexpr T kA = cst<T>(A), kB = cst<T>(B), kAA = cst<T>(AA), kBB = cst<T>(BB), kAB = cst<T>(AB);
    T * const tj = tab + job * 12 * kRow + sB;
    if (kind == 2)
    {
      // U jobs: along u with l_0 (P0) and l_1 (P1); row r along v: l_(r & 1) of P0 (r < 2)
      // or of P1 (r >= 2)
      T P0[2][2], P1[2][2]; // [qw][qv]
#pragma unroll
      for (int qw = 0; qw < 2; ++qw)
#pragma unroll
        for (int qv = 0; qv < 2; ++qv)
        {
          P0[qw][qv] = dot2(kA, F[qw][qv][0], kB, F[qw][qv][1]);
          P1[qw][qv] = dot2(kB, F[qw][qv][0], kA, F[qw][qv][1]);
        }
#pragma unroll
      for (int r = 0; r < 4; ++r)
      {
        T const x0 = (r & 1) ? kB : kA, x1 = (r & 1) ? kA : kB;
        T R[2];
#pragma unroll
        for (int qw = 0; qw < 2; ++qw)
          R[qw] = r >= 2 ? dot2(x0, P1[qw][0], x1, P1[qw][1]) : dot2(x0, P0[qw][0], x1, P0[qw][1]);
        // classes along w
        tj[(r * 3 + 0) * kRow] = dot2(kAA, R[0], kBB, R[1]);
        tj[(r * 3 + 1) * kRow] = dot2(kBB, R[0], kAA, R[1]);
        tj[(r * 3 + 2) * kRow] = kAB * (R[0] + R[1]);
      }
    }
    else
    {
      // sum jobs: along u the sum (kind 0) or the alternating sum (kind 1); row r along v:
      // the classes W_r (AA, BB), (BB, AA), (AB, AB)
      T P0[2][2];
#pragma unroll
      for (int qw = 0; qw < 2; ++qw)
#pragma unroll
        for (int qv = 0; qv < 2; ++qv)
          P0[qw][qv] = kind == 1 ? F[qw][qv][0] - F[qw][qv][1] : F[qw][qv][0] + F[qw][qv][1];
      constexpr T kS0[3] = {kAA, kBB, kAB}, kS1[3] = {kBB, kAA, kAB};
#pragma unroll
      for (int r = 0; r < 3; ++r)
      {
        T R[2];
#pragma unroll
        for (int qw = 0; qw < 2; ++qw)
          R[qw] = r == 2 ? kAB * (P0[qw][0] + P0[qw][1]) : dot2(kS0[r], P0[qw][0], kS1[r], P0[qw][1]);
        tj[(r * 3 + 0) * kRow] = dot2(kAA, R[0], kBB, R[1]);
        tj[(r * 3 + 1) * kRow] = dot2(kBB, R[0], kAA, R[1]);
        tj[(r * 3 + 2) * kRow] = kAB * (R[0] + R[1]);
      }
    }
  }
  __syncthreads();

  // ---- C. entries: lane = slot s; a warp takes the pairs p = p0, p0 + 8, ... of 32 slots
  int const warp = threadIdx.x >> 5;
  int const s = 32 * (warp % SW) + (threadIdx.x & 31);
  int64_t const gs = (int64_t)blockIdx.x * NS + s;
  bool const liveS = gs < a.nelem;
  bool const needK = (a.op[0].on && a.op[0].stiff) || (a.op[1].on && a.op[1].stiff);
  bool const needM = (a.op[0].on && a.op[0].mass) || (a.op[1].on && a.op[1].mass);
  double const kfac = bvAll[s * kBvStride + 8]; // k_e of slot s (1 without a per-element coefficient)
  // operator coefficients in the arithmetic of the tables: the only FP64-pipe
  // instructions of an entry are then its conversion to double, the high float's
  // hardware conversion and the addition of the low float (toDoubleMixed; the FP64
  // pipe, at 1/64 of the FP32 rate, is the scarcer resource)
  T ks[2], ms[2];
#pragma unroll
  for (int m = 0; m < 2; ++m)
  {
    LhsDev const & op = a.op[m];
    ks[m] = fromDouble<T>(op.stiff ? (op.stiff == 2 ? op.sc * kfac : op.sc) : 0.);
    ms[m] = fromDouble<T>(op.mass ? massCoef(op, kfac) : 0.);
  }
  uint32_t const * const ss = slotw + s * kSlotWords;
  double const * const bs = bvAll + s * kBvStride;
  uint32_t const consS = ss[kSwCons];
  bool const anyBcS = consS && ((a.op[0].on && a.op[0].bc) || (a.op[1].on && a.op[1].bc));
  char const * const col = reinterpret_cast<char const *>(tab + s);
  char const * const rk = reinterpret_cast<char const *>(ss + kSwRank);
  uint4 const * const pt = sDesc;
  // pair p of slot s: the stiffness sum kv (nine table terms), the mass term mv, the
  // local indices and the positions of entries (i, j) and (j, i) in the value arrays
  auto pairTerms = [&](int p, bool withK, bool withM, T & kv, T & mv, int & i, int & j, uint32_t & pij,
                       uint32_t & pji) {
    uint4 const d0 = pt[6 * p], d1 = pt[6 * p + 1], d2 = pt[6 * p + 2];
    uint4 const d3 = pt[6 * p + 3], d4 = pt[6 * p + 4], d5 = pt[6 * p + 5];
    kv = cst<T>(0.0);
    mv = cst<T>(0.0);
    if (withK)
    {
      auto acc = sumStartS(ldTab<T>(col, d0.x), d2.y);
      sumAddS(acc, ldTab<T>(col, d0.y), d2.z);
      sumAddS(acc, ldTab<T>(col, d0.z), d2.w);
      sumAddS(acc, ldTab<T>(col, d0.w), d3.x);
      sumAddS(acc, ldTab<T>(col, d1.x), d3.y);
      sumAddS(acc, ldTab<T>(col, d1.y), d3.z);
      sumAddS(acc, ldTab<T>(col, d1.z), d3.w);
      sumAddS(acc, ldTab<T>(col, d1.w), d4.x);
      sumAddS(acc, ldTab<T>(col, d2.x), d4.y);
      kv = sumEnd(acc);
    }
    if (withM)
    {
      constexpr T kAB = cst<T>(AB), kA01 = cst<T>(kAlpha01), kB0 = cst<T>(kBeta0), kZero = cst<T>(0.0);
      uint32_t const cx = d5.x;
      T const alpha = cx == 2 ? kAB : kA01;
      T const beta = negIf(cx == 2 ? kZero : kB0, cx == 1);
      mv = dot2(alpha, ldTab<T>(col, d4.z), beta, ldTab<T>(col, d4.w));
    }
    i = d5.y & 7;
    j = d5.y >> 3;
    pij = ss[kSwRp + i] + *reinterpret_cast<uint16_t const *>(rk + (d5.z & 0xffffu));
    pji = ss[kSwRp + j] + *reinterpret_cast<uint16_t const *>(rk + (d5.z >> 16));
  };
  // The usual operator pair, a stiffness-only operator and then a mass-only one, in a
  // warp none of whose 32 elements has a Dirichlet node under an operator with BCs:
  // a loop without the per-entry operator branches and Dirichlet votes.
  bool const kmPair = a.op[0].on && a.op[0].stiff && !a.op[0].mass && a.op[1].on && !a.op[1].stiff && a.op[1].mass;
  if (kmPair && !__any_sync(kFull, anyBcS))
  {
    double * const vK = a.op[0].vals;
    double * const vM = a.op[1].vals;
    for (int p = warp / SW; p < 36; p += 8)
    {
      T kv, mv;
      int i, j;
      uint32_t pij, pji;
      pairTerms(p, true, true, kv, mv, i, j, pij, pji);
      double const valK = toDoubleMixed(ks[0] * kv), valM = toDoubleMixed(ms[1] * mv);
      if (liveS)
      {
        atomicAdd(vK + pij, valK);
        atomicAdd(vM + pij, valM);
        if (i != j)
        {
          atomicAdd(vK + pji, valK);
          atomicAdd(vM + pji, valM);
        }
      }
    }
    return;
  }
  for (int p = warp / SW; p < 36; p += 8)
  {
    T kv, mv;
    int i, j;
    uint32_t pij, pji;
    pairTerms(p, needK, needM, kv, mv, i, j, pij, pji);
    bool const ci = (consS >> i) & 1u, cj = (consS >> j) & 1u;
    // a warp none of whose elements has a constrained node in this pair takes the path
    // without the Dirichlet checks (every warp of a problem without BCs)
    bool const bcHere = anyBcS && (ci || cj);
    if (__any_sync(kFull, bcHere))
    {
#pragma unroll
      for (int m = 0; m < 2; ++m)
      {
        LhsDev const & op = a.op[m];
        if (!op.on)
          continue;
        double const val = toDoubleMixed(op.stiff ? (op.mass ? dot2(ks[m], kv, ms[m], mv) : ks[m] * kv) : ms[m] * mv);
        if (!liveS)
          continue;
        if (bcHere && op.bc)
        {
          condenseEntry(op.vals + pij, a.bcDiag, a.b, ss[kSwDof + i], ss[kSwDof + j], bs[i], bs[j], ci, cj, i == j,
                        val);
          continue;
        }
        atomicAdd(op.vals + pij, val);
        if (i != j)
          atomicAdd(op.vals + pji, val);
      }
    }
    else
    {
#pragma unroll
      for (int m = 0; m < 2; ++m)
      {
        LhsDev const & op = a.op[m];
        if (!op.on)
          continue;
        double const val = toDoubleMixed(op.stiff ? (op.mass ? dot2(ks[m], kv, ms[m], mv) : ks[m] * kv) : ms[m] * mv);
        if (liveS)
        {
          atomicAdd(op.vals + pij, val);
          if (i != j)
            atomicAdd(op.vals + pji, val);
        }
      }
    }
  }
}
} // namespace q1g

void launchAssembleQ1(AsmArgs const & a, cudaStream_t s, bool fp64, bool perThread, int threads)
{
  if (perThread)
  {
    unsigned const blocks = (unsigned)((a.nelem + 127) / 128);
    if (fp64)
      kAssembleQ1<double><<<blocks, 128, 0, s>>>(a);
    else
      kAssembleQ1<dfl><<<blocks, 128, 0, s>>>(a);
    return;
  }
  auto go = [&](auto kern, int nt, size_t smem) {
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    unsigned const blocks = (unsigned)((a.nelem * 8 + nt - 1) / nt);
    kern<<<blocks, nt, smem, s>>>(a);
  };
  if (fp64)
    go(q1g::kAssembleQ1Group<double, 256>, 256, q1g::smemBytes<256>());
  else if (threads == 512)
    go(q1g::kAssembleQ1Group<dfl, 512>, 512, q1g::smemBytes<512>());
  else
    go(q1g::kAssembleQ1Group<dfl, 256>, 256, q1g::smemBytes<256>());
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
