// Q1 hexahedron element kernel in FP64 arithmetic, one thread per element, written for
// GB300's FP64 rate (2 FP64 operations per clock per SM, 1/64 of FP32): every value
// the element produces is computed with IEEE binary64 operations, and the kernel is
// bound by the FP64 pipe, so its design goal is the fewest FP64 instructions per
// element.  It computes what proxpde's element loop computes for a Q1 hexahedron with
// the 2x2x2 Gauss rule (include/builder.hpp:53-153): CurFE::reinit (include/curfe.hpp:
// 50-103), AssemblyStiffness(FE) / AssemblyScalarMass / AssemblyMassFE
// (include/assembly_lhs.hpp:52-109, 207-221, 262-277), AssemblyRhsAnalytic and
// AssemblyS2SProjection (include/assembly_rhs.hpp:61-88, 130-159), the Dirichlet
// condensation (builder.hpp:76-124), and adds the result into the CSR values and the
// load vector with FP64 reductions.
//
// Notation: node / quadrature point = lattice triple (x, y, z) in {0,1}^3; Gauss nodes
// xi = s g, s = -1 (bit 0) or +1 (bit 1), g = 0.5773502691896258 (src/qr.cpp:27),
// weights 1.  l_a(xi) = (1 + e_a xi) / 2 with e_0 = -1, e_1 = +1 (src/reffe.cpp:246-253).
//
//  1. Trilinear map x(xi) = 1/8 sum_k H_k xi^kx eta^ky zeta^kz, H = the Walsh-Hadamard
//     transform of the eight vertices (24 additions per coordinate).  The Jacobian
//     columns at the Gauss points, c1(eta, zeta) = H100 + eta H110 + zeta H101 +
//     eta zeta H111 and its two companions, take 22 FMAs per coordinate (x8 scale).
//  2. Per point, the reference's own form (curfe.hpp:73-76): the Gram matrix J^T J
//     (its diagonal depends on two of the three point coordinates, so it is shared by
//     point pairs), its adjugate and determinant D; 1/|det J| = rsqrt(D) by one
//     third-order Newton step from the hardware estimate; |det J| = D rsqrt(D);
//     G = k |det J| (J^T J)^-1 = k adj(J^T J) rsqrt(D).
//  3. Stiffness by per-axis contractions of G (sum factorisation on the 2x2x2 rule):
//     S_x[cy][cz] = sum_q G_xx W_cy(qy) W_cz(qz), U_xy[jx][iy][cz] = sum_q G_xy
//     l_jx(qx) l_iy(qy) W_cz(qz), ..., with W_c = l_i l_j of the class c of (i, j):
//     00, 11 or mixed.  An entry is a signed sum of nine table values; entries sharing
//     the y/z indices of i and j share partial sums (about six additions per entry).
//  4. Mass table Mt[cx][cy][cz] = sum_q |det J_q| W W W from the moments of |det J|.
//  5. sin(pi x) sin(pi y) sin(pi z) at the reference's qpoint = origin + J xi
//     (curfe.hpp:80; origin = vertex average, geo.hpp:721-728) by the Taylor series of
//     sin(pi(o + d)) about the element origin in the offset d (degree 7, valid for
//     |pi d| <= 0.05 where its truncation is below 1e-15 relative; larger elements
//     take sinpi directly), then the transposed contractions to the nodes.
// All scale factors of the contractions (powers of two) are folded into compile-time
// constants.
#include <type_traits>

#include "pxg_internal.h"
#include "pxg_sinpi.h"

namespace pxg
{
namespace q1f
{
constexpr double g = 0.5773502691896258; // src/qr.cpp:27
constexpr double A = 0.5 * (1. + g);     // l_0 at -g, l_1 at +g
constexpr double B = 0.5 * (1. - g);     // l_0 at +g, l_1 at -g
constexpr double PI = 3.141592653589793;

// node <-> lattice position of proxpde's Q1 hexahedron (src/reffe.cpp:684-759)
__host__ __device__ constexpr int node(int x, int y, int z) { return z * 4 + (y ? (x ? 2 : 3) : (x ? 1 : 0)); }
__host__ __device__ constexpr int cls(int a, int b) { return a == b ? a : 2; }
__host__ __device__ constexpr double eps(int a) { return a ? 1.0 : -1.0; }
__host__ __device__ constexpr double sgn(int bit) { return bit ? 1.0 : -1.0; }

// 1/sqrt(x): hardware estimate (about 2^-22 relative), then one third-order Newton
// step y' = y (1 + e/2 + 3e^2/8), e = 1 - x y^2, whose truncation error is O(e^3)
__device__ __forceinline__ double rsqrtN(double x)
{
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double const e = fma(-(x * y), y, 1.0);
  return fma(y * e, fma(0.375, e, 0.5), y);
}

// 2-point contractions of a pair (v0 at s = -1, v1 at s = +1) with a common deferred
// scale, so that an output costs one FP64 operation: l_a / A (l_0 = A v0 + B v1 =
// A (v0 + (B/A) v1)), and W_c / A^2 for the three classes (W_00 = A^2 v0 + B^2 v1,
// W_11 = B^2 v0 + A^2 v1, W_01 = AB (v0 + v1)).  Every stiffness table is two l and
// one W contraction, or two W contractions, of G: all carry 1/A^4, which is folded
// into the per-element factor of G; the mass table (three W) and the load (three l)
// fold theirs into their own per-element factors.
constexpr double rB = B / A, rBB = rB * rB;
template <int a>
__device__ __forceinline__ double cL(double v0, double v1)
{
  return a == 0 ? fma(rB, v1, v0) : fma(rB, v0, v1);
}
__device__ __forceinline__ void cW3(double v0, double v1, double (&w)[3])
{
  w[0] = fma(rBB, v1, v0);
  w[1] = fma(rBB, v0, v1);
  w[2] = rB * (v0 + v1);
}
constexpr double A2 = A * A, A3 = A2 * A, A4 = A2 * A2, A6 = A4 * A2;

// Taylor coefficients of t -> sin(pi (o + kap t)) at t = 0, kap = pi g / 8 (the offset
// d = J xi = g u / 8 in the x8 column scale): c_k = pi^k kap'^k / k! times S or C
struct Taylor7
{
  double c[8];
};
constexpr double KAP = PI * g / 8.;
__device__ __forceinline__ Taylor7 taylorSin(double S, double C, double scale)
{
  // c_k = (+S, +C, -S, -C, +S, +C, -S, -C)[k] kap^k / k!
  constexpr double k1 = KAP, k2 = KAP * KAP / 2., k3 = KAP * KAP * KAP / 6.,
                   k4 = KAP * KAP * KAP * KAP / 24., k5 = KAP * KAP * KAP * KAP * KAP / 120.,
                   k6 = KAP * KAP * KAP * KAP * KAP * KAP / 720., k7 = KAP * KAP * KAP * KAP * KAP * KAP * KAP / 5040.;
  double const s = S * scale, c = C * scale;
  Taylor7 t;
  t.c[0] = s;
  t.c[1] = c * k1;
  t.c[2] = s * -k2;
  t.c[3] = c * -k3;
  t.c[4] = s * k4;
  t.c[5] = c * k5;
  t.c[6] = s * -k6;
  t.c[7] = c * -k7;
  return t;
}
__device__ __forceinline__ double horner7(Taylor7 const & t, double u)
{
  double f = fma(t.c[7], u, t.c[6]);
  f = fma(f, u, t.c[5]);
  f = fma(f, u, t.c[4]);
  f = fma(f, u, t.c[3]);
  f = fma(f, u, t.c[2]);
  f = fma(f, u, t.c[1]);
  return fma(f, u, t.c[0]);
}
// degree 6: for |kap u| <= 0.02 the truncation is below 0.02^7 / 7! = 2.6e-16 relative
__device__ __forceinline__ double horner6(Taylor7 const & t, double u)
{
  double f = fma(t.c[6], u, t.c[5]);
  f = fma(f, u, t.c[4]);
  f = fma(f, u, t.c[3]);
  f = fma(f, u, t.c[2]);
  f = fma(f, u, t.c[1]);
  return fma(f, u, t.c[0]);
}
// |kap u| below lim, tested on the high word (integer pipe)
template <int LIM_PERMILLE>
__device__ __forceinline__ bool inTaylorRange(double u)
{
  constexpr double lim = LIM_PERMILLE * 1e-3 / KAP;
  return (uint32_t)(__double2hiint(u) & 0x7fffffff) < (uint32_t)__double2hiint(lim);
}

// f at the qpoint origin + (g/8) u by the direct evaluation (offsets beyond the Taylor
// range, analytic functions other than sin3); out of line so that its FP64 code is not
// predicated into every element, with scalar arguments so that nothing of the caller
// has to live in memory
__device__ __noinline__ double evalAt(int fn, double rc, double o0, double o1, double o2, double u0, double u1,
                                      double u2)
{
  return evalFn(fn, rc, fma(g / 8., u0, o0), fma(g / 8., u1, o1), fma(g / 8., u2, o2));
}

// Dirichlet condensation of one entry (builder.hpp:76-124): a constrained diagonal takes
// bcDiag, a free row the lift -K_ij h_j; out of line (rarely taken)
__device__ __noinline__ void condense(double * pij, double bcDiag, double * b, uint32_t dofi, uint32_t dofj,
                                      double const * bcVal, bool ci, bool cj, bool isDiag, double val)
{
  if (isDiag)
  {
    atomicAdd(pij, bcDiag);
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

struct Tables
{
  double Sx[3][3], Sy[3][3], Sz[3][3]; // S_x[cy][cz], S_y[cx][cz], S_z[cx][cy]
  double Uxy[2][2][3];                 // [jx][iy][cz]
  double Uxz[2][2][3];                 // [jx][iz][cy]
  double Uyz[2][2][3];                 // [jy][iz][cx]
};

// K_ij for i = node(ix, iy, iz), j = node(jx, jy, jz), the x pairs of one y/z block
// (a = (iy, iz), b = (jy, jz)): K(ix, jx) = e_ix e_jx Sx + e_ix F[jx] + e_jx F'[ix] + T[c(ix, jx)]
template <int iy, int iz, int jy, int jz>
__device__ __forceinline__ void entryBlock(Tables const & t, double (&K)[2][2])
{
  constexpr int cy = cls(iy, jy), cz = cls(iz, jz);
  constexpr double eyy = eps(iy) * eps(jy), ezz = eps(iz) * eps(jz), eyz = eps(iy) * eps(jz),
                   ezy = eps(jy) * eps(iz);
  constexpr bool diag = iy == jy && iz == jz;
  double T[3];
#pragma unroll
  for (int cx = 0; cx < 3; ++cx)
  {
    double const s = fma(eyy, t.Sy[cx][cz], ezz * t.Sz[cx][cy]);
    if constexpr (diag)
      T[cx] = fma(2. * eyz, t.Uyz[jy][iz][cx], s);
    else
      T[cx] = fma(eyz, t.Uyz[jy][iz][cx], fma(ezy, t.Uyz[iy][jz][cx], s));
  }
  double F[2], Fp[2];
#pragma unroll
  for (int x = 0; x < 2; ++x)
  {
    F[x] = fma(eps(jy), t.Uxy[x][iy][cz], eps(jz) * t.Uxz[x][iz][cy]);
    Fp[x] = diag ? F[x] : fma(eps(iy), t.Uxy[x][jy][cz], eps(iz) * t.Uxz[x][jz][cy]);
  }
  double const sx = t.Sx[cy][cz];
#pragma unroll
  for (int ix = 0; ix < 2; ++ix)
#pragma unroll
    for (int jx = 0; jx < 2; ++jx)
    {
      if (diag && jx < ix)
        continue;
      // the +-1 factors are compile-time signs: the multiplications fold into the
      // operand negations of the additions
      K[ix][jx] = fma(eps(ix) * eps(jx), sx, fma(eps(ix), F[jx], fma(eps(jx), Fp[ix], T[cls(ix, jx)])));
    }
}

__device__ __forceinline__ void loadRankRow(uint16_t const * rk, int i, uint16_t (&r)[8])
{
  uint4 const v = reinterpret_cast<uint4 const *>(rk)[i];
  r[0] = v.x & 0xffff, r[1] = v.x >> 16, r[2] = v.y & 0xffff, r[3] = v.y >> 16;
  r[4] = v.z & 0xffff, r[5] = v.z >> 16, r[6] = v.w & 0xffff, r[7] = v.w >> 16;
}
} // namespace q1f

// NT threads per block, at least MINB blocks per SM (the register budget per thread:
// 128 x 1 -> 254 registers, 8 warps per SM; 64 x 6 -> 170 registers, 12 warps per SM)
template <int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) kAssembleQ1F64(AsmArgs a)
{
  using namespace q1f;
  int64_t const i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i0 >= a.nelem)
    return;
  int64_t const e = elemOf(a, i0);

  // ---- inputs: vertex ids, DOFs (two 16-byte loads each), coordinates, coefficient
  uint32_t v[8], dof[8];
  {
    uint4 const c0 = reinterpret_cast<uint4 const *>(a.conn)[2 * e];
    uint4 const c1 = reinterpret_cast<uint4 const *>(a.conn)[2 * e + 1];
    v[0] = c0.x, v[1] = c0.y, v[2] = c0.z, v[3] = c0.w, v[4] = c1.x, v[5] = c1.y, v[6] = c1.z, v[7] = c1.w;
    uint4 const d0 = reinterpret_cast<uint4 const *>(a.emap)[2 * e];
    uint4 const d1 = reinterpret_cast<uint4 const *>(a.emap)[2 * e + 1];
    dof[0] = d0.x, dof[1] = d0.y, dof[2] = d0.z, dof[3] = d0.w, dof[4] = d1.x, dof[5] = d1.y, dof[6] = d1.z,
    dof[7] = d1.w;
  }
  LhsDev const & op0 = a.op[0];
  LhsDev const & op1 = a.op[1];
  bool const k0 = op0.on && op0.stiff, k1 = op1.on && op1.stiff;
  bool const m0 = op0.on && op0.mass, m1 = op1.on && op1.mass;
  bool const needK = k0 || k1, needM = m0 || m1;
  double const kfac = ((usesCoef(op0) || usesCoef(op1)) && a.kE) ? a.kE[e] : 1.0;
  uint32_t cons = 0;
  if (a.bcMask)
  {
#pragma unroll
    for (int n = 0; n < 8; ++n)
      if (a.bcMask[dof[n]])
        cons |= 1u << n;
  }
  int32_t rp[8];
#pragma unroll
  for (int n = 0; n < 8; ++n)
    rp[n] = a.rowPtr[dof[n]];

  // ---- 1. Walsh-Hadamard transform of the vertices: H[kx][ky][kz][r]
  double H[2][2][2][3];
#pragma unroll
  for (int x = 0; x < 2; ++x)
#pragma unroll
    for (int y = 0; y < 2; ++y)
#pragma unroll
      for (int z = 0; z < 2; ++z)
      {
        int64_t const id = v[node(x, y, z)];
#pragma unroll
        for (int r = 0; r < 3; ++r)
          H[x][y][z][r] = a.xyz[3 * id + r];
      }
#pragma unroll
  for (int r = 0; r < 3; ++r)
  {
#pragma unroll
    for (int y = 0; y < 2; ++y)
#pragma unroll
      for (int z = 0; z < 2; ++z)
      {
        double const p0 = H[0][y][z][r], p1 = H[1][y][z][r];
        H[0][y][z][r] = p0 + p1, H[1][y][z][r] = p1 - p0;
      }
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
      for (int z = 0; z < 2; ++z)
      {
        double const p0 = H[x][0][z][r], p1 = H[x][1][z][r];
        H[x][0][z][r] = p0 + p1, H[x][1][z][r] = p1 - p0;
      }
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
      for (int y = 0; y < 2; ++y)
      {
        double const p0 = H[x][y][0][r], p1 = H[x][y][1][r];
        H[x][y][0][r] = p0 + p1, H[x][y][1][r] = p1 - p0;
      }
  }
  double o[3]; // element origin = vertex average (geo.hpp:721-728)
#pragma unroll
  for (int r = 0; r < 3; ++r)
    o[r] = 0.125 * H[0][0][0][r];

  // ---- 2. Jacobian columns (x8): c1[qy][qz], c2[qx][qz], c3[qx][qy]
  double c1[2][2][3], c2[2][2][3], c3[2][2][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int p = 0; p < 2; ++p)
    {
      double const sg = sgn(p) * g;
      double const u1 = fma(sg, H[1][1][0][r], H[1][0][0][r]), w1 = fma(sg, H[1][1][1][r], H[1][0][1][r]);
      double const u2 = fma(sg, H[1][1][0][r], H[0][1][0][r]), w23 = fma(sg, H[1][1][1][r], H[0][1][1][r]);
      double const u3 = fma(sg, H[1][0][1][r], H[0][0][1][r]);
#pragma unroll
      for (int t = 0; t < 2; ++t)
      {
        double const tg = sgn(t) * g;
        c1[p][t][r] = fma(tg, w1, u1);  // (qy = p, qz = t)
        c2[p][t][r] = fma(tg, w23, u2); // (qx = p, qz = t)
        c3[p][t][r] = fma(tg, w23, u3); // (qx = p, qy = t)
      }
    }

  // ---- 3. per point: Gram matrix, adjugate, determinant, G and |det J|
  // the coefficient of a single stiffness operator is folded into G
  bool const foldK = k0 != k1;
  double const ks0 = k0 ? (op0.stiff == 2 ? op0.sc * kfac : op0.sc) : 0.;
  double const ks1 = k1 ? (op1.stiff == 2 ? op1.sc * kfac : op1.sc) : 0.;
  // the tables' common 1/A^4 and the 1/32 of G's scale (l' l' = 1/4, x8) folded in
  double const kk = (foldK ? (k0 ? ks0 : ks1) : 1.0) * (A4 / 32.);
  double d11[2][2], d22[2][2], d33[2][2];
#pragma unroll
  for (int p = 0; p < 2; ++p)
#pragma unroll
    for (int t = 0; t < 2; ++t)
    {
      d11[p][t] = fma(c1[p][t][0], c1[p][t][0], fma(c1[p][t][1], c1[p][t][1], c1[p][t][2] * c1[p][t][2]));
      d22[p][t] = fma(c2[p][t][0], c2[p][t][0], fma(c2[p][t][1], c2[p][t][1], c2[p][t][2] * c2[p][t][2]));
      d33[p][t] = fma(c3[p][t][0], c3[p][t][0], fma(c3[p][t][1], c3[p][t][1], c3[p][t][2] * c3[p][t][2]));
    }
  // xx yy zz xy xz yz of k |det J| (J^T J)^-1, x8; the diagonal three unscaled, their
  // scale sG folded into the first contraction of their tables
  double G[6][8], sG[8];
  double ad[8];   // |det J|, x512
  double u[8][3]; // J xi / (g / 8): the qpoint offset
#pragma unroll
  for (int q = 0; q < 8; ++q)
  {
    int const qx = q & 1, qy = (q >> 1) & 1, qz = q >> 2;
    double const(&ca)[3] = c1[qy][qz];
    double const(&cb)[3] = c2[qx][qz];
    double const(&cc)[3] = c3[qx][qy];
    double const g11 = d11[qy][qz], g22 = d22[qx][qz], g33 = d33[qx][qy];
    double const g12 = fma(ca[0], cb[0], fma(ca[1], cb[1], ca[2] * cb[2]));
    double const g13 = fma(ca[0], cc[0], fma(ca[1], cc[1], ca[2] * cc[2]));
    double const g23 = fma(cb[0], cc[0], fma(cb[1], cc[1], cb[2] * cc[2]));
    double const A11 = fma(-g23, g23, g22 * g33);
    double const A22 = fma(-g13, g13, g11 * g33);
    double const A33 = fma(-g12, g12, g11 * g22);
    double const A12 = fma(g13, g23, -(g12 * g33));
    double const A13 = fma(g12, g23, -(g13 * g22));
    double const A23 = fma(g12, g13, -(g11 * g23));
    double const D = fma(g11, A11, fma(g12, A12, g13 * A13));
    double const rs = rsqrtN(D);
    ad[q] = D * rs;
    double const s = kk * rs;
    G[0][q] = A11, G[1][q] = A22, G[2][q] = A33, sG[q] = s;
    G[3][q] = s * A12, G[4][q] = s * A13, G[5][q] = s * A23;
#pragma unroll
    for (int r = 0; r < 3; ++r)
      u[q][r] = sgn(qx) * ca[r] + (sgn(qy) * cb[r] + sgn(qz) * cc[r]);
  }

  // ---- 5. load vector (buildLhs' BC values and buildRhs), before the tables so that
  // the offsets die early
  pdlWait(); // the writes start here
  bool const bcOps = (op0.on && op0.bc) || (op1.on && op1.bc);
  if (a.b && cons && bcOps)
  {
    // Dirichlet values at the constrained DOFs, once per operator with BCs
#pragma unroll
    for (int m = 0; m < 2; ++m)
    {
      if (!a.op[m].on || !a.op[m].bc)
        continue;
#pragma unroll
      for (int n = 0; n < 8; ++n)
        if ((cons >> n) & 1u)
        {
          double const h = a.bcVal[dof[n]];
          if (h != 0.)
            atomicAdd(a.b + dof[n], h);
        }
    }
  }
  if (a.rkind)
  {
    // r_q = |det J_q| f_q (x512), then Fe_i = sum_q r_q l_ix l_iy l_iz by three common-
    // scale contractions: rcS carries their A^3 and the 1/512 of |det J|
    double const rcS = a.rc * (A3 / 512.);
    double rq[8];
    if (a.rkind == 1 && a.fn == PXG_FN_SIN3)
    {
      bool ok = true, small = true;
#pragma unroll
      for (int q = 0; q < 8; ++q)
#pragma unroll
        for (int r = 0; r < 3; ++r)
        {
          ok = ok && inTaylorRange<50>(u[q][r]);
          small = small && inTaylorRange<20>(u[q][r]);
        }
      if (ok)
      {
        Taylor7 tc[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
        {
          double S, C;
          sinCosPiTab(o[r], S, C);
          tc[r] = taylorSin(S, C, r == 0 ? rcS : 1.0);
        }
        // degree 6 when every element of the warp allows it (uniform control flow)
        if (__all_sync(__activemask(), small))
        {
#pragma unroll
          for (int q = 0; q < 8; ++q)
            rq[q] = ad[q] * (horner6(tc[0], u[q][0]) * (horner6(tc[1], u[q][1]) * horner6(tc[2], u[q][2])));
        }
        else
        {
#pragma unroll
          for (int q = 0; q < 8; ++q)
            rq[q] = ad[q] * (horner7(tc[0], u[q][0]) * (horner7(tc[1], u[q][1]) * horner7(tc[2], u[q][2])));
        }
      }
      else
      {
#pragma unroll 1
        for (int q = 0; q < 8; ++q)
          rq[q] = (rcS * ad[q]) * evalAt(a.fn, 1.0, o[0], o[1], o[2], u[q][0], u[q][1], u[q][2]);
      }
    }
    else if (a.rkind == 1 && a.fn == PXG_FN_CONST)
    {
#pragma unroll
      for (int q = 0; q < 8; ++q)
        rq[q] = rcS * ad[q];
    }
    else if (a.rkind == 1)
    {
#pragma unroll 1
      for (int q = 0; q < 8; ++q)
        rq[q] = (rcS * ad[q]) * evalAt(a.fn, 1.0, o[0], o[1], o[2], u[q][0], u[q][1], u[q][2]);
    }
    else
    {
      // projection of a DOF field: f_q = coef sum_n phi_n(q) field_n, by the same
      // per-axis contractions (nodes -> points)
      double f[2][2][2];
#pragma unroll
      for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y)
#pragma unroll
          for (int z = 0; z < 2; ++z)
            f[x][y][z] = a.field[dof[node(x, y, z)]];
      double t1[2][2][2], t2[2][2][2];
#pragma unroll
      for (int y = 0; y < 2; ++y)
#pragma unroll
        for (int z = 0; z < 2; ++z)
        {
          // value at point bit p along x: l_0(p) f0 + l_1(p) f1, l_0(0) = A, l_0(1) = B
          t1[0][y][z] = fma(A, f[0][y][z], B * f[1][y][z]);
          t1[1][y][z] = fma(B, f[0][y][z], A * f[1][y][z]);
        }
#pragma unroll
      for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int z = 0; z < 2; ++z)
        {
          t2[x][0][z] = fma(A, t1[x][0][z], B * t1[x][1][z]);
          t2[x][1][z] = fma(B, t1[x][0][z], A * t1[x][1][z]);
        }
#pragma unroll
      for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y)
        {
          double const fz0 = fma(A, t2[x][y][0], B * t2[x][y][1]);
          double const fz1 = fma(B, t2[x][y][0], A * t2[x][y][1]);
          rq[x + 2 * y] = ad[x + 2 * y] * (rcS * fz0);
          rq[x + 2 * y + 4] = ad[x + 2 * y + 4] * (rcS * fz1);
        }
    }
    // contract to the nodes: x, then y, then z
    double b1[2][2][2], b2[2][2][2];
#pragma unroll
    for (int y = 0; y < 2; ++y)
#pragma unroll
      for (int z = 0; z < 2; ++z)
      {
        double const v0 = rq[2 * y + 4 * z], v1 = rq[1 + 2 * y + 4 * z];
        b1[0][y][z] = cL<0>(v0, v1);
        b1[1][y][z] = cL<1>(v0, v1);
      }
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
      for (int z = 0; z < 2; ++z)
      {
        b2[x][0][z] = cL<0>(b1[x][0][z], b1[x][1][z]);
        b2[x][1][z] = cL<1>(b1[x][0][z], b1[x][1][z]);
      }
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
      for (int y = 0; y < 2; ++y)
#pragma unroll
        for (int z = 0; z < 2; ++z)
        {
          int const n = node(x, y, z);
          if (a.rbc && ((cons >> n) & 1u))
            continue;
          double const fe = z ? cL<1>(b2[x][y][0], b2[x][y][1]) : cL<0>(b2[x][y][0], b2[x][y][1]);
          atomicAdd(a.b + dof[n], fe);
        }
  }

  uint16_t const * rk = a.rank + e * 64;
  bool const anyBc = cons && bcOps;
  // ---- 4. mass: the 3x3x3 class table by three common-scale W contractions of
  // |det J| (x512) times a single mass operator's coefficient; the factor also
  // carries the contractions' A^6 and the 1/512
  bool const foldM = m0 != m1;
  double const ms0 = m0 ? massCoef(op0, kfac) : 0., ms1 = m1 ? massCoef(op1, kfac) : 0.;
  double Mt[3][3][3];
  if (needM)
  {
    double const mcf = (foldM ? (m0 ? ms0 : ms1) : 1.0) * (A6 / 512.);
    double Vm[2][2][3]; // [qx][qy][cz]
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
      for (int y = 0; y < 2; ++y)
        cW3(mcf * ad[x + 2 * y], mcf * ad[x + 2 * y + 4], Vm[x][y]);
    double Ym[2][3][3]; // [qx][cy][cz]
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
      for (int cz = 0; cz < 3; ++cz)
      {
        double w[3];
        cW3(Vm[x][0][cz], Vm[x][1][cz], w);
        Ym[x][0][cz] = w[0], Ym[x][1][cz] = w[1], Ym[x][2][cz] = w[2];
      }
#pragma unroll
    for (int cy = 0; cy < 3; ++cy)
#pragma unroll
      for (int cz = 0; cz < 3; ++cz)
      {
        double w[3];
        cW3(Ym[0][cy][cz], Ym[1][cy][cz], w);
        Mt[0][cy][cz] = w[0], Mt[1][cy][cz] = w[1], Mt[2][cy][cz] = w[2];
      }
  }

  // ---- 3. stiffness tables (their scale is in G)
  Tables t;
  if (needK)
  {
    // S_x: sum over qx, then W over qy and qz
    {
      double R[3][2];
#pragma unroll
      for (int z = 0; z < 2; ++z)
      {
        double w[3];
        cW3(fma(sG[4 * z], G[0][4 * z], sG[1 + 4 * z] * G[0][1 + 4 * z]),
            fma(sG[2 + 4 * z], G[0][2 + 4 * z], sG[3 + 4 * z] * G[0][3 + 4 * z]), w);
        R[0][z] = w[0], R[1][z] = w[1], R[2][z] = w[2];
      }
#pragma unroll
      for (int c = 0; c < 3; ++c)
        cW3(R[c][0], R[c][1], t.Sx[c]);
    }
    // S_y: sum over qy, then W over qx and qz
    {
      double R[3][2];
#pragma unroll
      for (int z = 0; z < 2; ++z)
      {
        double w[3];
        cW3(fma(sG[4 * z], G[1][4 * z], sG[2 + 4 * z] * G[1][2 + 4 * z]),
            fma(sG[1 + 4 * z], G[1][1 + 4 * z], sG[3 + 4 * z] * G[1][3 + 4 * z]), w);
        R[0][z] = w[0], R[1][z] = w[1], R[2][z] = w[2];
      }
#pragma unroll
      for (int c = 0; c < 3; ++c)
        cW3(R[c][0], R[c][1], t.Sy[c]);
    }
    // S_z: sum over qz, then W over qx and qy
    {
      double R[3][2];
#pragma unroll
      for (int y = 0; y < 2; ++y)
      {
        double w[3];
        cW3(fma(sG[2 * y], G[2][2 * y], sG[2 * y + 4] * G[2][2 * y + 4]),
            fma(sG[1 + 2 * y], G[2][1 + 2 * y], sG[1 + 2 * y + 4] * G[2][1 + 2 * y + 4]), w);
        R[0][y] = w[0], R[1][y] = w[1], R[2][y] = w[2];
      }
#pragma unroll
      for (int c = 0; c < 3; ++c)
        cW3(R[c][0], R[c][1], t.Sz[c]);
    }
    // U_xy[jx][iy][cz]: l over qx, l over qy, W over qz
    {
      double Y[2][2][2]; // [jx][iy][qz]
#pragma unroll
      for (int z = 0; z < 2; ++z)
      {
        double X0[2][2]; // [jx][qy]
#pragma unroll
        for (int y = 0; y < 2; ++y)
        {
          double const v0 = G[3][2 * y + 4 * z], v1 = G[3][1 + 2 * y + 4 * z];
          X0[0][y] = cL<0>(v0, v1), X0[1][y] = cL<1>(v0, v1);
        }
#pragma unroll
        for (int jx = 0; jx < 2; ++jx)
          Y[jx][0][z] = cL<0>(X0[jx][0], X0[jx][1]), Y[jx][1][z] = cL<1>(X0[jx][0], X0[jx][1]);
      }
#pragma unroll
      for (int jx = 0; jx < 2; ++jx)
#pragma unroll
        for (int iy = 0; iy < 2; ++iy)
          cW3(Y[jx][iy][0], Y[jx][iy][1], t.Uxy[jx][iy]);
    }
    // U_xz[jx][iz][cy]: l over qx, l over qz, W over qy
    {
      double Y[2][2][2]; // [jx][iz][qy]
#pragma unroll
      for (int y = 0; y < 2; ++y)
      {
        double X0[2][2]; // [jx][qz]
#pragma unroll
        for (int z = 0; z < 2; ++z)
        {
          double const v0 = G[4][2 * y + 4 * z], v1 = G[4][1 + 2 * y + 4 * z];
          X0[0][z] = cL<0>(v0, v1), X0[1][z] = cL<1>(v0, v1);
        }
#pragma unroll
        for (int jx = 0; jx < 2; ++jx)
          Y[jx][0][y] = cL<0>(X0[jx][0], X0[jx][1]), Y[jx][1][y] = cL<1>(X0[jx][0], X0[jx][1]);
      }
#pragma unroll
      for (int jx = 0; jx < 2; ++jx)
#pragma unroll
        for (int iz = 0; iz < 2; ++iz)
          cW3(Y[jx][iz][0], Y[jx][iz][1], t.Uxz[jx][iz]);
    }
    // U_yz[jy][iz][cx]: l over qy, l over qz, W over qx
    {
      double Y[2][2][2]; // [jy][iz][qx]
#pragma unroll
      for (int x = 0; x < 2; ++x)
      {
        double X0[2][2]; // [jy][qz]
#pragma unroll
        for (int z = 0; z < 2; ++z)
        {
          double const v0 = G[5][x + 4 * z], v1 = G[5][x + 2 + 4 * z];
          X0[0][z] = cL<0>(v0, v1), X0[1][z] = cL<1>(v0, v1);
        }
#pragma unroll
        for (int jy = 0; jy < 2; ++jy)
          Y[jy][0][x] = cL<0>(X0[jy][0], X0[jy][1]), Y[jy][1][x] = cL<1>(X0[jy][0], X0[jy][1]);
      }
#pragma unroll
      for (int jy = 0; jy < 2; ++jy)
#pragma unroll
        for (int iz = 0; iz < 2; ++iz)
          cW3(Y[jy][iz][0], Y[jy][iz][1], t.Uyz[jy][iz]);
    }
  }

  // ---- 6. entries and scatter.  The operator values: a folded coefficient is already
  // in the table; otherwise the operator's coefficient multiplies the unit entry.
  bool const foldedPair = foldK && foldM && ((k0 && !m0 && m1 && !k1) || (k1 && !m1 && m0 && !k0));
  // lanes of this warp with a constrained entry under an operator with BCs
  bool const bcWarp = __any_sync(__activemask(), anyBc);
  auto emit = [&](int i, int j, double kv, double mv, uint16_t rij, uint16_t rji) {
    int32_t const pij = rp[i] + rij, pji = rp[j] + rji;
    if (foldedPair && !bcWarp)
    {
      double * Kv = k0 ? op0.vals : op1.vals;
      double * Mv = k0 ? op1.vals : op0.vals;
      atomicAdd(Kv + pij, kv);
      atomicAdd(Mv + pij, mv);
      if (i != j)
      {
        atomicAdd(Kv + pji, kv);
        atomicAdd(Mv + pji, mv);
      }
      return;
    }
    bool const ci = (cons >> i) & 1u, cj = (cons >> j) & 1u;
#pragma unroll
    for (int m = 0; m < 2; ++m)
    {
      LhsDev const & op = a.op[m];
      if (!op.on)
        continue;
      double val;
      double const ksm = m ? ks1 : ks0, msm = m ? ms1 : ms0;
      if (op.stiff)
      {
        val = foldK ? kv : ksm * kv;
        if (op.mass)
          val = foldM ? val + mv : fma(msm, mv, val);
      }
      else
        val = foldM ? mv : msm * mv;
      if (anyBc && op.bc && (ci || cj))
      {
        condense(op.vals + pij, a.bcDiag, a.b, dof[i], dof[j], a.bcVal, ci, cj, i == j, val);
        continue;
      }
      atomicAdd(op.vals + pij, val);
      if (i != j)
        atomicAdd(op.vals + pji, val);
    }
  };
  // y/z blocks: a = (iy, iz), b = (jy, jz) with a <= b in the order (0,0) (1,0) (0,1) (1,1)
  auto block = [&](auto ay, auto az, auto by, auto bz) {
    constexpr int iy = decltype(ay)::value, iz = decltype(az)::value;
    constexpr int jy = decltype(by)::value, jz = decltype(bz)::value;
    constexpr bool diag = iy == jy && iz == jz;
    double K[2][2] = {{0., 0.}, {0., 0.}};
    if (needK)
      entryBlock<iy, iz, jy, jz>(t, K);
    uint16_t ri[2][8], rj[2][8];
#pragma unroll
    for (int x = 0; x < 2; ++x)
    {
      loadRankRow(rk, node(x, iy, iz), ri[x]);
      if (!diag)
        loadRankRow(rk, node(x, jy, jz), rj[x]);
    }
#pragma unroll
    for (int ix = 0; ix < 2; ++ix)
#pragma unroll
      for (int jx = 0; jx < 2; ++jx)
      {
        if (diag && jx < ix)
          continue;
        int const i = node(ix, iy, iz), j = node(jx, jy, jz);
        double const mv = needM ? Mt[cls(ix, jx)][cls(iy, jy)][cls(iz, jz)] : 0.;
        emit(i, j, K[ix][jx], mv, ri[ix][j], diag ? ri[jx][i] : rj[jx][i]);
      }
  };
  using I0 = std::integral_constant<int, 0>;
  using I1 = std::integral_constant<int, 1>;
  block(I0{}, I0{}, I0{}, I0{});
  block(I1{}, I0{}, I1{}, I0{});
  block(I0{}, I1{}, I0{}, I1{});
  block(I1{}, I1{}, I1{}, I1{});
  block(I0{}, I0{}, I1{}, I0{});
  block(I0{}, I0{}, I0{}, I1{});
  block(I0{}, I0{}, I1{}, I1{});
  block(I1{}, I0{}, I0{}, I1{});
  block(I1{}, I0{}, I1{}, I1{});
  block(I0{}, I1{}, I1{}, I1{});
}

void launchAssembleQ1F64(AsmArgs const & a, cudaStream_t s, int threads)
{
  if (a.nelem <= 0)
    return;
  if (threads == 64)
    launchElemKernel(kAssembleQ1F64<64, 6>, (unsigned)((a.nelem + 63) / 64), 64, 0, s, a);
  else
    launchElemKernel(kAssembleQ1F64<128, 1>, (unsigned)((a.nelem + 127) / 128), 128, 0, s, a);
}

} // namespace pxg
