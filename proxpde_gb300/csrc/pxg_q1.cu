// Q1 hexahedron element kernel with the 2x2x2 Gauss rule, written for GB300's FP64
// rate (about 1.2 TFLOP/s, 1/58 of FP32): it computes the same element matrices as
// the generic kernel (and as proxpde's CurFE + AssemblyStiffness(FE) + AssemblyMass
// + AssemblyRhsAnalytic, include/curfe.hpp:50-103, include/assembly_lhs.hpp:52-109,
// 207-221, include/assembly_rhs.hpp:61-88) with about 2.5x fewer FP64 instructions,
// by using the tensor-product structure of Q1 on the 2x2x2 rule.
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
#include "pxg_internal.h"

namespace pxg
{

namespace q1
{
constexpr double g = 0.5773502691896258;
constexpr double A = 0.5 * (1. + g);
constexpr double B = 0.5 * (1. - g);
constexpr double AA = A * A, BB = B * B, AB = A * B;

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
// W_c(q) = l_i(q) l_j(q)
__host__ __device__ constexpr double W(int c, int q) { return c == 2 ? AB : (c == q ? AA : BB); }
// sign of l'_a l'_b / (1/4)
__host__ __device__ constexpr double sgn(int a, int b) { return a == b ? 1.0 : -1.0; }

// 2-point contraction of a pair (v0 at q = 0, v1 at q = 1) with l_a
__device__ __forceinline__ double cL(int a, double v0, double v1) { return a == 0 ? A * v0 + B * v1 : B * v0 + A * v1; }
// ... with W_c
__device__ __forceinline__ double cW(int c, double v0, double v1)
{
  return c == 2 ? AB * (v0 + v1) : (c == 0 ? AA * v0 + BB * v1 : BB * v0 + AA * v1);
}

// sin(pi x) near a point whose sincospi is known: x = o + d
__device__ __forceinline__ double sinpiNear(double so, double co, double o, double d)
{
  double const u = 3.141592653589793 * d;
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

// Per-element geometry at the 8 Gauss points: G[0..5][q] = xx yy zz xy xz yz entries
// of adj(J) adj(J)^T / (4 |det J|), ad[q] = |det J_q|, off[q] = J_q xi_q.
struct Q1Geo
{
  double G[6][8];
  double ad[8];
  double off[8][3];
};

__device__ __forceinline__ void q1Geometry(double const (&X)[8][3], Q1Geo & geo)
{
  // ---- Jacobian columns: Jc[axis][p][t][r] with p, t the quadrature coordinates of
  // the two other axes in increasing order and r the physical coordinate; column
  // `axis` of J is the bilinear interpolation of half the edge differences along it
  double Jc[3][2][2][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
  {
    double dd[3][2][2];
#pragma unroll
    for (int s = 0; s < 2; ++s)
#pragma unroll
      for (int t = 0; t < 2; ++t)
      {
        dd[0][s][t] = X[node(1, s, t)][r] - X[node(0, s, t)][r]; // along x, at (y, z)
        dd[1][s][t] = X[node(s, 1, t)][r] - X[node(s, 0, t)][r]; // along y, at (x, z)
        dd[2][s][t] = X[node(s, t, 1)][r] - X[node(s, t, 0)][r]; // along z, at (x, y)
      }
#pragma unroll
    for (int ax = 0; ax < 3; ++ax)
    {
      double h[2][2];
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int t = 0; t < 2; ++t)
          h[p][t] = (0.5 * L(0, p)) * dd[ax][0][t] + (0.5 * L(1, p)) * dd[ax][1][t];
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int t = 0; t < 2; ++t)
          Jc[ax][p][t][r] = L(0, t) * h[p][0] + L(1, t) * h[p][1];
    }
  }

  // ---- per quadrature point: adjugate, |det|, geometric factors
#pragma unroll
  for (int q = 0; q < 8; ++q)
  {
    int const qx = q & 1, qy = (q >> 1) & 1, qz = q >> 2;
    double J[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
    {
      J[r][0] = Jc[0][qy][qz][r];
      J[r][1] = Jc[1][qx][qz][r];
      J[r][2] = Jc[2][qx][qy][r];
    }
    double C[3][3]; // adj(J) = J^-1 det J
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
    double const adet = fabs(det);
    geo.ad[q] = adet;
    double const s = 0.25 / adet;
    geo.G[0][q] = s * (C[0][0] * C[0][0] + C[0][1] * C[0][1] + C[0][2] * C[0][2]);
    geo.G[1][q] = s * (C[1][0] * C[1][0] + C[1][1] * C[1][1] + C[1][2] * C[1][2]);
    geo.G[2][q] = s * (C[2][0] * C[2][0] + C[2][1] * C[2][1] + C[2][2] * C[2][2]);
    geo.G[3][q] = s * (C[0][0] * C[1][0] + C[0][1] * C[1][1] + C[0][2] * C[1][2]);
    geo.G[4][q] = s * (C[0][0] * C[2][0] + C[0][1] * C[2][1] + C[0][2] * C[2][2]);
    geo.G[5][q] = s * (C[1][0] * C[2][0] + C[1][1] * C[2][1] + C[1][2] * C[2][2]);
    double const xq = qx ? g : -g, yq = qy ? g : -g, zq = qz ? g : -g;
#pragma unroll
    for (int r = 0; r < 3; ++r)
      geo.off[q][r] = J[r][0] * xq + J[r][1] * yq + J[r][2] * zq;
  }

}

// Element stiffness with unit coefficient (upper triangle j >= i of Kl).
__device__ __forceinline__ void q1Stiffness(Q1Geo const & geo, double (&Kl)[8][8])
{
  // ---- stiffness (unit coefficient), upper triangle
  {
    // diagonal-direction tables S_a[c1][c2] (c1, c2 = classes of the two other axes)
    double S[3][3][3];
#pragma unroll
    for (int ax = 0; ax < 3; ++ax)
    {
      // sum over the derivative axis, then contract the two others with W
      double H[2][2]; // [p][t] over the remaining axes in increasing order
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
      double R[2][3];
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          R[p][c] = cW(c, H[p][0], H[p][1]);
#pragma unroll
      for (int c1 = 0; c1 < 3; ++c1)
#pragma unroll
        for (int c2 = 0; c2 < 3; ++c2)
          S[ax][c1][c2] = cW(c1, R[0][c2], R[1][c2]);
    }
    // cross tables, generic in the axis pair (a < b), third axis t:
    //   U_ab[first index][second index][class], entries sum_q G_ab l(qa) l(qb) W(qt)
    double U[3][2][2][3]; // pair 0 = xy, 1 = xz, 2 = yz
#pragma unroll
    for (int pr = 0; pr < 3; ++pr)
    {
      int const axA = pr == 2 ? 1 : 0, axB = pr == 0 ? 1 : 2;
      int const axT = 3 - axA - axB;
      auto qidx = [&](int va, int vb, int vt) {
        int c[3];
        c[axA] = va, c[axB] = vb, c[axT] = vt;
        return c[0] + 2 * c[1] + 4 * c[2];
      };
      double V[2][2][3]; // [qa][qb][class of the third axis]
#pragma unroll
      for (int qa = 0; qa < 2; ++qa)
#pragma unroll
        for (int qb = 0; qb < 2; ++qb)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            V[qa][qb][c] = cW(c, geo.G[3 + pr][qidx(qa, qb, 0)], geo.G[3 + pr][qidx(qa, qb, 1)]);
      double Y[2][2][3]; // [qa][b][c]
#pragma unroll
      for (int qa = 0; qa < 2; ++qa)
#pragma unroll
        for (int bb = 0; bb < 2; ++bb)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            Y[qa][bb][c] = cL(bb, V[qa][0][c], V[qa][1][c]);
#pragma unroll
      for (int aa = 0; aa < 2; ++aa)
#pragma unroll
        for (int bb = 0; bb < 2; ++bb)
#pragma unroll
          for (int c = 0; c < 3; ++c)
            U[pr][aa][bb][c] = cL(aa, Y[0][bb][c], Y[1][bb][c]);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = i; j < 8; ++j)
      {
        int const ix = nx(i), iy = ny(i), iz = nz(i), jx = nx(j), jy = ny(j), jz = nz(j);
        int const cx = cls(ix, jx), cy = cls(iy, jy), cz = cls(iz, jz);
        double k = sgn(ix, jx) * S[0][cy][cz];
        k += sgn(iy, jy) * S[1][cx][cz];
        k += sgn(iz, jz) * S[2][cx][cy];
        // D_i,x D_j,y G_xy + D_i,y D_j,x G_yx (third axis z)
        k += sgn(ix, jy) * U[0][jx][iy][cz];
        k += sgn(iy, jx) * U[0][ix][jy][cz];
        // x, z (third axis y)
        k += sgn(ix, jz) * U[1][jx][iz][cy];
        k += sgn(iz, jx) * U[1][ix][jz][cy];
        // y, z (third axis x)
        k += sgn(iy, jz) * U[2][jy][iz][cx];
        k += sgn(iz, jy) * U[2][iy][jz][cx];
        Kl[i][j] = k;
      }
  }

}

} // namespace q1

__global__ void __launch_bounds__(128) kAssembleQ1(AsmArgs a)
{
  using namespace q1;
  int64_t const e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= a.nelem)
    return;

  // ---- inputs: vertex ids, coordinates, DOF ids, BC flags
  double X[8][3];
  uint32_t dof[8];
  {
    uint4 const c0 = reinterpret_cast<uint4 const *>(a.conn)[2 * e];
    uint4 const c1 = reinterpret_cast<uint4 const *>(a.conn)[2 * e + 1];
    uint32_t const v[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
#pragma unroll
    for (int n = 0; n < 8; ++n)
#pragma unroll
      for (int d = 0; d < 3; ++d)
        X[n][d] = a.xyz[3 * (int64_t)v[n] + d];
    uint4 const d0 = reinterpret_cast<uint4 const *>(a.emap)[2 * e];
    uint4 const d1 = reinterpret_cast<uint4 const *>(a.emap)[2 * e + 1];
    dof[0] = d0.x, dof[1] = d0.y, dof[2] = d0.z, dof[3] = d0.w;
    dof[4] = d1.x, dof[5] = d1.y, dof[6] = d1.z, dof[7] = d1.w;
  }
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

  Q1Geo geo;
  q1Geometry(X, geo);
  double Kl[8][8];
  if (needK)
    q1Stiffness(geo, Kl);
  double const (&ad)[8] = geo.ad;
  double const (&off)[8][3] = geo.off;

  // ---- mass table Mt[cx][cy][cz] (unit coefficient)
  double Mt[3][3][3];
  if (needM)
  {
    double Vm[2][2][3]; // [qx][qy][cz]
#pragma unroll
    for (int qx = 0; qx < 2; ++qx)
#pragma unroll
      for (int qy = 0; qy < 2; ++qy)
#pragma unroll
        for (int c = 0; c < 3; ++c)
          Vm[qx][qy][c] = cW(c, ad[qx + 2 * qy], ad[qx + 2 * qy + 4]);
    double Ym[2][3][3]; // [qx][cy][cz]
#pragma unroll
    for (int qx = 0; qx < 2; ++qx)
#pragma unroll
      for (int cy = 0; cy < 3; ++cy)
#pragma unroll
        for (int cz = 0; cz < 3; ++cz)
          Ym[qx][cy][cz] = cW(cy, Vm[qx][0][cz], Vm[qx][1][cz]);
#pragma unroll
    for (int cx = 0; cx < 3; ++cx)
#pragma unroll
      for (int cy = 0; cy < 3; ++cy)
#pragma unroll
        for (int cz = 0; cz < 3; ++cz)
          Mt[cx][cy][cz] = cW(cx, Ym[0][cy][cz], Ym[1][cy][cz]);
  }

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
    double const ks = op.stiff ? (op.stiff == 2 ? op.sc * kfac : op.sc) : 0.;
    double const ms = op.mass ? op.mc : 0.;
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = i; j < 8; ++j)
      {
        double val = 0.;
        if (op.stiff)
          val = ks * Kl[i][j];
        if (op.mass)
          val = fma(ms, Mt[cls(nx(i), nx(j))][cls(ny(i), ny(j))][cls(nz(i), nz(j))], val);
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
    double rq[8];
    if (a.rkind == 1)
    {
      double o[3];
#pragma unroll
      for (int d = 0; d < 3; ++d)
        o[d] = .125 * (X[0][d] + X[1][d] + X[2][d] + X[3][d] + X[4][d] + X[5][d] + X[6][d] + X[7][d]);
      if (a.fn == PXG_FN_SIN3)
      {
        double so[3], co[3];
#pragma unroll
        for (int d = 0; d < 3; ++d)
          sincospi(o[d], &so[d], &co[d]);
#pragma unroll
        for (int q = 0; q < 8; ++q)
        {
          double const f = sinpiNear(so[0], co[0], o[0], off[q][0]) * sinpiNear(so[1], co[1], o[1], off[q][1]) *
                           sinpiNear(so[2], co[2], o[2], off[q][2]);
          rq[q] = ad[q] * (a.rc * f);
        }
      }
      else
      {
#pragma unroll
        for (int q = 0; q < 8; ++q)
          rq[q] = ad[q] * evalFn(a.fn, a.rc, o[0] + off[q][0], o[1] + off[q][1], o[2] + off[q][2]);
      }
    }
    else
    {
      // projection of a DOF field: f_q = coef * sum_n phi_n(q) field_n
      double loc[8];
#pragma unroll
      for (int n = 0; n < 8; ++n)
        loc[n] = a.field[dof[n]];
#pragma unroll
      for (int q = 0; q < 8; ++q)
      {
        int const qx = q & 1, qy = (q >> 1) & 1, qz = q >> 2;
        double s = 0.;
#pragma unroll
        for (int n = 0; n < 8; ++n)
          s += (L(nx(n), qx) * L(ny(n), qy) * L(nz(n), qz)) * loc[n];
        rq[q] = ad[q] * (a.rc * s);
      }
    }
    double Fv[2][2][2]; // contract z, then y, then x
    double Ry[2][2][2]; // [qx][qy][iz]
#pragma unroll
    for (int qx = 0; qx < 2; ++qx)
#pragma unroll
      for (int qy = 0; qy < 2; ++qy)
#pragma unroll
        for (int iz = 0; iz < 2; ++iz)
          Ry[qx][qy][iz] = cL(iz, rq[qx + 2 * qy], rq[qx + 2 * qy + 4]);
    double Rx[2][2][2]; // [qx][iy][iz]
#pragma unroll
    for (int qx = 0; qx < 2; ++qx)
#pragma unroll
      for (int iy = 0; iy < 2; ++iy)
#pragma unroll
        for (int iz = 0; iz < 2; ++iz)
          Rx[qx][iy][iz] = cL(iy, Ry[qx][0][iz], Ry[qx][1][iz]);
#pragma unroll
    for (int ix = 0; ix < 2; ++ix)
#pragma unroll
      for (int iy = 0; iy < 2; ++iy)
#pragma unroll
        for (int iz = 0; iz < 2; ++iz)
          Fv[ix][iy][iz] = cL(ix, Rx[0][iy][iz], Rx[1][iy][iz]);
#pragma unroll
    for (int i = 0; i < 8; ++i)
    {
      if (a.rbc && ((cons >> i) & 1u))
        continue;
      atomicAdd(a.b + dof[i], Fv[nx(i)][ny(i)][nz(i)]);
    }
  }
}

void launchAssembleQ1(AsmArgs const & a, cudaStream_t s)
{
  unsigned const blocks = (unsigned)((a.nelem + 127) / 128);
  kAssembleQ1<<<blocks, 128, 0, s>>>(a);
}

// Adjoint gradient g_e = -(C u)_e^T K_e (C lambda)_e, K_e = k_e K0_e (Q1, 2x2x2 rule):
// the same element stiffness as kAssembleQ1, contracted with the two local vectors.
__global__ void __launch_bounds__(128) kAdjointGradQ1(AdjArgs a)
{
  using namespace q1;
  int64_t const e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= a.nelem)
    return;
  double X[8][3], ue[8], le[8];
  {
    uint4 const c0 = reinterpret_cast<uint4 const *>(a.conn)[2 * e];
    uint4 const c1 = reinterpret_cast<uint4 const *>(a.conn)[2 * e + 1];
    uint32_t const v[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
#pragma unroll
    for (int n = 0; n < 8; ++n)
#pragma unroll
      for (int d = 0; d < 3; ++d)
        X[n][d] = a.xyz[3 * (int64_t)v[n] + d];
    uint4 const d0 = reinterpret_cast<uint4 const *>(a.emap)[2 * e];
    uint4 const d1 = reinterpret_cast<uint4 const *>(a.emap)[2 * e + 1];
    uint32_t const dof[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
#pragma unroll
    for (int i = 0; i < 8; ++i)
    {
      bool const c = a.bcMask && a.bcMask[dof[i]];
      ue[i] = c ? 0. : a.u[dof[i]];
      le[i] = c ? 0. : a.lam[dof[i]];
    }
  }
  Q1Geo geo;
  q1Geometry(X, geo);
  double Kl[8][8];
  q1Stiffness(geo, Kl);
  double s = 0.;
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = i; j < 8; ++j)
      s = fma(Kl[i][j], (i == j) ? ue[i] * le[i] : fma(ue[i], le[j], ue[j] * le[i]), s);
  a.g[e] = -(a.kE[e] * s);
}

void launchAdjointGradQ1(AdjArgs const & a, cudaStream_t s)
{
  kAdjointGradQ1<<<(unsigned)((a.nelem + 127) / 128), 128, 0, s>>>(a);
}

} // namespace pxg
