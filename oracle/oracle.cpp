// CPU oracle for the proxpde finite-element assembly path.
//
// TEST INFRASTRUCTURE ONLY. This file restates, in plain C++17 without Eigen, the
// algorithm of proxpde's serial element loop so that the GPU engine can be checked
// against it. It is called by tests/, by __graft_entry__.smoke() and by the CPU
// baseline legs of bench.py, and never by the engine in proxpde_gb300/.
//
// What is restated, and from where (paths inside the proxpde project):
//   - quadrature rules Tet4, Tet11, Hex8, Hex27 .............. src/qr.cpp:27, 38, 199-320
//     and their selection per element (RecommendedQR) ........ include/fe.hpp:96-131
//   - reference elements P1/P2 tet, Q1/Q2 hex (phi, dphi,
//     mapping = dphi, dofPts/mappingPts ordering) ............ include/reffe.hpp:687-993,
//                                                              src/reffe.cpp:246-253, 374-383, 510-1003
//   - element origin (tet: pts[0], hex: vertex average) ...... include/geo.hpp:583-588, 721-728
//   - CurFE::reinit (jac, jacPlus=(J^T J)^-1 J^T,
//     detJ=sqrt(det(J^T J)), JxW, qpoint=origin+J*xi, dphi) . include/curfe.hpp:50-103
//   - AssemblyStiffness / AssemblyStiffnessFE (P0 coefficient)
//     / AssemblyScalarMass ................................... include/assembly_lhs.hpp:52-65, 93-109, 207-221
//     FEVar P0 evaluate (phi=1 times the element value) ....... include/var.hpp:111-127, 264-285
//   - AssemblyRhsAnalytic / AssemblyS2SProjection ........... include/assembly_rhs.hpp:61-88, 130-159
//   - Builder::buildLhs / buildRhs element loop, Dirichlet
//     condensation and triplet emission ...................... include/builder.hpp:31-154, 279-364
//   - Builder::closeMatrix = Eigen setFromTriplets (duplicates
//     summed in emission order) + prune(1, 1e-16) ............ include/builder.hpp:366-371
//   - DOF::setupElemMap first-touch numbering ............... include/dof.hpp:111-329
//   - buildCube for hexahedra and 5-tet cubes ............... src/mesh.cpp:355-534
//   - interpolateAnalyticFunction (Lagrange: value at dofPts) include/fespace.hpp:195-271
//
// Floating point: every operation is IEEE double and follows the loop order of the
// reference expressions. Eigen may evaluate small fixed-size products in another
// summation order, so agreement with the reference is to round-off (parity tests use
// 1e-12 relative), not bit for bit. Compile without -ffast-math and with
// -ffp-contract=off so that both machines give identical results.

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace
{

enum ElemType : int
{
  P1TET = 0,
  P2TET = 1,
  Q1HEX = 2,
  Q2HEX = 3,
};

constexpr double PI = 3.14159265358979323846;

// ---------------------------------------------------------------- quadrature
// src/qr.cpp:27 and :38 (the reference stores these truncated literals).
constexpr double sqrt13rd = 0.5773502691896258;
constexpr double sqrt35th = 0.774596669241483;

struct QRule
{
  int n;
  std::vector<std::array<double, 3>> node;
  std::vector<double> w;
};

QRule makeTet4()
{
  // src/qr.cpp:209-221
  QRule r;
  r.n = 4;
  double const a = 0.1381966011250105, b = 0.5854101966249685;
  r.node = {{a, a, a}, {b, a, a}, {a, b, a}, {a, a, b}};
  r.w.assign(4, .25 / 6);
  return r;
}

QRule makeTet11()
{
  // src/qr.cpp:223-246
  QRule r;
  r.n = 11;
  double const c1 = 0.0714285714285714, c2 = 0.7857142857142857;
  double const d1 = 0.399403576166799, d2 = 0.100596423833201;
  r.node = {
      {0.25, 0.25, 0.25},
      {c1, c1, c1},
      {c2, c1, c1},
      {c1, c2, c1},
      {c1, c1, c2},
      {d1, d1, d2},
      {d1, d2, d1},
      {d2, d1, d1},
      {d1, d2, d2},
      {d2, d1, d2},
      {d2, d2, d1},
  };
  double const w0 = -0.0131555555555556, w1 = 0.0076222222222222, w2 = 0.024888888888889;
  r.w = {w0, w1, w1, w1, w1, w2, w2, w2, w2, w2, w2};
  return r;
}

QRule makeHex8()
{
  // src/qr.cpp:260-280: x fastest, then y, then z; unit weights.
  QRule r;
  r.n = 8;
  for (int k = 0; k < 2; ++k)
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i)
        r.node.push_back(
            {i ? sqrt13rd : -sqrt13rd, j ? sqrt13rd : -sqrt13rd, k ? sqrt13rd : -sqrt13rd});
  r.w.assign(8, 1.0);
  return r;
}

QRule makeHex27()
{
  // src/qr.cpp:282-320: tensor Gauss-3, x fastest; weights (5,8,5)^3 / 729.
  QRule r;
  r.n = 27;
  double const x[3] = {-sqrt35th, 0.0, sqrt35th};
  double const w1[3] = {5., 8., 5.};
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i)
      {
        r.node.push_back({x[i], x[j], x[k]});
        r.w.push_back((w1[i] * w1[j] * w1[k]) / 729.);
      }
  return r;
}

// ---------------------------------------------------------- reference elements
// 1D Lagrange factors of the hexahedral elements (src/reffe.cpp:246-253, 374-383).
inline double fQ1(int a, double x) { return a == 0 ? 0.5 * (1. - x) : 0.5 * (1. + x); }
inline double dfQ1(int a, double) { return a == 0 ? -0.5 : +0.5; }
inline double fQ2(int a, double x)
{
  return a == 0 ? 0.5 * x * (x - 1.) : (a == 1 ? 0.5 * x * (x + 1.) : 1. - x * x);
}
inline double dfQ2(int a, double x) { return a == 0 ? x - 0.5 : (a == 1 ? x + 0.5 : -2. * x); }

// Q1 node -> 1D factor index per axis (src/reffe.cpp:684-759).
constexpr int q1idx[8][3] = {
    {0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
// Q2 node -> 1D factor index per axis (src/reffe.cpp:762-1003).
constexpr int q2idx[27][3] = {
    {0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1},
    {0, 1, 1}, {2, 0, 0}, {1, 2, 0}, {2, 1, 0}, {0, 2, 0}, {0, 0, 2}, {1, 0, 2},
    {1, 1, 2}, {0, 1, 2}, {2, 0, 1}, {1, 2, 1}, {2, 1, 1}, {0, 2, 1}, {2, 2, 0},
    {0, 2, 2}, {2, 0, 2}, {1, 2, 2}, {2, 1, 2}, {2, 2, 1}, {2, 2, 2}};
// tet P2 edge dofs (include/reffe.hpp:725-777, include/geo.hpp:526-529)
constexpr int tetEdge[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
// hex edges and faces (include/geo.hpp:640-665)
constexpr int hexEdge[12][2] = {
    {0, 1}, {1, 2}, {2, 3}, {3, 0}, {0, 4}, {1, 5}, {2, 6}, {3, 7}, {4, 5}, {5, 6}, {6, 7}, {7, 4}};
constexpr int hexFace[6][4] = {
    {0, 3, 2, 1}, {3, 0, 4, 7}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {4, 5, 6, 7}};

int numDofs(int t) { return t == P1TET ? 4 : t == P2TET ? 10 : t == Q1HEX ? 8 : 27; }
int numVerts(int t) { return (t == P1TET || t == P2TET) ? 4 : 8; }
bool isHex(int t) { return t == Q1HEX || t == Q2HEX; }

QRule const & rule(int t)
{
  static QRule const tet4 = makeTet4(), tet11 = makeTet11(), hex8 = makeHex8(), hex27 = makeHex27();
  return t == P1TET ? tet4 : t == P2TET ? tet11 : t == Q1HEX ? hex8 : hex27;
}

// phi_i(p) and grad phi_i(p) on the reference element, as written in src/reffe.cpp.
void shape(int t, double const * p, double * phi, double * dphi)
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
      int const a = tetEdge[e][0], b = tetEdge[e][1];
      phi[4 + e] = 4. * l[a] * l[b];
      for (int d = 0; d < 3; ++d)
        dphi[3 * (4 + e) + d] = 4. * (l[a] * dl[b][d] + dl[a][d] * l[b]);
    }
    return;
  }
  int const n = numDofs(t);
  for (int i = 0; i < n; ++i)
  {
    int const * ix = (t == Q1HEX) ? q1idx[i] : q2idx[i];
    double fx, fy, fz, gx, gy, gz;
    if (t == Q1HEX)
    {
      fx = fQ1(ix[0], x), fy = fQ1(ix[1], y), fz = fQ1(ix[2], z);
      gx = dfQ1(ix[0], x), gy = dfQ1(ix[1], y), gz = dfQ1(ix[2], z);
    }
    else
    {
      fx = fQ2(ix[0], x), fy = fQ2(ix[1], y), fz = fQ2(ix[2], z);
      gx = dfQ2(ix[0], x), gy = dfQ2(ix[1], y), gz = dfQ2(ix[2], z);
    }
    phi[i] = fx * fy * fz;
    dphi[3 * i + 0] = gx * fy * fz;
    dphi[3 * i + 1] = fx * gy * fz;
    dphi[3 * i + 2] = fx * fy * gz;
  }
}

// RefFE::mappingPts == dofPts (include/reffe.hpp:710-715, 748-767, 902-917, 960-988).
void mappingPoints(int t, double const (*X)[3], double (*P)[3])
{
  int const nv = numVerts(t);
  for (int v = 0; v < nv; ++v)
    for (int d = 0; d < 3; ++d)
      P[v][d] = X[v][d];
  if (t == P2TET)
  {
    for (int e = 0; e < 6; ++e)
      for (int d = 0; d < 3; ++d)
        P[4 + e][d] = .5 * (X[tetEdge[e][0]][d] + X[tetEdge[e][1]][d]);
  }
  else if (t == Q2HEX)
  {
    for (int e = 0; e < 12; ++e)
      for (int d = 0; d < 3; ++d)
        P[8 + e][d] = 0.5 * (X[hexEdge[e][0]][d] + X[hexEdge[e][1]][d]);
    for (int f = 0; f < 6; ++f)
      for (int d = 0; d < 3; ++d)
        P[20 + f][d] = 0.25 * (X[hexFace[f][0]][d] + X[hexFace[f][1]][d] + X[hexFace[f][2]][d] +
                               X[hexFace[f][3]][d]);
    for (int d = 0; d < 3; ++d)
      P[26][d] = .125 * (X[0][d] + X[1][d] + X[2][d] + X[3][d] + X[4][d] + X[5][d] + X[6][d] +
                         X[7][d]);
  }
}

// GeoElem::origin (include/geo.hpp:588 tet, :721-728 hex).
void origin(int t, double const (*X)[3], double * o)
{
  if (!isHex(t))
  {
    for (int d = 0; d < 3; ++d)
      o[d] = X[0][d];
    return;
  }
  for (int d = 0; d < 3; ++d)
    o[d] = .125 * (X[0][d] + X[1][d] + X[2][d] + X[3][d] + X[4][d] + X[5][d] + X[6][d] + X[7][d]);
}

// -------------------------------------------------------------------- CurFE
struct CurFE
{
  int t, qrt, N, nq; // element type, element type whose rule is used (FESpace's QR)
  // constant tables (curfe.hpp:20-45)
  std::vector<double> phiRef;  // nq x N
  std::vector<double> dphiRef; // nq x N x 3 (also the mapping table: mapping = dphiFun)
  // per element
  std::vector<double> JxW;   // nq
  std::vector<double> qpt;   // nq x 3
  std::vector<double> dphi;  // nq x N x 3
  std::vector<double> dofPts; // N x 3

  explicit CurFE(int type, int qrType = -1):
      t(type), qrt(qrType < 0 ? type : qrType), N(numDofs(type)), nq(rule(qrt).n)
  {
    phiRef.resize(nq * N);
    dphiRef.resize(nq * N * 3);
    for (int q = 0; q < nq; ++q)
      shape(t, rule(qrt).node[q].data(), &phiRef[q * N], &dphiRef[q * N * 3]);
    JxW.resize(nq);
    qpt.resize(nq * 3);
    dphi.resize(nq * N * 3);
    dofPts.resize(N * 3);
  }

  // curfe.hpp:50-103
  void reinit(double const (*X)[3])
  {
    auto P = reinterpret_cast<double(*)[3]>(dofPts.data());
    mappingPoints(t, X, P);
    double o[3];
    origin(t, X, o);
    QRule const & qr = rule(qrt);
    for (int q = 0; q < nq; ++q)
    {
      double J[3][3] = {};
      double const * M = &dphiRef[q * N * 3];
      for (int n = 0; n < N; ++n)
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c)
            J[r][c] += P[n][r] * M[3 * n + c];
      // J^T J, its inverse, sqrt(det), J^+ = (J^T J)^-1 J^T
      double A[3][3];
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
          A[a][b] = J[0][a] * J[0][b] + J[1][a] * J[1][b] + J[2][a] * J[2][b];
      double const c00 = A[1][1] * A[2][2] - A[1][2] * A[2][1];
      double const c01 = A[1][2] * A[2][0] - A[1][0] * A[2][2];
      double const c02 = A[1][0] * A[2][1] - A[1][1] * A[2][0];
      double const det = A[0][0] * c00 + A[0][1] * c01 + A[0][2] * c02;
      double Ai[3][3];
      Ai[0][0] = c00 / det;
      Ai[1][0] = c01 / det;
      Ai[2][0] = c02 / det;
      Ai[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) / det;
      Ai[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) / det;
      Ai[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) / det;
      Ai[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) / det;
      Ai[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) / det;
      Ai[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) / det;
      double Jp[3][3]; // dim x 3
      for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c)
          Jp[a][c] = Ai[a][0] * J[c][0] + Ai[a][1] * J[c][1] + Ai[a][2] * J[c][2];
      double const detJ = std::sqrt(det);
      JxW[q] = detJ * qr.w[q];
      double const * xi = qr.node[q].data();
      for (int r = 0; r < 3; ++r)
        qpt[3 * q + r] = o[r] + (J[r][0] * xi[0] + J[r][1] * xi[1] + J[r][2] * xi[2]);
      double * D = &dphi[q * N * 3];
      for (int i = 0; i < N; ++i)
        for (int c = 0; c < 3; ++c)
          D[3 * i + c] = M[3 * i + 0] * Jp[0][c] + M[3 * i + 1] * Jp[1][c] + M[3 * i + 2] * Jp[2][c];
    }
  }
};

// --------------------------------------------------------- analytic functions
// Registry of the analytic right-hand sides (the reference passes a std::function,
// assembly_rhs.hpp:50-59; the GPU engine keeps the same functions as numbered ids).
double rhsFun(int fn, double c, double const * p)
{
  switch (fn)
  {
  case 0: // constant
    return c;
  case 1: // c sin(pi x) sin(pi y) sin(pi z)
    return c * (std::sin(PI * p[0]) * std::sin(PI * p[1]) * std::sin(PI * p[2]));
  case 2: // the proxpde poisson3d tests: 2.5 pi^2 sin(pi x / 2) sin(3 pi y / 2)
    return c * (2.5 * PI * PI * std::sin(0.5 * PI * p[0]) * std::sin(1.5 * PI * p[1]));
  case 3: // exact solution of those tests: sin(pi x / 2) sin(3 pi y / 2)
    return c * (std::sin(0.5 * PI * p[0]) * std::sin(1.5 * PI * p[1]));
  default:
    return NAN;
  }
}

} // namespace

// ============================================================== C interface
extern "C"
{

struct orc_lhs
{
  int32_t stiff_kind;  // 0 none, 1 constant coefficient, 2 per-element coefficient (P0 FEVar)
  double stiff_c;      // the constant (kind 1)
  double const * k_e;  // per-element values (kind 2)
  int32_t mass_kind;   // 0 none, 1 constant coefficient, 2 per-element coefficient (P0 FEVar)
  double mass_c;       // the constant (kind 1)
  int32_t apply_bc;    // condense with the essential BC set (builder.hpp:76-124)
  double const * m_e;  // per-element values (mass kind 2)
};

struct orc_rhs
{
  int32_t kind;          // 0 none, 1 analytic function (AssemblyRhsAnalytic), 2 L2 projection (AssemblyS2SProjection)
  int32_t fn;            // analytic function id (kind 1)
  double c;              // scale of the function (kind 1) / projection coefficient (kind 2)
  double const * field;  // DOF vector projected (kind 2)
  int32_t apply_bc;      // zero constrained rows (builder.hpp:319-347)
};

int orc_num_dofs(int t) { return numDofs(t); }
int orc_num_verts(int t) { return numVerts(t); }
int orc_num_qpts(int t) { return rule(t).n; }

int orc_quadrature(int t, double * nodes, double * weights)
{
  QRule const & r = rule(t);
  for (int q = 0; q < r.n; ++q)
  {
    for (int d = 0; d < 3; ++d)
      nodes[3 * q + d] = r.node[q][d];
    weights[q] = r.w[q];
  }
  return r.n;
}

int orc_shape(int t, double const * p, double * phi, double * dphi)
{
  shape(t, p, phi, dphi);
  return numDofs(t);
}

// Structured cube of n^3 hexahedra on [0,1]^3 (src/mesh.cpp:456-534).
// xyz: (n+1)^3 x 3, conn: n^3 x 8.
int64_t orc_cube_hex(int n, double * xyz, uint32_t * conn)
{
  int const np = n + 1;
  double const h = 1.0 / n;
  for (int k = 0; k < np; ++k)
    for (int j = 0; j < np; ++j)
      for (int i = 0; i < np; ++i)
      {
        int64_t const id = i + (int64_t)np * j + (int64_t)np * np * k;
        xyz[3 * id + 0] = 0. + i * h;
        xyz[3 * id + 1] = 0. + j * h;
        xyz[3 * id + 2] = 0. + k * h;
      }
  int64_t const dx = 1, dy = np, dz = (int64_t)np * np;
  int64_t c = 0;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
      {
        int64_t const b = i + j * (int64_t)np + k * (int64_t)np * np;
        int64_t const v[8] = {b, b + dx, b + dx + dy, b + dy, b + dz, b + dx + dz, b + dx + dy + dz, b + dy + dz};
        for (int a = 0; a < 8; ++a)
          conn[8 * c + a] = (uint32_t)v[a];
        ++c;
      }
  return c;
}

// Structured cube of n^3 cubes, each split in 5 tetrahedra (src/mesh.cpp:355-454).
int64_t orc_cube_tet5(int n, double * xyz, uint32_t * conn)
{
  int const np = n + 1;
  double const h = 1.0 / n;
  for (int k = 0; k < np; ++k)
    for (int j = 0; j < np; ++j)
      for (int i = 0; i < np; ++i)
      {
        int64_t const id = i + (int64_t)np * j + (int64_t)np * np * k;
        xyz[3 * id + 0] = 0. + i * h;
        xyz[3 * id + 1] = 0. + j * h;
        xyz[3 * id + 2] = 0. + k * h;
      }
  int64_t const dx = 1, dy = np, dz = (int64_t)np * np;
  int64_t c = 0;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
      {
        int64_t const b = i + j * (int64_t)np + k * (int64_t)np * np;
        int64_t t[5][4];
        if ((i + j + k) % 2)
        {
          int64_t const odd[5][4] = {
              {b + dx, b + dy, b + dz, b + dx + dy + dz},
              {b, b + dx, b + dy, b + dz},
              {b + dx, b + dx + dy, b + dy, b + dx + dy + dz},
              {b + dx, b + dz, b + dx + dz, b + dx + dy + dz},
              {b + dy, b + dz, b + dx + dy + dz, b + dy + dz}};
          std::memcpy(t, odd, sizeof(t));
        }
        else
        {
          int64_t const even[5][4] = {
              {b, b + dx + dy, b + dx + dz, b + dy + dz},
              {b, b + dx, b + dx + dy, b + dx + dz},
              {b, b + dx + dy, b + dy, b + dy + dz},
              {b, b + dz, b + dx + dz, b + dy + dz},
              {b + dx + dy, b + dx + dz, b + dx + dy + dz, b + dy + dz}};
          std::memcpy(t, even, sizeof(t));
        }
        for (int r = 0; r < 5; ++r)
        {
          for (int a = 0; a < 4; ++a)
            conn[4 * c + a] = (uint32_t)t[r][a];
          ++c;
        }
      }
  return c;
}

// First-touch DOF numbering (dof.hpp:111-329, scalar space, BLOCK ordering).
// elemMap: nelem x numDofs(t). Returns the number of DOFs.
int64_t orc_dofmap(int t, int64_t nnodes, uint32_t const * conn, int64_t nelem, uint32_t * elemMap)
{
  int const nv = numVerts(t), N = numDofs(t);
  uint32_t const unset = 0xffffffffu;
  std::vector<uint32_t> ptMap(nnodes, unset);
  std::map<std::array<uint32_t, 2>, uint32_t> edgeDofs;
  std::map<std::array<uint32_t, 4>, uint32_t> faceDofs;
  uint32_t size = 0;
  for (int64_t e = 0; e < nelem; ++e)
  {
    uint32_t const * v = conn + e * nv;
    uint32_t * m = elemMap + e * N;
    int l = 0;
    for (int a = 0; a < nv; ++a) // points
    {
      if (ptMap[v[a]] == unset)
        ptMap[v[a]] = size++;
      m[l++] = ptMap[v[a]];
    }
    if (t == P2TET || t == Q2HEX) // edges, identified by the set of their points
    {
      int const ne = (t == P2TET) ? 6 : 12;
      for (int k = 0; k < ne; ++k)
      {
        int const * ed = (t == P2TET) ? tetEdge[k] : hexEdge[k];
        std::array<uint32_t, 2> key = {v[ed[0]], v[ed[1]]};
        std::sort(key.begin(), key.end());
        auto it = edgeDofs.find(key);
        if (it == edgeDofs.end())
          it = edgeDofs.emplace(key, size++).first;
        m[l++] = it->second;
      }
    }
    if (t == Q2HEX) // faces, then the element itself
    {
      for (int f = 0; f < 6; ++f)
      {
        std::array<uint32_t, 4> key = {v[hexFace[f][0]], v[hexFace[f][1]], v[hexFace[f][2]], v[hexFace[f][3]]};
        std::sort(key.begin(), key.end());
        auto it = faceDofs.find(key);
        if (it == faceDofs.end())
          it = faceDofs.emplace(key, size++).first;
        m[l++] = it->second;
      }
      m[l++] = size++;
    }
  }
  return size;
}

// DOF coordinates (dofPts of every element scattered by elemMap), used by
// interpolateAnalyticFunction (fespace.hpp:195-271) and by BC selection.
int orc_dof_coords(int t, double const * xyz, uint32_t const * conn, int64_t nelem,
                   uint32_t const * elemMap, double * dofxyz)
{
  int const nv = numVerts(t), N = numDofs(t);
  double X[8][3], P[27][3];
  for (int64_t e = 0; e < nelem; ++e)
  {
    for (int a = 0; a < nv; ++a)
      for (int d = 0; d < 3; ++d)
        X[a][d] = xyz[3 * (int64_t)conn[e * nv + a] + d];
    mappingPoints(t, X, P);
    for (int i = 0; i < N; ++i)
      for (int d = 0; d < 3; ++d)
        dofxyz[3 * (int64_t)elemMap[e * N + i] + d] = P[i][d];
  }
  return 0;
}

int orc_interpolate(int t, double const * xyz, uint32_t const * conn, int64_t nelem,
                    uint32_t const * elemMap, int fn, double c, double * v)
{
  int const nv = numVerts(t), N = numDofs(t);
  double X[8][3], P[27][3];
  for (int64_t e = 0; e < nelem; ++e)
  {
    for (int a = 0; a < nv; ++a)
      for (int d = 0; d < 3; ++d)
        X[a][d] = xyz[3 * (int64_t)conn[e * nv + a] + d];
    mappingPoints(t, X, P);
    for (int i = 0; i < N; ++i)
      v[elemMap[e * N + i]] = rhsFun(fn, c, P[i]);
  }
  return 0;
}

// Local element matrices/vector of one element, before any BC treatment.
// Ke/Me: N x N row-major, Fe: N. Any output may be NULL.
int orc_element(int t, double const * xyz, uint32_t const * conn, int64_t e,
                orc_lhs const * lhs, orc_rhs const * rhs, uint32_t const * elemMap,
                double * Ke, double * Fe)
{
  int const nv = numVerts(t), N = numDofs(t);
  thread_local CurFE * fe = nullptr;
  thread_local int feType = -1;
  if (feType != t)
  {
    delete fe;
    fe = new CurFE(t);
    feType = t;
  }
  double X[8][3];
  for (int a = 0; a < nv; ++a)
    for (int d = 0; d < 3; ++d)
      X[a][d] = xyz[3 * (int64_t)conn[e * nv + a] + d];
  fe->reinit(X);
  int const nq = fe->nq;
  if (Ke)
  {
    for (int i = 0; i < N * N; ++i)
      Ke[i] = 0.;
    if (lhs && lhs->stiff_kind)
    {
      // AssemblyStiffness (assembly_lhs.hpp:52-65) / AssemblyStiffnessFE with a P0
      // coefficient (:93-109; FEVar::evaluate = 1 * k_e, var.hpp:264-285)
      double const c = lhs->stiff_kind == 1 ? lhs->stiff_c : 1.0 * lhs->k_e[e];
      for (int q = 0; q < nq; ++q)
      {
        double const s = c * fe->JxW[q];
        double const * D = &fe->dphi[q * N * 3];
        for (int i = 0; i < N; ++i)
        {
          double const a0 = s * D[3 * i], a1 = s * D[3 * i + 1], a2 = s * D[3 * i + 2];
          for (int j = 0; j < N; ++j)
            Ke[i * N + j] += a0 * D[3 * j] + a1 * D[3 * j + 1] + a2 * D[3 * j + 2];
        }
      }
    }
    if (lhs && lhs->mass_kind)
    {
      // AssemblyScalarMass (assembly_lhs.hpp:207-221) / AssemblyMassFE with a P0
      // coefficient (:262-277: coef = 1, FEVar::evaluate = 1 * m_e)
      double const c = lhs->mass_kind == 1 ? lhs->mass_c : 1.0 * lhs->m_e[e];
      for (int q = 0; q < nq; ++q)
      {
        double const s = c * fe->JxW[q];
        double const * p = &fe->phiRef[q * N];
        for (int i = 0; i < N; ++i)
        {
          double const a = s * p[i];
          for (int j = 0; j < N; ++j)
            Ke[i * N + j] += a * p[j];
        }
      }
    }
  }
  if (Fe)
  {
    for (int i = 0; i < N; ++i)
      Fe[i] = 0.;
    if (rhs && rhs->kind == 1)
    {
      // AssemblyRhsAnalytic (assembly_rhs.hpp:61-88)
      for (int q = 0; q < nq; ++q)
      {
        double const f = rhsFun(rhs->fn, rhs->c, &fe->qpt[3 * q]);
        double const * p = &fe->phiRef[q * N];
        for (int i = 0; i < N; ++i)
          Fe[i] += fe->JxW[q] * p[i] * f;
      }
    }
    else if (rhs && rhs->kind == 3)
    {
      // AssemblyRhsAnalytic (assembly_rhs.hpp:61-88) with f(qpoint) given: values of
      // an arbitrary function at this element's CurFE::qpoint, field[e * nq + q]
      for (int q = 0; q < nq; ++q)
      {
        double const f = rhs->c * rhs->field[e * nq + q];
        double const * p = &fe->phiRef[q * N];
        for (int i = 0; i < N; ++i)
          Fe[i] += fe->JxW[q] * p[i] * f;
      }
    }
    else if (rhs && rhs->kind == 2)
    {
      // AssemblyS2SProjection (assembly_rhs.hpp:130-159)
      double loc[27];
      for (int n = 0; n < N; ++n)
        loc[n] = rhs->field[elemMap[e * N + n]];
      for (int q = 0; q < nq; ++q)
      {
        double const * p = &fe->phiRef[q * N];
        double rq = 0.;
        for (int n = 0; n < N; ++n)
          rq += p[n] * loc[n];
        for (int i = 0; i < N; ++i)
          Fe[i] += rhs->c * fe->JxW[q] * p[i] * rq;
      }
    }
  }
  return 0;
}

// CurFE::qpoint (curfe.hpp:80) of every element and quadrature point:
// out[(e * nq + q) * 3 + d]
void orc_qpoints(int t, double const * xyz, uint32_t const * conn, int64_t nelem, double * out)
{
  int const nv = numVerts(t);
  CurFE fe(t);
  for (int64_t e = 0; e < nelem; ++e)
  {
    double X[8][3];
    for (int a = 0; a < nv; ++a)
      for (int d = 0; d < 3; ++d)
        X[a][d] = xyz[3 * (int64_t)conn[e * nv + a] + d];
    fe.reinit(X);
    for (int k = 0; k < fe.nq * 3; ++k)
      out[e * fe.nq * 3 + k] = fe.qpt[k];
  }
}

// ------------------------------------------------------------------ builder
struct OrcTriplet
{
  int32_t r, c;
  double v;
};

struct orc_csr
{
  int64_t n;
  int64_t nnz;
  std::vector<int32_t> rowPtr;
  std::vector<int32_t> col;
  std::vector<double> val;
};

// Builder::buildLhs + buildRhs + closeMatrix for one matrix and one vector.
//   lhs may be NULL (no matrix), rhs may be NULL (no load vector).
//   bc_mask[ndof] != 0 marks constrained DOFs with values bc_val (NULL: no BCs).
//   b[ndof] is accumulated into (caller zeroes it), as Builder::b is.
//   nthreads > 1 runs the element loop and the triplet sort with OpenMP; the
//   result is identical to the serial run (each row keeps the emission order).
// Returns an opaque CSR handle (read it with orc_csr_*), or NULL without lhs.
void * orc_build(int t, double const * xyz, uint32_t const * conn, int64_t nelem,
                 uint32_t const * elemMap, int64_t ndof, orc_lhs const * lhs,
                 orc_rhs const * rhs, uint8_t const * bc_mask, double const * bc_val,
                 double bc_diag, int nthreads, double * b)
{
  int const N = numDofs(t);
  int64_t const NN = (int64_t)N * N;
#ifdef _OPENMP
  if (nthreads < 1)
    nthreads = 1;
#else
  nthreads = 1;
#endif
  std::vector<OrcTriplet> trip;
  if (lhs)
    trip.resize((size_t)(nelem * NN));
  // buildLhs adds its own Fe into b (builder.hpp:137); buildRhs adds C*Fe.
  // b is accumulated serially in element order after the parallel loop.
  std::vector<double> feL, feR;
  if (b && lhs && lhs->apply_bc && bc_mask)
    feL.assign((size_t)(nelem * N), 0.);
  if (b && rhs && rhs->kind)
    feR.assign((size_t)(nelem * N), 0.);

#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int64_t e = 0; e < nelem; ++e)
  {
    double Ke[27 * 27], Fe[27], h[27];
    bool cons[27];
    uint32_t const * id = elemMap + e * N;
    bool const bcL = lhs && lhs->apply_bc && bc_mask;
    bool const bcR = rhs && rhs->kind && rhs->apply_bc && bc_mask;
    for (int i = 0; i < N; ++i)
    {
      cons[i] = bc_mask && bc_mask[id[i]];
      h[i] = cons[i] ? bc_val[id[i]] : 0.;
    }
    if (lhs)
    {
      orc_element(t, xyz, conn, e, lhs, nullptr, elemMap, Ke, nullptr);
      if (bcL)
      {
        // Fe = C (0 - Ke h); Ke = C Ke C; then Ke(i,i) = diag, Fe(i) = h (builder.hpp:83-124)
        double fl[27];
        for (int i = 0; i < N; ++i)
        {
          double kh = 0.;
          for (int j = 0; j < N; ++j)
            kh += Ke[i * N + j] * h[j];
          fl[i] = cons[i] ? 0. : (0. - kh);
        }
        for (int i = 0; i < N; ++i)
          for (int j = 0; j < N; ++j)
            if (cons[i] || cons[j])
              Ke[i * N + j] = 0.;
        for (int i = 0; i < N; ++i)
          if (cons[i])
          {
            Ke[i * N + i] = bc_diag;
            fl[i] = h[i];
          }
        if (!feL.empty())
          for (int i = 0; i < N; ++i)
            feL[e * N + i] = fl[i];
      }
      OrcTriplet * tp = trip.data() + e * NN;
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
          tp[i * N + j] = OrcTriplet{(int32_t)id[i], (int32_t)id[j], Ke[i * N + j]};
    }
    if (!feR.empty())
    {
      orc_element(t, xyz, conn, e, nullptr, rhs, elemMap, nullptr, Fe);
      for (int i = 0; i < N; ++i)
        feR[e * N + i] = (bcR && cons[i]) ? 0. : Fe[i];
    }
  }
  if (b)
  {
    if (!feL.empty())
      for (int64_t e = 0; e < nelem; ++e)
        for (int i = 0; i < N; ++i)
          b[elemMap[e * N + i]] += feL[e * N + i];
    if (!feR.empty())
      for (int64_t e = 0; e < nelem; ++e)
        for (int i = 0; i < N; ++i)
          b[elemMap[e * N + i]] += feR[e * N + i];
  }
  if (!lhs)
    return nullptr;

  // closeMatrix: setFromTriplets (stable bucket by row, duplicates summed in
  // emission order) then prune(1., 1e-16): keep |v| > 1e-16.
  int64_t const nt = (int64_t)trip.size();
  std::vector<int64_t> rowStart(ndof + 1, 0);
  int const T = nthreads;
  std::vector<std::vector<int64_t>> cnt(T, std::vector<int64_t>(ndof + 1, 0));
#pragma omp parallel num_threads(T)
  {
#ifdef _OPENMP
    int const tid = omp_get_thread_num();
#else
    int const tid = 0;
#endif
    int64_t const lo = nt * tid / T, hi = nt * (tid + 1) / T;
    for (int64_t k = lo; k < hi; ++k)
      cnt[tid][trip[k].r]++;
  }
  // prefix over (row, thread) keeps emission order inside each row
  int64_t acc = 0;
  for (int64_t r = 0; r < ndof; ++r)
  {
    rowStart[r] = acc;
    for (int th = 0; th < T; ++th)
    {
      int64_t const c = cnt[th][r];
      cnt[th][r] = acc;
      acc += c;
    }
  }
  rowStart[ndof] = acc;
  std::vector<int32_t> bcol(nt);
  std::vector<double> bval(nt);
#pragma omp parallel num_threads(T)
  {
#ifdef _OPENMP
    int const tid = omp_get_thread_num();
#else
    int const tid = 0;
#endif
    int64_t const lo = nt * tid / T, hi = nt * (tid + 1) / T;
    for (int64_t k = lo; k < hi; ++k)
    {
      int64_t const p = cnt[tid][trip[k].r]++;
      bcol[p] = trip[k].c;
      bval[p] = trip[k].v;
    }
  }
  std::vector<OrcTriplet>().swap(trip);
  // collapse duplicates per row in insertion order, sort columns, prune
  auto * out = new orc_csr;
  out->n = ndof;
  std::vector<int64_t> rowCount(ndof, 0);
  std::vector<std::vector<std::pair<int32_t, double>>> rows(T);
#pragma omp parallel num_threads(T)
  {
    std::vector<int64_t> slot(ndof, -1);
    std::vector<std::pair<int32_t, double>> tmp;
#pragma omp for schedule(static)
    for (int64_t r = 0; r < ndof; ++r)
    {
      tmp.clear();
      for (int64_t k = rowStart[r]; k < rowStart[r + 1]; ++k)
      {
        int32_t const c = bcol[k];
        if (slot[c] < 0)
        {
          slot[c] = (int64_t)tmp.size();
          tmp.emplace_back(c, bval[k]);
        }
        else
          tmp[slot[c]].second += bval[k];
      }
      for (auto & pr: tmp)
        slot[pr.first] = -1;
      std::sort(tmp.begin(), tmp.end(), [](auto const & x, auto const & y) { return x.first < y.first; });
      int64_t kept = 0;
      for (int64_t k = rowStart[r]; k < rowStart[r] + (int64_t)tmp.size(); ++k)
      {
        auto const & pr = tmp[k - rowStart[r]];
        if (std::fabs(pr.second) > 1e-16 * std::fabs(1.0))
        {
          bcol[rowStart[r] + kept] = pr.first;
          bval[rowStart[r] + kept] = pr.second;
          kept++;
        }
      }
      rowCount[r] = kept;
    }
  }
  out->rowPtr.assign(ndof + 1, 0);
  for (int64_t r = 0; r < ndof; ++r)
    out->rowPtr[r + 1] = (int32_t)(out->rowPtr[r] + rowCount[r]);
  out->nnz = out->rowPtr[ndof];
  out->col.resize(out->nnz);
  out->val.resize(out->nnz);
#pragma omp parallel for schedule(static) num_threads(T)
  for (int64_t r = 0; r < ndof; ++r)
  {
    std::memcpy(&out->col[out->rowPtr[r]], &bcol[rowStart[r]], rowCount[r] * sizeof(int32_t));
    std::memcpy(&out->val[out->rowPtr[r]], &bval[rowStart[r]], rowCount[r] * sizeof(double));
  }
  return out;
}

int64_t orc_csr_nnz(void * h) { return h ? static_cast<orc_csr *>(h)->nnz : -1; }

int orc_csr_copy(void * h, int32_t * rowPtr, int32_t * col, double * val)
{
  auto * c = static_cast<orc_csr *>(h);
  if (!c)
    return -1;
  std::memcpy(rowPtr, c->rowPtr.data(), (c->n + 1) * sizeof(int32_t));
  std::memcpy(col, c->col.data(), c->nnz * sizeof(int32_t));
  std::memcpy(val, c->val.data(), c->nnz * sizeof(double));
  return 0;
}

void orc_csr_free(void * h) { delete static_cast<orc_csr *>(h); }

// Adjoint gradient from the oracle element matrices:
//   g_e = - k_e * (C lambda)_e^T K0_e (C u)_e  = - (C u)_e^T K_e (C lambda)_e
// with K_e the element stiffness (per-element coefficient k_e) and C zeroing the
// constrained DOFs (dK/dk_e of the condensed matrix is C K0_e C).
int orc_adjoint_grad(int t, double const * xyz, uint32_t const * conn, int64_t nelem,
                     uint32_t const * elemMap, double const * k_e, uint8_t const * bc_mask,
                     double const * u, double const * lam, int nthreads, double * g)
{
  int const N = numDofs(t);
  orc_lhs L{2, 0., k_e, 0, 0., 0};
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (int64_t e = 0; e < nelem; ++e)
  {
    double Ke[27 * 27], ue[27], le[27];
    orc_element(t, xyz, conn, e, &L, nullptr, elemMap, Ke, nullptr);
    for (int i = 0; i < N; ++i)
    {
      uint32_t const d = elemMap[e * N + i];
      bool const c = bc_mask && bc_mask[d];
      ue[i] = c ? 0. : u[d];
      le[i] = c ? 0. : lam[d];
    }
    double s = 0.;
    for (int i = 0; i < N; ++i)
    {
      double r = 0.;
      for (int j = 0; j < N; ++j)
        r += Ke[i * N + j] * le[j];
      s += ue[i] * r;
    }
    g[e] = -s;
  }
  return 0;
}

} // extern "C"

// ====================================================== vector spaces and coupling
// A system of FE spaces on one mesh (FESpace<..., dim> with its offset in the global
// vector, include/fespace.hpp:15-60; BLOCK DOF ordering: component d of local DOF i is
// elemMap(e, i) + d * ndof, include/dof.hpp:312-327) and one Builder call over it:
//   - buildLhs (row space == column space, include/builder.hpp:31-154): Diagonal
//     assemblies, Dirichlet condensation with the diagonal set on constrained DOFs;
//   - buildCoupling (include/builder.hpp:156-277): rows of one space, columns of
//     another, Fe = -Crow Ke h, Ke = Crow Ke Cclm, no diagonal.
// Assemblies (coef c; JxW, dphi, phi of the row space's CurFE unless stated):
//   1 AssemblyStiffness       Ke(i+dN, j+dN)   += c JxW dphi_i . dphi_j          (assembly_lhs.hpp:52-65)
//   2 AssemblyTensorStiffness Ke(i+dN, j+dN)   += c JxW dphi_i . dphi_j,
//                             Ke(i+d1N, j+d2N) += c JxW dphi_i[d1] dphi_j[d2]    (assembly_lhs.hpp:116-161)
//   3 AssemblyMass            Ke(i+dN, j+dN)   += c JxW phi_i phi_j              (assembly_lhs.hpp:347-365)
//   4 AssemblyGrad            Ke(i+dN, j)      += c JxW dphi_i[d] psi_j          (assembly_coupling.hpp:42-86)
//   5 AssemblyDiv             Ke(i, j+dN)      += c JxW phi_i dpsi_j[d]          (assembly_coupling.hpp:89-132)
// (psi: the column space's functions at the same quadrature points.)  The triplets
// of the call are returned in emission order; orc_system_close sums and prunes them.
namespace
{
struct SysTrip
{
  std::vector<OrcTriplet> t;
};
} // namespace

extern "C"
{

// Space s: type ts[s], quadrature of type qs[s], dims[s] components, offsets[s],
// ndofs[s] scalar DOFs, elemMaps[s] (nelem x numDofs(ts[s])), optional BC mask and
// values over its ndofs[s] * dims[s] component DOFs.  ops: kinds[k], coefs[k].
void * orc_system_call(void * acc, int row, int col, int const * ts, int const * qs, int const * dims,
                       int64_t const * offsets, int64_t const * ndofs, uint32_t const * const * elemMaps,
                       uint8_t const * const * bcMask, double const * const * bcVal, double bcDiag,
                       double const * xyz, uint32_t const * conn, int64_t nelem, int nops, int const * kinds,
                       double const * coefs, double * b)
{
  auto * T = acc ? static_cast<SysTrip *>(acc) : new SysTrip;
  int const tr = ts[row], tc = ts[col], dr = dims[row], dc = dims[col];
  int const Nr = numDofs(tr), Nc = numDofs(tc), Lr = Nr * dr, Lc = Nc * dc;
  int const nv = numVerts(tr);
  bool const diagCall = row == col;
  CurFE fr(tr, qs[row]), fc(tc, qs[col]);
  std::vector<double> Ke((size_t)Lr * Lc), Fe(Lr), h(Lc);
  std::vector<char> consR(Lr), consC(Lc);
  for (int64_t e = 0; e < nelem; ++e)
  {
    double X[8][3];
    for (int v = 0; v < nv; ++v)
      for (int d = 0; d < 3; ++d)
        X[v][d] = xyz[3 * (int64_t)conn[e * nv + v] + d];
    fr.reinit(X);
    if (!diagCall)
      fc.reinit(X);
    std::fill(Ke.begin(), Ke.end(), 0.);
    for (int k = 0; k < nops; ++k)
    {
      double const c = coefs[k];
      for (int q = 0; q < fr.nq; ++q)
      {
        double const w = c * fr.JxW[q];
        double const * Dr = &fr.dphi[q * Nr * 3];
        double const * Pr = &fr.phiRef[q * Nr];
        double const * Dc = diagCall ? Dr : &fc.dphi[q * Nc * 3];
        double const * Pc = diagCall ? Pr : &fc.phiRef[q * Nc];
        switch (kinds[k])
        {
        case 1:
        case 2:
          for (int d = 0; d < dr; ++d)
            for (int i = 0; i < Nr; ++i)
              for (int j = 0; j < Nr; ++j)
                Ke[(size_t)(i + d * Nr) * Lc + j + d * Nr] +=
                    w * (Dr[3 * i] * Dr[3 * j] + Dr[3 * i + 1] * Dr[3 * j + 1] + Dr[3 * i + 2] * Dr[3 * j + 2]);
          if (kinds[k] == 2)
            for (int d1 = 0; d1 < dr; ++d1)
              for (int d2 = 0; d2 < dr; ++d2)
                for (int i = 0; i < Nr; ++i)
                  for (int j = 0; j < Nr; ++j)
                    Ke[(size_t)(i + d1 * Nr) * Lc + j + d2 * Nr] += w * Dr[3 * i + d1] * Dr[3 * j + d2];
          break;
        case 3:
          for (int d = 0; d < dr; ++d)
            for (int i = 0; i < Nr; ++i)
              for (int j = 0; j < Nr; ++j)
                Ke[(size_t)(i + d * Nr) * Lc + j + d * Nr] += w * Pr[i] * Pr[j];
          break;
        case 4:
          for (int d = 0; d < dr; ++d)
            for (int i = 0; i < Nr; ++i)
              for (int j = 0; j < Nc; ++j)
                Ke[(size_t)(i + d * Nr) * Lc + j] += w * Dr[3 * i + d] * Pc[j];
          break;
        case 5:
          for (int d = 0; d < dc; ++d)
            for (int i = 0; i < Nr; ++i)
              for (int j = 0; j < Nc; ++j)
                Ke[(size_t)i * Lc + j + d * Nc] += w * Pr[i] * Dc[3 * j + d];
          break;
        default:
          return nullptr;
        }
      }
    }
    // constraints: component DOF of local (i, d) is elemMap(e, i) + d * ndof
    uint32_t const * er = elemMaps[row] + e * Nr;
    uint32_t const * ec = elemMaps[col] + e * Nc;
    for (int d = 0; d < dr; ++d)
      for (int i = 0; i < Nr; ++i)
      {
        int64_t const id = er[i] + (int64_t)d * ndofs[row];
        consR[i + d * Nr] = bcMask[row] && bcMask[row][id];
      }
    for (int d = 0; d < dc; ++d)
      for (int j = 0; j < Nc; ++j)
      {
        int64_t const id = ec[j] + (int64_t)d * ndofs[col];
        consC[j + d * Nc] = bcMask[col] && bcMask[col][id];
        h[j + d * Nc] = consC[j + d * Nc] ? bcVal[col][id] : 0.;
      }
    // Fe = -C Ke h ; Ke = C Ke C (rows / columns)
    for (int I = 0; I < Lr; ++I)
    {
      double kh = 0.;
      for (int J = 0; J < Lc; ++J)
        kh += Ke[(size_t)I * Lc + J] * h[J];
      Fe[I] = consR[I] ? 0. : (0. - kh);
    }
    for (int I = 0; I < Lr; ++I)
      for (int J = 0; J < Lc; ++J)
        if (consR[I] || consC[J])
          Ke[(size_t)I * Lc + J] = 0.;
    if (diagCall)
      for (int I = 0; I < Lr; ++I)
        if (consR[I])
        {
          Ke[(size_t)I * Lc + I] = bcDiag;
          Fe[I] = h[I];
        }
    // emission (builder.hpp:139-152 / 254-274): i, d1, then j, d2
    for (int i = 0; i < Nr; ++i)
      for (int d1 = 0; d1 < dr; ++d1)
      {
        int32_t const idI = (int32_t)(offsets[row] + er[i] + (int64_t)d1 * ndofs[row]);
        if (b)
          b[idI] += Fe[i + d1 * Nr];
        for (int j = 0; j < Nc; ++j)
          for (int d2 = 0; d2 < dc; ++d2)
          {
            int32_t const idJ = (int32_t)(offsets[col] + ec[j] + (int64_t)d2 * ndofs[col]);
            T->t.push_back({idI, idJ, Ke[(size_t)(i + d1 * Nr) * Lc + j + d2 * Nc]});
          }
      }
  }
  return T;
}

// closeMatrix over the accumulated calls: duplicates summed in emission order, columns
// sorted, |v| <= 1e-16 pruned.  Frees the accumulator; returns a CSR handle.
void * orc_system_close(void * acc, int64_t ntot)
{
  auto * T = static_cast<SysTrip *>(acc);
  auto * out = new orc_csr;
  out->n = ntot;
  std::vector<std::vector<std::pair<int32_t, double>>> rows(ntot);
  std::vector<int64_t> slot(ntot, -1);
  if (T)
    for (auto const & tr: T->t)
    {
      auto & R = rows[tr.r];
      (void)slot;
      bool found = false;
      for (auto & pr: R)
        if (pr.first == tr.c)
        {
          pr.second += tr.v;
          found = true;
          break;
        }
      if (!found)
        R.emplace_back(tr.c, tr.v);
    }
  delete T;
  out->rowPtr.assign(ntot + 1, 0);
  for (int64_t r = 0; r < ntot; ++r)
  {
    auto & R = rows[r];
    std::sort(R.begin(), R.end(), [](auto const & x, auto const & y) { return x.first < y.first; });
    for (auto const & pr: R)
      if (std::fabs(pr.second) > 1e-16)
      {
        out->col.push_back(pr.first);
        out->val.push_back(pr.second);
      }
    out->rowPtr[r + 1] = (int32_t)out->col.size();
  }
  out->nnz = out->rowPtr[ntot];
  return out;
}

} // extern "C"
