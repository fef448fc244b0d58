// Q2 hexahedron element kernel in FP64 arithmetic with sum factorisation: one warp per
// element.  It computes what proxpde's element loop computes for a Q2 hexahedron with
// the 3x3x3 Gauss rule (include/builder.hpp:53-153): CurFE::reinit (include/curfe.hpp:
// 50-103), AssemblyStiffness(FE) / AssemblyScalarMass / AssemblyMassFE
// (include/assembly_lhs.hpp:52-109, 207-221, 262-277), AssemblyRhsAnalytic and
// AssemblyS2SProjection (include/assembly_rhs.hpp:61-88, 130-159) and the Dirichlet
// condensation (builder.hpp:76-124), in IEEE binary64, with FP64 reductions into the
// CSR values and the load vector.
//
// The Q2 basis is a tensor product of the 1D functions l_0 = x(x-1)/2, l_1 = x(x+1)/2,
// l_2 = 1 - x^2 (src/reffe.cpp:374-383), and the rule a tensor product of the 3-point
// Gauss rule, so every sum over the 27 points factors into three 3-term sums:
//  - per point (lane q): J of the trilinear map from the Walsh-Hadamard transform of
//    the vertices (the 27 mapping points lie on the trilinear image, so this is the
//    reference's J), J^T J, its adjugate and determinant D, 1/|det J| = rsqrt(D) (one
//    third-order Newton step), w_q |det J_q|, G_q = k w_q |det J| (J^T J)^-1;
//  - stiffness tables, each three one-axis contractions of one G component with the
//    1D products D_ab = l'_a l'_b, P_ab = l_a l_b (6 symmetric classes): S_x = sum
//    G_xx D P P, S_y, S_z (216 values each).  The mixed terms of K_ij,
//    sum G_xy (E_ix,jx E_jy,iy + E_jx,ix E_iy,jy) P with E_ab = l'_a l_b, split E into
//    its symmetric part S_ab = (l_a l_b)'/2 (6 classes) and antisymmetric part
//    A_ab = (l'_a l_b - l'_b l_a)/2 (3 classes, a < b, and its sign): the sum is
//    2 sum G S S P - 2 s_x s_y sum G A A P, so each of G_xy, G_xz, G_yz gives a table SS
//    (216 values) and a table AA (54), sharing their first stage (the 6-class P axis),
//    instead of the 486 values of sum G E E P;
//    the stiffness stages use each class's three coefficients divided by the first, so
//    that an output costs two FP64 operations, and an entry K_ij, a sum of nine table
//    values (three S, an SS and an AA per mixed component), multiplies each by its
//    deferred scale (the product of the three classes' first coefficients, with the
//    factor 2 and the sign) in the FMA that adds it;
//  - mass table sum |det J| w P P P (216), M_ij one value of it;
//  - the load r_q = w_q |det J_q| f(qpoint_q), contracted to the nodes with l_a.
// About 16k FP64 operations per element against about 100k for the per-point form.
// A contraction stage maps [3][m] (point axis first) to [m][C] (C classes last), so
// three stages turn [qx][qy][qz] into [cx][cy][cz]; the lanes take the stage's outputs
// in turn.
#include <vector>

#include "pxg_internal.h"
#include "pxg_sinpi.h"

namespace pxg
{
namespace q2f
{
constexpr int NQ = 27, N = 27, NP = N * (N + 1) / 2;

// 1D tables at the three Gauss points t_0 < t_1 = 0 < t_2 (from initQ2F64Tables):
// [0, 9) l_a(t_k) at 3a + k; [9, 27) P classes; [27, 45) D classes; [45, 63) S classes;
// [63, 72) A classes.  Symmetric classes: (0,0) (1,1) (2,2) (0,1) (0,2) (1,2);
// antisymmetric: (0,1) (0,2) (1,2).
__device__ double gCoef[72];
__device__ double gCoefN[72];      // P, D, S, A classes divided by their first coefficient
// the deferred scales: S_x S_y S_z (216 each), then per mixed component its SS table
// (216) and its AA table (128: index a for a positive orientation, 64 + a for a
// negative one, 54 for the pairs without an AA term, whose scale is 0)
constexpr int kAA = 128;
constexpr int kTab = 3 * 216 + 3 * (216 + kAA);
__device__ double gScale[kTab];
__device__ double gT[3];           // t_k
__device__ double gWl[NQ];         // weights in lattice order qx * 9 + qy * 3 + qz
__device__ uint8_t gRuleOfLat[NQ]; // the rule's point index of each lattice point
__device__ uint8_t gLatOfNode[N];  // node n -> ax * 9 + ay * 3 + az (1D function indices)
__device__ uint8_t gNodeOfLat[N];
__device__ uint16_t gPairsF[NP];   // (i << 8 | j), i <= j
// per pair, its index into each table (the layouts of the contractions below): the S
// tables' (shared by the mass and S_x, S_y, S_z), then SS_xy, AA_xy, SS_xz, AA_xz,
// SS_yz, AA_yz (an AA index with the orientation, as gScale lays them out); 8 per pair
// (one padding)
__device__ uint16_t gPairIdx[NP * 8];
constexpr int kPairsPerLane = (NP + 31) / 32; // 12


__host__ __device__ constexpr int symCls(int a, int b)
{
  return a == b ? a : (a + b == 1 ? 3 : (a + b == 2 ? 4 : 5));
}

// 1/sqrt(x) by the hardware estimate and one third-order Newton step
__device__ __forceinline__ double rsqrtN(double x)
{
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double const e = fma(-(x * y), y, 1.0);
  return fma(y * e, fma(0.375, e, 0.5), y);
}

// out[r * C + c] = sum_k coef[3c + k] in[k * m + r] (r < m, c < C), lanes in turn
__device__ __forceinline__ void stage(double const * in, int m, int C, double const * coef, double * out, int lane)
{
  for (int o = lane; o < m * C; o += 32)
  {
    int const r = o / C, c = o - r * C;
    double const * k = coef + 3 * c;
    out[o] = fma(k[2], in[2 * m + r], fma(k[1], in[m + r], k[0] * in[r]));
  }
  __syncwarp();
}
// the same with normalised coefficients (coef[3c] = 1): two operations per output
__device__ __forceinline__ void stageN(double const * in, int m, int C, double const * coef, double * out, int lane)
{
  for (int o = lane; o < m * C; o += 32)
  {
    int const r = o / C, c = o - r * C;
    double const * k = coef + 3 * c;
    out[o] = fma(k[2], in[2 * m + r], fma(k[1], in[m + r], in[r]));
  }
  __syncwarp();
}
__device__ __forceinline__ void contract3N(double const * in, int c0, double const * k0, int c1, double const * k1,
                                           int c2, double const * k2, double * out, double * scr0, double * scr1,
                                           int lane)
{
  stageN(in, 9, c0, k0, scr0, lane);
  stageN(scr0, 3 * c0, c1, k1, scr1, lane);
  stageN(scr1, c0 * c1, c2, k2, out, lane);
}
// three stages of a [3][3][3] array with the coefficient tables of the three axes
__device__ __forceinline__ void contract3(double const * in, int c0, double const * k0, int c1, double const * k1,
                                          int c2, double const * k2, double * out, double * scr0, double * scr1,
                                          int lane)
{
  stage(in, 9, c0, k0, scr0, lane);       // [3][3][c0]
  stage(scr0, 3 * c0, c1, k1, scr1, lane); // [3][c0][c1]
  stage(scr1, c0 * c1, c2, k2, out, lane); // [c0][c1][c2]
}

__device__ __noinline__ void condenseF(double * pij, double bcDiag, double * b, uint32_t dofi, uint32_t dofj,
                                       double bvi, double bvj, bool ci, bool cj, bool isDiag, double val)
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

// f at the point, out of line (its FP64 code is only run for the load)
__device__ __noinline__ double evalPoint(int fn, double rc, double x, double y, double z)
{
  return evalFn(fn, rc, x, y, z);
}

struct Smem
{
  double coef[72];
  double coefN[72];
  double w[NQ];
  double X[8][3];
  double H[8][3]; // Walsh-Hadamard transform of the vertices, [kx + 2 ky + 4 kz][r]
  double G[6][NQ];
  double ad[NQ];
  double tab[272]; // one table at a time: the mass, S_x, S_y, S_z, then SS [0, 216) and
                   // AA [216, 270) of each mixed component, tab[270] = 0
  double scr[2][243];
  double bv[N];
  uint32_t dof[N];
  int32_t rp[N];
  uint8_t latOfNode[N];
  uint8_t nodeOfLat[N];
  uint8_t ruleOfLat[NQ];
};
} // namespace q2f

__global__ void __launch_bounds__(32) kAssembleQ2F64(AsmArgs a)
{
  using namespace q2f;
  __shared__ Smem S;
  int const lane = threadIdx.x;
  for (int k = lane; k < 72; k += 32)
    S.coef[k] = gCoef[k], S.coefN[k] = gCoefN[k];
  if (lane < NQ)
  {
    S.w[lane] = gWl[lane];
    S.latOfNode[lane] = gLatOfNode[lane];
    S.nodeOfLat[lane] = gNodeOfLat[lane];
    S.ruleOfLat[lane] = gRuleOfLat[lane];
  }
  int64_t const e = elemOf(a, blockIdx.x);
  // ---- inputs
  if (lane < 24)
  {
    uint32_t const id = a.conn[e * 8 + lane / 3];
    S.X[lane / 3][lane % 3] = a.xyz[3 * (int64_t)id + lane % 3];
  }
  bool mine = false;
  if (lane < N)
  {
    uint32_t const d = a.emap[e * N + lane];
    S.dof[lane] = d;
    S.rp[lane] = a.rowPtr[d];
    mine = a.bcMask && a.bcMask[d];
    S.bv[lane] = mine ? a.bcVal[d] : 0.;
  }
  uint32_t const cons = __ballot_sync(0xffffffffu, mine);
  __syncwarp();
  LhsDev const & op0 = a.op[0];
  LhsDev const & op1 = a.op[1];
  bool const k0 = op0.on && op0.stiff, k1 = op1.on && op1.stiff;
  bool const m0 = op0.on && op0.mass, m1 = op1.on && op1.mass;
  bool const needK = k0 || k1, needM = m0 || m1;
  double const kfac = ((usesCoef(op0) || usesCoef(op1)) && a.kE) ? a.kE[e] : 1.0;
  bool const foldK = k0 != k1, foldM = m0 != m1;
  double const ks0 = k0 ? (op0.stiff == 2 ? op0.sc * kfac : op0.sc) : 0.;
  double const ks1 = k1 ? (op1.stiff == 2 ? op1.sc * kfac : op1.sc) : 0.;
  double const ms0 = m0 ? massCoef(op0, kfac) : 0., ms1 = m1 ? massCoef(op1, kfac) : 0.;

  // ---- the Walsh-Hadamard transform of the vertices, x(xi) = 1/8 sum_k H_k xi^kx
  // eta^ky zeta^kz: lane 3 lat + r holds coordinate r of the vertex at lattice point
  // lat = vx + 2 vy + 4 vz (proxpde's Q1 vertex order, src/reffe.cpp:684-759), and
  // each stage pairs the lanes whose lattice points differ along one axis
  {
    int const lat = lane / 3, r = lane % 3;
    int const vx = lat & 1, vy = (lat >> 1) & 1, vz = lat >> 2;
    int const v = vz * 4 + (vy ? (vx ? 2 : 3) : (vx ? 1 : 0));
    double h = lane < 24 ? S.X[v][r] : 0.;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax)
    {
      int const bit = (lat >> ax) & 1, step = 3 << ax;
      double const o = __shfl_sync(0xffffffffu, h, lane < 24 ? (bit ? lane - step : lane + step) : lane);
      h = bit ? h - o : h + o;
    }
    if (lane < 24)
      S.H[lat][r] = h;
  }
  __syncwarp();
  // ---- per point: lane q = qx * 9 + qy * 3 + qz; the Jacobian columns (x8)
  // c1 = H100 + eta H110 + zeta H101 + eta zeta H111, ...
  if (lane < NQ)
  {
    int const qx = lane / 9, qy = (lane / 3) % 3, qz = lane % 3;
    double const xi = gT[qx], eta = gT[qy], zeta = gT[qz];
    double c[3][3]; // c[col][r]
    double o[3];    // the element origin, the vertex average (geo.hpp:721-728)
#pragma unroll
    for (int r = 0; r < 3; ++r)
    {
      // H[kx + 2 ky + 4 kz]
      double const H000 = S.H[0][r], H100 = S.H[1][r], H010 = S.H[2][r], H110 = S.H[3][r];
      double const H001 = S.H[4][r], H101 = S.H[5][r], H011 = S.H[6][r], H111 = S.H[7][r];
      c[0][r] = fma(zeta, fma(eta, H111, H101), fma(eta, H110, H100));
      c[1][r] = fma(zeta, fma(xi, H111, H011), fma(xi, H110, H010));
      c[2][r] = fma(eta, fma(xi, H111, H011), fma(xi, H101, H001));
      o[r] = 0.125 * H000;
    }
    double const g11 = fma(c[0][0], c[0][0], fma(c[0][1], c[0][1], c[0][2] * c[0][2]));
    double const g22 = fma(c[1][0], c[1][0], fma(c[1][1], c[1][1], c[1][2] * c[1][2]));
    double const g33 = fma(c[2][0], c[2][0], fma(c[2][1], c[2][1], c[2][2] * c[2][2]));
    double const g12 = fma(c[0][0], c[1][0], fma(c[0][1], c[1][1], c[0][2] * c[1][2]));
    double const g13 = fma(c[0][0], c[2][0], fma(c[0][1], c[2][1], c[0][2] * c[2][2]));
    double const g23 = fma(c[1][0], c[2][0], fma(c[1][1], c[2][1], c[1][2] * c[2][2]));
    double const A11 = fma(-g23, g23, g22 * g33);
    double const A22 = fma(-g13, g13, g11 * g33);
    double const A33 = fma(-g12, g12, g11 * g22);
    double const A12 = fma(g13, g23, -(g12 * g33));
    double const A13 = fma(g12, g23, -(g13 * g22));
    double const A23 = fma(g12, g13, -(g11 * g23));
    double const D = fma(g11, A11, fma(g12, A12, g13 * A13));
    double const rs = rsqrtN(D);
    double const wq = S.w[lane];
    S.ad[lane] = (D * rs) * wq; // w |det J| x 512
    // k w |det J| (J^T J)^-1 = k w adj rsqrt(D) / 8 (the columns carry x8)
    double const sG = ((foldK ? (k0 ? ks0 : ks1) : 1.0) * 0.125) * (wq * rs);
    S.G[0][lane] = sG * A11, S.G[1][lane] = sG * A22, S.G[2][lane] = sG * A33;
    // G_xy as [qz][qx][qy] and G_xz as [qy][qx][qz]: their tables contract the P axis first
    S.G[3][qz * 9 + qx * 3 + qy] = sG * A12, S.G[4][qy * 9 + qx * 3 + qz] = sG * A13, S.G[5][lane] = sG * A23;
    // the qpoint origin + J xi (curfe.hpp:80), for the analytic load
    if (a.rkind == 1)
    {
      double const x = fma(0.125, fma(xi, c[0][0], fma(eta, c[1][0], zeta * c[2][0])), o[0]);
      double const y = fma(0.125, fma(xi, c[0][1], fma(eta, c[1][1], zeta * c[2][1])), o[1]);
      double const z = fma(0.125, fma(xi, c[0][2], fma(eta, c[1][2], zeta * c[2][2])), o[2]);
      S.scr[0][lane] = x, S.scr[0][32 + lane] = y, S.scr[0][64 + lane] = z;
    }
  }
  __syncwarp();
  double const * const cL = S.coef;
  double const * const cP = S.coef + 9;

  // ---- load vector (buildLhs' BC values, buildRhs); the writes start here
  pdlWait();
  bool const bcOps = (op0.on && op0.bc) || (op1.on && op1.bc);
  if (a.b && cons && bcOps && lane < N && ((cons >> lane) & 1u))
  {
#pragma unroll
    for (int m = 0; m < 2; ++m)
      if (a.op[m].on && a.op[m].bc && S.bv[lane] != 0.)
        atomicAdd(a.b + S.dof[lane], S.bv[lane]);
  }
  if (a.rkind)
  {
    // r_q = w_q |det J_q| f_q (x512: the 1/512 is in rc), then Fe = sum_q r_q l l l
    double const rc = a.rc * (1. / 512.);
    double * const rq = S.scr[1];
    if (lane < NQ)
    {
      double f;
      if (a.rkind == 1 && a.fn == PXG_FN_SIN3)
        f = rc * (sinPiTab(S.scr[0][lane]) * sinPiTab(S.scr[0][32 + lane]) * sinPiTab(S.scr[0][64 + lane]));
      else if (a.rkind == 1)
        f = evalPoint(a.fn, rc, S.scr[0][lane], S.scr[0][32 + lane], S.scr[0][64 + lane]);
      else if (a.rkind == 3)
        f = rc * a.field[e * NQ + S.ruleOfLat[lane]];
      else
      {
        // projection: the field at the point, sum_n phi_n(q) field_n with phi_n = l l l
        int const qx = lane / 9, qy = (lane / 3) % 3, qz = lane % 3;
        double s = 0.;
        for (int n = 0; n < N; ++n)
        {
          int const L = S.latOfNode[n];
          s = fma(cL[3 * (L / 9) + qx] * cL[3 * ((L / 3) % 3) + qy] * cL[3 * (L % 3) + qz], a.field[S.dof[n]], s);
        }
        f = rc * s;
      }
      rq[lane] = S.ad[lane] * f;
    }
    __syncwarp();
    double * const bn = S.scr[0] + 96; // [ax][ay][az]
    stage(rq, 9, 3, cL, S.scr[0], lane);
    stage(S.scr[0], 9, 3, cL, S.scr[0] + 128, lane);
    stage(S.scr[0] + 128, 9, 3, cL, bn, lane);
    if (lane < N)
    {
      int const n = S.nodeOfLat[lane];
      if (!(a.rbc && ((cons >> n) & 1u)))
        atomicAdd(a.b + S.dof[n], bn[lane]);
    }
    __syncwarp();
  }

  // ---- the tables one at a time into S.tab, each lane adding them into the entries
  // of its pairs p = lane + 32 k (kv, mv in registers): the mass table w |det J| (times
  // a single mass operator's coefficient, and the 1/512) contracted with P over the
  // three axes, then the six stiffness tables (normalised stages; each value times its
  // deferred scale, gScale in the tables' concatenated layout)
  double kv[kPairsPerLane], mv[kPairsPerLane];
#pragma unroll
  for (int k = 0; k < kPairsPerLane; ++k)
    kv[k] = 0., mv[k] = 0.;
  auto addTable = [&](int slot0, int slot1, int scaleBase, bool toMass) {
#pragma unroll
    for (int k = 0; k < kPairsPerLane; ++k)
    {
      int const p = lane + 32 * k;
      if (p >= NP)
        break;
      int const t0 = gPairIdx[8 * p + slot0];
      if (toMass)
        mv[k] = S.tab[t0];
      else
      {
        kv[k] = fma(S.tab[t0], __ldg(gScale + scaleBase + t0), kv[k]);
        if (slot1 >= 0)
        {
          // the AA value of the pair's orientation (index mod 64) and its signed scale
          int const t1 = gPairIdx[8 * p + slot1];
          kv[k] = fma(S.tab[216 + (t1 & 63)], __ldg(gScale + scaleBase + 216 + t1), kv[k]);
        }
      }
    }
    __syncwarp(); // before the next table overwrites S.tab
  };
  if (needM)
  {
    double const mcf = (foldM ? (m0 ? ms0 : ms1) : 1.0) * (1. / 512.);
    if (lane < NQ)
      S.scr[1][lane] = mcf * S.ad[lane];
    __syncwarp();
    contract3(S.scr[1], 6, cP, 6, cP, 6, cP, S.tab, S.scr[0], S.scr[1], lane);
    addTable(0, -1, 0, true);
  }
  if (needK)
  {
    double const * const nP = S.coefN + 9;
    double const * const nD = S.coefN + 27;
    double const * const nS = S.coefN + 45;
    double const * const nA = S.coefN + 63;
    contract3N(S.G[0], 6, nD, 6, nP, 6, nP, S.tab, S.scr[0], S.scr[1], lane); // [px][py][pz]
    addTable(0, -1, 0, false);
    contract3N(S.G[1], 6, nP, 6, nD, 6, nP, S.tab, S.scr[0], S.scr[1], lane);
    addTable(0, -1, 216, false);
    contract3N(S.G[2], 6, nP, 6, nP, 6, nD, S.tab, S.scr[0], S.scr[1], lane);
    addTable(0, -1, 432, false);
    // a mixed component: SS into tab[0, 216), then AA from the same first stage (scr[0])
    // into tab[216, 270), and the zero that pairs without an AA term read
    auto mixed = [&](double const * g) {
      contract3N(g, 6, nP, 6, nS, 6, nS, S.tab, S.scr[0], S.scr[1], lane);
      stageN(S.scr[0], 18, 3, nA, S.scr[1], lane);
      stageN(S.scr[1], 18, 3, nA, S.tab + 216, lane);
      if (lane == 0)
        S.tab[270] = 0.;
      __syncwarp();
    };
    mixed(S.G[3]); // [pz][sx][sy], [pz][ax][ay]
    addTable(1, 2, 648, false);
    mixed(S.G[4]); // [py][sx][sz], [py][ax][az]
    addTable(3, 4, 648 + (216 + kAA), false);
    mixed(S.G[5]); // [px][sy][sz], [px][ay][az]
    addTable(5, 6, 648 + 2 * (216 + kAA), false);
  }

  // ---- the scatter of the entries i <= j
  uint16_t const * rk = a.rank + e * (int64_t)(N * N);
  bool const anyBc = cons && bcOps;
#pragma unroll
  for (int k = 0; k < kPairsPerLane; ++k)
  {
    int const p = lane + 32 * k;
    if (p >= NP)
      break;
    uint16_t const pr = gPairsF[p];
    int const i = pr >> 8, j = pr & 0xff;
    int32_t const pij = S.rp[i] + rk[i * N + j], pji = S.rp[j] + rk[j * N + i];
    bool const ci = (cons >> i) & 1u, cj = (cons >> j) & 1u;
#pragma unroll
    for (int m = 0; m < 2; ++m)
    {
      LhsDev const & op = a.op[m];
      if (!op.on)
        continue;
      double val;
      if (op.stiff)
      {
        val = foldK ? kv[k] : (m ? ks1 : ks0) * kv[k];
        if (op.mass)
          val = foldM ? val + mv[k] : fma(m ? ms1 : ms0, mv[k], val);
      }
      else
        val = foldM ? mv[k] : (m ? ms1 : ms0) * mv[k];
      if (anyBc && op.bc && (ci || cj))
      {
        condenseF(op.vals + pij, a.bcDiag, a.b, S.dof[i], S.dof[j], S.bv[i], S.bv[j], ci, cj, i == j, val);
        continue;
      }
      atomicAdd(op.vals + pij, val);
      if (i != j)
        atomicAdd(op.vals + pji, val);
    }
  }
}

// The 1D tables, the lattice maps and the pair list, from the reference's rule and
// basis (the engine's host restatement of src/qr.cpp and src/reffe.cpp).
pxg_status initQ2F64Tables(pxg_ctx * c)
{
  using namespace q2f;
  std::vector<double> xi, w;
  hostRule(Q2HEX, xi, w);
  if ((int)w.size() != NQ)
    return fail(c, PXG_ERR_UNSUPPORTED, "Q2 rule: %d points", (int)w.size());
  // the three 1D points, ascending
  double t[3] = {1e300, 0., -1e300};
  for (int q = 0; q < NQ; ++q)
  {
    t[0] = xi[3 * q] < t[0] ? xi[3 * q] : t[0];
    t[2] = xi[3 * q] > t[2] ? xi[3 * q] : t[2];
  }
  auto idx = [&](double v) { return v == t[0] ? 0 : (v == t[2] ? 2 : 1); };
  t[1] = 0.;
  double wl[NQ];
  uint8_t ruleOfLat[NQ];
  for (int q = 0; q < NQ; ++q)
  {
    int const L = idx(xi[3 * q]) * 9 + idx(xi[3 * q + 1]) * 3 + idx(xi[3 * q + 2]);
    wl[L] = w[q];
    ruleOfLat[L] = (uint8_t)q;
  }
  // 1D functions of src/reffe.cpp:374-383 (index 0: node -1, 1: node +1, 2: node 0)
  auto f = [](int a, double x) { return a == 0 ? 0.5 * x * (x - 1.) : (a == 1 ? 0.5 * x * (x + 1.) : 1. - x * x); };
  auto df = [](int a, double x) { return a == 0 ? x - 0.5 : (a == 1 ? x + 0.5 : -2. * x); };
  int const cls[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  std::vector<double> coef(72);
  for (int a = 0; a < 3; ++a)
    for (int k = 0; k < 3; ++k)
      coef[3 * a + k] = f(a, t[k]);
  for (int cc = 0; cc < 6; ++cc)
    for (int k = 0; k < 3; ++k)
    {
      coef[9 + 3 * cc + k] = f(cls[cc][0], t[k]) * f(cls[cc][1], t[k]);
      coef[27 + 3 * cc + k] = df(cls[cc][0], t[k]) * df(cls[cc][1], t[k]);
    }
  int const anti[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  for (int cc = 0; cc < 6; ++cc)
    for (int k = 0; k < 3; ++k)
    {
      int const a = cls[cc][0], b = cls[cc][1];
      coef[45 + 3 * cc + k] = 0.5 * (df(a, t[k]) * f(b, t[k]) + df(b, t[k]) * f(a, t[k]));
    }
  for (int cc = 0; cc < 3; ++cc)
    for (int k = 0; k < 3; ++k)
    {
      int const a = anti[cc][0], b = anti[cc][1];
      coef[63 + 3 * cc + k] = 0.5 * (df(a, t[k]) * f(b, t[k]) - df(b, t[k]) * f(a, t[k]));
    }
  // node n -> the 1D functions of its three factors: the lattice point where phi_n = 1
  uint8_t latOfNode[N], nodeOfLat[N];
  double const node1d[3] = {-1., 1., 0.};
  for (int L = 0; L < N; ++L)
  {
    double const p[3] = {node1d[L / 9], node1d[(L / 3) % 3], node1d[L % 3]};
    double phi[N], dphi[3 * N];
    hostShape(Q2HEX, p, phi, dphi);
    int found = -1;
    for (int n = 0; n < N; ++n)
      if (phi[n] > 0.5)
        found = n;
    if (found < 0)
      return fail(c, PXG_ERR_UNSUPPORTED, "Q2 node lattice");
    latOfNode[found] = (uint8_t)L;
    nodeOfLat[L] = (uint8_t)found;
  }
  std::vector<uint16_t> pairs;
  for (int i = 0; i < N; ++i)
    for (int j = i; j < N; ++j)
      pairs.push_back((uint16_t)(i << 8 | j));
  // the P, D, S, A classes divided by their first coefficient (the value at t_0, nonzero
  // for every class), and the deferred scale of each stiffness table value: the
  // product of its three classes' first coefficients, in the tables' layouts
  std::vector<double> coefN(coef);
  auto first = [&](int base, int cc) { return coef[base + 3 * cc]; };
  for (int k = 9; k < 72; k += 3)
    if (coef[k] == 0.)
      return fail(c, PXG_ERR_UNSUPPORTED, "Q2 tables: a class vanishes at the first Gauss point");
  for (int base : {9, 27, 45})
    for (int cc = 0; cc < 6; ++cc)
      for (int k = 0; k < 3; ++k)
        coefN[base + 3 * cc + k] = coef[base + 3 * cc + k] / first(base, cc);
  for (int cc = 0; cc < 3; ++cc)
    for (int k = 0; k < 3; ++k)
      coefN[63 + 3 * cc + k] = coef[63 + 3 * cc + k] / first(63, cc);
  std::vector<double> scale(kTab, 0.);
  auto sP = [&](int cc) { return first(9, cc); };
  auto sD = [&](int cc) { return first(27, cc); };
  auto sS = [&](int cc) { return first(45, cc); };
  auto sA = [&](int cc) { return first(63, cc); };
  for (int x = 0; x < 6; ++x)
    for (int y = 0; y < 6; ++y)
      for (int z = 0; z < 6; ++z)
      {
        int const k = x * 36 + y * 6 + z;
        scale[k] = sD(x) * sP(y) * sP(z);
        scale[216 + k] = sP(x) * sD(y) * sP(z);
        scale[432 + k] = sP(x) * sP(y) * sD(z);
      }
  // mixed component m: 2 x SS, and -2 x orientation x AA (index 64 + a: the negative
  // orientation; 54: no AA term, scale 0)
  for (int m = 0; m < 3; ++m)
  {
    int const base = 648 + m * (216 + kAA);
    for (int p = 0; p < 6; ++p)
    {
      for (int s1 = 0; s1 < 6; ++s1)
        for (int s2 = 0; s2 < 6; ++s2)
          scale[base + p * 36 + s1 * 6 + s2] = 2. * sP(p) * sS(s1) * sS(s2);
      for (int a1 = 0; a1 < 3; ++a1)
        for (int a2 = 0; a2 < 3; ++a2)
        {
          double const v = 2. * sP(p) * sA(a1) * sA(a2);
          scale[base + 216 + p * 9 + a1 * 3 + a2] = -v;
          scale[base + 216 + 64 + p * 9 + a1 * 3 + a2] = v;
        }
    }
  }
  PXG_CUDA(c, cudaMemcpyToSymbol(gCoef, coef.data(), 72 * 8));
  PXG_CUDA(c, cudaMemcpyToSymbol(gCoefN, coefN.data(), 72 * 8));
  PXG_CUDA(c, cudaMemcpyToSymbol(gScale, scale.data(), scale.size() * 8));
  PXG_CUDA(c, cudaMemcpyToSymbol(gT, t, 24));
  PXG_CUDA(c, cudaMemcpyToSymbol(gWl, wl, NQ * 8));
  PXG_CUDA(c, cudaMemcpyToSymbol(gRuleOfLat, ruleOfLat, NQ));
  PXG_CUDA(c, cudaMemcpyToSymbol(gLatOfNode, latOfNode, N));
  PXG_CUDA(c, cudaMemcpyToSymbol(gNodeOfLat, nodeOfLat, N));
  PXG_CUDA(c, cudaMemcpyToSymbol(gPairsF, pairs.data(), pairs.size() * 2));
  // each pair's index into the tables: S (and mass) [px][py][pz]; for the mixed
  // components xy, xz, yz the SS tables [pz][sx][sy], [py][sx][sz], [px][sy][sz] (the
  // symmetric classes of the two derivative axes) and the AA tables [pz][ax][ay], ... with
  // the antisymmetric class a + b - 1 of {a, b}, plus 64 when the orientation
  // sign(j_1 - i_1) sign(j_2 - i_2) is negative, and 54 when either axis pair is
  // diagonal (no AA term)
  std::vector<uint16_t> pidx(pairs.size() * 8, 0);
  auto aaIdx = [](int lead, int i1, int j1, int i2, int j2) -> uint16_t {
    if (i1 == j1 || i2 == j2)
      return 54;
    int const v = lead * 9 + (i1 + j1 - 1) * 3 + (i2 + j2 - 1);
    return (uint16_t)(((i1 < j1) == (i2 < j2)) ? v : 64 + v);
  };
  for (size_t q = 0; q < pairs.size(); ++q)
  {
    int const i = pairs[q] >> 8, j = pairs[q] & 0xff;
    int const Li = latOfNode[i], Lj = latOfNode[j];
    int const ix = Li / 9, iy = (Li / 3) % 3, iz = Li % 3, jx = Lj / 9, jy = (Lj / 3) % 3, jz = Lj % 3;
    int const px = symCls(ix, jx), py = symCls(iy, jy), pz = symCls(iz, jz);
    uint16_t * const o = &pidx[8 * q];
    o[0] = (uint16_t)(px * 36 + py * 6 + pz);
    o[1] = (uint16_t)(pz * 36 + px * 6 + py);
    o[2] = aaIdx(pz, ix, jx, iy, jy);
    o[3] = (uint16_t)(py * 36 + px * 6 + pz);
    o[4] = aaIdx(py, ix, jx, iz, jz);
    o[5] = (uint16_t)(px * 36 + py * 6 + pz);
    o[6] = aaIdx(px, iy, jy, iz, jz);
  }
  PXG_CUDA(c, cudaMemcpyToSymbol(gPairIdx, pidx.data(), pidx.size() * 2));
  return PXG_OK;
}

void launchAssembleQ2F64(AsmArgs const & a, cudaStream_t s)
{
  if (a.nelem > 0)
    launchElemKernel(kAssembleQ2F64, (unsigned)a.nelem, 32, 0, s, a);
}

} // namespace pxg
