// Internal declarations of the GB300 assembly engine (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <utility>
#include <vector>

#include "../../include/pxg.h"

namespace pxg
{

enum : int
{
  P1TET = 0,
  P2TET = 1,
  Q1HEX = 2,
  Q2HEX = 3,
};

// Element traits: vertices, DOFs, quadrature points (LagrangeFE<...>::RecommendedQR,
// include/fe.hpp:96-131 of proxpde).
template <int T>
struct Elem;
template <>
struct Elem<P1TET>
{
  static constexpr int NV = 4, N = 4, NQ = 4;
  static constexpr bool hex = false;
};
template <>
struct Elem<P2TET>
{
  static constexpr int NV = 4, N = 10, NQ = 11;
  static constexpr bool hex = false;
};
template <>
struct Elem<Q1HEX>
{
  static constexpr int NV = 8, N = 8, NQ = 8;
  static constexpr bool hex = true;
};
template <>
struct Elem<Q2HEX>
{
  static constexpr int NV = 8, N = 27, NQ = 27;
  static constexpr bool hex = true;
};

inline int numVerts(int t) { return (t == P1TET || t == P2TET) ? 4 : 8; }
inline int numDofs(int t) { return t == P1TET ? 4 : t == P2TET ? 10 : t == Q1HEX ? 8 : 27; }
inline int numQpts(int t) { return t == P1TET ? 4 : t == P2TET ? 11 : t == Q1HEX ? 8 : 27; }
inline bool isHex(int t) { return t == Q1HEX || t == Q2HEX; }

// Local topology (include/geo.hpp:520-529, 640-665 of proxpde).
__host__ __device__ constexpr int tetEdgeV(int e, int k)
{
  constexpr int t[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
  return t[e][k];
}
__host__ __device__ constexpr int hexEdgeV(int e, int k)
{
  constexpr int t[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {0, 4}, {1, 5},
                            {2, 6}, {3, 7}, {4, 5}, {5, 6}, {6, 7}, {7, 4}};
  return t[e][k];
}
__host__ __device__ constexpr int hexFaceV(int f, int k)
{
  constexpr int t[6][4] = {{0, 3, 2, 1}, {3, 0, 4, 7}, {0, 1, 5, 4},
                           {1, 2, 6, 5}, {2, 3, 7, 6}, {4, 5, 6, 7}};
  return t[f][k];
}

// Mapping points = DOF points of the Lagrange elements, built from the vertices
// (RefFE::dofPts / mappingPts, include/reffe.hpp:748-767, 960-988 of proxpde).
template <int T>
__host__ __device__ inline void mappingPoints(double const (*X)[3], double (*P)[3])
{
  constexpr int NV = Elem<T>::NV;
#pragma unroll
  for (int v = 0; v < NV; ++v)
#pragma unroll
    for (int d = 0; d < 3; ++d)
      P[v][d] = X[v][d];
  if constexpr (T == P2TET)
  {
#pragma unroll
    for (int e = 0; e < 6; ++e)
#pragma unroll
      for (int d = 0; d < 3; ++d)
        P[4 + e][d] = .5 * (X[tetEdgeV(e, 0)][d] + X[tetEdgeV(e, 1)][d]);
  }
  if constexpr (T == Q2HEX)
  {
#pragma unroll
    for (int e = 0; e < 12; ++e)
#pragma unroll
      for (int d = 0; d < 3; ++d)
        P[8 + e][d] = 0.5 * (X[hexEdgeV(e, 0)][d] + X[hexEdgeV(e, 1)][d]);
#pragma unroll
    for (int f = 0; f < 6; ++f)
#pragma unroll
      for (int d = 0; d < 3; ++d)
        P[20 + f][d] = 0.25 * (X[hexFaceV(f, 0)][d] + X[hexFaceV(f, 1)][d] +
                               X[hexFaceV(f, 2)][d] + X[hexFaceV(f, 3)][d]);
#pragma unroll
    for (int d = 0; d < 3; ++d)
      P[26][d] = .125 * (X[0][d] + X[1][d] + X[2][d] + X[3][d] + X[4][d] + X[5][d] +
                         X[6][d] + X[7][d]);
  }
}

// Analytic functions by id (pxg_fn).  sinpi(x) is sin(pi x) without the rounding of
// pi x; it agrees with the reference's std::sin(M_PI * x) to round-off.
__host__ __device__ inline double evalFn(int fn, double c, double x, double y, double z)
{
#ifdef __CUDA_ARCH__
  switch (fn)
  {
  case PXG_FN_CONST:
    return c;
  case PXG_FN_SIN3:
    return c * (sinpi(x) * sinpi(y) * sinpi(z));
  case PXG_FN_POISSON_RHS:
    return c * (2.5 * 3.141592653589793 * 3.141592653589793 * sinpi(0.5 * x) * sinpi(1.5 * y));
  case PXG_FN_POISSON_EXACT:
    return c * (sinpi(0.5 * x) * sinpi(1.5 * y));
  case PXG_FN_COORD_X:
    return c * x;
  case PXG_FN_COORD_Y:
    return c * y;
  case PXG_FN_COORD_Z:
    return c * z;
  }
  return __longlong_as_double(0x7ff8000000000000ll);
#else
  (void)fn;
  (void)c;
  (void)x;
  (void)y;
  (void)z;
  return 0.0;
#endif
}

// ------------------------------------------------------------ device buffer
template <typename T>
struct DevBuf
{
  T * p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(DevBuf const &) = delete;
  DevBuf & operator=(DevBuf const &) = delete;
  ~DevBuf() { reset(); }
  void reset()
  {
    if (p)
      cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count)
  {
    reset();
    if (count == 0)
      return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess)
    {
      p = nullptr;
      return e;
    }
    n = count;
    return cudaSuccess;
  }
  size_t bytes() const { return n * sizeof(T); }
};

} // namespace pxg

// CG work vectors, device scalars and the internal stream used for graph capture
struct CgWork
{
  int64_t n = 0;
  pxg::DevBuf<double> r, z, p, q, dinv, part, scal;
  cudaStream_t stream = nullptr;
  cudaEvent_t evIn = nullptr, evOut = nullptr;
  ~CgWork()
  {
    if (stream)
      cudaStreamDestroy(stream);
    if (evIn)
      cudaEventDestroy(evIn);
    if (evOut)
      cudaEventDestroy(evOut);
  }
};

// state kept by pxg_adjoint_forward for pxg_adjoint_backward (the saved tensors)
struct AdjState
{
  int64_t n = 0, nnz = 0;
  pxg::DevBuf<double> K, M, b, u, w, Mw, lam, part;
  double rtol = 1e-10;
  int maxIter = 0;
  bool valid = false;
};

// a context's mesh declared as a batch of independent problems (pxg_batch_set)
struct BatchState
{
  bool ready = false;
  int64_t nprob = 0;
  int probBase = 0; // global id of this batch's first problem in the last solve
  pxg::DevBuf<int64_t> elemOff, dofOff;
  std::vector<int64_t> dofOffHost;
  pxg::DevBuf<int32_t> rowProb;
  pxg::DevBuf<double> K, M, b, u, lam, r, z, p, q, dinv, w, Mw;
};

// arguments a captured batch graph was built for
struct GraphKey
{
  int nctx = 0;
  void * ctx[2] = {nullptr, nullptr};
  double const * ut[2] = {nullptr, nullptr};
  double * grad[2] = {nullptr, nullptr};
  pxg_rhs_op rhs{};
  double rtol = 0.;
  int maxIter = 0;
  int scatter[2] = {0, 0}, threads[2] = {0, 0}; // the element kernels captured in the graph
  int arith[2] = {0, 0};
  bool operator==(GraphKey const & o) const
  {
    return nctx == o.nctx && ctx[0] == o.ctx[0] && ctx[1] == o.ctx[1] && ut[0] == o.ut[0] && ut[1] == o.ut[1] &&
           grad[0] == o.grad[0] && grad[1] == o.grad[1] && rhs.kind == o.rhs.kind && rhs.fn == o.rhs.fn &&
           rhs.coef == o.rhs.coef && rhs.field == o.rhs.field && rtol == o.rtol && maxIter == o.maxIter &&
           scatter[0] == o.scatter[0] && scatter[1] == o.scatter[1] && threads[0] == o.threads[0] &&
           threads[1] == o.threads[1] && arith[0] == o.arith[0] && arith[1] == o.arith[1];
  }
};

// per-problem solver state of the persistent batch kernel (on the first context)
struct BatchShared
{
  int nprob = 0;
  pxg::DevBuf<double> acc;
  pxg::DevBuf<int> done, itF, itA, err;
  pxg::DevBuf<unsigned> bar;
  // problem table (global problem id -> system, first row, rows) and the per-iteration
  // row chunks of the running problems, two tables used by alternate iterations
  pxg::DevBuf<int> probSys;
  pxg::DevBuf<int64_t> probRow0, probRows;
  int64_t capChunks = 0;
  pxg::DevBuf<int> chunkProb[2], chunkRows[2], nchunk;
  pxg::DevBuf<int64_t> chunkRow0[2];
  cudaGraphExec_t exec = nullptr;
  GraphKey key;
  ~BatchShared()
  {
    if (exec)
      cudaGraphExecDestroy(exec);
  }
};

// ----------------------------------------------------------------- context
struct pxg_ctx
{
  int device = 0;
  std::string err;
  // mesh
  int etype = -1;
  int nv = 0, N = 0;
  int64_t nnodes = 0, nelem = 0;
  pxg::DevBuf<double> xyz;
  pxg::DevBuf<uint32_t> conn;
  // DOF map
  int64_t ndof = 0;
  pxg::DevBuf<uint32_t> emap;
  // structural pattern + per-element scatter ranks (rank[e][i][j]: position of
  // column emap[e][j] inside row emap[e][i])
  int64_t nnz = 0;
  int maxRowLen = 0;
  pxg::DevBuf<int32_t> rowPtr, colIdx;
  pxg::DevBuf<uint16_t> rank;
  // coefficient and BCs
  pxg::DevBuf<double> kE;
  bool hasCoef = false;
  pxg::DevBuf<uint8_t> bcMask;
  pxg::DevBuf<double> bcVal;
  int64_t nbc = 0;
  double bcDiag = 1.0;
  // small device scratch (counters, flags)
  pxg::DevBuf<unsigned long long> counter;
  // scatter strategy and elements per CTA of the element kernels (pxg_set_scatter,
  // pxg_autotune); threads = 0 is the kernel's default
  int scatter = 0; // PXG_SCATTER_REDUCE or PXG_SCATTER_COLOUR
  int threads = 0;
  // element colouring of the colour-ordered scatter: elements sorted by colour,
  // start[k] .. start[k + 1] the k-th colour class
  struct ColourState
  {
    int ncol = 0;
    std::vector<int64_t> start;
    pxg::DevBuf<uint32_t> perm;
    bool built = false;
  } colour;
  // warp-group scatter map of the P2 FP64 kernel (pxg_group.cu): for each group of 32
  // consecutive elements, its distinct CSR positions in ascending order (off: first
  // index of each group, pos, beg: offset of the first contribution in the group) and
  // the contributions in the same order as codes (element lane | local entry); built
  // on first use
  struct GroupState
  {
    bool built = false;
    int64_t ngroups = 0, ndistinct = 0;
    pxg::DevBuf<int32_t> off, pos;
    pxg::DevBuf<uint16_t> beg, item;
    void reset()
    {
      built = false;
      ngroups = ndistinct = 0;
      off.reset();
      pos.reset();
      beg.reset();
      item.reset();
    }
  } groups;
  // boundary facets in key order: element * faces-per-element + local face, and markers
  struct FacetState
  {
    bool built = false;
    int64_t n = 0;
    pxg::DevBuf<uint32_t> face;
    pxg::DevBuf<int32_t> marker;
  } facets;
  // arithmetic of the element kernels (pxg_set_arithmetic): PXG_ARITH_FP64 (default)
  // or PXG_ARITH_DFL (double-float, opt-in).  Cross-check kernels, chosen in the
  // environment when the context is created: PXG_Q1_GENERIC=1 (the per-quadrature-point
  // FP64 kernel), PXG_Q1_THREAD=1 (the one-thread tensor-product kernel in the
  // context's arithmetic), PXG_Q1_GROUP=1 (the eight-lanes-per-element kernel in the
  // context's arithmetic; the double-float default), PXG_TET_GENERIC=1 and
  // PXG_Q2_GENERIC=1 (the per-quadrature-point FP64 kernels)
  int arith = PXG_ARITH_FP64;
  bool q1Generic = false;
  bool q1Thread = false;
  bool q1Group = false;
  bool tetGeneric = false;
  bool q2Generic = false;
  // P2 FP64: sum each warp's contributions per distinct position before the reductions
  bool groupScatter = true;
  // zero the outputs with a kernel that the FP64 element kernel overlaps (else memsets)
  bool zeroOverlap = true;
  // positions with at most this many contributions get one reduction per contribution
  // (L2 adds them) instead of FP64 additions on the SM: 2 measured best at 64^3 x 6
  int groupRedMax = 2;
  int sms = 0; // SMs of the device (persistent grids)
  // What produced each value array pxg_assemble wrote (its recipe): the lhs operators
  // added into it since it was last overwritten, with the versions of the coordinates,
  // the coefficient and the BCs they used.  pxg_close_matrix recomputes the array's
  // near-zero entries in the reference's evaluation order from it (pxg_assemble.cu).
  struct LhsRec
  {
    int stiff, mass, bc;
    double sc, mc;
  };
  struct Recipe
  {
    double const * vals = nullptr;
    std::vector<LhsRec> ops;
    uint64_t meshVer = 0, coefVer = 0, bcVer = 0;
    bool valid = false;
  };
  std::vector<Recipe> recipes;
  uint64_t meshVer = 1, coefVer = 1, bcVer = 1;
  // element ids of each DOF in ascending order (built on the first recomputation)
  pxg::DevBuf<int32_t> dofElemPtr;
  pxg::DevBuf<uint32_t> dofElem;
  CgWork cg;
  AdjState adj;
  BatchState batch;
  BatchShared bshared;
};

// arguments of the element kernels
namespace pxg
{
struct LhsDev
{
  int on, stiff, mass, bc;
  double sc, mc;
  double * vals;
};

// The mass coefficient of an operator for an element whose P0 coefficient is kfac:
// AssemblyScalarMass(mc) (kind 1) or AssemblyMassFE with the per-element coefficient
// (kind 2, include/assembly_lhs.hpp:234-277), times mc.
__host__ __device__ __forceinline__ double massCoef(LhsDev const & op, double kfac)
{
  return op.mass == 2 ? op.mc * kfac : op.mc;
}
// whether an operator reads the per-element coefficient
__host__ __device__ __forceinline__ bool usesCoef(LhsDev const & op)
{
  return op.on && (op.stiff == 2 || op.mass == 2);
}

struct AsmArgs
{
  int64_t nelem;
  double const * xyz;
  uint32_t const * conn;
  uint32_t const * emap;
  int32_t const * rowPtr;
  uint16_t const * rank;
  double const * kE;
  uint8_t const * bcMask;
  double const * bcVal;
  double bcDiag;
  LhsDev op[2];
  int rkind, fn, rbc;
  double rc;
  double const * field;
  double * b;
  // colour-ordered scatter: the launch covers elements perm[permBase .. permBase + nelem)
  uint32_t const * perm;
  int64_t permBase;
  // warp-group scatter map (P2 FP64 kernel, element order only; null: plain reductions)
  int32_t const * grpOff;
  int32_t const * grpPos;
  uint16_t const * grpBeg;
  uint16_t const * grpItem;
  int grpRedMax;
  // launched as a programmatic dependent of the zeroing of its outputs (pdlWait)
  int pdl;
};

// The default FP64 element kernels run as programmatic dependents of the kernel that
// zeroes their outputs: their blocks start while the (DRAM-bound) zeroing runs, compute
// their element values, and wait for it only before their first write.  On a plain
// launch the wait returns at once.
__device__ __forceinline__ void pdlWait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// launch an element kernel, as a programmatic dependent of the stream's previous
// launch when a.pdl is set
template <typename Kern>
inline cudaError_t launchElemKernel(Kern kern, unsigned blocks, unsigned threads, size_t smem, cudaStream_t s,
                                    AsmArgs const & a)
{
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = a.pdl ? at : nullptr;
  cfg.numAttrs = a.pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, a);
}

// P2 tetrahedron local numbering (src/reffe.cpp:542-642): vertices 0-3, then the edges
// 01 12 20 03 13 23 as nodes 4-9; end k of edge node n
__host__ __device__ constexpr int p2EdgeEnd(int n, int k)
{
  return k == 0 ? (n == 4 ? 0 : n == 5 ? 1 : n == 6 ? 2 : n == 7 ? 0 : n == 8 ? 1 : 2)
                : (n == 4 ? 1 : n == 5 ? 2 : n == 6 ? 0 : 3);
}
__host__ __device__ constexpr bool p2EdgesMeet(int i, int j)
{
  return p2EdgeEnd(i, 0) == p2EdgeEnd(j, 0) || p2EdgeEnd(i, 0) == p2EdgeEnd(j, 1) ||
         p2EdgeEnd(i, 1) == p2EdgeEnd(j, 0) || p2EdgeEnd(i, 1) == p2EdgeEnd(j, 1);
}
// the seven classes of the P2 mass matrix: vertex-vertex (same, other), vertex-edge
// (on, off), edge-edge (same, sharing a vertex, disjoint)
__host__ __device__ constexpr int p2MassClass(int i, int j)
{
  return j < i   ? p2MassClass(j, i)
         : j < 4 ? (i == j ? 0 : 1)
         : i < 4 ? ((i == p2EdgeEnd(j, 0) || i == p2EdgeEnd(j, 1)) ? 2 : 3)
         : i == j ? 4
                  : (p2EdgesMeet(i, j) ? 5 : 6);
}
// index of the pair (min, max) among the 55 pairs i <= j of the P2 element, row by row
__host__ __device__ constexpr int p2UpperIdx(int i, int j)
{
  return j < i ? p2UpperIdx(j, i) : i * 10 - i * (i - 1) / 2 + (j - i);
}
// warp-group scatter of the P2 kernel: per warp, the 55 stiffness entries and the 7 mass
// values of each lane's element in shared memory, value-major (value v of lane l at
// v * 32 + l), then the group's 3,200 contribution codes; a code is
// lane | pair index << 5 | mass class << 11
constexpr int kP2GroupValues = 55 + 7;
constexpr int kP2GroupItems = 32 * 100;
constexpr size_t kP2GroupSmemPerWarp = kP2GroupValues * 32 * sizeof(double) + kP2GroupItems * sizeof(uint16_t);
__host__ __device__ constexpr uint16_t p2GroupCode(int lane, int i, int j)
{
  return (uint16_t)(lane | (p2UpperIdx(i, j) << 5) | (p2MassClass(i, j) << 11));
}

// element id of the launch's i-th element
__device__ __forceinline__ int64_t elemOf(AsmArgs const & a, int64_t i)
{
  return a.perm ? (int64_t)a.perm[a.permBase + i] : i;
}

void launchAssembleQ1(AsmArgs const & a, cudaStream_t s, bool fp64, bool perThread, int threads);
// the FP64 one-thread-per-element Q1 kernel (pxg_q1f64.cu), the default
void launchAssembleQ1F64(AsmArgs const & a, cudaStream_t s, int threads);
// element colouring (pxg_colour.cu); built once per mesh
pxg_status buildColouring(pxg_ctx * c);

struct AdjArgs
{
  int64_t nelem;
  double const * xyz;
  uint32_t const * conn;
  uint32_t const * emap;
  double const * kE;
  uint8_t const * bcMask;
  double const * u;
  double const * lam;
  double * g;
};
void launchAdjointGradQ1(AdjArgs const & a, cudaStream_t s, bool fp64);
} // namespace pxg

// Row-segment CSR product shared by the solvers: LPR consecutive lanes of a warp
// work on one row (coalesced reads of the row's values and column ids), then reduce
// with shuffles; every lane of the group returns the row's result.  All 32 lanes of
// the warp must call it (valid = false for lanes without a row).
namespace pxg
{
constexpr int kLpr = 4;  // lanes per row
constexpr int kUnr = 8;  // entries per lane and load round
// LPR lanes per row (a power of two), UNR entries per lane and round.  The FP64 pipe
// issues every slot of a round, used or not (GB300: 1/64 of the FP32 rate), so LPR x
// UNR should just cover the typical row: 4 x 7 for Q1 hexahedra (27 entries), 2 x 8
// for P1 tetrahedra (15).
template <bool L2ONLY, int LPR = kLpr, int UNR = kUnr, bool REDUCE = true>
__device__ __forceinline__ double rowDot(int32_t const * __restrict__ rp, int32_t const * __restrict__ ci,
                                         double const * __restrict__ a, double const * x, int64_t row, bool valid)
{
  // UNR strided entries per lane and round: their column ids and values are loaded
  // together, then the gathers, so each lane keeps many loads in flight (a row of up
  // to LPR * UNR entries takes one round)
  int const sub = threadIdx.x & (LPR - 1);
  double t = 0.;
  if (valid)
  {
    int32_t const e = rp[row + 1];
    for (int32_t base = rp[row] + sub; base < e; base += UNR * LPR)
    {
      int32_t cc[UNR];
      double av[UNR];
#pragma unroll
      for (int u = 0; u < UNR; ++u)
      {
        int32_t const k = base + u * LPR;
        bool const ok = k < e;
        // the matrix is streamed once per product: evict-first loads, so that it does not
        // push the gathered vector out of L2
        cc[u] = ok ? __ldcs(ci + k) : -1;
        av[u] = ok ? __ldcs(a + k) : 0.;
      }
#pragma unroll
      for (int u = 0; u < UNR; ++u)
        if (cc[u] >= 0)
          t = fma(av[u], L2ONLY ? __ldcg(x + cc[u]) : x[cc[u]], t);
    }
  }
  if constexpr (REDUCE)
  {
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1)
      t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  return t;
}

// The lane partials t[k] of LPR rows (row k of the lane's group in the k-th of LPR
// consecutive row batches), reduced so that the lane whose position in its group is
// `sub` returns the whole sum of row `sub`: log2(LPR) halving stages, in each of which
// a lane keeps the half of its rows its partner does not and adds the partner's share
// of them.  LPR - 1 additions per lane for LPR rows, where the butterfly of rowDot
// takes log2(LPR) per row; the lanes are paired as in that butterfly (xor LPR/2 first),
// so every row sum is the same double.
template <int LPR>
__device__ __forceinline__ double transposeReduce(double (&t)[LPR], int sub)
{
  if constexpr (LPR == 1)
    return t[0];
  else
  {
    constexpr int H = LPR / 2;
    bool const upper = (sub & H) != 0;
    double keep[H];
#pragma unroll
    for (int k = 0; k < H; ++k)
    {
      double const send = upper ? t[k] : t[k + H];
      keep[k] = (upper ? t[k + H] : t[k]) + __shfl_xor_sync(0xffffffffu, send, H);
    }
    return transposeReduce<H>(keep, sub);
  }
}
} // namespace pxg

// status helpers shared by the translation units
namespace pxg
{
pxg_status fail(pxg_ctx * c, pxg_status s, char const * fmt, ...);
pxg_status cudaFail(pxg_ctx * c, cudaError_t e, char const * what);
pxg_status ensureDevice(pxg_ctx * c);

// pattern / dofmap (pxg_pattern.cu)
pxg_status buildDofmap(pxg_ctx * c);
pxg_status buildPattern(pxg_ctx * c);

// reference tables (pxg_assemble.cu)
pxg_status initTables(pxg_ctx * c);
// quadrature rule (nodes xi[3 q + d], weights) and shape functions of element type t
// on the reference element, as proxpde defines them (host)
void hostRule(int t, std::vector<double> & xi, std::vector<double> & w);
pxg_status initQ2Tables(pxg_ctx * c);                      // pxg_q2.cu
void launchAssembleQ2(AsmArgs const & a, cudaStream_t s, int sms); // pxg_q2.cu
pxg_status initQ2F64Tables(pxg_ctx * c);                          // pxg_q2f64.cu
void launchAssembleQ2F64(AsmArgs const & a, cudaStream_t s);      // pxg_q2f64.cu
pxg_status buildScatterGroups(pxg_ctx * c);                       // pxg_group.cu
void hostShape(int t, double const * p, double * phi, double * dphi);
// g_e = -(C u)_e^T K_e (C lambda)_e for every element (pxg_assemble.cu)
pxg_status launchAdjointGrad(pxg_ctx * c, double const * u, double const * lam, double * g, cudaStream_t s);
// prune + compaction of a structural CSR into caller buffers (pxg_assemble.cu)
pxg_status closeCsr(pxg_ctx * c, int32_t const * rowPtr, int32_t const * colIdx, int64_t n, double const * vals,
                    int32_t * rp, int32_t * ci, double * vout, int64_t * nnzOut, cudaStream_t s);
// Jacobi-PCG (pxg_solve.cu)
pxg_status cgSolve(pxg_ctx * c, int32_t const * rp, int32_t const * ci, double const * a, int64_t n,
                   double const * b, double * x, double rtol, int maxIter, int * itersOut, double * relOut,
                   cudaStream_t user);
} // namespace pxg

#define PXG_CUDA(ctx, call)                                                                    \
  do                                                                                           \
  {                                                                                            \
    cudaError_t _e = (call);                                                                   \
    if (_e != cudaSuccess)                                                                     \
      return pxg::cudaFail((ctx), _e, #call);                                                  \
  } while (0)
