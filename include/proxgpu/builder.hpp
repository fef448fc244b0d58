// proxgpu/builder.hpp — header-only C++20 drop-in for proxpde's assembly call surface,
// running on the GB300 engine through its C ABI (include/pxg.h, libpxg.so).
//
// The names and the call sequence follow proxpde (include/builder.hpp:12-391, the
// Assembly* types of include/assembly_lhs.hpp / assembly_rhs.hpp, and the setup and
// solve calls of its tests, e.g. test/poisson3dhex.cpp:20-104):
//
//   using namespace proxgpu;
//   using Mesh_T = Mesh<Hexahedron>;
//   using FESpace_T = FESpace<Mesh_T, LagrangeFE<Hexahedron, 1>::RefFE_T,
//                             LagrangeFE<Hexahedron, 1>::RecommendedQR>;
//   std::unique_ptr<Mesh_T> mesh{new Mesh_T};
//   buildHyperCube(*mesh, {0., 0., 0.}, {1., 1., 1.}, {n, n, n});      // mesh.hpp:385-421
//   FESpace_T feSpace{*mesh};                                          // fespace.hpp:27-193
//   auto bcLeft = BCEss{feSpace, side::LEFT};
//   bcLeft << [](Vec3 const &) { return 0.; };                         // bc.hpp:63
//   Builder builder{feSpace.dof.size};                                 // builder.hpp:19
//   builder.buildLhs(std::tuple{AssemblyStiffness(1.0, feSpace)}, bcs);
//   builder.buildRhs(std::tuple{AssemblyRhsAnalytic(rhs, feSpace)}, bcs);  // any f(Vec3)
//   builder.closeMatrix();
//   LUSolver solver;                                                   // sparse_matrix.hpp:44
//   solver.analyzePattern(builder.A);
//   solver.factorize(builder.A);
//   sol.data = solver.solve(builder.b);
//
// Differences from proxpde, all forced by running on a GPU or by what the engine
// replaces:
//  - a host function rhs (std::function or lambda) is evaluated on the host at the
//    quadrature points the device reports (pxg_get_qpoints) and integrated on the
//    device; device functions chosen by id (pxg_fn) are the faster form; unrecognised
//    assembly types do not compile (no CPU fallback);
//  - A is returned as CSR arrays; proxpde's default ClmMajor storage is CSC, and for
//    the symmetric matrices assembled here the CSC arrays are the same arrays;
//  - LUSolver is the device Jacobi-preconditioned CG (pxg_cg) behind UmfPackLU's
//    analyzePattern / factorize / solve, to a relative residual of 1e-14 by default;
//  - Vec is a std::vector<double> with the few Eigen operations the tests use;
//  - errors throw proxgpu::Error (carrying the pxg_status) instead of aborting.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <functional>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "../pxg.h"

namespace proxgpu
{

struct Error : std::runtime_error
{
  pxg_status status;
  Error(pxg_status s, std::string const & what): std::runtime_error(what), status(s) {}
};

inline void check(pxg_status s, pxg_ctx const * ctx, char const * what)
{
  if (s != PXG_OK)
    throw Error(s, std::string(what) + ": " + pxg_status_string(s) + (ctx ? std::string(" (") + pxg_last_error(ctx) + ")" : ""));
}

struct Tetrahedron
{
  static constexpr int numPts = 4;
};
struct Hexahedron
{
  static constexpr int numPts = 8;
};

enum class StorageType
{
  ClmMajor,
  RowMajor
};

// Boundary markers of the structured cube (include/mesh.hpp:178-188) and the plane
// markFacetsCube gives each (include/mesh.hpp:442-498).
namespace side
{
enum : int
{
  NONE = 0,
  BOTTOM,
  RIGHT,
  TOP,
  LEFT,
  BACK,
  FRONT
};
} // namespace side

// Point / vector value of the BC functions (the Vec3 of the reference's Fun<3, 3>)
struct Vec3
{
  double v[3] = {0., 0., 0.};
  Vec3() = default;
  Vec3(double x, double y, double z): v{x, y, z} {}
  double operator()(int i) const { return v[i]; }
  double & operator()(int i) { return v[i]; }
  static Vec3 Constant(double c) { return Vec3(c, c, c); }
};

template <typename Elem>
struct Mesh
{
  std::vector<double> xyz;     // nnodes x 3
  std::vector<uint32_t> conn;  // nelem x numPts, proxpde's local vertex order
  int64_t nnodes() const { return (int64_t)xyz.size() / 3; }
  int64_t nelem() const { return (int64_t)conn.size() / Elem::numPts; }
};

// buildHyperCube(mesh, origin, length, {nx, ny, nz}) (include/mesh.hpp:385-421, with
// buildCube of src/mesh.cpp:355-534): the box origin + [0, length] split into
// nx x ny x nz cubes, node (i, j, k) at id i + (nx+1) j + (nx+1)(ny+1) k; hexahedra, or
// 5 tetrahedra per cube alternating with the parity of (i + j + k).
template <typename Elem>
void buildHyperCube(Mesh<Elem> & m, Vec3 const & origin, Vec3 const & length, std::array<uint32_t, 3> const & n)
{
  if (n[0] == 0 || n[1] == 0 || n[2] == 0)
    throw Error(PXG_ERR_INVALID_ARG, "buildHyperCube: zero elements along an axis");
  uint32_t const nx = n[0], ny = n[1], nz = n[2];
  uint32_t const px = nx + 1, py = ny + 1, pz = nz + 1;
  double const h[3] = {length(0) / nx, length(1) / ny, length(2) / nz};
  m.xyz.assign((size_t)px * py * pz * 3, 0.);
  m.conn.clear();
  for (uint32_t k = 0; k < pz; ++k)
    for (uint32_t j = 0; j < py; ++j)
      for (uint32_t i = 0; i < px; ++i)
      {
        size_t const id = i + (size_t)px * j + (size_t)px * py * k;
        m.xyz[3 * id] = origin(0) + i * h[0];
        m.xyz[3 * id + 1] = origin(1) + j * h[1];
        m.xyz[3 * id + 2] = origin(2) + k * h[2];
      }
  uint32_t const dx = 1, dy = px, dz = px * py;
  for (uint32_t k = 0; k < nz; ++k)
    for (uint32_t j = 0; j < ny; ++j)
      for (uint32_t i = 0; i < nx; ++i)
      {
        uint32_t const b = i + j * dy + k * dz;
        if constexpr (std::is_same_v<Elem, Hexahedron>)
        {
          for (uint32_t v : {b, b + dx, b + dx + dy, b + dy, b + dz, b + dx + dz, b + dx + dy + dz, b + dy + dz})
            m.conn.push_back(v);
        }
        else
        {
          uint32_t const odd[5][4] = {{b + dx, b + dy, b + dz, b + dx + dy + dz},
                                      {b, b + dx, b + dy, b + dz},
                                      {b + dx, b + dx + dy, b + dy, b + dx + dy + dz},
                                      {b + dx, b + dz, b + dx + dz, b + dx + dy + dz},
                                      {b + dy, b + dz, b + dx + dy + dz, b + dy + dz}};
          uint32_t const even[5][4] = {{b, b + dx + dy, b + dx + dz, b + dy + dz},
                                       {b, b + dx, b + dx + dy, b + dx + dz},
                                       {b, b + dx + dy, b + dy, b + dy + dz},
                                       {b, b + dz, b + dx + dz, b + dy + dz},
                                       {b + dx + dy, b + dx + dz, b + dx + dy + dz, b + dy + dz}};
          auto const & t = ((i + j + k) % 2) ? odd : even;
          for (auto const & row: t)
            for (uint32_t v : row)
              m.conn.push_back(v);
        }
      }
}

// the unit cube with n^3 cubes, and the box origin + [0, length] with n^3 cubes
template <typename Elem>
Mesh<Elem> buildHyperCube(int n)
{
  Mesh<Elem> m;
  buildHyperCube(m, Vec3(0., 0., 0.), Vec3(1., 1., 1.), {(uint32_t)n, (uint32_t)n, (uint32_t)n});
  return m;
}
template <typename Elem>
Mesh<Elem> buildHyperCube(std::array<double, 3> const & origin, std::array<double, 3> const & length, int n)
{
  Mesh<Elem> m;
  buildHyperCube(m, Vec3(origin[0], origin[1], origin[2]), Vec3(length[0], length[1], length[2]),
                 {(uint32_t)n, (uint32_t)n, (uint32_t)n});
  return m;
}

// Vec (Eigen::VectorXd in proxpde, include/def.hpp:157-160) with the operations the
// tests use, and Var (a named vector, include/var.hpp:14-52)
struct Vec : std::vector<double>
{
  using std::vector<double>::vector;
  Vec(std::vector<double> v): std::vector<double>(std::move(v)) {}
  double norm() const
  {
    double s = 0.;
    for (double x: *this)
      s += x * x;
    return std::sqrt(s);
  }
  Vec operator-(Vec const & o) const
  {
    if (o.size() != size())
      throw Error(PXG_ERR_INVALID_ARG, "Vec: sizes differ");
    Vec r(size());
    for (size_t k = 0; k < size(); ++k)
      r[k] = (*this)[k] - o[k];
    return r;
  }
  Vec operator+(Vec const & o) const
  {
    if (o.size() != size())
      throw Error(PXG_ERR_INVALID_ARG, "Vec: sizes differ");
    Vec r(size());
    for (size_t k = 0; k < size(); ++k)
      r[k] = (*this)[k] + o[k];
    return r;
  }
};
struct Var
{
  std::string name;
  Vec data;
  explicit Var(std::string n, size_t size = 0): name(std::move(n)), data(size, 0.0) {}
};
using scalarFun_T = std::function<double(Vec3 const &)>;
using vectorFun_T = std::function<Vec3(Vec3 const &)>;

// checkError (include/def.hpp:357-385): each error within tol of its expected value;
// returns the failure bitset (0 = pass), printing each comparison
inline int checkError(std::vector<double> const & errors, std::vector<double> const & expected, double tol = 1.e-12)
{
  if (errors.size() != expected.size())
    throw Error(PXG_ERR_INVALID_ARG, "checkError: sizes differ");
  int fails = 0;
  for (size_t k = 0; k < errors.size(); ++k)
  {
    bool const ok = std::fabs(errors[k] - expected[k]) < tol;
    std::printf("error: %.16e, expected: %.16e, difference: %.3e %s\n", errors[k], expected[k],
                std::fabs(errors[k] - expected[k]), ok ? "ok" : "FAIL");
    if (!ok)
      fails |= 1 << k;
  }
  return fails;
}

// Device array owned through the C ABI.
template <typename T>
struct DeviceArray
{
  pxg_ctx * ctx = nullptr;
  T * p = nullptr;
  size_t n = 0;
  DeviceArray() = default;
  DeviceArray(pxg_ctx * c, size_t count): ctx(c), n(count)
  {
    void * v = nullptr;
    check(pxg_device_alloc(c, count * sizeof(T), &v), c, "pxg_device_alloc");
    p = static_cast<T *>(v);
  }
  DeviceArray(DeviceArray const &) = delete;
  DeviceArray & operator=(DeviceArray const &) = delete;
  DeviceArray(DeviceArray && o) noexcept: ctx(o.ctx), p(o.p), n(o.n) { o.p = nullptr; }
  DeviceArray & operator=(DeviceArray && o) noexcept
  {
    std::swap(ctx, o.ctx);
    std::swap(p, o.p);
    std::swap(n, o.n);
    return *this;
  }
  ~DeviceArray()
  {
    if (p)
      pxg_device_free(ctx, p);
  }
  void zero()
  {
    std::vector<T> z(n, T{});
    check(pxg_memcpy(ctx, p, z.data(), n * sizeof(T), 0, nullptr), ctx, "pxg_memcpy");
  }
  std::vector<T> host() const
  {
    std::vector<T> h(n);
    check(pxg_memcpy(ctx, h.data(), p, n * sizeof(T), 1, nullptr), ctx, "pxg_memcpy");
    return h;
  }
};

// A Lagrange space on the device: the mesh, the first-touch DOF map and the CSR
// pattern live in one engine context.  Elem and Order give the reference element, Dim
// components (BLOCK ordering), QrOrder the order of the element type whose quadrature
// rule the space uses; offset is the space's offset in a global system.  Users write
// FESpace<Mesh_T, RefFE_T, QR_T, Dim> (below), as in proxpde.
template <typename Elem, int Order, int Dim = 1, int QrOrder = Order>
struct FESpaceImpl
{
  static constexpr int typeOf(int order)
  {
    return std::is_same_v<Elem, Tetrahedron> ? (order == 1 ? PXG_P1TET : PXG_P2TET)
                                             : (order == 1 ? PXG_Q1HEX : PXG_Q2HEX);
  }
  static constexpr int elemType = typeOf(Order);
  static constexpr int qrType = typeOf(QrOrder);
  static constexpr int dim = Dim;
  pxg_ctx * ctx = nullptr;
  struct
  {
    int64_t size = 0;
  } dof;
  int64_t nnz = 0;
  int64_t offset = 0;
  int64_t nelem = 0;
  double lo[3] = {0., 0., 0.}, hi[3] = {0., 0., 0.}; // bounding box of the mesh

  explicit FESpaceImpl(Mesh<Elem> const & m, int64_t off = 0, int device = 0): offset(off), nelem(m.nelem())
  {
    check(pxg_create(&ctx, device), nullptr, "pxg_create");
    check(pxg_set_mesh(ctx, elemType, m.xyz.data(), m.nnodes(), m.conn.data(), m.nelem(), PXG_MEM_HOST), ctx,
          "pxg_set_mesh");
    check(pxg_build_dofmap(ctx, &dof.size), ctx, "pxg_build_dofmap");
    check(pxg_build_pattern(ctx, &nnz), ctx, "pxg_build_pattern");
    // boundary facets marked on the planes of the bounding box, as markFacetsCube does
    // for buildHyperCube (include/mesh.hpp:443-481)
    for (int d = 0; d < 3; ++d)
      lo[d] = 1e300, hi[d] = -1e300;
    for (size_t k = 0; k < m.xyz.size(); ++k)
    {
      lo[k % 3] = std::min(lo[k % 3], m.xyz[k]);
      hi[k % 3] = std::max(hi[k % 3], m.xyz[k]);
    }
    double const len[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    check(pxg_mark_facets_box(ctx, lo, len), ctx, "pxg_mark_facets_box");
  }
  FESpaceImpl(FESpaceImpl const &) = delete;
  FESpaceImpl & operator=(FESpaceImpl const &) = delete;
  ~FESpaceImpl()
  {
    if (ctx)
      pxg_destroy(ctx);
  }

  // Lagrange interpolation of a device function (interpolateAnalyticFunction,
  // include/fespace.hpp:195-271)
  std::vector<double> interpolate(int fn, double coef = 1.0) const
  {
    DeviceArray<double> v(ctx, (size_t)dof.size);
    check(pxg_interpolate(ctx, fn, coef, v.p, nullptr), ctx, "pxg_interpolate");
    return v.host();
  }
  // CurFE::qpoint of every element and quadrature point (nelem x nq x 3)
  std::vector<double> qpoints() const
  {
    int const nq = elemType == PXG_P1TET ? 4 : elemType == PXG_P2TET ? 11 : elemType == PXG_Q1HEX ? 8 : 27;
    std::vector<double> q((size_t)nelem * nq * 3);
    check(pxg_get_qpoints(ctx, q.data(), PXG_MEM_HOST, nullptr), ctx, "pxg_get_qpoints");
    return q;
  }
};

// Reference elements and quadrature rules as type tags, with proxpde's names:
// LagrangeFE<Elem, Order>::RefFE_T / ::RecommendedQR (include/fe.hpp:96-131),
// GaussQR<Elem, points> (include/qr.hpp), RefTetrahedronP1 ... (include/reffe.hpp).
template <typename Elem, int Order>
struct RefLagrange
{
  using Elem_T = Elem;
  static constexpr int order = Order;
};
template <typename Elem, int NumPts>
struct GaussQR
{
  static_assert(NumPts == 4 || NumPts == 11 || NumPts == 8 || NumPts == 27, "rules of the Lagrange elements only");
  using Elem_T = Elem;
  static constexpr int order = (NumPts == 4 || NumPts == 8) ? 1 : 2; // the element order it belongs to
};
template <typename Elem, int Order>
struct LagrangeFE
{
  static_assert(Order == 1 || Order == 2, "P1/P2 tetrahedra and Q1/Q2 hexahedra");
  using RefFE_T = RefLagrange<Elem, Order>;
  using RecommendedQR =
      GaussQR<Elem, std::is_same_v<Elem, Tetrahedron> ? (Order == 1 ? 4 : 11) : (Order == 1 ? 8 : 27)>;
};
using RefTetrahedronP1 = RefLagrange<Tetrahedron, 1>;
using RefTetrahedronP2 = RefLagrange<Tetrahedron, 2>;
using RefHexahedronQ1 = RefLagrange<Hexahedron, 1>;
using RefHexahedronQ2 = RefLagrange<Hexahedron, 2>;

// FESpace<Mesh_T, RefFE_T, QR_T, Dim> (include/fespace.hpp:15-60)
template <typename Mesh_T, typename RefFE_T, typename QR_T, unsigned Dim = 1>
struct FESpace: FESpaceImpl<typename RefFE_T::Elem_T, RefFE_T::order, (int)Dim, QR_T::order>
{
  static_assert(std::is_same_v<Mesh_T, Mesh<typename RefFE_T::Elem_T>>, "the mesh and the element must match");
  static_assert(std::is_same_v<typename QR_T::Elem_T, typename RefFE_T::Elem_T>, "the rule and the element must match");
  using FESpaceImpl<typename RefFE_T::Elem_T, RefFE_T::order, (int)Dim, QR_T::order>::FESpaceImpl;
};

// interpolateAnalyticFunction(f, feSpace, v) (include/fespace.hpp:195-271) for a host
// function of the point: f at the DOF points (from the device); a vector space takes
// f returning Vec3 and fills every component (BLOCK ordering)
template <typename F, typename FE, typename = std::enable_if_t<std::is_invocable_v<F const &, Vec3 const &>>>
void interpolateAnalyticFunction(F const & f, FE const & fe, std::vector<double> & v)
{
  std::vector<double> const x = fe.interpolate(PXG_FN_COORD_X), y = fe.interpolate(PXG_FN_COORD_Y),
                            z = fe.interpolate(PXG_FN_COORD_Z);
  size_t const n = x.size();
  v.assign(n * FE::dim, 0.0);
  for (size_t k = 0; k < n; ++k)
  {
    auto const r = f(Vec3(x[k], y[k], z[k]));
    if constexpr (std::is_arithmetic_v<std::decay_t<decltype(r)>>)
      v[k] = r;
    else
      for (int c = 0; c < FE::dim; ++c)
        v[k + c * n] = r(c);
  }
}

// BCEss (include/bc.hpp:81-97) on the DOFs of the boundary facets with a marker, or on
// an explicit list.  Marker with a constant on a scalar space: the constrained set is
// built on the device from the facet markers (pxg_set_bc_markers).  Marker with a
// function of the point (scalar, or Vec3 on a vector space) and optional components:
// evaluated at the DOF points on the host (setup, as the reference does).  `dofs` /
// `values` always hold the constrained component DOFs (k + c * ndof) and their values,
// which the system builder uses.
struct BCEss
{
  int marker = side::NONE; // set: the scalar device path applies
  double value = 0.0;
  std::vector<uint32_t> dofs;
  std::vector<double> values;
  double diag = 1.0; // BCEss::diag (bc.hpp:301)

  template <typename FE>
  BCEss(FE const & fe, int m, double v = 0.0): value(v)
  {
    if (m < side::BOTTOM || m > side::FRONT)
      throw Error(PXG_ERR_INVALID_ARG, "BCEss: unknown side marker");
    if constexpr (FE::dim == 1)
      marker = m;
    collect(fe, m, [v](Vec3 const &) { return Vec3::Constant(v); }, {});
  }
  template <typename FE, typename F, typename = std::enable_if_t<std::is_invocable_v<F const &, Vec3 const &>>>
  BCEss(FE const & fe, int m, F const & fun, std::vector<int> comps = {})
  {
    if (m < side::BOTTOM || m > side::FRONT)
      throw Error(PXG_ERR_INVALID_ARG, "BCEss: unknown side marker");
    collect(fe, m, fun, comps);
  }
  BCEss(std::vector<uint32_t> d, std::vector<double> v): dofs(std::move(d)), values(std::move(v)) {}

  // BCEss << f (include/bc.hpp:63-79): new values, f at the constrained DOFs' points
  // (scalar f, or Vec3 f whose component c goes to the DOFs of component c)
  template <typename F, typename = std::enable_if_t<std::is_invocable_v<F const &, Vec3 const &>>>
  BCEss & operator<<(F const & fun)
  {
    if (pts.size() != 3 * dofs.size())
      throw Error(PXG_ERR_INVALID_ARG, "BCEss <<: the condition was given as an explicit DOF list");
    for (size_t k = 0; k < dofs.size(); ++k)
    {
      auto const r = fun(Vec3(pts[3 * k], pts[3 * k + 1], pts[3 * k + 2]));
      if constexpr (std::is_arithmetic_v<std::decay_t<decltype(r)>>)
        values[k] = r;
      else
        values[k] = r(comp[k]);
    }
    marker = side::NONE; // the values are a function now: the explicit list applies
    return *this;
  }

private:
  std::vector<double> pts; // the constrained DOFs' points
  std::vector<int> comp;   // and components

  // the DOFs on the marker's plane of the box (markFacetsCube), for every component
  template <typename FE, typename F>
  void collect(FE const & fe, int m, F const & fun, std::vector<int> comps)
  {
    int const axis = (m == side::RIGHT || m == side::LEFT) ? 0 : (m == side::BOTTOM || m == side::TOP) ? 1 : 2;
    bool const upper = m == side::RIGHT || m == side::TOP || m == side::FRONT;
    double const plane = upper ? fe.hi[axis] : fe.lo[axis], tol = 1e-6 * (fe.hi[axis] - fe.lo[axis]);
    std::vector<double> const x = fe.interpolate(PXG_FN_COORD_X), y = fe.interpolate(PXG_FN_COORD_Y),
                              z = fe.interpolate(PXG_FN_COORD_Z);
    if (comps.empty())
      for (int c = 0; c < FE::dim; ++c)
        comps.push_back(c);
    std::vector<double> const & xa = axis == 0 ? x : axis == 1 ? y : z;
    for (int c: comps)
      for (size_t k = 0; k < xa.size(); ++k)
        if (std::fabs(xa[k] - plane) <= tol)
        {
          auto const r = fun(Vec3(x[k], y[k], z[k]));
          double val;
          if constexpr (std::is_arithmetic_v<std::decay_t<decltype(r)>>)
            val = r;
          else
            val = r(c);
          dofs.push_back((uint32_t)(k + (size_t)c * xa.size()));
          values.push_back(val);
          pts.insert(pts.end(), {x[k], y[k], z[k]});
          comp.push_back(c);
        }
  }
};

// ------------------------------------------------------------------ assemblies
template <typename FE>
struct AssemblyStiffness
{
  double coef;
  FE const * feSpace;
  AssemblyStiffness(double c, FE const & fe): coef(c), feSpace(&fe) {}
};

// AssemblyStiffnessFE with a P0 coefficient: one value per element
template <typename FE>
struct AssemblyStiffnessFE
{
  std::vector<double> const * coefP0;
  FE const * feSpace;
  AssemblyStiffnessFE(std::vector<double> const & k, FE const & fe): coefP0(&k), feSpace(&fe) {}
};

template <typename FE>
struct AssemblyScalarMass
{
  double coef;
  FE const * feSpace;
  AssemblyScalarMass(double c, FE const & fe): coef(c), feSpace(&fe) {}
};
template <typename FE>
using AssemblyMass = AssemblyScalarMass<FE>;

// AssemblyMassFE with a P0 coefficient: one value per element (the space holds one
// per-element coefficient: with AssemblyStiffnessFE in the same call, both take the
// same values)
template <typename FE>
struct AssemblyMassFE
{
  std::vector<double> const * coefP0;
  FE const * feSpace;
  AssemblyMassFE(std::vector<double> const & k, FE const & fe): coefP0(&k), feSpace(&fe) {}
};

// AssemblyRhsAnalytic(f, feSpace, comps) (include/assembly_rhs.hpp:34-91).  f is any
// function of the point, as in the reference (a lambda or std::function returning a
// double on a scalar space, a Vec3 on a vector space): it is evaluated on the host at
// the quadrature points the device reports, and the values are integrated on the
// device (rhs kind 3).  f may also be a device function chosen by id (pxg_fn): one id
// on a scalar space, one id and one coefficient per component on a vector space.  Only
// the listed components (default: all) get a load, component c into block c.
template <typename FE>
struct AssemblyRhsAnalytic
{
  int fn;
  double coef;
  FE const * feSpace;
  std::vector<int> fns;      // per component (-1: values at the quadrature points)
  std::vector<double> coefs; // per component
  std::vector<int> comps;
  std::vector<std::vector<double>> qvals; // per component: f at the quadrature points
  template <typename F, typename = std::enable_if_t<std::is_invocable_v<F const &, Vec3 const &>>>
  AssemblyRhsAnalytic(F const & f, FE const & fe, std::vector<int> cmp = {}):
      fn(-1), coef(1.0), feSpace(&fe), fns(FE::dim, -1), coefs(FE::dim, 1.0), comps(std::move(cmp))
  {
    if (comps.empty())
      for (int d = 0; d < FE::dim; ++d)
        comps.push_back(d);
    for (int d: comps)
      if (d < 0 || d >= FE::dim)
        throw Error(PXG_ERR_INVALID_ARG, "AssemblyRhsAnalytic: component out of range");
    std::vector<double> const qp = fe.qpoints();
    size_t const n = qp.size() / 3;
    qvals.assign(FE::dim, std::vector<double>(n));
    for (size_t k = 0; k < n; ++k)
    {
      auto const r = f(Vec3(qp[3 * k], qp[3 * k + 1], qp[3 * k + 2]));
      if constexpr (std::is_arithmetic_v<std::decay_t<decltype(r)>>)
      {
        static_assert(FE::dim == 1, "a vector space takes a function returning Vec3");
        qvals[0][k] = r;
      }
      else
        for (int c = 0; c < FE::dim; ++c)
          qvals[(size_t)c][k] = r(c);
    }
  }
  AssemblyRhsAnalytic(int f, FE const & fe, double c = 1.0): fn(f), coef(c), feSpace(&fe), fns{f}, coefs{c}, comps{0}
  {
    static_assert(FE::dim == 1, "this ctor is available only for scalar fe spaces.");
  }
  AssemblyRhsAnalytic(std::array<int, FE::dim> const & f, FE const & fe, std::array<double, FE::dim> const & c,
                      std::vector<int> cmp = {}):
      fn(f[0]), coef(c[0]), feSpace(&fe), fns(f.begin(), f.end()), coefs(c.begin(), c.end()), comps(std::move(cmp))
  {
    if (comps.empty())
      for (int d = 0; d < FE::dim; ++d)
        comps.push_back(d);
    for (int d: comps)
      if (d < 0 || d >= FE::dim)
        throw Error(PXG_ERR_INVALID_ARG, "AssemblyRhsAnalytic: component out of range");
  }
};

// AssemblyS2SProjection / AssemblyProjection(c, field, feSpace, comps)
// (include/assembly_rhs.hpp:93-163).  On a vector space the field holds every
// component (BLOCK ordering), and the j-th listed component (default: all) is projected
// into block j, as the reference's running block index does.
template <typename FE>
struct AssemblyProjection
{
  double coef;
  std::vector<double> const * field;
  FE const * feSpace;
  std::vector<int> comps;
  AssemblyProjection(double c, std::vector<double> const & r, FE const & fe, std::vector<int> cmp = {}):
      coef(c), field(&r), feSpace(&fe), comps(std::move(cmp))
  {
    if (comps.empty())
      for (int d = 0; d < FE::dim; ++d)
        comps.push_back(d);
    for (int d: comps)
      if (d < 0 || d >= FE::dim)
        throw Error(PXG_ERR_INVALID_ARG, "AssemblyProjection: component out of range");
    if ((int64_t)r.size() != FE::dim * fe.dof.size)
      throw Error(PXG_ERR_INVALID_ARG, "AssemblyProjection: the field must hold every component");
  }
};

template <typename FE>
struct AssemblyTensorStiffness
{
  double coef;
  FE const * feSpace;
  AssemblyTensorStiffness(double c, FE const & fe): coef(c), feSpace(&fe) {}
};

// AssemblyGrad(c, vector space, scalar space) (include/assembly_coupling.hpp:42-86)
template <typename FE1, typename FE2>
struct AssemblyGrad
{
  double coef;
  FE1 const * feSpace1;
  FE2 const * feSpace2;
  AssemblyGrad(double c, FE1 const & a, FE2 const & b): coef(c), feSpace1(&a), feSpace2(&b) {}
  static constexpr int kind = PXG_OP_GRAD;
};

// AssemblyDiv(c, scalar space, vector space) (include/assembly_coupling.hpp:89-132)
template <typename FE1, typename FE2>
struct AssemblyDiv
{
  double coef;
  FE1 const * feSpace1;
  FE2 const * feSpace2;
  AssemblyDiv(double c, FE1 const & a, FE2 const & b): coef(c), feSpace1(&a), feSpace2(&b) {}
  static constexpr int kind = PXG_OP_DIV;
};

// The closed matrix on the host, with the parts of Eigen::SparseMatrix's interface that
// proxpde's tests use on builder.A (rows/cols/nonZeros/isCompressed, coeff, A * x,
// norm, block; test/cavitytime.cpp:192, test/solver_test.cpp:74, test/stokes3dhex.cpp:77).
// The storage is compressed rows (outer = row pointers, inner = column indices), where
// Eigen's default is compressed columns: the two coincide for the symmetric matrices of
// the Poisson and Stokes tests, and coeff, operator* and block follow the row-major
// meaning in every case.  ctx is the engine context (GPU) that assembled it.
struct CsrMatrix
{
  int64_t nrows = 0, ncols = 0;
  std::vector<int32_t> outer; // row_ptr
  std::vector<int32_t> inner; // col_idx
  std::vector<double> values;
  pxg_ctx * ctx = nullptr;

  int64_t rows() const { return nrows; }
  int64_t cols() const { return ncols; }
  int64_t nonZeros() const { return (int64_t)values.size(); }
  bool isCompressed() const { return true; }
  int32_t const * outerIndexPtr() const { return outer.data(); }
  int32_t const * innerIndexPtr() const { return inner.data(); }
  double const * valuePtr() const { return values.data(); }
  // entry (i, j), 0 where the pattern has none (columns are sorted within a row)
  double coeff(int64_t i, int64_t j) const
  {
    auto const b0 = inner.begin() + outer[i], b1 = inner.begin() + outer[i + 1];
    auto const it = std::lower_bound(b0, b1, (int32_t)j);
    return (it != b1 && *it == j) ? values[it - inner.begin()] : 0.;
  }
  Vec operator*(Vec const & x) const
  {
    if ((int64_t)x.size() != ncols)
      throw Error(PXG_ERR_INVALID_ARG, "CsrMatrix * Vec: sizes differ");
    Vec y((size_t)nrows, 0.);
    for (int64_t i = 0; i < nrows; ++i)
    {
      double s = 0.;
      for (int32_t k = outer[i]; k < outer[i + 1]; ++k)
        s += values[k] * x[inner[k]];
      y[i] = s;
    }
    return y;
  }
  // the Frobenius norm
  double norm() const
  {
    double s = 0.;
    for (double v: values)
      s += v * v;
    return std::sqrt(s);
  }
  // a copy of rows r0 .. r0 + nr, columns c0 .. c0 + nc
  CsrMatrix block(int64_t r0, int64_t c0, int64_t nr, int64_t nc) const
  {
    if (r0 < 0 || c0 < 0 || r0 + nr > nrows || c0 + nc > ncols)
      throw Error(PXG_ERR_INVALID_ARG, "CsrMatrix::block: out of range");
    CsrMatrix B;
    B.nrows = nr;
    B.ncols = nc;
    B.ctx = ctx;
    B.outer.push_back(0);
    for (int64_t i = r0; i < r0 + nr; ++i)
    {
      for (int32_t k = outer[i]; k < outer[i + 1]; ++k)
        if (inner[k] >= c0 && inner[k] < c0 + nc)
        {
          B.inner.push_back((int32_t)(inner[k] - c0));
          B.values.push_back(values[k]);
        }
      B.outer.push_back((int32_t)B.inner.size());
    }
    return B;
  }
};

// UmfPackLU's interface as the tests use it (include/sparse_matrix.hpp:44:
// analyzePattern, factorize, solve) over the engine's device Jacobi-preconditioned CG
// (pxg_cg): factorize copies the matrix to the GPU that assembled it, and each solve
// runs the CG from x = 0 to the relative residual rtol (1e-14 by default), throwing
// PXG_ERR_NOT_CONVERGED if it stops at maxIter.  The CG needs a symmetric positive
// definite matrix, which a direct LU does not; iterations and relRes report the last
// solve.
struct LUSolver
{
  double rtol = 1e-14;
  int maxIter = 0; // 0: 10 * rows + 1000
  int iterations = 0;
  double relRes = 0.;

  void analyzePattern(CsrMatrix const & A)
  {
    if (!A.ctx || A.rows() != A.cols() || (int64_t)A.outer.size() != A.rows() + 1)
      throw Error(PXG_ERR_INVALID_ARG, "LUSolver: a square matrix closed by a Builder is needed");
    ctx = A.ctx;
    n = A.rows();
  }
  void factorize(CsrMatrix const & A)
  {
    if (A.ctx != ctx || A.rows() != n)
      throw Error(PXG_ERR_INVALID_ARG, "LUSolver: factorize a matrix of the analysed pattern");
    rp = DeviceArray<int32_t>(ctx, A.outer.size());
    ci = DeviceArray<int32_t>(ctx, std::max<size_t>(A.inner.size(), 1));
    va = DeviceArray<double>(ctx, std::max<size_t>(A.values.size(), 1));
    check(pxg_memcpy(ctx, rp.p, A.outer.data(), A.outer.size() * 4, 0, nullptr), ctx, "pxg_memcpy");
    check(pxg_memcpy(ctx, ci.p, A.inner.data(), A.inner.size() * 4, 0, nullptr), ctx, "pxg_memcpy");
    check(pxg_memcpy(ctx, va.p, A.values.data(), A.values.size() * 8, 0, nullptr), ctx, "pxg_memcpy");
  }
  void compute(CsrMatrix const & A)
  {
    analyzePattern(A);
    factorize(A);
  }
  Vec solve(std::vector<double> const & b)
  {
    if (!rp.p || (int64_t)b.size() != n)
      throw Error(PXG_ERR_INVALID_ARG, "LUSolver: factorize first; b must have one value per row");
    DeviceArray<double> bd(ctx, (size_t)n), xd(ctx, (size_t)n);
    check(pxg_memcpy(ctx, bd.p, b.data(), (size_t)n * 8, 0, nullptr), ctx, "pxg_memcpy");
    int const mi = maxIter > 0 ? maxIter : (int)std::min<int64_t>(10 * n + 1000, 1 << 30);
    check(pxg_cg(ctx, rp.p, ci.p, va.p, n, bd.p, xd.p, rtol, mi, &iterations, &relRes, nullptr), ctx, "pxg_cg");
    return Vec(xd.host());
  }

private:
  pxg_ctx * ctx = nullptr;
  int64_t n = 0;
  DeviceArray<int32_t> rp, ci;
  DeviceArray<double> va;
};

template <typename FE, StorageType Storage = StorageType::ClmMajor>
struct Builder
{
  FE & fe;
  DeviceArray<double> vals; // accumulated values on the structural pattern
  DeviceArray<double> bDev;
  CsrMatrix A;
  Vec b;

  explicit Builder(FE & f):
      fe(f), vals(f.ctx, (size_t)f.nnz), bDev(f.ctx, (size_t)f.dof.size), b((size_t)f.dof.size, 0.0)
  {
    vals.zero();
    bDev.zero();
  }

  template <typename... Asm>
  void buildLhs(std::tuple<Asm...> const & assemblies, std::vector<BCEss> const & bcs = {})
  {
    static_assert(sizeof...(Asm) > 0, "we need at least 1 assembly.");
    pxg_lhs_op op{0, 0.0, 0, 0.0, bcs.empty() ? 0 : 1};
    p0 = nullptr;
    std::apply([&](auto const &... a) { (addLhs(op, a), ...); }, assemblies);
    setBcs(bcs);
    check(pxg_assemble(fe.ctx, &op, vals.p, nullptr, nullptr, nullptr, bcs.empty() ? nullptr : bDev.p,
                       PXG_ACCUMULATE, nullptr),
          fe.ctx, "pxg_assemble");
  }

  template <typename... Asm>
  void buildRhs(std::tuple<Asm...> const & assemblies, std::vector<BCEss> const & bcs = {})
  {
    setBcs(bcs);
    std::apply([&](auto const &... a) { (addRhs(a, bcs.empty() ? 0 : 1), ...); }, assemblies);
  }

  // setFromTriplets + prune(1., 1e-16) (builder.hpp:366-371)
  void closeMatrix()
  {
    int64_t const n = fe.dof.size;
    DeviceArray<int32_t> rp(fe.ctx, (size_t)n + 1), ci(fe.ctx, (size_t)fe.nnz);
    DeviceArray<double> vo(fe.ctx, (size_t)fe.nnz);
    int64_t nnz = 0;
    check(pxg_close_matrix(fe.ctx, vals.p, rp.p, ci.p, vo.p, &nnz, nullptr), fe.ctx, "pxg_close_matrix");
    A.nrows = A.ncols = n;
    A.ctx = fe.ctx;
    A.outer = rp.host();
    A.inner = ci.host();
    A.inner.resize((size_t)nnz);
    A.values = vo.host();
    A.values.resize((size_t)nnz);
    b = bDev.host();
    vals.zero(); // the triplets were consumed (builder.hpp:370)
  }

  void clearRhs()
  {
    bDev.zero();
    b.assign(b.size(), 0.0);
  }
  void clearLhs() { vals.zero(); }
  void clear()
  {
    clearLhs();
    clearRhs();
  }

private:
  void setBcs(std::vector<BCEss> const & bcs)
  {
    size_t nm = 0;
    double diag = 1.0;
    for (auto const & bc: bcs)
    {
      nm += bc.marker != side::NONE;
      diag = bc.diag;
    }
    if (nm && nm == bcs.size())
    {
      // on the device: the marked facets' DOFs, constant values (later ones win)
      std::vector<int32_t> m, f;
      std::vector<double> c;
      for (auto const & bc: bcs)
      {
        m.push_back(bc.marker);
        f.push_back(PXG_FN_CONST);
        c.push_back(bc.value);
      }
      check(pxg_set_bc_markers(fe.ctx, m.data(), f.data(), c.data(), (int)m.size(), diag), fe.ctx,
            "pxg_set_bc_markers");
      return;
    }
    std::vector<uint32_t> d;
    std::vector<double> v;
    for (auto const & bc: bcs)
    {
      d.insert(d.end(), bc.dofs.begin(), bc.dofs.end());
      v.insert(v.end(), bc.values.begin(), bc.values.end());
    }
    check(pxg_set_bc(fe.ctx, d.data(), v.data(), (int64_t)d.size(), diag, PXG_MEM_HOST), fe.ctx, "pxg_set_bc");
  }

  template <typename X>
  void addLhs(pxg_lhs_op & op, AssemblyStiffness<X> const & a)
  {
    op.stiffness = 1;
    op.stiff_coef = a.coef;
  }
  // the per-element coefficient of the current buildLhs call
  std::vector<double> const * p0 = nullptr;
  void setP0(std::vector<double> const & k)
  {
    if (p0 && p0 != &k && *p0 != k)
      throw Error(PXG_ERR_UNSUPPORTED, "the per-element coefficients of one buildLhs call must be the same");
    if ((int64_t)k.size() != fe.nelem)
      throw Error(PXG_ERR_INVALID_ARG, "a per-element coefficient needs one value per element");
    p0 = &k;
    check(pxg_set_coef(fe.ctx, k.data(), PXG_MEM_HOST, nullptr), fe.ctx, "pxg_set_coef");
  }
  template <typename X>
  void addLhs(pxg_lhs_op & op, AssemblyStiffnessFE<X> const & a)
  {
    setP0(*a.coefP0);
    op.stiffness = 2;
    op.stiff_coef = 1.0;
  }
  template <typename X>
  void addLhs(pxg_lhs_op & op, AssemblyMassFE<X> const & a)
  {
    setP0(*a.coefP0);
    op.mass = 2;
    op.mass_coef = 1.0;
  }
  template <typename X>
  void addLhs(pxg_lhs_op & op, AssemblyScalarMass<X> const & a)
  {
    op.mass = 1;
    op.mass_coef = a.coef;
  }

  template <typename X>
  void addRhs(AssemblyRhsAnalytic<X> const & a, int bc)
  {
    if (!a.qvals.empty())
    {
      // a host function: its values at the quadrature points, integrated on the device
      DeviceArray<double> f(fe.ctx, a.qvals[0].size());
      check(pxg_memcpy(fe.ctx, f.p, a.qvals[0].data(), f.n * sizeof(double), 0, nullptr), fe.ctx, "pxg_memcpy");
      pxg_rhs_op r{3, 0, a.coef, f.p, bc};
      check(pxg_assemble(fe.ctx, nullptr, nullptr, nullptr, nullptr, &r, bDev.p, PXG_ACCUMULATE, nullptr), fe.ctx,
            "pxg_assemble");
      return; // f is released here; freeing device memory waits for the assembly that reads it
    }
    pxg_rhs_op r{1, a.fn, a.coef, nullptr, bc};
    check(pxg_assemble(fe.ctx, nullptr, nullptr, nullptr, nullptr, &r, bDev.p, PXG_ACCUMULATE, nullptr), fe.ctx,
          "pxg_assemble");
  }
  template <typename X>
  void addRhs(AssemblyProjection<X> const & a, int bc)
  {
    DeviceArray<double> f(fe.ctx, a.field->size());
    check(pxg_memcpy(fe.ctx, f.p, a.field->data(), f.n * sizeof(double), 0, nullptr), fe.ctx, "pxg_memcpy");
    pxg_rhs_op r{2, 0, a.coef, f.p, bc};
    check(pxg_assemble(fe.ctx, nullptr, nullptr, nullptr, nullptr, &r, bDev.p, PXG_ACCUMULATE, nullptr), fe.ctx,
          "pxg_assemble");
    // f is released here; freeing device memory waits for the assembly that reads it
  }
};

template <typename FE, std::enable_if_t<!std::is_arithmetic_v<std::remove_cv_t<FE>>, int> = 0>
Builder(FE &) -> Builder<FE, StorageType::ClmMajor>;

// Builder{numDOFs} over spaces with offsets (vector spaces, buildCoupling): the calls
// are recorded and run on a device system (pxg_sys) by closeMatrix, when all the
// spaces are known.
template <StorageType Storage>
struct Builder<void, Storage>
{
  int64_t size;
  CsrMatrix A;
  Vec b;

  explicit Builder(int64_t n): size(n), b((size_t)n, 0.0) {}

  template <typename... Asm>
  void buildLhs(std::tuple<Asm...> const & assemblies, std::vector<BCEss> const & bcs = {})
  {
    static_assert(sizeof...(Asm) > 0, "we need at least 1 assembly.");
    Call c;
    std::apply([&](auto const &... a) { (addSquare(c, a), ...); }, assemblies);
    c.col = c.row;
    c.bcRow = c.bcCol = bcs;
    calls.push_back(std::move(c));
  }

  template <typename Asm>
  void buildCoupling(Asm const & a, std::vector<BCEss> const & bcsRow, std::vector<BCEss> const & bcsCol)
  {
    Call c;
    c.row = spaceOf(*a.feSpace1);
    c.col = spaceOf(*a.feSpace2);
    c.kinds.push_back(Asm::kind);
    c.coefs.push_back(a.coef);
    c.bcRow = bcsRow;
    c.bcCol = bcsCol;
    calls.push_back(std::move(c));
  }

  // buildRhs (builder.hpp:279-364) on one space of the system, scalar or vector: the
  // loads are recorded and added to b by closeMatrix.  Block c of a vector space's
  // load is condensed with the DOFs constrained in component c.
  template <typename... Asm>
  void buildRhs(std::tuple<Asm...> const & assemblies, std::vector<BCEss> const & bcs = {})
  {
    static_assert(sizeof...(Asm) > 0, "we need at least 1 assembly.");
    std::apply([&](auto const &... a) { (addRhsCall(a, bcs), ...); }, assemblies);
  }

  // setFromTriplets + prune(1., 1e-16) (builder.hpp:366-371) over the recorded calls
  void closeMatrix()
  {
    std::vector<int> order(spaces.size());
    for (size_t k = 0; k < order.size(); ++k)
      order[k] = (int)k;
    std::sort(order.begin(), order.end(), [&](int x, int y) { return spaces[x].offset < spaces[y].offset; });
    std::vector<pxg_ctx *> ctxs;
    std::vector<int> dims, qrs, slot(spaces.size());
    int64_t off = 0;
    for (size_t k = 0; k < order.size(); ++k)
    {
      Space const & sp = spaces[order[k]];
      if (sp.offset != off)
        throw Error(PXG_ERR_INVALID_ARG, "Builder: the spaces' offsets do not tile the system");
      off += sp.ndof * sp.dim;
      ctxs.push_back(sp.ctx);
      dims.push_back(sp.dim);
      qrs.push_back(sp.qr);
      slot[order[k]] = (int)k;
    }
    if (off != size)
      throw Error(PXG_ERR_INVALID_ARG, "Builder: size differs from the spaces' DOFs");
    pxg_ctx * c0 = ctxs[0];
    pxg_sys * S = nullptr;
    int64_t ntot = 0, nnz = 0;
    check(pxg_sys_create(&S, ctxs.data(), dims.data(), qrs.data(), (int)ctxs.size(), &ntot, &nnz), c0,
          "pxg_sys_create");
    struct Guard
    {
      pxg_sys * s;
      ~Guard() { pxg_sys_destroy(s); }
    } guard{S};
    DeviceArray<double> vals(c0, (size_t)nnz), bd(c0, (size_t)ntot);
    vals.zero();
    bd.zero();
    auto setBcs = [&](int s, std::vector<BCEss> const & bcs) {
      std::vector<uint32_t> d;
      std::vector<double> v;
      double diag = 1.0;
      for (auto const & bc: bcs)
      {
        d.insert(d.end(), bc.dofs.begin(), bc.dofs.end());
        v.insert(v.end(), bc.values.begin(), bc.values.end());
        diag = bc.diag;
      }
      check(pxg_sys_set_bc(S, s, d.data(), v.data(), (int64_t)d.size(), diag), c0, "pxg_sys_set_bc");
    };
    for (auto const & c: calls)
    {
      setBcs(slot[c.row], c.bcRow);
      if (c.col != c.row)
        setBcs(slot[c.col], c.bcCol);
      check(pxg_sys_assemble(S, slot[c.row], slot[c.col], c.kinds.data(), c.coefs.data(), (int)c.kinds.size(),
                             vals.p, bd.p, PXG_ACCUMULATE, nullptr),
            c0, "pxg_sys_assemble");
    }
    for (auto const & r: rhsCalls)
    {
      Space const & sp = spaces[r.space];
      for (auto const & part: r.parts)
      {
        // the constrained DOFs of component part.block, as the space's own DOF ids
        std::vector<uint32_t> d;
        std::vector<double> v;
        double diag = 1.0;
        int64_t const lo = part.block * sp.ndof;
        for (auto const & bc: r.bcs)
        {
          for (size_t k = 0; k < bc.dofs.size(); ++k)
            if ((int64_t)bc.dofs[k] >= lo && (int64_t)bc.dofs[k] < lo + sp.ndof)
            {
              d.push_back((uint32_t)(bc.dofs[k] - lo));
              v.push_back(bc.values[k]);
            }
          diag = bc.diag;
        }
        check(pxg_set_bc(sp.ctx, d.data(), v.data(), (int64_t)d.size(), diag, PXG_MEM_HOST), sp.ctx, "pxg_set_bc");
        DeviceArray<double> f;
        if (part.kind == 3)
        {
          f = DeviceArray<double>(sp.ctx, part.qvals.size());
          check(pxg_memcpy(sp.ctx, f.p, part.qvals.data(), part.qvals.size() * sizeof(double), 0, nullptr), sp.ctx,
                "pxg_memcpy");
        }
        else if (part.field)
        {
          f = DeviceArray<double>(sp.ctx, (size_t)sp.ndof);
          check(pxg_memcpy(sp.ctx, f.p, part.field + (size_t)part.fieldComp * sp.ndof, (size_t)sp.ndof * sizeof(double),
                           0, nullptr),
                sp.ctx, "pxg_memcpy");
        }
        pxg_rhs_op op{part.kind, part.fn, part.coef, f.p, r.bcs.empty() ? 0 : 1};
        check(pxg_assemble(sp.ctx, nullptr, nullptr, nullptr, nullptr, &op, bd.p + sp.offset + lo, PXG_ACCUMULATE,
                           nullptr),
              sp.ctx, "pxg_assemble");
        // f is released here; freeing device memory waits for the assembly that reads it
      }
    }
    DeviceArray<int32_t> rpo(c0, (size_t)ntot + 1), cio(c0, (size_t)nnz);
    DeviceArray<double> vo(c0, (size_t)nnz);
    int64_t kept = 0;
    check(pxg_sys_close_matrix(S, vals.p, rpo.p, cio.p, vo.p, &kept, nullptr), c0, "pxg_sys_close_matrix");
    A.nrows = A.ncols = ntot;
    A.ctx = c0;
    A.outer = rpo.host();
    A.inner = cio.host();
    A.inner.resize((size_t)kept);
    A.values = vo.host();
    A.values.resize((size_t)kept);
    b = bd.host();
    calls.clear(); // the triplets were consumed (builder.hpp:370)
    rhsCalls.clear();
  }

private:
  struct Space
  {
    pxg_ctx * ctx;
    int dim, qr;
    int64_t offset, ndof;
  };
  struct Call
  {
    int row = -1, col = -1;
    std::vector<int> kinds;
    std::vector<double> coefs;
    std::vector<BCEss> bcRow, bcCol;
  };
  struct RhsPart
  {
    int block, kind, fn;
    double coef;
    double const * field; // projection: the whole field on the host, else null
    int fieldComp;
    std::vector<double> qvals; // kind 3: a copy of the values at the quadrature points
  };
  struct RhsCall
  {
    int space;
    std::vector<RhsPart> parts;
    std::vector<BCEss> bcs;
  };
  std::vector<Space> spaces;
  std::vector<Call> calls;
  std::vector<RhsCall> rhsCalls;

  template <typename FE>
  static void checkRule()
  {
    // the element kernels integrate loads with the element's own rule
    if (FE::qrType != FE::elemType)
      throw Error(PXG_ERR_UNSUPPORTED, "buildRhs on a space with another quadrature rule");
  }
  template <typename X>
  void addRhsCall(AssemblyRhsAnalytic<X> const & a, std::vector<BCEss> const & bcs)
  {
    checkRule<X>();
    RhsCall r{spaceOf(*a.feSpace), {}, bcs};
    // the calls run at closeMatrix: the parts keep what they need (the assembly object
    // may be a temporary of the buildRhs call)
    for (int c: a.comps)
      if (a.qvals.empty())
        r.parts.push_back(RhsPart{c, 1, a.fns[(size_t)c], a.coefs[(size_t)c], nullptr, 0, {}});
      else
        r.parts.push_back(RhsPart{c, 3, 0, a.coefs[(size_t)c], nullptr, c, a.qvals[(size_t)c]});
    rhsCalls.push_back(std::move(r));
  }
  template <typename X>
  void addRhsCall(AssemblyProjection<X> const & a, std::vector<BCEss> const & bcs)
  {
    checkRule<X>();
    RhsCall r{spaceOf(*a.feSpace), {}, bcs};
    for (size_t j = 0; j < a.comps.size(); ++j)
      r.parts.push_back(RhsPart{(int)j, 2, 0, a.coef, a.field->data(), a.comps[j], {}});
    rhsCalls.push_back(std::move(r));
  }

  template <typename FE>
  int spaceOf(FE const & fe)
  {
    for (size_t k = 0; k < spaces.size(); ++k)
      if (spaces[k].ctx == fe.ctx)
        return (int)k;
    spaces.push_back(Space{fe.ctx, FE::dim, FE::qrType, fe.offset, fe.dof.size});
    return (int)spaces.size() - 1;
  }
  template <typename FE>
  void setRow(Call & c, FE const & fe)
  {
    int const s = spaceOf(fe);
    if (c.row >= 0 && c.row != s)
      throw Error(PXG_ERR_INVALID_ARG, "buildLhs: the assemblies of one call share one space");
    c.row = s;
  }
  template <typename X>
  void addSquare(Call & c, AssemblyStiffness<X> const & a)
  {
    setRow(c, *a.feSpace);
    c.kinds.push_back(PXG_OP_STIFFNESS);
    c.coefs.push_back(a.coef);
  }
  template <typename X>
  void addSquare(Call & c, AssemblyTensorStiffness<X> const & a)
  {
    setRow(c, *a.feSpace);
    c.kinds.push_back(PXG_OP_TENSOR_STIFFNESS);
    c.coefs.push_back(a.coef);
  }
  template <typename X>
  void addSquare(Call & c, AssemblyScalarMass<X> const & a)
  {
    setRow(c, *a.feSpace);
    c.kinds.push_back(PXG_OP_MASS);
    c.coefs.push_back(a.coef);
  }
};

template <typename I, std::enable_if_t<std::is_integral_v<I>, int> = 0>
Builder(I) -> Builder<void, StorageType::ClmMajor>;

} // namespace proxgpu
