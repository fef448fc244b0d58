// proxgpu/builder.hpp — header-only C++20 drop-in for proxpde's assembly call surface,
// running on the GB300 engine through its C ABI (include/pxg.h, libpxg.so).
//
// The names and the call sequence follow proxpde (include/builder.hpp:12-391 and the
// Assembly* types of include/assembly_lhs.hpp / assembly_rhs.hpp):
//
//   auto mesh = proxgpu::buildHyperCube<proxgpu::Hexahedron>(n);       // mesh.hpp:385-421
//   proxgpu::FESpace<proxgpu::Hexahedron, 1> feSpace{mesh};            // fespace.hpp:27-193
//   auto bcs = std::vector{proxgpu::BCEss{feSpace, proxgpu::side::LEFT},
//                          proxgpu::BCEss{feSpace, proxgpu::side::BOTTOM}};
//   proxgpu::Builder builder{feSpace};                                 // builder.hpp:19
//   builder.buildLhs(std::tuple{proxgpu::AssemblyStiffness(1.0, feSpace)}, bcs);
//   builder.buildRhs(std::tuple{proxgpu::AssemblyRhsAnalytic(PXG_FN_POISSON_RHS, feSpace)}, bcs);
//   builder.closeMatrix();
//   builder.A (CSR arrays on the host), builder.b
//
// Differences from proxpde, all forced by running on a GPU:
//  - right-hand sides are device functions chosen by id (pxg_fn) instead of a host
//    std::function; unrecognised assembly types do not compile (no CPU fallback);
//  - A is returned as CSR arrays; proxpde's default ClmMajor storage is CSC, and for
//    the symmetric matrices assembled here the CSC arrays are the same arrays;
//  - errors throw proxgpu::Error (carrying the pxg_status) instead of aborting.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
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

template <typename Elem>
struct Mesh
{
  std::vector<double> xyz;     // nnodes x 3
  std::vector<uint32_t> conn;  // nelem x numPts, proxpde's local vertex order
  int64_t nnodes() const { return (int64_t)xyz.size() / 3; }
  int64_t nelem() const { return (int64_t)conn.size() / Elem::numPts; }
};

// buildCube on [0,1]^3 with n^3 cubes (src/mesh.cpp:355-534): hexahedra, or 5
// tetrahedra per cube alternating with the parity of (i + j + k).
template <typename Elem>
Mesh<Elem> buildHyperCube(int n)
{
  Mesh<Elem> m;
  int const np = n + 1;
  double const h = 1.0 / n;
  m.xyz.resize((size_t)np * np * np * 3);
  for (int k = 0; k < np; ++k)
    for (int j = 0; j < np; ++j)
      for (int i = 0; i < np; ++i)
      {
        size_t const id = i + (size_t)np * j + (size_t)np * np * k;
        m.xyz[3 * id] = 0. + i * h;
        m.xyz[3 * id + 1] = 0. + j * h;
        m.xyz[3 * id + 2] = 0. + k * h;
      }
  uint32_t const dx = 1, dy = np, dz = np * np;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
      {
        uint32_t const b = i + j * np + k * np * np;
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
  return m;
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

// FESpace<Mesh, LagrangeFE<Elem, Order>::RefFE_T, RecommendedQR> on the device: the
// mesh, the first-touch DOF map and the CSR pattern live in one engine context.
template <typename Elem, int Order>
struct FESpace
{
  static constexpr int elemType =
      std::is_same_v<Elem, Tetrahedron> ? (Order == 1 ? PXG_P1TET : PXG_P2TET) : (Order == 1 ? PXG_Q1HEX : PXG_Q2HEX);
  pxg_ctx * ctx = nullptr;
  struct
  {
    int64_t size = 0;
  } dof;
  int64_t nnz = 0;

  explicit FESpace(Mesh<Elem> const & m, int device = 0)
  {
    check(pxg_create(&ctx, device), nullptr, "pxg_create");
    check(pxg_set_mesh(ctx, elemType, m.xyz.data(), m.nnodes(), m.conn.data(), m.nelem(), PXG_MEM_HOST), ctx,
          "pxg_set_mesh");
    check(pxg_build_dofmap(ctx, &dof.size), ctx, "pxg_build_dofmap");
    check(pxg_build_pattern(ctx, &nnz), ctx, "pxg_build_pattern");
    // boundary facets marked on the planes of the bounding box, as markFacetsCube does
    // for buildHyperCube (include/mesh.hpp:443-481)
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (size_t k = 0; k < m.xyz.size(); ++k)
    {
      lo[k % 3] = std::min(lo[k % 3], m.xyz[k]);
      hi[k % 3] = std::max(hi[k % 3], m.xyz[k]);
    }
    double const len[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    check(pxg_mark_facets_box(ctx, lo, len), ctx, "pxg_mark_facets_box");
  }
  FESpace(FESpace const &) = delete;
  FESpace & operator=(FESpace const &) = delete;
  ~FESpace()
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
};

// BCEss{feSpace, marker, value} (include/bc.hpp:81-97): the DOFs of the boundary facets
// with that marker, set up on the device (pxg_set_bc_markers); or an explicit DOF list.
struct BCEss
{
  int marker = side::NONE; // NONE: the explicit list below
  double value = 0.0;
  std::vector<uint32_t> dofs;
  std::vector<double> values;
  double diag = 1.0; // BCEss::diag (bc.hpp:301)

  template <typename FE>
  BCEss(FE const &, int m, double v = 0.0): marker(m), value(v)
  {
    if (m < side::BOTTOM || m > side::FRONT)
      throw Error(PXG_ERR_INVALID_ARG, "BCEss: unknown side marker");
  }
  BCEss(std::vector<uint32_t> d, std::vector<double> v): dofs(std::move(d)), values(std::move(v)) {}
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

template <typename FE>
struct AssemblyRhsAnalytic
{
  int fn;
  double coef;
  FE const * feSpace;
  AssemblyRhsAnalytic(int f, FE const & fe, double c = 1.0): fn(f), coef(c), feSpace(&fe) {}
};

template <typename FE>
struct AssemblyProjection
{
  double coef;
  std::vector<double> const * field;
  FE const * feSpace;
  AssemblyProjection(double c, std::vector<double> const & r, FE const & fe): coef(c), field(&r), feSpace(&fe) {}
};

// CSR matrix on the host
struct CsrMatrix
{
  int64_t rows = 0, cols = 0;
  std::vector<int32_t> outer; // row_ptr
  std::vector<int32_t> inner; // col_idx
  std::vector<double> values;
  int64_t nonZeros() const { return (int64_t)values.size(); }
};

template <typename FE, StorageType Storage = StorageType::ClmMajor>
struct Builder
{
  FE & fe;
  DeviceArray<double> vals; // accumulated values on the structural pattern
  DeviceArray<double> bDev;
  CsrMatrix A;
  std::vector<double> b;

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
    A.rows = A.cols = n;
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
    if (nm && nm != bcs.size())
      throw Error(PXG_ERR_UNSUPPORTED, "BCEss: marker and DOF-list conditions in one call");
    if (nm)
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
  template <typename X>
  void addLhs(pxg_lhs_op & op, AssemblyStiffnessFE<X> const & a)
  {
    check(pxg_set_coef(fe.ctx, a.coefP0->data(), PXG_MEM_HOST, nullptr), fe.ctx, "pxg_set_coef");
    op.stiffness = 2;
    op.stiff_coef = 1.0;
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

template <typename FE>
Builder(FE &) -> Builder<FE, StorageType::ClmMajor>;

} // namespace proxgpu
