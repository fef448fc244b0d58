// proxpde's test/stokes3dhex.cpp and test/stokes3dtet.cpp on the proxgpu shim: the
// Taylor-Hood Stokes problem (Poiseuille inflow in the box [0,1] x [0,2] x [0,1],
// 4^3 cells) assembled on the device through Builder{numDOFs}, buildLhs and
// buildCoupling.  The closed matrix, b and the interpolated exact solution go to a
// binary file; the solve and the error norms are done by the test harness.
#include <cstdio>
#include <string>

#include "proxgpu/builder.hpp"

using namespace proxgpu;

template <typename Elem_T>
int run(char const * out)
{
  double const ly = 2.;
  using Mesh_T = Mesh<Elem_T>;
  using QR = typename LagrangeFE<Elem_T, 2>::RecommendedQR;
  Mesh_T mesh;
  buildHyperCube(mesh, {0., 0., 0.}, {1., ly, 1.}, {4, 4, 4});
  FESpace<Mesh_T, typename LagrangeFE<Elem_T, 2>::RefFE_T, QR, 3> feSpaceVel{mesh};
  FESpace<Mesh_T, typename LagrangeFE<Elem_T, 1>::RefFE_T, QR> feSpaceP{mesh, 3 * feSpaceVel.dof.size};

  auto const zero = [](Vec3 const &) { return Vec3::Constant(0.); };
  auto const inlet = [](Vec3 const & p) { return Vec3(0., 0.5 * (1. - p(0) * p(0)), 0.); };
  auto const bcsVel = std::vector{
      BCEss{feSpaceVel, side::BOTTOM, inlet},
      BCEss{feSpaceVel, side::RIGHT, zero},
      BCEss{feSpaceVel, side::TOP, zero, {0, 2}},
      BCEss{feSpaceVel, side::LEFT, zero, {0, 2}},
      BCEss{feSpaceVel, side::BACK, zero, {2}},
      BCEss{feSpaceVel, side::FRONT, zero, {2}},
  };
  auto const bcsP = std::vector<BCEss>{};

  auto const dofU = feSpaceVel.dof.size;
  auto const dofP = feSpaceP.dof.size;
  int64_t const numDOFs = 3 * dofU + dofP;
  Builder builder{numDOFs};
  double const nu = 0.1;
  builder.buildLhs(std::tuple{AssemblyTensorStiffness{nu, feSpaceVel}}, bcsVel);
  builder.buildCoupling(AssemblyGrad{-1.0, feSpaceVel, feSpaceP}, bcsVel, bcsP);
  builder.buildCoupling(AssemblyDiv{-1.0, feSpaceP, feSpaceVel}, bcsP, bcsVel);
  builder.closeMatrix();

  // exact solution: inlet profile on the velocity DOFs, nu (ly - y) on the pressure's
  std::vector<double> ex((size_t)numDOFs, 0.);
  auto const xv = feSpaceVel.interpolate(PXG_FN_COORD_X);
  for (int64_t k = 0; k < dofU; ++k)
    ex[(size_t)(dofU + k)] = inlet(Vec3(xv[(size_t)k], 0., 0.))(1);
  auto const yp = feSpaceP.interpolate(PXG_FN_COORD_Y);
  for (int64_t k = 0; k < dofP; ++k)
    ex[(size_t)(3 * dofU + k)] = nu * (ly - yp[(size_t)k]);

  FILE * f = std::fopen(out, "wb");
  if (!f)
    return 1;
  int64_t const hdr[3] = {builder.A.rows(), builder.A.nonZeros(), dofU};
  std::fwrite(hdr, 8, 3, f);
  std::fwrite(builder.A.outer.data(), 4, builder.A.outer.size(), f);
  std::fwrite(builder.A.inner.data(), 4, builder.A.inner.size(), f);
  std::fwrite(builder.A.values.data(), 8, builder.A.values.size(), f);
  std::fwrite(builder.b.data(), 8, builder.b.size(), f);
  std::fwrite(ex.data(), 8, ex.size(), f);
  std::fclose(f);
  return 0;
}

int main(int argc, char * argv[])
{
  if (argc < 3)
  {
    std::fprintf(stderr, "usage: stokes3d <hex|tet> <output>\n");
    return 2;
  }
  try
  {
    return std::string(argv[1]) == "hex" ? run<Hexahedron>(argv[2]) : run<Tetrahedron>(argv[2]);
  }
  catch (Error const & e)
  {
    std::fprintf(stderr, "proxgpu error: %s\n", e.what());
    return 1;
  }
}
