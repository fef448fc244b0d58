// Loads on a vector space through the proxgpu shim's Builder{numDOFs}: on the unit
// cube (3^3 cells), a 3-component P2 / Q2 space and a P1 / Q1 space behind it.
// buildRhs takes AssemblyRhsAnalytic with one device function and one coefficient per
// component on components 0 and 2, and the projection of a vector field's components
// (2, 0) into blocks (0, 1), under BCEss on the bottom (every component) and the left
// (components 0 and 2); the scalar space gets a constant load without BCs
// (include/assembly_rhs.hpp:34-163, include/builder.hpp:279-364).  Writes b to a binary
// file; the pytest wrapper compares it with the oracle block by block.
//
//   vector_loads <hex|tet> <output>
#include <cmath>
#include <cstdio>
#include <string>

#include "proxgpu/builder.hpp"

using namespace proxgpu;

template <typename Elem_T>
int run(char const * out)
{
  using Mesh_T = Mesh<Elem_T>;
  auto const mesh = buildHyperCube<Elem_T>(3);
  FESpace<Mesh_T, typename LagrangeFE<Elem_T, 2>::RefFE_T, typename LagrangeFE<Elem_T, 2>::RecommendedQR, 3> feSpaceVel{mesh};
  FESpace<Mesh_T, typename LagrangeFE<Elem_T, 1>::RefFE_T, typename LagrangeFE<Elem_T, 1>::RecommendedQR> feSpaceP{
      mesh, 3 * feSpaceVel.dof.size};
  auto const dofU = feSpaceVel.dof.size;
  auto const dofP = feSpaceP.dof.size;

  auto const one = [](Vec3 const &) { return Vec3::Constant(1.); };
  auto const zero = [](Vec3 const &) { return Vec3::Constant(0.); };
  auto const bcsVel = std::vector{
      BCEss{feSpaceVel, side::BOTTOM, one},
      BCEss{feSpaceVel, side::LEFT, zero, {0, 2}},
  };
  std::vector<double> field((size_t)(3 * dofU));
  for (size_t k = 0; k < field.size(); ++k)
    field[k] = std::sin(0.37 * (double)k) + 0.1 * (double)(k % 7);

  Builder builder{3 * dofU + dofP};
  builder.buildLhs(std::tuple{AssemblyScalarMass{1.0, feSpaceVel}});
  builder.buildRhs(
      std::tuple{
          AssemblyRhsAnalytic{std::array<int, 3>{PXG_FN_SIN3, PXG_FN_CONST, PXG_FN_POISSON_RHS}, feSpaceVel,
                              std::array{1.0, 2.0, -0.5}, {0, 2}},
          AssemblyProjection{0.7, field, feSpaceVel, {2, 0}},
      },
      bcsVel);
  builder.buildRhs(std::tuple{AssemblyRhsAnalytic{PXG_FN_CONST, feSpaceP, 3.0}});
  builder.closeMatrix();

  FILE * f = std::fopen(out, "wb");
  if (!f)
    return 1;
  int64_t const hdr[3] = {(int64_t)builder.b.size(), dofU, dofP};
  std::fwrite(hdr, 8, 3, f);
  std::fwrite(builder.b.data(), 8, builder.b.size(), f);
  std::fclose(f);
  return 0;
}

int main(int argc, char * argv[])
{
  if (argc < 3)
  {
    std::fprintf(stderr, "usage: vector_loads <hex|tet> <output>\n");
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
