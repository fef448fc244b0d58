// proxpde's poisson3dhex / poisson3dhex_q2 tests (test/poisson3dhex.cpp:18-75,
// test/poisson3dhex_q2.cpp:18-80) written against the proxgpu drop-in shim: the same
// call sequence, assembled by the GB300 engine.  Writes the closed matrix, the load
// vector and the interpolated exact solution to a binary file; the solve and the
// golden-norm check are done by the pytest wrapper.
//
//   poisson3d <order 1|2> <n> <output file>
#include <cstdio>
#include <cstdlib>

#include "proxgpu/builder.hpp"

template <int Order>
int run(int n, char const * out)
{
  using namespace proxgpu;
  using Mesh_T = Mesh<Hexahedron>;
  using FESpace_T =
      FESpace<Mesh_T, typename LagrangeFE<Hexahedron, Order>::RefFE_T, typename LagrangeFE<Hexahedron, Order>::RecommendedQR>;
  auto const mesh = buildHyperCube<Hexahedron>(n);
  FESpace_T feSpace{mesh};
  auto const bcs = std::vector{BCEss{feSpace, side::LEFT}, BCEss{feSpace, side::BOTTOM}};
  Builder builder{feSpace};
  builder.buildLhs(std::tuple{AssemblyStiffness(1.0, feSpace)}, bcs);
  builder.buildRhs(std::tuple{AssemblyRhsAnalytic(PXG_FN_POISSON_RHS, feSpace)}, bcs);
  builder.closeMatrix();
  auto const exact = feSpace.interpolate(PXG_FN_POISSON_EXACT);

  FILE * f = std::fopen(out, "wb");
  if (!f)
    return 2;
  int64_t const hdr[2] = {builder.A.rows(), builder.A.nonZeros()};
  std::fwrite(hdr, sizeof(hdr), 1, f);
  std::fwrite(builder.A.outer.data(), 4, builder.A.outer.size(), f);
  std::fwrite(builder.A.inner.data(), 4, builder.A.inner.size(), f);
  std::fwrite(builder.A.values.data(), 8, builder.A.values.size(), f);
  std::fwrite(builder.b.data(), 8, builder.b.size(), f);
  std::fwrite(exact.data(), 8, exact.size(), f);
  std::fclose(f);
  return 0;
}

int main(int argc, char ** argv)
{
  if (argc < 4)
  {
    std::fprintf(stderr, "usage: poisson3d <order 1|2> <n> <output>\n");
    return 2;
  }
  int const order = std::atoi(argv[1]), n = std::atoi(argv[2]);
  try
  {
    return order == 1 ? run<1>(n, argv[3]) : run<2>(n, argv[3]);
  }
  catch (proxgpu::Error const & e)
  {
    std::fprintf(stderr, "proxgpu error: %s\n", e.what());
    return 1;
  }
}
