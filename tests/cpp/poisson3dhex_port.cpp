// proxpde's test/poisson3dhex.cpp (lines 18-104) on the proxgpu shim with the namespace
// changed: the same mesh, space, boundary conditions (BCEss << lambda), Builder{size},
// the host-lambda right-hand side, LUSolver, interpolateAnalyticFunction of a lambda
// and checkError against the golden norm.  What the port leaves out is outside the
// assembly path: the YAML configuration (n is an argument), MilliTimer and the
// XDMF/HDF5 output.
//
//   poisson3dhex_port <n> <expected error>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <memory>

#include "proxgpu/builder.hpp"

using namespace proxgpu;

int test(uint n, double expected)
{
  using Elem_T = Hexahedron;
  using Mesh_T = Mesh<Elem_T>;
  using FESpace_T = FESpace<Mesh_T, LagrangeFE<Elem_T, 1>::RefFE_T, LagrangeFE<Elem_T, 1>::RecommendedQR>;

  scalarFun_T const rhs = [](Vec3 const & p)
  { return 2.5 * M_PI * M_PI * std::sin(0.5 * M_PI * p(0)) * std::sin(1.5 * M_PI * p(1)); };

  scalarFun_T const exactSol = [](Vec3 const & p)
  { return std::sin(0.5 * M_PI * p(0)) * std::sin(1.5 * M_PI * p(1)); };

  std::unique_ptr<Mesh_T> mesh{new Mesh_T};
  buildHyperCube(*mesh, {0., 0., 0.}, {1., 1., 1.}, {n, n, n});

  FESpace_T feSpace{*mesh};

  auto bcLeft = BCEss{feSpace, side::LEFT};
  bcLeft << [](Vec3 const &) { return 0.; };
  auto bcBottom = BCEss{feSpace, side::BOTTOM};
  bcBottom << [](Vec3 const &) { return 0.; };
  auto const bcs = std::vector{bcLeft, bcBottom};

  Builder builder{feSpace.dof.size};
  builder.buildLhs(std::tuple{AssemblyStiffness(1.0, feSpace)}, bcs);
  builder.buildRhs(std::tuple{AssemblyRhsAnalytic(rhs, feSpace)}, bcs);
  builder.closeMatrix();

  Var sol{"u"};
  LUSolver solver;
  solver.analyzePattern(builder.A);
  solver.factorize(builder.A);
  sol.data = solver.solve(builder.b);

  Var exact{"exact"};
  interpolateAnalyticFunction(exactSol, feSpace, exact.data);
  Var error{"e"};
  error.data = sol.data - exact.data;

  double norm = error.data.norm();
  std::printf("cg iterations %d, relative residual %.3e\n", solver.iterations, solver.relRes);

  // the residual of the solution with the closed matrix, as test/cavitytime.cpp:192 forms it
  Vec const res = builder.A * sol.data - builder.b;
  std::printf("host residual %.3e (A: %lld x %lld, %lld nonzeros, compressed %d, A(0,0) = %.6f)\n",
              res.norm() / builder.b.norm(), (long long)builder.A.rows(), (long long)builder.A.cols(),
              (long long)builder.A.nonZeros(), (int)builder.A.isCompressed(), builder.A.coeff(0, 0));
  if (!(res.norm() <= 1e-12 * builder.b.norm()) || builder.A.block(0, 0, 2, 2).nonZeros() < 1)
    return 4;

  return checkError({norm}, {expected});
}

int main(int argc, char ** argv)
{
  if (argc < 3)
  {
    std::fprintf(stderr, "usage: poisson3dhex_port <n> <expected error>\n");
    return 2;
  }
  try
  {
    return test((uint)std::atoi(argv[1]), std::atof(argv[2]));
  }
  catch (proxgpu::Error const & e)
  {
    std::fprintf(stderr, "proxgpu error: %s\n", e.what());
    return 3;
  }
}
