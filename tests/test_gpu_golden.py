"""proxpde's golden tests run end to end on the GPU engine through the Builder mirror:
assemble on the device, solve with the mirror's LUSolver (UmfPackLU's interface over the
device CG, to a relative residual of 1e-14), compare ||u - I_h u_exact||_2 with the
pinned value (tolerance 1e-12, include/def.hpp:357-385).  A scipy direct solve of the
same system is the cross-check; the Stokes systems are indefinite, which the CG does
not take, and are solved by scipy."""
import os

import numpy as np
import pytest
import scipy.sparse.linalg as spla

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def poisson_rhs(p):
    """The reference's rhs lambda (test/poisson3dhex.cpp:25-30), on the host."""
    return 2.5 * np.pi ** 2 * np.sin(0.5 * np.pi * p[:, 0]) * np.sin(1.5 * np.pi * p[:, 1])


def run(px, mesh, order, rhs_kind):
    fe = px.FESpace(mesh, order)
    bcs = [px.BCEss(fe, px.side.LEFT), px.BCEss(fe, px.side.BOTTOM)]
    builder = px.Builder(fe)
    builder.buildLhs((px.AssemblyStiffness(1.0, fe),), bcs)
    if rhs_kind == "analytic":
        builder.buildRhs((px.AssemblyRhsAnalytic(px.FN_POISSON_RHS, fe),), bcs)
    elif rhs_kind == "callable":
        builder.buildRhs((px.AssemblyRhsAnalytic(poisson_rhs, fe),), bcs)
    else:
        proj = px.interpolateAnalyticFunction(px.FN_POISSON_RHS, fe)
        builder.buildRhs((px.AssemblyProjection(1.0, proj, fe),), bcs)
    builder.closeMatrix()
    solver = px.LUSolver()
    solver.analyzePattern(builder)
    solver.factorize(builder)
    u = solver.solve(builder.b)
    assert solver.rel_res <= 1e-14
    exact = px.interpolateAnalyticFunction(px.FN_POISSON_EXACT, fe)
    ud = spla.spsolve(builder.A.tocsc(), builder.b)
    return float(np.linalg.norm(u - exact)), float(np.linalg.norm(ud - exact))


@pytest.mark.parametrize("elem,order,n,rhs,expected", [
    ("hex", 1, 4, "analytic", 0.1352139631934435),        # test/poisson3dhex.cpp:118
    ("hex", 1, 4, "callable", 0.1352139631934435),        # the same with the rhs as a host function
    ("hex", 2, 4, "analytic", 0.0070042836287997),        # test/poisson3dhex_q2.cpp:120
    ("hex", 2, 8, "analytic", 0.001164556821288369),      # test/poisson3dhex_q2.cpp:126
    ("tet", 2, 4, "proj", 0.08097818482375403),           # test/poisson3dtet_p2.cpp:124
    ("tet", 2, 8, "proj", 0.02265721054353444),           # test/poisson3dtet_p2.cpp:134
])
def test_golden_structured(engine, elem, order, n, rhs, expected):
    px = engine
    mesh = px.buildHyperCube(px.Hexahedron if elem == "hex" else px.Tetrahedron, n)
    e_dev, e_host = run(px, mesh, order, rhs)
    assert abs(e_dev - expected) < 1e-12, (e_dev, expected)
    assert abs(e_host - expected) < 1e-12, (e_host, expected)


def test_golden_unstructured_p1(engine):
    """test/poisson3dtet.cpp with data/cube_uns.msh (data/poisson3dtet.yaml:8-11)."""
    px = engine
    d = np.load(os.path.join(GOLDEN, "cube_uns.npz"))
    mesh = px.Mesh(px.Tetrahedron, d["xyz"], d["tets"], facets=(d["tris"], d["tri_tags"]))
    e_dev, e_host = run(px, mesh, 1, "proj")
    assert abs(e_dev - 0.88528925443) < 1e-12 and abs(e_host - 0.88528925443) < 1e-12, (e_dev, e_host)


@pytest.mark.parametrize("elem,expected", [
    # test/stokes3dhex.cpp:135-140
    ("hex", [1.309442419567852e-15, 1.021847252919293e-14, 1.800953966048908e-15, 1.097009563518918e-14]),
    # test/stokes3dtet.cpp:122-127
    ("tet", [1.191610761242353e-15, 4.347071660478249e-15, 1.168951507916659e-15, 5.36156027085171e-14]),
])
def test_golden_stokes(engine, elem, expected):
    """test/stokes3dhex.cpp and stokes3dtet.cpp written against the mirror: Taylor-Hood
    spaces with offsets, Builder{numDOFs}, tensor stiffness, grad / div couplings and six
    component-wise BCEss; solved on the host, error norms against the pinned values."""
    px = engine
    ly, nu = 2.0, 0.1
    E = px.Hexahedron if elem == "hex" else px.Tetrahedron
    mesh = px.buildHyperCube(E, 4, length=(1.0, ly, 1.0))
    vel = px.FESpace(mesh, 2, dim=3)
    p = px.FESpace(mesh, 1, offset=3 * vel.dof.size, qr_order=2)
    inlet = lambda X: np.stack([0 * X[:, 0], 0.5 * (1.0 - X[:, 0] ** 2), 0 * X[:, 0]], axis=1)
    zero = lambda X: np.zeros((X.shape[0], 3))
    s = px.side
    bcsVel = [px.BCEss(vel, s.BOTTOM, inlet), px.BCEss(vel, s.RIGHT, zero), px.BCEss(vel, s.TOP, zero, comps=[0, 2]),
              px.BCEss(vel, s.LEFT, zero, comps=[0, 2]), px.BCEss(vel, s.BACK, zero, comps=[2]),
              px.BCEss(vel, s.FRONT, zero, comps=[2])]
    bcsP = []
    n = 3 * vel.dof.size + p.dof.size
    builder = px.Builder(n)
    builder.buildLhs((px.AssemblyTensorStiffness(nu, vel),), bcsVel)
    builder.buildCoupling(px.AssemblyGrad(-1.0, vel, p), bcsVel, bcsP)
    builder.buildCoupling(px.AssemblyDiv(-1.0, p, vel), bcsP, bcsVel)
    builder.closeMatrix()
    sol = spla.spsolve(builder.A.tocsc(), builder.b)
    nd = vel.dof.size
    X = vel.dofPts()
    ue = inlet(X)
    pe = nu * (ly - p.dofPts()[:, 1])
    err = [np.linalg.norm(sol[c * nd:(c + 1) * nd] - ue[:, c]) for c in range(3)]
    err.append(np.linalg.norm(sol[3 * nd:] - pe))
    for e, r in zip(err, expected):
        assert abs(e - r) < 1e-12
