"""proxpde's golden tests run end to end on the GPU engine through the Builder mirror:
assemble on the device, solve on the host (scipy direct solve, like the reference's
UmfPackLU), compare ||u - I_h u_exact||_2 with the pinned value (tolerance 1e-12,
include/def.hpp:357-385)."""
import os

import numpy as np
import pytest
import scipy.sparse.linalg as spla

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def run(px, mesh, order, rhs_kind):
    fe = px.FESpace(mesh, order)
    bcs = [px.BCEss(fe, px.side.LEFT), px.BCEss(fe, px.side.BOTTOM)]
    builder = px.Builder(fe)
    builder.buildLhs((px.AssemblyStiffness(1.0, fe),), bcs)
    if rhs_kind == "analytic":
        builder.buildRhs((px.AssemblyRhsAnalytic(px.FN_POISSON_RHS, fe),), bcs)
    else:
        proj = px.interpolateAnalyticFunction(px.FN_POISSON_RHS, fe)
        builder.buildRhs((px.AssemblyProjection(1.0, proj, fe),), bcs)
    builder.closeMatrix()
    u = spla.spsolve(builder.A.tocsc(), builder.b)
    exact = px.interpolateAnalyticFunction(px.FN_POISSON_EXACT, fe)
    return float(np.linalg.norm(u - exact))


@pytest.mark.parametrize("elem,order,n,rhs,expected", [
    ("hex", 1, 4, "analytic", 0.1352139631934435),        # test/poisson3dhex.cpp:118
    ("hex", 2, 4, "analytic", 0.0070042836287997),        # test/poisson3dhex_q2.cpp:120
    ("hex", 2, 8, "analytic", 0.001164556821288369),      # test/poisson3dhex_q2.cpp:126
    ("tet", 2, 4, "proj", 0.08097818482375403),           # test/poisson3dtet_p2.cpp:124
    ("tet", 2, 8, "proj", 0.02265721054353444),           # test/poisson3dtet_p2.cpp:134
])
def test_golden_structured(engine, elem, order, n, rhs, expected):
    px = engine
    mesh = px.buildHyperCube(px.Hexahedron if elem == "hex" else px.Tetrahedron, n)
    assert abs(run(px, mesh, order, rhs) - expected) < 1e-12


def test_golden_unstructured_p1(engine):
    """test/poisson3dtet.cpp with data/cube_uns.msh (data/poisson3dtet.yaml:8-11)."""
    px = engine
    d = np.load(os.path.join(GOLDEN, "cube_uns.npz"))
    mesh = px.Mesh(px.Tetrahedron, d["xyz"], d["tets"], facets=(d["tris"], d["tri_tags"]))
    assert abs(run(px, mesh, 1, "proj") - 0.88528925443) < 1e-12
