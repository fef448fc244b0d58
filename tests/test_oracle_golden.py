"""The oracle reproduces proxpde's golden solution-error norms (checkError, absolute
tolerance 1e-12, include/def.hpp:357-385): assemble with the restated element loop,
solve directly, compare ||u - I_h u_exact||_2 with the value the reference test pins.
"""
import os

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def left_bottom(em, ndof, dx):
    # BCEss{feSpace, side::LEFT} + BCEss{feSpace, side::BOTTOM}: planes x=0 and y=0
    return O.plane_bc_mask(dx, [("x", 0.0), ("y", 0.0)])


@pytest.mark.parametrize("t,n,gen,rhs,expected", [
    # test/poisson3dhex.cpp:114-120
    (O.Q1HEX, 4, O.cube_hex, "analytic", 0.1352139631934435),
    # test/poisson3dhex_q2.cpp:115-129
    (O.Q2HEX, 4, O.cube_hex, "analytic", 0.0070042836287997),
    (O.Q2HEX, 8, O.cube_hex, "analytic", 0.001164556821288369),
    # test/poisson3dtet_p2.cpp:117-136 (structured 5-tet cube, projected rhs)
    (O.P2TET, 4, O.cube_tet5, "proj", 0.08097818482375403),
    (O.P2TET, 8, O.cube_tet5, "proj", 0.02265721054353444),
])
def test_structured_goldens(oracle_lib, t, n, gen, rhs, expected):
    xyz, conn = gen(n)
    val = O.poisson_golden(t, xyz, conn, left_bottom, rhs)
    assert abs(val - expected) < 1e-12


def test_unstructured_p1_golden(oracle_lib):
    """test/poisson3dtet.cpp + data/poisson3dtet.yaml:8-11 (data/cube_uns.msh)."""
    d = np.load(os.path.join(GOLDEN, "cube_uns.npz"))
    xyz, conn = d["xyz"], d["tets"]
    facets = [(tuple(t), int(m)) for t, m in zip(d["tris"], d["tri_tags"])]

    def bc(em, ndof, dx):
        return O.facet_bc_mask(O.P1TET, conn, em, ndof, facets, {1, 4})  # BOTTOM, LEFT

    val = O.poisson_golden(O.P1TET, xyz, conn, bc, "proj")
    assert abs(val - 0.88528925443) < 1e-12


@pytest.mark.parametrize("elem,expected", [
    # test/stokes3dhex.cpp:135-140 (checkError, absolute 1e-12)
    ("hex", [1.309442419567852e-15, 1.021847252919293e-14, 1.800953966048908e-15, 1.097009563518918e-14]),
    # test/stokes3dtet.cpp:122-127
    ("tet", [1.191610761242353e-15, 4.347071660478249e-15, 1.168951507916659e-15, 5.36156027085171e-14]),
])
def test_oracle_stokes_goldens(elem, expected):
    """Vector spaces (BLOCK ordering), tensor stiffness and the grad / div couplings of
    the oracle, through proxpde's Taylor-Hood Stokes tests: Poiseuille flow in the box
    [0,1] x [0,2] x [0,1], 4^3 cells, with the tests' six BCEss (component lists)."""
    err, _, _ = O.stokes_golden(elem)
    for e, r in zip(err, expected):
        assert abs(e - r) < 1e-12
