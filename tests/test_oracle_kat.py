"""The oracle against proxpde's own known-answer tests.

Quadrature rows restated from test/qr.cpp:216-291 (monomials integrated exactly on
the reference tetrahedron / hexahedron) and the basis checks of
test/reffe_test.cpp:13-76 (phi_j(x_i) = delta_ij, sum_j grad phi_j = 0 at the DOF
points).  Pure CPU.
"""
import numpy as np
import pytest

import oracle as O

# (rule, (i,j,k), exact value, tolerance) -- test/qr.cpp:216-291
TET = [
    (O.P1TET, (0, 0, 0), 1 / 6, 1e-15), (O.P1TET, (1, 0, 0), 1 / 24, 1e-15),
    (O.P1TET, (2, 0, 0), 1 / 60, 1e-15), (O.P1TET, (1, 1, 0), 1 / 120, 1e-15),
    (O.P2TET, (0, 0, 0), 1 / 6, 1e-15), (O.P2TET, (1, 0, 0), 1 / 24, 1e-15),
    (O.P2TET, (2, 0, 0), 1 / 60, 1e-15), (O.P2TET, (1, 1, 0), 1 / 120, 1e-15),
    (O.P2TET, (3, 0, 0), 1 / 120, 1e-15), (O.P2TET, (2, 1, 0), 1 / 360, 1e-15),
    (O.P2TET, (1, 1, 1), 1 / 720, 1e-15), (O.P2TET, (4, 0, 0), 1 / 210, 1e-15),
    (O.P2TET, (3, 1, 0), 1 / 840, 1e-15), (O.P2TET, (2, 2, 0), 1 / 1260, 1e-15),
    (O.P2TET, (2, 1, 1), 1 / 2520, 1e-15),
]
HEX = [
    (O.Q1HEX, (0, 0, 0), 8.0, 1e-15), (O.Q1HEX, (1, 0, 0), 0.0, 1e-15), (O.Q1HEX, (2, 0, 0), 8 / 3, 1e-15),
    (O.Q1HEX, (0, 2, 0), 8 / 3, 1e-15), (O.Q1HEX, (0, 0, 2), 8 / 3, 1e-15), (O.Q1HEX, (1, 1, 1), 0.0, 1e-15),
    (O.Q1HEX, (3, 0, 0), 0.0, 1e-15), (O.Q1HEX, (2, 1, 0), 0.0, 1e-15),
    (O.Q2HEX, (0, 0, 0), 8.0, 1e-14), (O.Q2HEX, (2, 0, 0), 8 / 3, 1e-14), (O.Q2HEX, (0, 0, 2), 8 / 3, 1e-14),
    (O.Q2HEX, (1, 1, 1), 0.0, 1e-15), (O.Q2HEX, (4, 0, 0), 8 / 5, 1e-14), (O.Q2HEX, (2, 2, 0), 8 / 9, 1e-14),
    (O.Q2HEX, (3, 1, 0), 0.0, 1e-15), (O.Q2HEX, (2, 1, 1), 0.0, 1e-15),
]


@pytest.mark.parametrize("rule,pw,exact,tol", TET + HEX)
def test_quadrature_monomials(oracle_lib, rule, pw, exact, tol):
    nodes, w = O.quadrature(rule)
    # the reference sums in long double (test/qr.cpp:79-86)
    val = np.longdouble(0)
    for q in range(len(w)):
        m = nodes[q, 0] ** pw[0] * nodes[q, 1] ** pw[1] * nodes[q, 2] ** pw[2]
        val += np.longdouble(w[q]) * np.longdouble(m)
    assert abs(float(val) - exact) <= tol


REF_VERTS = {
    O.P1TET: np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float),
    O.P2TET: np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float),
    O.Q1HEX: np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                       [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], float),
}
REF_VERTS[O.Q2HEX] = REF_VERTS[O.Q1HEX]


@pytest.mark.parametrize("t", [O.P1TET, O.P2TET, O.Q1HEX, O.Q2HEX])
def test_basis_delta_and_partition(oracle_lib, t):
    """test/reffe_test.cpp:13-76 on the reference element."""
    X = REF_VERTS[t]
    conn = np.arange(X.shape[0], dtype=np.uint32)[None, :]
    em, ndof = O.dofmap(t, X.shape[0], conn)
    pts = O.dof_coords(t, X, conn, em, ndof)[em[0]]
    N = O.num_dofs(t)
    mat = np.zeros((N, N))
    dsum = np.zeros((N, 3))
    for i in range(N):
        phi, dphi = O.shape(t, pts[i])
        mat[i] = phi
        dsum[i] = dphi.sum(axis=0)
    assert np.linalg.norm(mat - np.eye(N)) <= 1e-16
    assert np.linalg.norm(dsum) <= 1e-15
