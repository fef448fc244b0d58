"""Boundary facets, markers and Dirichlet conditions set up on the device
(buildFacets / markFacetsCube, mesh.hpp:226-498; BCEss::setupDofMap, bc.hpp:252-295):
facet counts and markers of the structured cube, and assembled systems with
marker-based conditions against the oracle with the same constrained set."""
import numpy as np
import pytest

import oracle as O
from helpers import assert_close, compare_csr, oracle_lhs, problem

pytestmark = pytest.mark.gpu

TYPES = [(O.P1TET, "tet6", 4, 12), (O.P2TET, "tet5", 3, 12), (O.Q1HEX, "hex", 5, 6), (O.Q2HEX, "hex", 3, 6)]
IDS = ["p1tet", "p2tet", "q1hex", "q2hex"]
BOTTOM, RIGHT, TOP, LEFT, BACK, FRONT = 1, 2, 3, 4, 5, 6


@pytest.mark.parametrize("t,gen,n,per_square", TYPES, ids=IDS)
def test_facets_and_box_markers(engine, t, gen, n, per_square):
    from proxpde_gb300 import Context

    xyz, conn, _ = problem(gen, n, 0.2, seed=5)
    ctx = Context(0)
    ctx.set_mesh(t, xyz, conn)
    nb = ctx.build_facets()
    assert nb == per_square * n * n  # 6 faces x n^2 squares, 2 triangles per square
    ctx.mark_facets_box()
    faces, markers = ctx.get_facets()
    nf = 6 if t in (O.Q1HEX, O.Q2HEX) else 4
    assert np.all(faces // nf < conn.shape[0]) and np.unique(faces).size == nb
    counts = np.bincount(markers, minlength=7)
    assert counts[0] == 0
    assert np.all(counts[1:] == nb // 6)


@pytest.mark.parametrize("t,gen,n,per_square", TYPES, ids=IDS)
def test_marker_conditions_match_oracle(engine, t, gen, n, per_square):
    """Three conditions with shared DOFs (later ones win): LEFT = 0.5, TOP = 2 x,
    FRONT = sin sin sin; K(k_e) and the load with the lift against the oracle."""
    import torch

    from proxpde_gb300 import Context
    from proxpde_gb300._lib import FN_COORD_X

    xyz, conn, k = problem(gen, n, 0.2, seed=6, sigma=1.0)
    ctx = Context(0)
    ctx.set_mesh(t, xyz, conn)
    ndof = ctx.build_dofmap()
    nnz = ctx.build_pattern()
    ctx.set_coef(k)
    ctx.mark_facets_box()
    ctx.set_bc_markers([(LEFT, O.FN_CONST, 0.5), (TOP, FN_COORD_X, 2.0), (FRONT, O.FN_SIN3, 1.0)], diag=1.0)
    K = torch.empty(nnz, dtype=torch.float64, device="cuda")
    b = torch.empty(ndof, dtype=torch.float64, device="cuda")
    op = {"stiffness": 2, "stiff_coef": 1.0, "apply_bc": 1}
    rhs = {"kind": 1, "fn": O.FN_SIN3, "coef": 1.0, "apply_bc": 1}
    ctx.assemble(op0=op, vals0=K, rhs=rhs, b=b)
    torch.cuda.synchronize()
    # expected constrained set and values from the DOF coordinates
    em, _ = O.dofmap(t, xyz.shape[0], conn)
    dx = O.dof_coords(t, xyz, conn, em, ndof)
    on = lambda a, v: np.abs(dx[:, a] - v) <= 1e-12
    mask = (on(0, 0.0) | on(1, 1.0) | on(2, 1.0)).astype(np.uint8)
    val = np.zeros(ndof)
    val[on(0, 0.0)] = 0.5
    val[on(1, 1.0)] = 2.0 * dx[on(1, 1.0), 0]
    f = on(2, 1.0)
    val[f] = np.sin(np.pi * dx[f, 0]) * np.sin(np.pi * dx[f, 1]) * np.sin(np.pi * dx[f, 2])
    csr, bo = O.build(t, xyz, conn, em, ndof, lhs=oracle_lhs(op, k), bc_mask=mask, bc_val=val)
    _, bo = O.build(t, xyz, conn, em, ndof, rhs={"kind": 1, "fn": O.FN_SIN3, "c": 1.0, "apply_bc": 1},
                    bc_mask=mask, bc_val=val, b=bo)
    rp, ci = ctx.get_pattern()
    import scipy.sparse as sp

    A = sp.csr_matrix((K.cpu().numpy(), ci, rp), shape=(ndof, ndof))
    B = sp.csr_matrix((csr[2], csr[1], csr[0]), shape=(ndof, ndof))
    assert abs(A - B).max() <= 1e-12 * abs(B).max()
    assert_close(b.cpu().numpy(), bo, what="rhs with lift")


def test_marker_conditions_need_facets(engine):
    from proxpde_gb300 import Context, PxgError

    xyz, conn, _ = problem("hex", 2)
    ctx = Context(0)
    ctx.set_mesh(O.Q1HEX, xyz, conn)
    ctx.build_dofmap()
    with pytest.raises(PxgError):
        ctx.set_bc_markers([(LEFT, O.FN_CONST, 0.0)])
    ctx.mark_facets_box()
    with pytest.raises(PxgError):
        ctx.set_bc_markers([(LEFT, 99, 0.0)])  # unknown function id
