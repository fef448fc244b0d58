"""Builder semantics the oracle restates (include/builder.hpp), checked on small
cases: duplicate summation and prune at closeMatrix, BC condensation with
multiplicity on the diagonal, first-touch DOF numbering, serial == OpenMP."""
import numpy as np
import pytest

import oracle as O
from proxpde_gb300 import meshgen


def test_mesh_builders_match_reference_restatement(oracle_lib):
    for n in (1, 2, 5):
        a = O.cube_hex(n)
        b = meshgen.cube_hex(n)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        a = O.cube_tet5(n)
        b = meshgen.cube_tet5(n)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_kuhn_split_volume():
    xyz, conn = meshgen.cube_tet6(3)
    X = xyz[conn.astype(np.int64)]
    v = np.abs(np.einsum("ij,ij->i", np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]), X[:, 3] - X[:, 0])) / 6
    assert abs(v.sum() - 1.0) < 1e-14 and np.all(v > 0)


def test_first_touch_numbering_hex(oracle_lib):
    # element 0 = nodes (0,1,2+n,1+n, ...) gets DOFs 0..7 in its local order
    xyz, conn = O.cube_hex(2)
    em, ndof = O.dofmap(O.Q1HEX, xyz.shape[0], conn)
    assert ndof == 27
    assert list(em[0]) == list(range(8))
    # element 1 shares 4 nodes with element 0 and creates 4 new DOFs 8..11
    assert sorted(set(em[1]) - set(em[0])) == [8, 9, 10, 11]


@pytest.mark.parametrize("t", [O.P2TET, O.Q2HEX])
def test_first_touch_interleaves_entities(oracle_lib, t):
    gen = O.cube_tet5 if t == O.P2TET else O.cube_hex
    xyz, conn = gen(2)
    em, ndof = O.dofmap(t, xyz.shape[0], conn)
    assert list(em[0]) == list(range(O.num_dofs(t)))
    assert em.max() + 1 == ndof and len(np.unique(em)) == ndof


def test_prune_and_duplicate_sum(oracle_lib):
    # unperturbed Q1 stiffness with k=1: face-neighbour entries cancel exactly and
    # are pruned; every other structural entry survives
    xyz, conn = O.cube_hex(3)
    em, ndof = O.dofmap(O.Q1HEX, xyz.shape[0], conn)
    csr, _ = O.build(O.Q1HEX, xyz, conn, em, ndof, lhs={"stiff_kind": 1, "stiff_c": 1.0})
    rp, col, val = csr
    assert np.all(np.abs(val) > 1e-16)
    keys = np.unique(em[:, :, None].astype(np.int64) * ndof + em[:, None, :])
    assert len(keys) > len(val)  # some structural entries were pruned
    A = O.csr_to_scipy(csr, ndof)
    assert abs(A - A.T).max() < 1e-15
    assert np.abs(A @ np.ones(ndof)).max() < 1e-14  # constants are in the kernel


def test_bc_diagonal_multiplicity(oracle_lib):
    xyz, conn = O.cube_hex(2)
    em, ndof = O.dofmap(O.Q1HEX, xyz.shape[0], conn)
    dx = O.dof_coords(O.Q1HEX, xyz, conn, em, ndof)
    mask = O.plane_bc_mask(dx, [("x", 0.0)])
    csr, b = O.build(O.Q1HEX, xyz, conn, em, ndof, lhs={"stiff_kind": 1, "stiff_c": 1.0, "apply_bc": 1},
                     bc_mask=mask, bc_val=np.full(ndof, 2.0))
    A = O.csr_to_scipy(csr, ndof).toarray()
    mult = np.bincount(em.reshape(-1), minlength=ndof)
    for d in np.nonzero(mask)[0]:
        assert A[d, d] == mult[d]  # diag = 1.0 once per touching element
        assert np.count_nonzero(A[d]) == 1 and np.count_nonzero(A[:, d]) == 1
        assert b[d] == 2.0 * mult[d]


def test_openmp_equals_serial(oracle_lib):
    xyz, conn = meshgen.cube_tet6(4)
    xyz = meshgen.perturb(xyz, 4, 0.2, 7)
    k = meshgen.lognormal(8, conn.shape[0])
    em, ndof = O.dofmap(O.P1TET, xyz.shape[0], conn)
    lhs = {"stiff_kind": 2, "k_e": k, "mass_kind": 1, "mass_c": 1.0}
    rhs = {"kind": 1, "fn": O.FN_SIN3, "c": 1.0}
    a, ba = O.build(O.P1TET, xyz, conn, em, ndof, lhs=lhs, rhs=rhs, nthreads=1)
    b, bb = O.build(O.P1TET, xyz, conn, em, ndof, lhs=lhs, rhs=rhs, nthreads=4)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert np.array_equal(ba, bb)


@pytest.mark.parametrize("t,gen,closed", [(O.Q1HEX, "hex", "nnz_q1_cube"), (O.P2TET, "tet6", "nnz_p2_kuhn6")])
def test_structural_nnz_closed_forms(t, gen, closed):
    """The closed forms the full-size GPU tests use, against brute-force counts of the
    DOF pairs that share an element."""
    import helpers as H

    for n in range(1, 7):
        xyz, conn = H.GEN[gen](n)
        em, ndof = O.dofmap(t, xyz.shape[0], conn)
        N = em.shape[1]
        i = np.repeat(em, N, axis=1).reshape(-1).astype(np.int64)
        j = np.tile(em, (1, N)).reshape(-1).astype(np.int64)
        assert np.unique(i * ndof + j).size == getattr(H, closed)(n), n


def test_q1_quadrature_helper_matches_oracle():
    """The numpy quadrature of the full-size checks reproduces the oracle's element loop."""
    import helpers as H

    xyz, conn, k = H.problem("hex", 5, 0.2, seed=3, sigma=1.0)
    em, ndof = O.dofmap(O.Q1HEX, xyz.shape[0], conn)
    vol, kvol, rsum = H.q1_quadrature(xyz, conn, k)
    K, b = O.build(O.Q1HEX, xyz, conn, em, ndof, lhs={"stiff_kind": 2, "k_e": k},
                   rhs={"kind": 1, "fn": O.FN_SIN3, "c": 1.0})
    Ks = O.csr_to_scipy(K, ndof)
    X = np.empty((ndof, 3))
    X[em.reshape(-1)] = xyz[conn.reshape(-1).astype(np.int64)]
    assert abs(vol - 1.0) <= 1e-13
    for d in range(3):
        u = X[:, d] - 0.5
        assert abs(u @ (Ks @ u) - kvol) <= 1e-12 * kvol
    assert abs(b.sum() - rsum) <= 1e-13 * rsum


@pytest.mark.parametrize("elem", ["hex", "tet"])
def test_vector_load_expectation(oracle_lib, elem):
    """The oracle side of the vector-load case (buildRhs on a vector space): blocks
    condensed per component, the unconstrained constant load integrates to c * |cube|,
    and block 1 holds only the projection of field component 0."""
    from helpers import vector_load_expect, vector_load_field

    xyz, conn = O.cube_hex(3) if elem == "hex" else O.cube_tet5(3)
    tv = O.Q2HEX if elem == "hex" else O.P2TET
    nd = O.dofmap(tv, xyz.shape[0], conn)[1]
    field = vector_load_field(3 * nd)
    b, masks = vector_load_expect(elem, xyz, conn, field)
    for c in range(3):
        blk = b[c * nd:(c + 1) * nd]
        assert masks[c].any() and np.all(blk[masks[c] == 1] == 0.0) and np.any(blk != 0.0)
    assert masks[1].sum() < masks[0].sum() == masks[2].sum()
    assert abs(b[3 * nd:].sum() - 3.0) < 1e-12
    # projection is linear in the field: doubling component 0 doubles block 1 only
    f2 = field.copy()
    f2[:nd] *= 2.0
    b2, _ = vector_load_expect(elem, xyz, conn, f2)
    assert np.allclose(b2[nd:2 * nd], 2.0 * b[nd:2 * nd], rtol=1e-14, atol=1e-300)
    assert np.array_equal(np.delete(b2, np.s_[nd:2 * nd]), np.delete(b, np.s_[nd:2 * nd]))


@pytest.mark.parametrize("t,gen", [(O.P1TET, "tet6"), (O.P2TET, "tet6"), (O.Q1HEX, "hex"), (O.Q2HEX, "hex")])
def test_mass_fe_coefficient(oracle_lib, t, gen):
    """AssemblyMassFE with a P0 coefficient (assembly_lhs.hpp:262-277): a constant
    coefficient reproduces AssemblyScalarMass, and the element matrix scales with the
    element's own value only."""
    from helpers import problem

    xyz, conn, k = problem(gen, 2, 0.15, seed=3, sigma=1.0)
    em, ndof = O.dofmap(t, xyz.shape[0], conn)
    c = np.full(conn.shape[0], 2.5)
    a, _ = O.build(t, xyz, conn, em, ndof, lhs={"mass_kind": 2, "m_e": c})
    b, _ = O.build(t, xyz, conn, em, ndof, lhs={"mass_kind": 1, "mass_c": 2.5})
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    for e in (0, conn.shape[0] - 1):
        Me, _ = O.element(t, xyz, conn, e, lhs={"mass_kind": 2, "m_e": k})
        M1, _ = O.element(t, xyz, conn, e, lhs={"mass_kind": 1, "mass_c": 1.0})
        assert np.allclose(Me, k[e] * M1, rtol=1e-15, atol=0.0)


@pytest.mark.parametrize("t,gen", [(O.P1TET, "tet6"), (O.P2TET, "tet5"), (O.Q1HEX, "hex"), (O.Q2HEX, "hex")])
def test_values_at_qpoints_reproduce_analytic_load(t, gen):
    """rhs kind 3 (values at CurFE::qpoint, evaluated by the caller) reproduces
    AssemblyRhsAnalytic of the same function evaluated inside the oracle (kind 1):
    the points are the reference's qpoint = origin + J xi (curfe.hpp:80)."""
    from proxpde_gb300 import meshgen

    xyz, conn = {"tet6": meshgen.cube_tet6, "tet5": meshgen.cube_tet5, "hex": meshgen.cube_hex}[gen](3)
    xyz = meshgen.perturb(xyz, 3, 0.15, 47)
    em, nd = O.dofmap(t, xyz.shape[0], conn)
    qp = O.qpoints(t, xyz, conn).reshape(-1, 3)
    v = np.sin(np.pi * qp[:, 0]) * np.sin(np.pi * qp[:, 1]) * np.sin(np.pi * qp[:, 2])
    _, b3 = O.build(t, xyz, conn, em, nd, rhs={"kind": 3, "c": 2.0, "field": v})
    _, b1 = O.build(t, xyz, conn, em, nd, rhs={"kind": 1, "fn": O.FN_SIN3, "c": 2.0})
    assert np.abs(b3 - b1).max() <= 1e-15 * np.abs(b1).max()
