"""Vector spaces and coupled (mixed) systems on the device (pxg_sys) against the oracle:
proxpde's Taylor-Hood Stokes tests (Q2-Q1 hexahedra, P2-P1 tetrahedra; tensor
stiffness, grad / div couplings, component-wise Dirichlet data) assembled through the C
ABI, compared entry by entry with the oracle and solved against the pinned golden error
norms; plus vector stiffness + mass with a Dirichlet set."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle as O
from helpers import assert_close, compare_csr

pytestmark = pytest.mark.gpu

GOLDEN = {
    "hex": [1.309442419567852e-15, 1.021847252919293e-14, 1.800953966048908e-15, 1.097009563518918e-14],
    "tet": [1.191610761242353e-15, 4.347071660478249e-15, 1.168951507916659e-15, 5.36156027085171e-14],
}


def device_closed(sysm, vals):
    """closeMatrix on the host: prune |v| <= 1e-16 from the structural values."""
    rp, ci = sysm.get_pattern()
    A = sp.csr_matrix((vals.cpu().numpy(), ci, rp), shape=(sysm.ntot, sysm.ntot))
    A.data[np.abs(A.data) <= 1e-16] = 0.0
    A.eliminate_zeros()
    A.sort_indices()
    return A


@pytest.mark.parametrize("elem", ["hex", "tet"])
def test_stokes_system_matches_oracle_and_goldens(engine, elem):
    import torch

    from proxpde_gb300 import Context
    from proxpde_gb300._lib import OP_DIV, OP_GRAD, OP_TENSOR_STIFFNESS, System

    P = O.stokes_problem(elem)
    cv, cp = Context(0), Context(0)
    cv.set_mesh(P["tv"], P["xyz"], P["conn"])
    cp.set_mesh(P["tp"], P["xyz"], P["conn"])
    assert cv.build_dofmap() == P["ndv"] and cp.build_dofmap() == P["ndp"]
    S = System([cv, cp], [3, 1], qr_types=[P["tv"], P["tv"]])
    assert S.ntot == 3 * P["ndv"] + P["ndp"] and S.offsets == [0, 3 * P["ndv"]]
    dofs = np.nonzero(P["bc_mask"])[0]
    S.set_bc(0, dofs, P["bc_vals"][dofs], 1.0)
    vals = torch.zeros(S.nnz, dtype=torch.float64, device="cuda")
    b = torch.zeros(S.ntot, dtype=torch.float64, device="cuda")
    S.assemble(0, 0, [(OP_TENSOR_STIFFNESS, 0.1)], vals, b, accumulate=True)
    S.assemble(0, 1, [(OP_GRAD, -1.0)], vals, b, accumulate=True)
    S.assemble(1, 0, [(OP_DIV, -1.0)], vals, b, accumulate=True)
    torch.cuda.synchronize()
    A = device_closed(S, vals)
    err_o, csr_o, b_o = O.stokes_golden(elem)
    compare_csr((A.indptr, A.indices, A.data), csr_o, S.ntot)
    assert_close(b.cpu().numpy(), b_o, what="rhs")
    sol = spla.spsolve(A.tocsc(), b.cpu().numpy())
    for e, r in zip(O.stokes_errors(P, sol), GOLDEN[elem]):
        assert abs(e - r) < 1e-12


@pytest.mark.parametrize("t,gen,n", [(O.Q1HEX, O.cube_hex, 3), (O.P2TET, O.cube_tet5, 2)], ids=["q1hex", "p2tet"])
def test_vector_stiffness_mass(engine, t, gen, n):
    """AssemblyStiffness + AssemblyMass on a 3-component space with constrained
    components (BLOCK ordering) against the oracle."""
    import torch

    from proxpde_gb300 import Context
    from proxpde_gb300._lib import OP_MASS, OP_STIFFNESS, System

    xyz, conn = gen(n)
    em, nd = O.dofmap(t, xyz.shape[0], conn)
    x = O.dof_coords(t, xyz, conn, em, nd)
    ids = np.nonzero(np.abs(x[:, 0]) <= 1e-12)[0]
    dofs = np.concatenate([ids, ids + 2 * nd])  # components 0 and 2 on x = 0
    bvals = np.concatenate([1.0 + x[ids, 1], -x[ids, 2]])
    mask = np.zeros(3 * nd, dtype=np.uint8)
    mask[dofs] = 1
    mv = np.zeros(3 * nd)
    mv[dofs] = bvals
    S_o = O.System(xyz, conn, [dict(t=t, qr=t, dim=3, offset=0, ndof=nd, em=em)], 3 * nd)
    S_o.set_bc(0, mask, mv, 1.0)
    S_o.call(0, 0, [(O.STIFF, 2.0), (O.MASS, 0.5)])
    csr_o = S_o.close()
    c = Context(0)
    c.set_mesh(t, xyz, conn)
    c.build_dofmap()
    S = System([c], [3])
    S.set_bc(0, dofs, bvals, 1.0)
    vals = torch.zeros(S.nnz, dtype=torch.float64, device="cuda")
    b = torch.zeros(S.ntot, dtype=torch.float64, device="cuda")
    S.assemble(0, 0, [(OP_STIFFNESS, 2.0), (OP_MASS, 0.5)], vals, b)
    torch.cuda.synchronize()
    A = device_closed(S, vals)
    compare_csr((A.indptr, A.indices, A.data), csr_o, S.ntot)
    assert_close(b.cpu().numpy(), S_o.b, what="rhs")


def test_system_rejects_mismatched_operators(engine):
    import torch

    from proxpde_gb300 import Context, PxgError
    from proxpde_gb300._lib import OP_GRAD, OP_TENSOR_STIFFNESS, System

    xyz, conn = O.cube_hex(2)
    cv, cp = Context(0), Context(0)
    cv.set_mesh(O.Q2HEX, xyz, conn)
    cp.set_mesh(O.Q1HEX, xyz, conn)
    cv.build_dofmap()
    cp.build_dofmap()
    S = System([cv, cp], [3, 1], qr_types=[O.Q2HEX, O.Q2HEX])
    vals = torch.zeros(S.nnz, dtype=torch.float64, device="cuda")
    with pytest.raises(PxgError):
        S.assemble(0, 1, [(OP_TENSOR_STIFFNESS, 1.0)], vals)  # a square operator on a coupling call
    with pytest.raises(PxgError):
        S.assemble(1, 0, [(OP_GRAD, 1.0)], vals)  # grad needs vector rows


@pytest.mark.parametrize("elem", ["hex", "tet"])
def test_vector_loads_match_oracle(engine, elem):
    """buildRhs on a vector space through Builder{numDOFs}: an analytic load with one
    function per component on two of the three components, and the L2 projection of a
    vector field with its components listed out of order, under component-wise Dirichlet
    sets; a scalar load on the second space (tests/helpers.py:vector_load_expect). Each
    block is compared with the oracle's scalar load of that component, condensed with
    that component's constrained DOFs."""
    import proxpde_gb300 as px
    from helpers import vector_load_expect, vector_load_field

    E = px.Hexahedron if elem == "hex" else px.Tetrahedron
    mesh = px.buildHyperCube(E, 3)
    vel = px.FESpace(mesh, 2, dim=3)
    p = px.FESpace(mesh, 1, offset=3 * vel.dof.size)
    nd, ndp = vel.dof.size, p.dof.size
    field = vector_load_field(3 * nd)
    expect, masks = vector_load_expect(elem, mesh.xyz, mesh.conn, field)
    assert expect.size == 3 * nd + ndp
    s = px.side
    bcs = [px.BCEss(vel, s.BOTTOM, lambda X: np.ones((X.shape[0], 3))), px.BCEss(vel, s.LEFT, 0.0, comps=[0, 2])]
    builder = px.Builder(3 * nd + ndp)
    builder.buildLhs((px.AssemblyMass(1.0, vel),))
    builder.buildRhs((px.AssemblyRhsAnalytic([px.FN_SIN3, px.FN_CONST, px.FN_POISSON_RHS], vel,
                                             coef=[1.0, 2.0, -0.5], comps=[0, 2]),
                      px.AssemblyS2SProjection(0.7, field, vel, comps=[2, 0])), bcs)
    builder.buildRhs((px.AssemblyRhsAnalytic(px.FN_CONST, p, 3.0),))
    builder.closeMatrix()
    b = builder.b
    for c in range(3):
        assert masks[c].any() and np.all(b[c * nd:(c + 1) * nd][masks[c] == 1] == 0.0)
    assert_close(b, expect, what="vector and scalar loads")
    with pytest.raises(ValueError):
        px.AssemblyRhsAnalytic(px.FN_CONST, vel)  # a vector space takes one id per component
    with pytest.raises(ValueError):
        px.AssemblyS2SProjection(1.0, field[:nd], vel)  # the field holds every component
    pq = px.FESpace(mesh, 1, offset=0, qr_order=2)
    with pytest.raises(px.PxgError):
        px.Builder(ndp).buildRhs((px.AssemblyRhsAnalytic(px.FN_CONST, pq),))  # loads use the element's rule


def test_system_close_above_noalloc_cap(engine):
    """pxg_sys_close_matrix (the system Builder's closeMatrix) has no row limit and no
    shared scratch: a 3-component P1 space with more rows than the allocation-free
    prune's 4,194,304, mass only (the component-cross blocks are structural zeros
    that the prune removes), matches the host-side prune of the same values, and two
    systems close one after the other on one stream with their own results."""
    import torch

    from proxpde_gb300 import Context, meshgen
    from proxpde_gb300._lib import OP_MASS, System

    xyz, conn = meshgen.cube_tet6(112)
    c = Context(0)
    c.set_mesh(O.P1TET, xyz, conn)
    nd = c.build_dofmap()
    S = System([c], [3])
    assert S.ntot == 3 * nd > 4_194_304
    vals = torch.zeros(S.nnz, dtype=torch.float64, device="cuda")
    S.assemble(0, 0, [(OP_MASS, 1.0)], vals)
    rp = torch.empty(S.ntot + 1, dtype=torch.int32, device="cuda")
    ci = torch.empty(S.nnz, dtype=torch.int32, device="cuda")
    vo = torch.empty(S.nnz, dtype=torch.float64, device="cuda")
    kept = S.close_matrix(vals, rp, ci, vo)
    torch.cuda.synchronize()
    A = device_closed(S, vals)
    assert kept == A.nnz and kept * 3 == S.nnz  # one block of three per row survives
    assert np.array_equal(rp.cpu().numpy(), A.indptr)
    assert np.array_equal(ci[:kept].cpu().numpy(), A.indices)
    assert np.array_equal(vo[:kept].cpu().numpy(), A.data)
    # a second, smaller system closed right after on the same stream keeps its own counts
    xyz2, conn2 = meshgen.cube_tet6(4)
    c2 = Context(0)
    c2.set_mesh(O.P1TET, xyz2, conn2)
    c2.build_dofmap()
    S2 = System([c2], [2])
    v2 = torch.zeros(S2.nnz, dtype=torch.float64, device="cuda")
    S2.assemble(0, 0, [(OP_MASS, 1.0)], v2)
    rp2 = torch.empty(S2.ntot + 1, dtype=torch.int32, device="cuda")
    ci2 = torch.empty(S2.nnz, dtype=torch.int32, device="cuda")
    vo2 = torch.empty(S2.nnz, dtype=torch.float64, device="cuda")
    assert S2.close_matrix(v2, rp2, ci2, vo2) * 2 == S2.nnz
    assert S.close_matrix(vals, rp, ci, vo) == kept
