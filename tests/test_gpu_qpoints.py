"""Analytic right-hand sides of any function (AssemblyRhsAnalytic with a host
std::function, include/assembly_rhs.hpp:50-59): the device reports CurFE::qpoint of
every element and quadrature point (pxg_get_qpoints, include/curfe.hpp:80), the
caller evaluates f there, and rhs kind 3 integrates the values on the device.

Against the oracle, for a function outside the device's pxg_fn list, on every element
type: the points agree to round-off, and the load vector (alone, with Dirichlet rows,
and beside stiffness + mass in the same call, with either scatter) agrees within the
tolerances of tests/helpers.py."""
import numpy as np
import pytest

import oracle as O
from helpers import assert_close, compare_csr, gpu_assemble, oracle_lhs, problem

pytestmark = pytest.mark.gpu

CASES = [(O.P1TET, "tet6", 4), (O.P2TET, "tet6", 3), (O.Q1HEX, "hex", 4), (O.Q2HEX, "hex", 3)]


def f_host(p):
    """Not one of the device functions: exp(x) cos(2y) + z^2 - xy."""
    return np.exp(p[:, 0]) * np.cos(2.0 * p[:, 1]) + p[:, 2] ** 2 - p[:, 0] * p[:, 1]


@pytest.mark.parametrize("t,gen,n", CASES, ids=[O.NAMES[c[0]] for c in CASES])
def test_qpoints_match_oracle(engine, t, gen, n):
    from proxpde_gb300 import Context

    xyz, conn, _ = problem(gen, n, 0.15, seed=41)
    ctx = Context(0)
    ctx.set_mesh(t, xyz, conn)
    qd = ctx.get_qpoints()
    qo = O.qpoints(t, xyz, conn)
    assert qd.shape == qo.shape == (conn.shape[0], O.lib().orc_num_qpts(t), 3)
    assert np.abs(qd - qo).max() <= 1e-15 * 8


@pytest.mark.parametrize("scatter", [0, 1], ids=["reduce", "colour"])
@pytest.mark.parametrize("t,gen,n", CASES, ids=[O.NAMES[c[0]] for c in CASES])
def test_host_function_load_matches_oracle(engine, t, gen, n, scatter):
    xyz, conn, k = problem(gen, n, 0.15, seed=43, sigma=1.0)
    em, ndof = O.dofmap(t, xyz.shape[0], conn)
    vals = f_host(O.qpoints(t, xyz, conn).reshape(-1, 3))
    # the load alone
    g = gpu_assemble(t, xyz, conn, [], rhs={"kind": 3, "coef": 1.5}, field=vals, scatter=scatter)
    _, b = O.build(t, xyz, conn, em, ndof, rhs={"kind": 3, "c": 1.5, "field": vals})
    assert_close(g["b"], b, what=f"kind3 {O.NAMES[t]} b")
    # with Dirichlet rows, beside K(k_e) with BCs and M in the same call
    dx = O.dof_coords(t, xyz, conn, em, ndof)
    mask = O.plane_bc_mask(dx, [("x", 0.0)])
    val = np.where(mask, 0.5 + dx[:, 1], 0.0)
    dofs = np.nonzero(mask)[0].astype(np.uint32)
    ops = [{"stiffness": 2, "stiff_coef": 1.0, "apply_bc": 1}, {"mass": 1, "mass_coef": 1.0}]
    g = gpu_assemble(t, xyz, conn, ops, rhs={"kind": 3, "coef": 1.5, "apply_bc": 1}, field=vals, k=k,
                     bc=(dofs, val[dofs]), scatter=scatter)
    csrK, b = O.build(t, xyz, conn, em, ndof, lhs=oracle_lhs(ops[0], k), bc_mask=mask, bc_val=val)
    csrM, _ = O.build(t, xyz, conn, em, ndof, lhs=oracle_lhs(ops[1], k))
    _, b = O.build(t, xyz, conn, em, ndof, rhs={"kind": 3, "c": 1.5, "field": vals, "apply_bc": 1}, bc_mask=mask,
                   bc_val=val, b=b)
    compare_csr(g["mats"][0], csrK, ndof, what=f"kind3 {O.NAMES[t]} K")
    compare_csr(g["mats"][1], csrM, ndof, what=f"kind3 {O.NAMES[t]} M")
    assert_close(g["b"], b, what=f"kind3 {O.NAMES[t]} b+bc")


def test_kind3_needs_values(engine):
    import torch

    from proxpde_gb300 import Context, PxgError

    xyz, conn, _ = problem("hex", 2)
    ctx = Context(0)
    ctx.set_mesh(O.Q1HEX, xyz, conn)
    ctx.build_dofmap()
    ctx.build_pattern()
    b = torch.zeros(ctx.ndof, dtype=torch.float64, device="cuda")
    with pytest.raises(PxgError):
        ctx.assemble(rhs={"kind": 3, "coef": 1.0}, b=b)
