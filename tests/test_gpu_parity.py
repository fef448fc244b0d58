"""GPU engine vs the CPU oracle on the same seeded inputs (C ABI path).

Covers every element type, the configurations' operator mixes at sizes the oracle
finishes in seconds, essential BCs (lift and multiplicity), projection loads,
accumulation, and the prune step of closeMatrix (exact cancellations on the
unperturbed P1 mesh with k = 1)."""
import numpy as np
import pytest

import oracle as O
from helpers import EPS, EPS_DFL, assert_close, compare_csr, gpu_assemble, oracle_lhs, problem, structural_pattern
from proxpde_gb300._lib import ARITH_DFL, ARITH_FP64

pytestmark = pytest.mark.gpu

K_OP = {"stiffness": 2, "stiff_coef": 1.0}
K1_OP = {"stiffness": 1, "stiff_coef": 1.0}
M_OP = {"mass": 1, "mass_coef": 1.0}

CASES = [
    # id, element, mesh generator, n, perturbation, k sigma, ops, rhs
    ("c1_p1tet_16", O.P1TET, "tet6", 16, 0.0, None, [K1_OP], {"kind": 1, "fn": O.FN_CONST, "coef": 1.0}),
    ("c2_q1hex_10", O.Q1HEX, "hex", 10, 0.2, 1.0, [K_OP, M_OP], {"kind": 1, "fn": O.FN_SIN3, "coef": 1.0}),
    ("c3_p2tet_5", O.P2TET, "tet6", 5, 0.15, 0.5, [K_OP, M_OP], {"kind": 1, "fn": O.FN_CONST, "coef": 1.0}),
    ("q2hex_3", O.Q2HEX, "hex", 3, 0.2, 1.0, [K_OP, M_OP], {"kind": 1, "fn": O.FN_SIN3, "coef": 1.0}),
    ("p1tet5_6", O.P1TET, "tet5", 6, 0.1, 1.0, [K_OP, {"mass": 1, "mass_coef": 2.5}],
     {"kind": 1, "fn": O.FN_POISSON_RHS, "coef": 1.0}),
    ("q1_mixed_op", O.Q1HEX, "hex", 5, 0.2, 1.0, [{"stiffness": 2, "stiff_coef": 0.5, "mass": 1, "mass_coef": 3.0}],
     None),
    # unperturbed hexahedra, k = 1: the face-neighbour stiffness entries cancel exactly,
    # so the prune step sees round-off residues
    ("q1hex_uniform_12", O.Q1HEX, "hex", 12, 0.0, None, [K1_OP, M_OP], {"kind": 1, "fn": O.FN_SIN3, "coef": 1.0}),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_parity(engine, case):
    _, t, gen, n, alpha, sig, ops, rhs = case
    xyz, conn, k = problem(gen, n, alpha, seed=11, sigma=sig)
    g = gpu_assemble(t, xyz, conn, ops, rhs=rhs, k=k)
    em, ndof = O.dofmap(t, xyz.shape[0], conn)
    assert g["ndof"] == ndof
    assert np.array_equal(g["em"], em), "first-touch DOF map differs"
    rp_s, ci_s = structural_pattern(em, ndof)
    assert np.array_equal(g["pattern"][0], rp_s) and np.array_equal(g["pattern"][1], ci_s)
    for m, (op, mat) in enumerate(zip(ops, g["mats"])):
        csr, _ = O.build(t, xyz, conn, em, ndof, lhs=oracle_lhs(op, k), nthreads=4)
        # the pruned pattern is bit-exact: no entry kept on one side only
        assert compare_csr(mat, csr, ndof, what=f"parity {case[0]} op{m}") == 0
        # entries near the prune threshold were recomputed in the reference's order:
        # bit for bit the oracle's values
        rows = np.repeat(np.arange(ndof), np.diff(csr[0]))
        rowmax = np.zeros(ndof)
        np.maximum.at(rowmax, rows, np.abs(csr[2]))
        near = np.abs(csr[2]) <= 1e-16 + 16 * 2.220446049250313e-16 * rowmax[rows]
        if near.any():
            assert np.array_equal(mat[2][near], csr[2][near])
    if rhs is not None:
        _, b = O.build(t, xyz, conn, em, ndof, rhs={"kind": rhs["kind"], "fn": rhs["fn"], "c": rhs["coef"]})
        assert_close(g["b"], b, what=f"parity {case[0]} rhs")


def test_prune_cancellation_margin(engine):
    """On the unperturbed P1 mesh with k = 1 many stiffness sums cancel; the engine
    prunes exactly the entries the oracle prunes, and no kept or pruned entry lies
    near the 1e-16 threshold (so summation order cannot flip one)."""
    xyz, conn, _ = problem("tet6", 16)
    g = gpu_assemble(O.P1TET, xyz, conn, [K1_OP])
    sv = np.abs(g["struct_vals"][0])
    nz = g["nnz"]
    assert g["mats"][0][1].size < nz  # something was pruned
    em, ndof = O.dofmap(O.P1TET, xyz.shape[0], conn)
    csr, _ = O.build(O.P1TET, xyz, conn, em, ndof, lhs={"stiff_kind": 1, "stiff_c": 1.0})
    assert compare_csr(g["mats"][0], csr, ndof) == 0  # bit-exact pruned pattern
    near = (sv > 1e-18) & (sv < 1e-14)
    assert not near.any(), f"{near.sum()} entries near the prune threshold"
    # the synchronous and the stream-ordered prune counts agree with the compaction
    import torch

    v = torch.as_tensor(g["struct_vals"][0]).cuda()
    out = torch.full((2,), -1, dtype=torch.int64, device="cuda")
    g["ctx"].prune_count_device(v, out[1:])
    assert g["ctx"].prune_count(v) == out[1].item() == nz - g["mats"][0][1].size
    assert out[0].item() == -1
    # the count's vector loads: a value array 8 bytes off a 16-byte boundary (first
    # entry alone, no odd tail) and the aligned one (odd tail), with zeroed ends
    assert nz % 2 == 1
    npruned = nz - g["mats"][0][1].size
    w = torch.zeros(nz + 2, dtype=torch.float64, device="cuda")  # zero sentinels count if read
    w[1:nz + 1] = v
    assert g["ctx"].prune_count(w[1:]) == npruned
    extra = int(abs(g["struct_vals"][0][0]) > 1e-16) + int(abs(g["struct_vals"][0][-1]) > 1e-16)
    w[1] = 0.0
    w[nz] = 0.0
    assert g["ctx"].prune_count(w[1:]) == npruned + extra
    assert g["ctx"].prune_count(w[1:nz + 1].clone()) == npruned + extra


@pytest.mark.parametrize("t,gen", [(O.P1TET, "tet6"), (O.P2TET, "tet5"), (O.Q1HEX, "hex"), (O.Q2HEX, "hex")])
def test_bc_lift_and_projection(engine, t, gen):
    """Inhomogeneous Dirichlet data on x=0 and y=0 (lift into b, diagonal
    multiplicity) with an L2-projection load on the same space."""
    n = 3
    xyz, conn, k = problem(gen, n, 0.15, seed=5, sigma=1.0)
    em, ndof = O.dofmap(t, xyz.shape[0], conn)
    dx = O.dof_coords(t, xyz, conn, em, ndof)
    mask = O.plane_bc_mask(dx, [("x", 0.0), ("y", 0.0)])
    val = np.where(mask, 1.0 + dx[:, 2], 0.0)
    field = np.sin(dx[:, 0] + 2 * dx[:, 1]) + dx[:, 2]
    op = {"stiffness": 2, "stiff_coef": 1.0, "mass": 1, "mass_coef": 0.5, "apply_bc": 1}
    rhs = {"kind": 2, "fn": 0, "coef": 2.0, "apply_bc": 1}
    dofs = np.nonzero(mask)[0].astype(np.uint32)
    g = gpu_assemble(t, xyz, conn, [op], rhs=rhs, k=k, bc=(dofs, val[dofs]), field=field)
    csr, b = O.build(t, xyz, conn, em, ndof, lhs=oracle_lhs(op, k), bc_mask=mask, bc_val=val)
    _, b = O.build(t, xyz, conn, em, ndof, rhs={"kind": 2, "c": 2.0, "field": field, "apply_bc": 1},
                   bc_mask=mask, bc_val=val, b=b)
    compare_csr(g["mats"][0], csr, ndof)
    assert_close(g["b"], b, what="rhs with lift")


def test_p2_group_scatter_overwrites_and_accumulates(engine):
    """The P2 warp-group scatter on outputs holding other values: an overwriting call
    matches the oracle, and an accumulating second call doubles K and M (to round-off
    of the reductions' order)."""
    import torch

    from proxpde_gb300 import Context

    xyz, conn, k = problem("tet6", 3, 0.15, seed=5, sigma=0.5)  # 162 elements: a partial last warp
    ctx = Context(0)
    ctx.set_mesh(O.P2TET, xyz, conn)
    ndof = ctx.build_dofmap()
    nnz = ctx.build_pattern()
    ctx.set_coef(k)
    K = torch.full((nnz,), 7.0, dtype=torch.float64, device="cuda")  # overwritten, not added to
    M = torch.full_like(K, -3.0)
    ctx.assemble(op0=K_OP, vals0=K, op1=M_OP, vals1=M)
    K1, M1 = K.clone(), M.clone()
    import scipy.sparse as sp

    em, _ = O.dofmap(O.P2TET, xyz.shape[0], conn)
    rp, ci = ctx.get_pattern()
    for op, v in ((K_OP, K1), (M_OP, M1)):
        csr, _ = O.build(O.P2TET, xyz, conn, em, ndof, lhs=oracle_lhs(op, k), nthreads=4)
        A = sp.csr_matrix((v.cpu().numpy(), ci, rp), shape=(ndof, ndof))
        B = sp.csr_matrix((csr[2], csr[1], csr[0]), shape=(ndof, ndof))
        assert abs(A - B).max() <= 1e-12 * abs(B).max()
    ctx.assemble(op0=K_OP, vals0=K, op1=M_OP, vals1=M, accumulate=True)
    for v, v1 in ((K, K1), (M, M1)):
        assert float((v - 2 * v1).abs().max()) <= 1e-14 * float(v1.abs().max())


def test_accumulate_and_single_element(engine):
    import torch

    from proxpde_gb300 import Context

    xyz, conn, k = problem("hex", 1, 0.0, sigma=None)
    ctx = Context(0)
    ctx.set_mesh(O.Q1HEX, xyz, conn)
    assert ctx.build_dofmap() == 8
    nnz = ctx.build_pattern()
    assert nnz == 64
    v = torch.zeros(nnz, dtype=torch.float64, device="cuda")
    ctx.assemble(op0=K1_OP, vals0=v)
    first = v.clone()
    ctx.assemble(op0=K1_OP, vals0=v, accumulate=True)
    assert torch.equal(v, 2 * first)
    Ke, _ = O.element(O.Q1HEX, xyz, conn, 0, lhs={"stiff_kind": 1, "stiff_c": 1.0})
    rp, ci = ctx.get_pattern()
    dense = np.zeros((8, 8))
    em = ctx.get_dofmap()[0]
    for r in range(8):
        for p in range(rp[r], rp[r + 1]):
            dense[r, ci[p]] = first[p].item()
    assert_close(dense[np.ix_(em, em)], Ke, what="single element")


def test_invalid_inputs_rejected(engine):
    from proxpde_gb300 import Context, PxgError

    xyz, conn, _ = problem("hex", 2)
    ctx = Context(0)
    bad = conn.copy()
    bad[3, 2] = xyz.shape[0]  # out-of-range node id
    with pytest.raises(PxgError) as ei:
        ctx.set_mesh(O.Q1HEX, xyz, bad)
    assert ei.value.status == 1
    with pytest.raises(PxgError):
        ctx.set_mesh(7, xyz, conn)  # unknown element type
    with pytest.raises(PxgError) as ei:
        ctx.set_mesh(O.Q1HEX, xyz, conn[:0])  # no elements
    assert ei.value.status == 1
    ctx.set_mesh(O.Q1HEX, xyz, conn)
    with pytest.raises(PxgError):
        ctx.build_pattern()  # before the DOF map
    ctx.build_dofmap()
    ctx.build_pattern()
    import torch

    v = torch.zeros(ctx.nnz, dtype=torch.float64, device="cuda")
    with pytest.raises(PxgError):
        ctx.assemble(op0={"stiffness": 2}, vals0=v)  # per-element coefficient not set
    b = torch.zeros(ctx.ndof, dtype=torch.float64, device="cuda")
    with pytest.raises(PxgError):
        ctx.assemble(rhs={"kind": 1, "fn": 99}, b=b)  # unknown analytic function
    with pytest.raises(PxgError):
        ctx.set_bc(np.array([ctx.ndof], np.uint32), np.zeros(1))  # DOF out of range
    # the context is still usable after the rejected calls
    ctx.assemble(op0=K1_OP, vals0=v)
    torch.cuda.synchronize()
    assert torch.isfinite(v).all()


Q1_KERNELS = ["fp64", "group-dfl", "group-fp64", "thread-dfl", "thread-fp64", "generic"]


def q1_kernel(monkeypatch, kernel):
    """Select a Q1 kernel for the contexts created next; returns its arithmetic."""
    monkeypatch.setenv("PXG_Q1_GENERIC", "1" if kernel == "generic" else "0")
    monkeypatch.setenv("PXG_Q1_THREAD", "1" if kernel.startswith("thread") else "0")
    monkeypatch.setenv("PXG_Q1_GROUP", "1" if kernel.startswith("group") else "0")
    return ARITH_DFL if kernel.endswith("dfl") else ARITH_FP64


@pytest.mark.parametrize("kernel", Q1_KERNELS)
@pytest.mark.parametrize("bc", [False, True], ids=["nobc", "bc"])
@pytest.mark.parametrize("n", [7, 40])
def test_q1_kernels_agree_with_oracle(engine, monkeypatch, kernel, bc, n):
    """The Q1 kernels against the oracle: the FP64 one-thread-per-element kernel
    (default), the eight-lanes-per-element tensor-product kernel and the older
    one-thread tensor-product kernel, each in double-float and in FP64, and the generic
    per-quadrature-point kernel; K(k_e) + M + sin3 load on a perturbed mesh, with and
    without inhomogeneous Dirichlet data.  n = 40 takes the short-series path of the
    load (small offsets), n = 7 the direct sinpi path; 7^3 elements also leave a partly
    filled last block."""
    arith = q1_kernel(monkeypatch, kernel)
    xyz, conn, k = problem("hex", n, 0.2, seed=21, sigma=1.0)
    em, ndof = O.dofmap(O.Q1HEX, xyz.shape[0], conn)
    bcarg, mask, val = None, None, None
    ops = [dict(K_OP), dict(M_OP)]
    rhs = {"kind": 1, "fn": O.FN_SIN3, "coef": 1.0}
    if bc:
        dx = O.dof_coords(O.Q1HEX, xyz, conn, em, ndof)
        mask = O.plane_bc_mask(dx, [("x", 0.0), ("z", 1.0)])
        val = np.where(mask, 0.5 + dx[:, 1], 0.0)
        dofs = np.nonzero(mask)[0].astype(np.uint32)
        bcarg = (dofs, val[dofs])
        ops[0]["apply_bc"] = 1
        rhs["apply_bc"] = 1
    g = gpu_assemble(O.Q1HEX, xyz, conn, ops, rhs=rhs, k=k, bc=bcarg, arith=arith)
    csrK, b = O.build(O.Q1HEX, xyz, conn, em, ndof, lhs=oracle_lhs(ops[0], k), bc_mask=mask, bc_val=val)
    csrM, _ = O.build(O.Q1HEX, xyz, conn, em, ndof, lhs=oracle_lhs(ops[1], k))
    _, b = O.build(O.Q1HEX, xyz, conn, em, ndof, rhs={"kind": 1, "fn": O.FN_SIN3, "c": 1.0, "apply_bc": int(bc)},
                   bc_mask=mask, bc_val=val, b=b)
    eps = EPS_DFL if arith == ARITH_DFL else EPS
    compare_csr(g["mats"][0], csrK, ndof, what=f"q1 {kernel} K", eps=eps)
    compare_csr(g["mats"][1], csrM, ndof, what=f"q1 {kernel} M", eps=eps)
    assert_close(g["b"], b, what=f"q1 {kernel} b", eps=eps)


@pytest.mark.parametrize("kernel", ["fp64", "fp64-plain", "dfl", "generic"])
@pytest.mark.parametrize("t,gen,n", [(O.P1TET, "tet6", 9), (O.P2TET, "tet6", 5), (O.P2TET, "tet5", 4)],
                         ids=["p1tet6", "p2tet6", "p2tet5"])
@pytest.mark.parametrize("bc", [False, True], ids=["nobc", "bc"])
@pytest.mark.parametrize("rhs_fn", ["const", "sin3"])
def test_tet_kernels_agree_with_oracle(engine, monkeypatch, kernel, t, gen, n, bc, rhs_fn):
    """The tetrahedron kernels against the oracle: reference-tensor entries in FP64
    (default; P2 with the warp-group scatter, and with plain reductions:
    PXG_NO_GROUP_SCATTER=1) and in double-float, and the per-quadrature-point FP64 kernel
    (PXG_TET_GENERIC=1); K(k_e) + M with a load (the constant load takes the closed-form
    path of the reference-tensor kernels), with and without inhomogeneous Dirichlet
    data.  750 P2 elements leave the last warp group partly filled."""
    monkeypatch.setenv("PXG_TET_GENERIC", "1" if kernel == "generic" else "0")
    monkeypatch.setenv("PXG_NO_GROUP_SCATTER", "1" if kernel == "fp64-plain" else "0")
    arith = ARITH_DFL if kernel == "dfl" else ARITH_FP64
    xyz, conn, k = problem(gen, n, 0.15, seed=23, sigma=0.5)
    em, ndof = O.dofmap(t, xyz.shape[0], conn)
    fn = O.FN_CONST if rhs_fn == "const" else O.FN_SIN3
    ops = [dict(K_OP), {"mass": 1, "mass_coef": 1.5}]
    rhs = {"kind": 1, "fn": fn, "coef": 2.0}
    bcarg, mask, val = None, None, None
    if bc:
        dx = O.dof_coords(t, xyz, conn, em, ndof)
        mask = O.plane_bc_mask(dx, [("x", 0.0), ("y", 1.0)])
        val = np.where(mask, 0.25 + dx[:, 2], 0.0)
        dofs = np.nonzero(mask)[0].astype(np.uint32)
        bcarg = (dofs, val[dofs])
        ops[0]["apply_bc"] = 1
        rhs["apply_bc"] = 1
    g = gpu_assemble(t, xyz, conn, ops, rhs=rhs, k=k, bc=bcarg, arith=arith)
    csrK, b = O.build(t, xyz, conn, em, ndof, lhs=oracle_lhs(ops[0], k), bc_mask=mask, bc_val=val)
    csrM, _ = O.build(t, xyz, conn, em, ndof, lhs=oracle_lhs(ops[1], k))
    _, b = O.build(t, xyz, conn, em, ndof, rhs={"kind": 1, "fn": fn, "c": 2.0, "apply_bc": int(bc)},
                   bc_mask=mask, bc_val=val, b=b)
    name = O.NAMES[t]
    eps = EPS_DFL if arith == ARITH_DFL else EPS
    compare_csr(g["mats"][0], csrK, ndof, what=f"{name} {kernel} K", eps=eps)
    compare_csr(g["mats"][1], csrM, ndof, what=f"{name} {kernel} M", eps=eps)
    assert_close(g["b"], b, what=f"{name} {kernel} b", eps=eps)


MASS_FE_KERNELS = [(O.P1TET, "tet6", 5, {}, ARITH_FP64), (O.P1TET, "tet6", 5, {}, ARITH_DFL),
                   (O.P2TET, "tet6", 3, {}, ARITH_FP64), (O.P2TET, "tet6", 3, {}, ARITH_DFL),
                   (O.P2TET, "tet6", 3, {"PXG_TET_GENERIC": "1"}, ARITH_FP64),
                   (O.Q1HEX, "hex", 5, {}, ARITH_FP64), (O.Q1HEX, "hex", 5, {}, ARITH_DFL),
                   (O.Q1HEX, "hex", 5, {"PXG_Q1_THREAD": "1"}, ARITH_DFL),
                   (O.Q1HEX, "hex", 4, {"PXG_Q1_GENERIC": "1"}, ARITH_FP64), (O.Q2HEX, "hex", 2, {}, ARITH_FP64),
                   (O.Q2HEX, "hex", 3, {}, ARITH_DFL)]
MASS_FE_IDS = ["p1", "p1_dfl", "p2", "p2_dfl", "p2_generic", "q1", "q1_group_dfl", "q1_thread_dfl", "q1_generic",
               "q2", "q2_dfl"]


@pytest.mark.parametrize("t,gen,n,env,arith", MASS_FE_KERNELS, ids=MASS_FE_IDS)
def test_mass_fe_coefficient_matches_oracle(engine, monkeypatch, t, gen, n, env, arith):
    """AssemblyMassFE with the per-element coefficient (mass kind 2, times mass_coef)
    in every element kernel against the oracle: alone (the mass coefficient folded
    where a kernel folds a single operator's), beside AssemblyStiffnessFE on the same
    coefficient, and in one operator with a constant stiffness, with Dirichlet data."""
    for v in ("PXG_TET_GENERIC", "PXG_Q1_THREAD", "PXG_Q1_GENERIC", "PXG_Q1_GROUP", "PXG_Q2_GENERIC"):
        monkeypatch.setenv(v, env.get(v, "0"))
    xyz, conn, k = problem(gen, n, 0.15, seed=29, sigma=1.0)
    em, ndof = O.dofmap(t, xyz.shape[0], conn)
    dx = O.dof_coords(t, xyz, conn, em, ndof)
    mask = O.plane_bc_mask(dx, [("z", 0.0)])
    val = np.where(mask, 1.0 - dx[:, 0], 0.0)
    dofs = np.nonzero(mask)[0].astype(np.uint32)
    for ops in ([{"mass": 2, "mass_coef": 0.75}],
                [{"stiffness": 2, "stiff_coef": 1.0}, {"mass": 2, "mass_coef": 2.0}],
                [{"stiffness": 1, "stiff_coef": 0.5, "mass": 2, "mass_coef": 3.0, "apply_bc": 1}]):
        bc = (dofs, val[dofs]) if any(o.get("apply_bc") for o in ops) else None
        g = gpu_assemble(t, xyz, conn, ops, k=k, bc=bc, arith=arith)
        for op, mat in zip(ops, g["mats"]):
            o = oracle_lhs(op, k)
            kw = dict(bc_mask=mask, bc_val=val) if op.get("apply_bc") else {}
            csr, b = O.build(t, xyz, conn, em, ndof, lhs=o, **kw)
            compare_csr(mat, csr, ndof, what=f"massFE {O.NAMES[t]} {env} arith{arith}",
                        eps=EPS_DFL if arith == ARITH_DFL else EPS)
            if op.get("apply_bc"):
                assert_close(g["b"], b, what="lift")


@pytest.mark.parametrize("kernel", ["fp64", "group-dfl", "group-fp64"])
def test_q1_two_stiffness_operators(engine, monkeypatch, kernel):
    """The Q1 kernels with two stiffness operators of different coefficients, one of
    them combined with a mass term of coefficient 2, and with the operators swapped
    (mass first), on a perturbed mesh with a partly filled last block."""
    arith = q1_kernel(monkeypatch, kernel)
    xyz, conn, k = problem("hex", 7, 0.2, seed=37, sigma=1.0)
    em, ndof = O.dofmap(O.Q1HEX, xyz.shape[0], conn)
    for ops in ([{"stiffness": 2, "stiff_coef": 0.75, "mass": 1, "mass_coef": 2.0}, {"stiffness": 1, "stiff_coef": 3.0}],
                [{"mass": 1, "mass_coef": 0.3}, {"stiffness": 2, "stiff_coef": 2.5}]):
        g = gpu_assemble(O.Q1HEX, xyz, conn, ops, k=k, arith=arith)
        for op, mat in zip(ops, g["mats"]):
            csr, _ = O.build(O.Q1HEX, xyz, conn, em, ndof, lhs=oracle_lhs(op, k))
            compare_csr(mat, csr, ndof, eps=EPS_DFL if arith == ARITH_DFL else EPS)


def test_tet_two_stiffness_operators(engine):
    """Two stiffness operators with different coefficients (no folding into G) and a
    combined stiffness + mass operator, on P2."""
    xyz, conn, k = problem("tet6", 4, 0.15, seed=29, sigma=0.5)
    em, ndof = O.dofmap(O.P2TET, xyz.shape[0], conn)
    ops = [{"stiffness": 2, "stiff_coef": 0.75, "mass": 1, "mass_coef": 2.0}, {"stiffness": 1, "stiff_coef": 3.0}]
    g = gpu_assemble(O.P2TET, xyz, conn, ops, k=k)
    for op, mat in zip(ops, g["mats"]):
        csr, _ = O.build(O.P2TET, xyz, conn, em, ndof, lhs=oracle_lhs(op, k))
        compare_csr(mat, csr, ndof)


@pytest.mark.parametrize("kernel", ["fp64", "dfl"])
@pytest.mark.parametrize("n", [3, 5])
@pytest.mark.parametrize("bc", [False, True], ids=["nobc", "bc"])
@pytest.mark.parametrize("rhs_kind", ["sin3", "projection"])
def test_q2_kernels_agree_with_oracle(engine, monkeypatch, kernel, n, bc, rhs_kind):
    """The Q2 kernels against the oracle: the FP64 element kernel (default) and the
    block-per-element double-float kernel; K(k_e) + M with an analytic or a projected
    load, with and without inhomogeneous Dirichlet data; n = 5 gives more elements than
    the persistent grid of the double-float kernel has blocks only on small GPUs, n = 3
    fewer."""
    arith = ARITH_DFL if kernel == "dfl" else ARITH_FP64
    xyz, conn, k = problem("hex", n, 0.2, seed=31, sigma=1.0)
    em, ndof = O.dofmap(O.Q2HEX, xyz.shape[0], conn)
    dx = O.dof_coords(O.Q2HEX, xyz, conn, em, ndof)
    ops = [dict(K_OP), {"mass": 1, "mass_coef": 0.75}]
    field = np.sin(dx[:, 0] + 2 * dx[:, 1]) + dx[:, 2]
    if rhs_kind == "sin3":
        rhs = {"kind": 1, "fn": O.FN_SIN3, "coef": 1.5}
        orhs = {"kind": 1, "fn": O.FN_SIN3, "c": 1.5}
    else:
        rhs = {"kind": 2, "fn": 0, "coef": 1.5}
        orhs = {"kind": 2, "c": 1.5, "field": field}
    bcarg, mask, val = None, None, None
    if bc:
        mask = O.plane_bc_mask(dx, [("y", 0.0), ("z", 1.0)])
        val = np.where(mask, 0.5 - dx[:, 0], 0.0)
        dofs = np.nonzero(mask)[0].astype(np.uint32)
        bcarg = (dofs, val[dofs])
        ops[0]["apply_bc"] = 1
        rhs["apply_bc"] = 1
        orhs["apply_bc"] = 1
    g = gpu_assemble(O.Q2HEX, xyz, conn, ops, rhs=rhs, k=k, bc=bcarg, field=field, arith=arith)
    csrK, b = O.build(O.Q2HEX, xyz, conn, em, ndof, lhs=oracle_lhs(ops[0], k), bc_mask=mask, bc_val=val)
    csrM, _ = O.build(O.Q2HEX, xyz, conn, em, ndof, lhs=oracle_lhs(ops[1], k))
    _, b = O.build(O.Q2HEX, xyz, conn, em, ndof, rhs=orhs, bc_mask=mask, bc_val=val, b=b)
    eps = EPS_DFL if arith == ARITH_DFL else EPS
    compare_csr(g["mats"][0], csrK, ndof, what=f"q2 {kernel} K", eps=eps)
    compare_csr(g["mats"][1], csrM, ndof, what=f"q2 {kernel} M", eps=eps)
    assert_close(g["b"], b, what=f"q2 {kernel} b", eps=eps)


def test_q2_two_stiffness_operators(engine):
    """Q2 with two stiffness operators of different coefficients (no folding into G) and
    a combined stiffness + mass operator."""
    xyz, conn, k = problem("hex", 3, 0.2, seed=37, sigma=0.5)
    em, ndof = O.dofmap(O.Q2HEX, xyz.shape[0], conn)
    ops = [{"stiffness": 2, "stiff_coef": 0.75, "mass": 1, "mass_coef": 2.0}, {"stiffness": 1, "stiff_coef": 3.0}]
    g = gpu_assemble(O.Q2HEX, xyz, conn, ops, k=k)
    for op, mat in zip(ops, g["mats"]):
        csr, _ = O.build(O.Q2HEX, xyz, conn, em, ndof, lhs=oracle_lhs(op, k))
        compare_csr(mat, csr, ndof)


def test_fp64_rate_probe(engine):
    """pxg_fp64_rate: the measured FP64 FMA rate is positive and below the FP32 rate
    bound of the device (128 lanes x 2 flops per SM per clock, here as FMAs: 128 per SM
    per clock); on a GB300 it is 1/64 of that."""
    import torch

    from proxpde_gb300._lib import fp64_rate

    rate, ms = fp64_rate(0)
    p = torch.cuda.get_device_properties(0)
    bound = p.multi_processor_count * 128 * 2.2e9
    assert 0 < rate < bound and ms > 0


def test_red_rate_probe(engine):
    """pxg_red_rate: FP64 reductions per second by lane pattern, on an L2-resident array
    (32 MB) and a 1 GB one: positive, sectors shared by four lanes at least as fast per
    reduction as one lane per sector (the scatter's design rests on it), and bad
    arguments rejected."""
    from proxpde_gb300._lib import PxgError, red_rate

    for nbytes in (32 << 20, 1 << 30):
        r1, ms1 = red_rate(1, nbytes)
        r4, ms4 = red_rate(4, nbytes)
        assert r1 > 0 and r4 > 0 and ms1 > 0 and ms4 > 0
        assert r4 >= r1
    for bad in ((3, 32 << 20), (1, 3 << 20), (1, 1024)):
        with pytest.raises(PxgError):
            red_rate(*bad)
