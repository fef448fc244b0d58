"""Checks at the full sizes of the reference workloads:

- entry by entry against the oracle (threaded over the host's cores): the Q1 128^3
  K(k_e), M and sin3 load, the P2 64^3 x 6 K(k_e) and M, and the Q2 48^3 K(k_e), M
  and sin3 load, each in the default FP64
  arithmetic and in the opt-in double-float one, with the normwise and entrywise
  tolerances of tests/helpers.py (1e-12 relative to each entry above the round-off
  floor of its row);
- through properties that hold at any size: the Q1 128^3 stiffness + mass + sin load (the benchmark workload) and the P2 64^3
  (6 Kuhn tetrahedra per cell) stiffness + mass: DOF and nnz counts against closed
  forms, a sorted, structurally symmetric pattern with every diagonal, K 1 = 0
  (partition of unity), x^T K x = sum_e k_e vol_e for each coordinate function x and
  x^T K y = 0 (grad x is constant and reproduced exactly; the quadrature of |det J| is
  exact), 1^T M 1 = 1 and x^T M 1 = 1/2 (exact integrals over the unit cube, whose
  boundary stays flat), K and M symmetric, and the load vector's sum against a numpy
  quadrature at the reference's quadrature points;
- the Q1 96^3 adjoint gradient: the device solutions' residuals in the oracle's
  condensed matrix, the loss and the gradient kernel against the oracle at the same
  u and lambda, and a directional central difference;
- the 256-problem batch: batched gradients against the plain path, problem by problem.

Tolerances are written at each check.  x^T K x sums element forms of size k h^3 from
entries of size k h, so it loses log2(1/h^2) bits to cancellation: 1e-10 relative.
"""
import numpy as np
import pytest

import oracle as O
from helpers import (EPS, EPS_DFL, assert_close, compare_csr, gpu_assemble, nnz_p2_kuhn6, nnz_q1_cube, oracle_lhs,
                     q1_quadrature)

pytestmark = pytest.mark.gpu


def spmv(rows, cols, v, x):
    """y = A x for A given by its entries (rows, cols, v), on the device."""
    import torch

    return torch.zeros(x.shape[0], dtype=torch.float64, device=x.device).index_add_(0, rows, v * x[cols])


def pattern_checks(rp, ci, n):
    """Sorted rows, every diagonal present, structural symmetry (on the device)."""
    import torch

    rows = torch.repeat_interleave(torch.arange(n, device=ci.device), (rp[1:] - rp[:-1]).long())
    cols = ci.long()
    key = rows * n + cols
    assert bool((key[1:] > key[:-1]).all()), "rows not strictly increasing in column"
    assert int((rows == cols).sum()) == n, "a diagonal entry is missing"
    keyT, perm = torch.sort(cols * n + rows)
    assert torch.equal(keyT, key), "pattern not symmetric"
    return rows, cols, perm  # perm: position of entry (j, i) for entry (i, j), in CSR order


def symmetric_values(v, perm, tol):
    d = (v - v[perm]).abs().max().item()
    assert d <= tol * v.abs().max().item(), d


def dof_coordinates(t, xyz, conn, em, ndof):
    """Coordinates of the DOF points: vertices, and the edge midpoints of P2
    (local edges 01 12 20 03 13 23)."""
    X = np.empty((ndof, 3))
    nv = 4 if t in (O.P1TET, O.P2TET) else 8
    X[em[:, :nv].reshape(-1)] = xyz[conn[:, :nv].reshape(-1).astype(np.int64)]
    if t == O.P2TET:
        c = conn.astype(np.int64)
        for k, (a, b) in enumerate([(0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3)]):
            X[em[:, 4 + k]] = 0.5 * (xyz[c[:, a]] + xyz[c[:, b]])
    return X


def assemble_full(t, xyz, conn, k, rhs):
    import torch

    from proxpde_gb300 import Context

    ctx = Context(0)
    ctx.set_mesh(t, xyz, conn)
    ndof = ctx.build_dofmap()
    nnz = ctx.build_pattern()
    ctx.set_coef(k)
    K = torch.empty(nnz, dtype=torch.float64, device="cuda")
    M = torch.empty_like(K)
    b = torch.empty(ndof, dtype=torch.float64, device="cuda")
    ctx.assemble(op0={"stiffness": 2, "stiff_coef": 1.0}, vals0=K, op1={"mass": 1, "mass_coef": 1.0}, vals1=M,
                 rhs=rhs, b=b)
    rp, ci = ctx.get_pattern()
    em = ctx.get_dofmap()
    torch.cuda.synchronize()
    return ctx, ndof, nnz, torch.as_tensor(rp).cuda(), torch.as_tensor(ci).cuda(), K, M, b, em


def operator_checks(t, xyz, conn, k, ndof, rp, ci, K, M, em, kvol):
    import torch

    rows, cols, perm = pattern_checks(rp, ci, ndof)
    symmetric_values(K, perm, 1e-14)
    symmetric_values(M, perm, 1e-14)
    one = torch.ones(ndof, dtype=torch.float64, device="cuda")
    rowabs = spmv(rows, cols, K.abs(), one)
    k1 = spmv(rows, cols, K, one).abs().max().item()
    assert k1 <= 1e-12 * rowabs.max().item(), k1  # K 1 = 0
    X = torch.as_tensor(dof_coordinates(t, xyz, conn, em, ndof)).cuda() - 0.5
    for d in range(3):
        u = X[:, d].contiguous()
        Ku = spmv(rows, cols, K, u)
        q = float(u @ Ku)
        assert abs(q - kvol) <= 1e-10 * kvol, (d, q, kvol)  # x^T K x = sum k_e vol_e
        w = X[:, (d + 1) % 3]
        assert abs(float(w @ Ku)) <= 1e-10 * kvol  # x^T K y = 0
    M1 = spmv(rows, cols, M, one)
    m1 = float(M1.sum())
    assert abs(m1 - 1.0) <= 1e-12, m1  # 1^T M 1 = |cube|
    xm = float((X[:, 0] + 0.5) @ M1)
    assert abs(xm - 0.5) <= 1e-12, xm  # x^T M 1 = int x


def test_q1_128_cube(engine):
    """The benchmark workload: perturbed Q1 128^3, K(k_e) + M + sin3 load."""
    from proxpde_gb300 import meshgen

    n = 128
    xyz, conn = meshgen.cube_hex(n)
    xyz = meshgen.perturb(xyz, n, 0.2, 20261205)
    k = meshgen.lognormal(20261206, conn.shape[0], 1.0)
    ctx, ndof, nnz, rp, ci, K, M, b, em = assemble_full(O.Q1HEX, xyz, conn, k, {"kind": 1, "fn": O.FN_SIN3, "coef": 1.0})
    assert ndof == (n + 1) ** 3
    assert nnz == nnz_q1_cube(n) == 57_066_625
    vol, kvol, rsum = q1_quadrature(xyz, conn, k)
    assert abs(vol - 1.0) <= 1e-12
    operator_checks(O.Q1HEX, xyz, conn, k, ndof, rp, ci, K, M, em, kvol)
    bs = float(b.sum())
    assert abs(bs - rsum) <= 1e-12 * rsum, (bs, rsum)  # sin3 > 0 on the cube: no cancellation


def test_p2_64_cube(engine):
    """Perturbed P2 64^3 x 6 Kuhn tetrahedra, k_e lognormal(0, 0.5), K(k_e) + M + unit load."""
    from proxpde_gb300 import meshgen

    n = 64
    xyz, conn = meshgen.cube_tet6(n)
    xyz = meshgen.perturb(xyz, n, 0.15, 20261207)
    k = meshgen.lognormal(20261208, conn.shape[0], 0.5)
    ctx, ndof, nnz, rp, ci, K, M, b, em = assemble_full(O.P2TET, xyz, conn, k, {"kind": 1, "fn": O.FN_CONST, "coef": 1.0})
    assert conn.shape[0] == 1_572_864
    assert ndof == (2 * n + 1) ** 3
    assert nnz == nnz_p2_kuhn6(n) == 60_859_905
    X = xyz[conn.astype(np.int64)]
    vol = np.abs(np.linalg.det(X[:, 1:4] - X[:, :1])) / 6.0
    kvol = float((k * vol).sum())
    operator_checks(O.P2TET, xyz, conn, k, ndof, rp, ci, K, M, em, kvol)
    bs = float(b.sum())
    assert abs(bs - 1.0) <= 1e-12, bs  # sum of the load vector of f = 1 is the volume


def _threads():
    import os

    return max(1, len(os.sched_getaffinity(0)))


@pytest.mark.parametrize("arith", ["fp64", "dfl"])
def test_q1_128_entrywise(engine, arith):
    """The benchmark workload (perturbed Q1 128^3, K(k_e) + M + sin3 load) entry by entry
    against the oracle: the DOF map, the pruned CSR patterns and every value."""
    from proxpde_gb300 import meshgen
    from proxpde_gb300._lib import ARITH_DFL, ARITH_FP64

    n = 128
    xyz, conn = meshgen.cube_hex(n)
    xyz = meshgen.perturb(xyz, n, 0.2, 20261205)
    k = meshgen.lognormal(20261206, conn.shape[0], 1.0)
    ops = [{"stiffness": 2, "stiff_coef": 1.0}, {"mass": 1, "mass_coef": 1.0}]
    rhs = {"kind": 1, "fn": O.FN_SIN3, "coef": 1.0}
    g = gpu_assemble(O.Q1HEX, xyz, conn, ops, rhs=rhs, k=k, arith=ARITH_DFL if arith == "dfl" else ARITH_FP64)
    em, ndof = O.dofmap(O.Q1HEX, xyz.shape[0], conn)
    assert ndof == g["ndof"] and np.array_equal(em, g["em"])
    nt = _threads()
    for m, op in enumerate(ops):
        csr, _ = O.build(O.Q1HEX, xyz, conn, em, ndof, lhs=oracle_lhs(op, k), nthreads=nt)
        compare_csr(g["mats"][m], csr, ndof, what=f"q1 128^3 {arith} {'KM'[m]}", eps=EPS_DFL if arith == "dfl" else EPS)
        del csr
    _, b = O.build(O.Q1HEX, xyz, conn, em, ndof, rhs={"kind": 1, "fn": O.FN_SIN3, "c": 1.0}, nthreads=nt)
    assert_close(g["b"], b, what=f"q1 128^3 {arith} b", eps=EPS_DFL if arith == "dfl" else EPS)


@pytest.mark.parametrize("arith", ["fp64", "dfl"])
def test_p2_64_entrywise(engine, arith):
    """Perturbed P2 64^3 x 6 Kuhn tetrahedra, K(k_e) + M, entry by entry against the
    oracle."""
    from proxpde_gb300 import meshgen
    from proxpde_gb300._lib import ARITH_DFL, ARITH_FP64

    n = 64
    xyz, conn = meshgen.cube_tet6(n)
    xyz = meshgen.perturb(xyz, n, 0.15, 20261207)
    k = meshgen.lognormal(20261208, conn.shape[0], 0.5)
    ops = [{"stiffness": 2, "stiff_coef": 1.0}, {"mass": 1, "mass_coef": 1.0}]
    g = gpu_assemble(O.P2TET, xyz, conn, ops, k=k, arith=ARITH_DFL if arith == "dfl" else ARITH_FP64)
    em, ndof = O.dofmap(O.P2TET, xyz.shape[0], conn)
    assert ndof == g["ndof"] and np.array_equal(em, g["em"])
    nt = _threads()
    for m, op in enumerate(ops):
        csr, _ = O.build(O.P2TET, xyz, conn, em, ndof, lhs=oracle_lhs(op, k), nthreads=nt)
        compare_csr(g["mats"][m], csr, ndof, what=f"p2 64^3x6 {arith} {'KM'[m]}", eps=EPS_DFL if arith == "dfl" else EPS)
        del csr


@pytest.mark.parametrize("arith", ["fp64", "dfl"])
def test_q2_48_entrywise(engine, arith):
    """The Q2 workload (perturbed Q2 48^3, K(k_e) + M + sin3 load: 110,592 elements,
    57 M structural entries) entry by entry against the oracle: the DOF map, the pruned
    CSR patterns and every value."""
    from proxpde_gb300 import meshgen
    from proxpde_gb300._lib import ARITH_DFL, ARITH_FP64

    n = 48
    xyz, conn = meshgen.cube_hex(n)
    xyz = meshgen.perturb(xyz, n, 0.2, 20261209)
    k = meshgen.lognormal(20261210, conn.shape[0], 1.0)
    ops = [{"stiffness": 2, "stiff_coef": 1.0}, {"mass": 1, "mass_coef": 1.0}]
    rhs = {"kind": 1, "fn": O.FN_SIN3, "coef": 1.0}
    g = gpu_assemble(O.Q2HEX, xyz, conn, ops, rhs=rhs, k=k, arith=ARITH_DFL if arith == "dfl" else ARITH_FP64)
    em, ndof = O.dofmap(O.Q2HEX, xyz.shape[0], conn)
    assert ndof == g["ndof"] and np.array_equal(em, g["em"])
    nt = _threads()
    eps = EPS_DFL if arith == "dfl" else EPS
    for m, op in enumerate(ops):
        csr, _ = O.build(O.Q2HEX, xyz, conn, em, ndof, lhs=oracle_lhs(op, k), nthreads=nt)
        compare_csr(g["mats"][m], csr, ndof, what=f"q2 48^3 {arith} {'KM'[m]}", eps=eps)
        del csr
    _, b = O.build(O.Q2HEX, xyz, conn, em, ndof, rhs={"kind": 1, "fn": O.FN_SIN3, "c": 1.0}, nthreads=nt)
    assert_close(g["b"], b, what=f"q2 48^3 {arith} b", eps=eps)


def test_q1_96_adjoint(engine):
    """The differentiation workload at full size (884,736 elements)."""
    import torch

    from proxpde_gb300 import meshgen
    from proxpde_gb300.adjoint import DiffusionProblem

    n = 96
    P = DiffusionProblem.cube_q1(n, rtol=1e-10)
    k = meshgen.lognormal(20261208, P.nelem, 1.0)
    P.ctx.set_coef(k)
    u = torch.empty(P.ndof, dtype=torch.float64, device="cuda")
    lam = torch.empty_like(u)
    g = torch.empty(P.nelem, dtype=torch.float64, device="cuda")
    J, itf = P.ctx.adjoint_forward(P.rhs, P.ut, 1e-10, 50000, u_out=u)
    itb = P.ctx.adjoint_backward(g, 1.0, lam_out=lam)
    torch.cuda.synchronize()
    assert itf > 0 and itb > 0
    # the oracle's system on the same mesh and DOF map
    xyz, conn = meshgen.cube_hex(n)
    xyz = meshgen.perturb(xyz, n, 0.2, 20261207)
    em, ndof = O.dofmap(O.Q1HEX, xyz.shape[0], conn)
    assert np.array_equal(em, P.ctx.get_dofmap()) and ndof == P.ndof
    mask = P.bc_mask
    Kc, b = O.build(O.Q1HEX, xyz, conn, em, ndof, lhs={"stiff_kind": 2, "k_e": k, "apply_bc": 1},
                    rhs={"kind": 1, "fn": O.FN_CONST, "c": 1.0, "apply_bc": 1}, bc_mask=mask, bc_val=np.zeros(ndof),
                    nthreads=8)
    Mc, _ = O.build(O.Q1HEX, xyz, conn, em, ndof, lhs={"mass_kind": 1, "mass_c": 1.0}, nthreads=8)
    K, M = O.csr_to_scipy(Kc, ndof), O.csr_to_scipy(Mc, ndof)
    ut = O.interpolate(O.Q1HEX, xyz, conn, em, ndof, O.FN_SIN3)
    uh, lh, gh = u.cpu().numpy(), lam.cpu().numpy(), g.cpu().numpy()
    # the device solves, measured in the oracle's matrix: the CG stops at 1e-10 on its
    # recursive residual; the true residual in the oracle's matrix adds the entry
    # differences times ||K|| ||u|| / ||b|| (~1e4 here)
    assert np.linalg.norm(K @ uh - b) <= 1e-8 * np.linalg.norm(b)
    w = uh - ut
    Mw = M @ w
    assert np.linalg.norm(K @ lh - Mw) <= 1e-8 * np.linalg.norm(Mw)
    # loss and gradient kernel at the same u, lambda
    Jo = 0.5 * float(w @ Mw)
    assert abs(J - Jo) <= 1e-12 * Jo, (J, Jo)
    go = O.adjoint_grad(O.Q1HEX, xyz, conn, em, k, mask, uh, lh, nthreads=8)
    assert np.linalg.norm(gh - go) <= 1e-10 * np.linalg.norm(go)
    # directional central difference along v = g / max|g| (step 1e-3 in log k: the CG's
    # 1e-10 tolerance swamps per-element differences of 1e-6 at this size)
    v = gh / np.abs(gh).max()
    d = 1e-3
    Js = []
    for sgn in (1.0, -1.0):
        P.ctx.set_coef(k * np.exp(sgn * d * v))
        Js.append(P.ctx.adjoint_forward(P.rhs, P.ut, 1e-12, 50000)[0])
    fd = (Js[0] - Js[1]) / (2 * d)
    dd = float(gh @ v)
    assert abs(fd - dd) <= 1e-4 * abs(dd), (fd, dd)


def test_batch_256_matches_plain(engine):
    """The batched workload at full size: 128 Q1 + 128 P1 cubes, n ~ U{8..48}."""
    import torch

    from proxpde_gb300 import batch
    from proxpde_gb300.adjoint import DiffusionLoss, DiffusionProblem

    probs = batch.make_problems()
    assert len(probs) == 256
    groups = [batch.Batch([p for p in probs if p["etype"] == O.Q1HEX]),
              batch.Batch([p for p in probs if p["etype"] == O.P1TET])]
    losses, _ = batch.batch_adjoint(groups)
    torch.cuda.synchronize()
    i = 0
    worst = 0.0
    for grp in groups:
        for q in range(grp.nprob):
            p = grp.problems[q]
            P = DiffusionProblem(p["etype"], p["xyz"], p["conn"], bc_nodes=p["bc_nodes"], rtol=1e-10)
            lk = torch.as_tensor(np.log(p["k"])).cuda().requires_grad_(True)
            J = DiffusionLoss.apply(lk, P)
            J.backward()
            gb, gp = grp.grad_of(q), lk.grad
            worst = max(worst, float(torch.linalg.norm(gb - gp) / torch.linalg.norm(gp)))
            Jv = float(J.detach())
            assert abs(float(losses[i]) - Jv) <= 1e-9 * abs(Jv)
            P.ctx.close()
            i += 1
    assert i == 256
    assert worst <= 1e-8, worst
