"""Scatter strategies and the autotuner: the element colouring is proper (no two
elements of a class share a vertex), the colour-ordered scatter matches the oracle for
every element type and is bitwise reproducible, every block-size variant matches the
oracle, the autotuner keeps a candidate that matches the oracle, and a batch assembled
with the colour-ordered scatter gives the same gradients."""
import numpy as np
import pytest

import oracle as O
from helpers import EPS, EPS_DFL, assert_close, compare_csr, gpu_assemble, oracle_lhs, problem

pytestmark = pytest.mark.gpu

K_OP = {"stiffness": 2, "stiff_coef": 1.0}
M_OP = {"mass": 1, "mass_coef": 1.0}
SIN3 = {"kind": 1, "fn": O.FN_SIN3, "coef": 1.0}
TYPES = [(O.P1TET, "tet6", 6), (O.P2TET, "tet5", 4), (O.Q1HEX, "hex", 7), (O.Q2HEX, "hex", 3)]
IDS = ["p1tet", "p2tet", "q1hex", "q2hex"]


def check_against_oracle(t, xyz, conn, k, g, eps=EPS):
    em, ndof = O.dofmap(t, xyz.shape[0], conn)
    for op, mat in zip([K_OP, M_OP], g["mats"]):
        csr, _ = O.build(t, xyz, conn, em, ndof, lhs=oracle_lhs(op, k), nthreads=4)
        compare_csr(mat, csr, ndof, eps=eps)
    _, b = O.build(t, xyz, conn, em, ndof, rhs={"kind": 1, "fn": O.FN_SIN3, "c": 1.0})
    assert_close(g["b"], b, what="rhs", eps=eps)


@pytest.mark.parametrize("t,gen,n", TYPES, ids=IDS)
def test_colouring_is_proper(engine, t, gen, n):
    from proxpde_gb300 import Context

    xyz, conn, _ = problem(gen, n, 0.1, seed=3)
    ctx = Context(0)
    ctx.set_mesh(t, xyz, conn)
    ncol, order, offs = ctx.colouring(with_order=True)
    assert 1 < ncol <= 128
    assert offs[0] == 0 and offs[-1] == conn.shape[0] and np.all(np.diff(offs) > 0)
    assert np.array_equal(np.sort(order), np.arange(conn.shape[0]))
    for c in range(ncol):
        cls = order[offs[c]:offs[c + 1]]
        assert np.all(np.diff(cls.astype(np.int64)) > 0)  # element order inside a class
        verts = conn[cls].reshape(-1)
        assert np.unique(verts).size == verts.size, f"class {c} has elements sharing a vertex"
    # built once per mesh, the same on a second query
    assert ctx.colouring()[0] == ncol


@pytest.mark.parametrize("t,gen,n", TYPES, ids=IDS)
def test_colour_scatter_matches_oracle_and_is_reproducible(engine, t, gen, n):
    from proxpde_gb300 import SCATTER_COLOUR

    xyz, conn, k = problem(gen, n, 0.15, seed=9, sigma=1.0)
    g1 = gpu_assemble(t, xyz, conn, [K_OP, M_OP], rhs=SIN3, k=k, scatter=SCATTER_COLOUR)
    check_against_oracle(t, xyz, conn, k, g1)
    g2 = gpu_assemble(t, xyz, conn, [K_OP, M_OP], rhs=SIN3, k=k, scatter=SCATTER_COLOUR)
    for a, b in zip(g1["struct_vals"], g2["struct_vals"]):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), "colour-ordered values differ between runs"
    assert np.array_equal(g1["b"].view(np.uint64), g2["b"].view(np.uint64))


@pytest.mark.parametrize("t,gen,n,threads,dfl", [(O.P1TET, "tet6", 6, 64, False), (O.P1TET, "tet6", 6, 256, False),
                                                 (O.P2TET, "tet5", 4, 64, False), (O.P2TET, "tet5", 4, 256, False),
                                                 (O.P2TET, "tet5", 4, 256, True),
                                                 (O.Q1HEX, "hex", 7, 64, False), (O.Q1HEX, "hex", 7, 128, False),
                                                 (O.Q1HEX, "hex", 7, 256, True), (O.Q1HEX, "hex", 7, 512, True)])
def test_block_size_variants_match_oracle(engine, t, gen, n, threads, dfl):
    """Every block size of the FP64 element kernels (and of the double-float ones,
    whose Q1 kernel has eight lanes per element) against the oracle."""
    from proxpde_gb300 import SCATTER_REDUCE
    from proxpde_gb300._lib import ARITH_DFL, ARITH_FP64

    xyz, conn, k = problem(gen, n, 0.15, seed=9, sigma=1.0)
    g = gpu_assemble(t, xyz, conn, [K_OP, M_OP], rhs=SIN3, k=k, scatter=SCATTER_REDUCE, threads=threads,
                     arith=ARITH_DFL if dfl else ARITH_FP64)
    check_against_oracle(t, xyz, conn, k, g, eps=EPS_DFL if dfl else EPS)


def test_bad_block_size_is_rejected(engine):
    from proxpde_gb300 import Context, PxgError

    xyz, conn, _ = problem("hex", 3)
    ctx = Context(0)
    ctx.set_mesh(O.Q1HEX, xyz, conn)
    with pytest.raises(PxgError):
        ctx.set_scatter(0, 96)
    with pytest.raises(PxgError):
        ctx.set_scatter(7, 0)


@pytest.mark.parametrize("t,gen,n", [(O.Q1HEX, "hex", 16), (O.P1TET, "tet6", 12)], ids=["q1hex", "p1tet"])
def test_autotune_keeps_a_correct_candidate(engine, t, gen, n):
    import torch

    from proxpde_gb300 import Context

    xyz, conn, k = problem(gen, n, 0.15, seed=4, sigma=1.0)
    ctx = Context(0)
    ctx.set_mesh(t, xyz, conn)
    ndof = ctx.build_dofmap()
    nnz = ctx.build_pattern()
    ctx.set_coef(k)
    rep = ctx.autotune(op0=K_OP, op1=M_OP, rhs=SIN3)
    assert rep["ncolours"] > 1
    nsizes = 2 if t == O.Q1HEX else 3  # block sizes of the element kernel
    assert len(rep["candidates"]) == 2 * nsizes  # x two scatters
    assert all(ms > 0 for _, _, ms in rep["candidates"])
    best = min(rep["candidates"], key=lambda c: c[2])
    assert (rep["threads"], rep["scatter"]) == best[:2]
    K = torch.empty(nnz, dtype=torch.float64, device="cuda")
    M = torch.empty_like(K)
    b = torch.empty(ndof, dtype=torch.float64, device="cuda")
    ctx.assemble(op0=K_OP, vals0=K, op1=M_OP, vals1=M, rhs=SIN3, b=b)
    em, _ = O.dofmap(t, xyz.shape[0], conn)
    rp, ci = ctx.get_pattern()
    for op, v in zip([K_OP, M_OP], [K, M]):
        csr, _ = O.build(t, xyz, conn, em, ndof, lhs=oracle_lhs(op, k), nthreads=4)
        import scipy.sparse as sp

        A = sp.csr_matrix((v.cpu().numpy(), ci, rp), shape=(ndof, ndof))
        B = sp.csr_matrix((csr[2], csr[1], csr[0]), shape=(ndof, ndof))
        assert abs(A - B).max() <= 1e-12 * abs(B).max()
    _, bo = O.build(t, xyz, conn, em, ndof, rhs={"kind": 1, "fn": O.FN_SIN3, "c": 1.0})
    assert_close(b.cpu().numpy(), bo, what="rhs")


def test_batch_with_colour_scatter(engine):
    """Colour-ordered assembly inside the captured batch graph: same gradients as the
    reduction scatter."""
    from proxpde_gb300 import SCATTER_COLOUR, batch

    probs = batch.make_problems(n_hex=3, n_tet=3, nmin=3, nmax=6, seed=41)
    B = [batch.Batch([p for p in probs if p["etype"] == O.Q1HEX]), batch.Batch([p for p in probs if p["etype"] == O.P1TET])]
    l1, _ = batch.batch_adjoint(B, rtol=1e-12)
    g1 = [b.grad.clone() for b in B]
    for b in B:
        b.ctx.set_scatter(SCATTER_COLOUR)
    for _ in range(2):  # capture, then replay
        l2, _ = batch.batch_adjoint(B, rtol=1e-12)
    for a, b in zip(g1, B):
        assert float((a - b.grad).norm() / a.norm()) <= 1e-10
    assert np.allclose(l1, l2, rtol=1e-10, atol=0)
