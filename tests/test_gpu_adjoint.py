"""Adjoint gradient of the diffusion loss (the differentiation configuration):
device Jacobi-CG against a direct solve, the GPU gradient against the gradient
assembled on the CPU from the oracle's element matrices (relative error <= 1e-8),
central finite differences (step 1e-6) on 64 seeded elements, and
torch.autograd.gradcheck of the forward/backward pair."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

import oracle as O
from helpers import problem

pytestmark = pytest.mark.gpu


def oracle_system(xyz, conn, k, bc_nodes, t=O.Q1HEX):
    """K (condensed), M, b and the target on the oracle, with the engine's DOF map."""
    em, ndof = O.dofmap(t, xyz.shape[0], conn)
    nv = conn.shape[1]
    node2dof = np.full(xyz.shape[0], -1, dtype=np.int64)
    node2dof[conn.reshape(-1).astype(np.int64)] = em[:, :nv].reshape(-1)
    mask = np.zeros(ndof, dtype=np.uint8)
    mask[node2dof[bc_nodes]] = 1
    K, b = O.build(t, xyz, conn, em, ndof, lhs={"stiff_kind": 2, "k_e": k, "apply_bc": 1},
                   rhs={"kind": 1, "fn": O.FN_CONST, "c": 1.0, "apply_bc": 1}, bc_mask=mask, bc_val=np.zeros(ndof))
    M, _ = O.build(t, xyz, conn, em, ndof, lhs={"mass_kind": 1, "mass_c": 1.0})
    ut = O.interpolate(t, xyz, conn, em, ndof, O.FN_SIN3)
    return em, ndof, mask, O.csr_to_scipy(K, ndof).tocsc(), O.csr_to_scipy(M, ndof), b, ut


def reference_gradient(xyz, conn, k, bc_nodes, t=O.Q1HEX):
    em, ndof, mask, K, M, b, ut = oracle_system(xyz, conn, k, bc_nodes, t)
    u = spla.spsolve(K, b)
    lam = spla.spsolve(K, M @ (u - ut))
    J = 0.5 * (u - ut) @ (M @ (u - ut))
    return J, O.adjoint_grad(t, xyz, conn, em, k, mask, u, lam, nthreads=4), u


def make(n, seed=31):
    from proxpde_gb300 import meshgen

    xyz, conn, k = problem("hex", n, 0.2, seed=seed, sigma=1.0)
    return xyz, conn, k, meshgen.boundary_nodes(n)


def test_cg_matches_direct_solve(engine):
    import torch

    from proxpde_gb300 import Context

    xyz, conn, k, bcn = make(10)
    em, ndof, mask, K, M, b, ut = oracle_system(xyz, conn, k, bcn)
    ctx = Context(0)
    ctx.set_mesh(O.Q1HEX, xyz, conn)
    ctx.build_dofmap()
    ctx.build_pattern()
    rp, ci = ctx.pattern_device()
    Kc = K.tocsr()
    Kc.sort_indices()
    # the oracle's closed matrix on the device (its own pattern)
    rp_t = torch.as_tensor(Kc.indptr.astype(np.int32)).cuda()
    ci_t = torch.as_tensor(Kc.indices.astype(np.int32)).cuda()
    v_t = torch.as_tensor(Kc.data).cuda()
    b_t = torch.as_tensor(b).cuda()
    x = torch.zeros(ndof, dtype=torch.float64, device="cuda")
    it, rel = ctx.cg(rp_t, ci_t, v_t, b_t, x, rtol=1e-13, max_iter=5000)
    assert rel <= 1e-13 and it > 0
    xr = spla.spsolve(K, b)
    assert np.linalg.norm(x.cpu().numpy() - xr) <= 1e-9 * np.linalg.norm(xr)


def test_gradient_matches_cpu_reference(engine):
    import torch

    from proxpde_gb300.adjoint import DiffusionLoss, DiffusionProblem

    xyz, conn, k, bcn = make(12)
    P = DiffusionProblem(O.Q1HEX, xyz, conn, bc_nodes=bcn, rtol=1e-12)
    logk = torch.as_tensor(np.log(k)).cuda().requires_grad_(True)
    J = DiffusionLoss.apply(logk, P)
    J.backward()
    Jr, gr, ur = reference_gradient(xyz, conn, k, bcn)
    assert abs(J.item() - Jr) <= 1e-9 * abs(Jr)
    g = logk.grad.cpu().numpy()
    assert np.linalg.norm(g - gr) <= 1e-8 * np.linalg.norm(gr), np.linalg.norm(g - gr) / np.linalg.norm(gr)
    assert P.iters[0] > 0 and P.iters[1] > 0


def test_gradient_finite_differences(engine):
    """Central differences of the discrete loss (step 1e-6 in log k_e) on 64 seeded
    elements: the losses use the engine's assembly with direct solves, the gradient
    is the engine's adjoint."""
    import torch

    from proxpde_gb300 import Context
    from proxpde_gb300.adjoint import DiffusionLoss, DiffusionProblem

    xyz, conn, k, bcn = make(8, seed=41)
    P = DiffusionProblem(O.Q1HEX, xyz, conn, bc_nodes=bcn, rtol=1e-13)
    logk = torch.as_tensor(np.log(k)).cuda().requires_grad_(True)
    DiffusionLoss.apply(logk, P).backward()
    g = logk.grad.cpu().numpy()

    em, ndof, mask, _, M, _, ut = oracle_system(xyz, conn, k, bcn)
    ctx = P.ctx
    nnz = ctx.nnz
    rph, cih = ctx.get_pattern()
    Kd = torch.empty(nnz, dtype=torch.float64, device="cuda")
    bd = torch.empty(ndof, dtype=torch.float64, device="cuda")

    def J_of(lk):
        ctx.set_coef(np.exp(lk))
        ctx.assemble(op0={"stiffness": 2, "stiff_coef": 1.0, "apply_bc": 1}, vals0=Kd,
                     rhs={"kind": 1, "fn": O.FN_CONST, "coef": 1.0, "apply_bc": 1}, b=bd)
        import scipy.sparse as sp

        A = sp.csr_matrix((Kd.cpu().numpy(), cih, rph), shape=(ndof, ndof)).tocsc()
        u = spla.spsolve(A, bd.cpu().numpy())
        w = u - ut
        return 0.5 * w @ (M @ w)

    rng = np.random.default_rng(20261208)
    sel = rng.choice(conn.shape[0], size=64, replace=False)
    lk0 = np.log(k)
    h = 1e-6
    fd = []
    for e in sel:
        lp, lm = lk0.copy(), lk0.copy()
        lp[e] += h
        lm[e] -= h
        fd.append((J_of(lp) - J_of(lm)) / (2 * h))
    fd = np.array(fd)
    err = np.abs(fd - g[sel]).max() / np.abs(g[sel]).max()
    assert err <= 1e-5, err


def test_autograd_gradcheck(engine):
    import torch

    from proxpde_gb300.adjoint import DiffusionLoss, DiffusionProblem

    xyz, conn, k, bcn = make(3, seed=5)
    P = DiffusionProblem(O.Q1HEX, xyz, conn, bc_nodes=bcn, rtol=1e-14, max_iter=2000)
    logk = torch.as_tensor(np.log(k)).cuda().requires_grad_(True)
    assert torch.autograd.gradcheck(lambda x: DiffusionLoss.apply(x, P), (logk,), eps=1e-6, atol=1e-9, rtol=1e-5)


@pytest.mark.parametrize("t,gen", [(O.P1TET, "tet6")])
def test_gradient_p1_tets(engine, t, gen):
    import torch

    from proxpde_gb300 import meshgen
    from proxpde_gb300.adjoint import DiffusionLoss, DiffusionProblem

    n = 4
    xyz, conn, k = problem(gen, n, 0.15, seed=9, sigma=1.0)
    bcn = meshgen.boundary_nodes(n)
    P = DiffusionProblem(t, xyz, conn, bc_nodes=bcn, rtol=1e-12)
    logk = torch.as_tensor(np.log(k)).cuda().requires_grad_(True)
    DiffusionLoss.apply(logk, P).backward()
    _, gr, _ = reference_gradient(xyz, conn, k, bcn, t)
    g = logk.grad.cpu().numpy()
    assert np.linalg.norm(g - gr) <= 1e-8 * np.linalg.norm(gr)


@pytest.mark.parametrize("t,gen", [(O.P1TET, "tet6"), (O.P2TET, "tet6"), (O.Q1HEX, "hex"), (O.Q2HEX, "hex")])
def test_gradient_kernel_all_types(engine, t, gen):
    """pxg_adjoint_grad on given u, lambda against the oracle's element-matrix formula."""
    import torch

    from proxpde_gb300 import Context

    xyz, conn, k = problem(gen, 3, 0.15, seed=13, sigma=1.0)
    ctx = Context(0)
    ctx.set_mesh(t, xyz, conn)
    ndof = ctx.build_dofmap()
    ctx.set_coef(k)
    em = ctx.get_dofmap()
    rng = np.random.default_rng(3)
    u, lam = rng.standard_normal(ndof), rng.standard_normal(ndof)
    mask = (rng.random(ndof) < 0.2).astype(np.uint8)
    dofs = np.nonzero(mask)[0].astype(np.uint32)
    ctx.set_bc(dofs, np.zeros(dofs.size))
    g = torch.empty(conn.shape[0], dtype=torch.float64, device="cuda")
    ctx.adjoint_grad(torch.as_tensor(u).cuda(), torch.as_tensor(lam).cuda(), g)
    gr = O.adjoint_grad(t, xyz, conn, em, k, mask, u, lam)
    assert np.abs(g.cpu().numpy() - gr).max() <= 1e-12 * np.abs(gr).max()
