"""Batches of independent diffusion problems (the batched adjoint configuration).

A batch of one element type is the disjoint union of its problems in one engine
context (elements grouped by problem, node ids offset), marked with pxg_batch_set.
`batch_adjoint` runs pxg_batch_adjoint over one or two batches: assembly of K(k),
M and b for every problem, forward and adjoint CG of all problems in one persistent
kernel, the gradient kernel, all captured in one CUDA graph.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import meshgen
from ._lib import FN_CONST, FN_SIN3, P1TET, Q1HEX, Context, PxgError, RhsOp, _ptr


def problem_sizes(n_hex=128, n_tet=128, nmin=8, nmax=48, seed=20261209):
    """The seeded cube size n ~ U{nmin..nmax} of every problem (hexahedra first)."""
    return nmin + (meshgen.splitmix64(seed, np.arange(n_hex + n_tet)) % np.uint64(nmax - nmin + 1)).astype(np.int64)


def shard(sizes, n_hex, rank, world):
    """The problems of `rank` when a batch is split over `world` ranks (one GPU each):
    independent problems, so no exchange between the ranks.  Largest first, each to
    the rank with the least work so far; the work of a problem is its nonzeros (27 per
    row for Q1 hexahedra, 15 for P1 tetrahedra, (n + 1)^3 rows) times n, as the CG
    iterations grow with n.  Returns ascending problem indices."""
    sizes = np.asarray(sizes, dtype=np.int64)
    cost = np.where(np.arange(sizes.size) < n_hex, 27.0, 15.0) * (sizes + 1.0) ** 3 * sizes
    load = np.zeros(world)
    owner = np.empty(sizes.size, dtype=np.int64)
    for p in sorted(range(sizes.size), key=lambda q: (-cost[q], q)):
        r = int(np.argmin(load))
        owner[p] = r
        load[r] += cost[p]
    return np.nonzero(owner == rank)[0]


def make_problems(n_hex=128, n_tet=128, nmin=8, nmax=48, alpha=0.2, seed=20261209, only=None):
    """Seeded problems: cube sizes n ~ U{nmin..nmax}; Q1 hexahedra first, then P1
    tetrahedra (6 per cube); nodes perturbed by U(-alpha h, alpha h); k_e = exp(N(0,1)).
    `only`: the indices of the problems to build (a rank's shard), default all."""
    sizes = problem_sizes(n_hex, n_tet, nmin, nmax, seed)
    keep = set(range(sizes.size)) if only is None else {int(q) for q in only}
    probs = []
    for p, n in enumerate(sizes.tolist()):
        if p not in keep:
            continue
        hexa = p < n_hex
        xyz, conn = meshgen.cube_hex(n) if hexa else meshgen.cube_tet6(n)
        xyz = meshgen.perturb(xyz, n, alpha, seed + 1 + 7 * p)
        k = meshgen.lognormal(seed + 2 + 7 * p, conn.shape[0], 1.0)
        probs.append({"etype": Q1HEX if hexa else P1TET, "n": n, "xyz": xyz, "conn": conn, "k": k,
                      "bc_nodes": meshgen.boundary_nodes(n)})
    return probs


class Batch:
    """The problems of one element type as one context."""

    def __init__(self, problems, device=0):
        assert problems and len({p["etype"] for p in problems}) == 1
        self.problems = problems
        self.etype = problems[0]["etype"]
        self.dev = f"cuda:{device}"
        xyzs, conns, ks, bcs, eoff = [], [], [], [], [0]
        node0 = 0
        for p in problems:
            xyzs.append(p["xyz"])
            conns.append(p["conn"].astype(np.int64) + node0)
            ks.append(p["k"])
            bcs.append(p["bc_nodes"] + node0)
            node0 += p["xyz"].shape[0]
            eoff.append(eoff[-1] + p["conn"].shape[0])
        self.xyz = np.ascontiguousarray(np.concatenate(xyzs))
        self.conn = np.ascontiguousarray(np.concatenate(conns).astype(np.uint32))
        self.k = np.ascontiguousarray(np.concatenate(ks))
        self.elem_off = np.array(eoff, dtype=np.int64)
        self.nprob = len(problems)
        self.nelem = self.conn.shape[0]
        ctx = self.ctx = Context(device)
        ctx.set_mesh(self.etype, self.xyz, self.conn)
        self.ndof = ctx.build_dofmap()
        self.nnz = ctx.build_pattern()
        st = ctx.L.pxg_batch_set(ctx.h, self.elem_off.ctypes.data_as(C.POINTER(C.c_int64)), self.nprob)
        ctx._check(st, "batch_set")
        em = ctx.get_dofmap()
        nv = self.conn.shape[1]
        node2dof = np.full(self.xyz.shape[0], -1, dtype=np.int64)
        node2dof[self.conn.reshape(-1).astype(np.int64)] = em[:, :nv].reshape(-1)
        dofs = np.unique(node2dof[np.concatenate(bcs)])
        ctx.set_bc(dofs.astype(np.uint32), np.zeros(dofs.size), 1.0)
        ctx.set_coef(self.k)
        self.ut = torch.zeros(self.ndof, dtype=torch.float64, device=self.dev)
        ctx.interpolate(FN_SIN3, 1.0, self.ut)
        self.grad = torch.zeros(self.nelem, dtype=torch.float64, device=self.dev)

    def grad_of(self, p):
        return self.grad[int(self.elem_off[p]):int(self.elem_off[p + 1])]


def batch_adjoint(batches, rtol=1e-10, max_iter=20000, use_graph=True, rhs=None, stream=None):
    """One call over all batches: returns (losses per problem, largest CG iteration count)."""
    rhs = rhs if rhs is not None else {"kind": 1, "fn": FN_CONST, "coef": 1.0}
    L = batches[0].ctx.L
    nb = len(batches)
    ctxs = (C.c_void_p * nb)(*[b.ctx.h.value for b in batches])
    uts = (C.c_void_p * nb)(*[b.ut.data_ptr() for b in batches])
    grads = (C.c_void_p * nb)(*[b.grad.data_ptr() for b in batches])
    nprob = sum(b.nprob for b in batches)
    losses = (C.c_double * nprob)()
    it = C.c_int()
    r = RhsOp(int(rhs.get("kind", 1)), int(rhs.get("fn", 0)), float(rhs.get("coef", 1.0)), _ptr(rhs.get("field")), 1)
    st = L.pxg_batch_adjoint(ctxs, nb, C.byref(r), uts, float(rtol), int(max_iter), losses, grads, C.byref(it),
                             1 if use_graph else 0, stream)
    if st != 0:
        raise PxgError(st, "batch_adjoint: " + L.pxg_last_error(batches[0].ctx.h).decode())
    return np.array(losses[:]), it.value
