"""Differentiable diffusion loss on the GPU engine.

    J(log k) = 1/2 (u - u_t)^T M (u - u_t),   K(k) u = b,   k_e = exp(log k_e)

with K the stiffness of a per-element coefficient (AssemblyStiffnessFE), homogeneous
or inhomogeneous essential BCs, M the mass matrix and b a load term.  Forward and
backward are the engine's C-ABI pair pxg_adjoint_forward / pxg_adjoint_backward
(device Jacobi-CG solves, adjoint gradient kernel); `DiffusionLoss` gives them the
torch.autograd.Function interface.
"""
from __future__ import annotations

import numpy as np
import torch

from . import meshgen
from ._lib import FN_CONST, FN_SIN3, Q1HEX, Context


class DiffusionProblem:
    """Mesh + DOF map + pattern + BCs + target on one GPU context."""

    def __init__(self, etype, xyz, conn, bc_nodes=None, fn_target=FN_SIN3, rhs=None, rtol=1e-10, max_iter=50000,
                 device=0):
        self.dev = f"cuda:{device}"
        self.ctx = Context(device)
        self.ctx.set_mesh(etype, xyz, conn)
        self.ndof = self.ctx.build_dofmap()
        self.nnz = self.ctx.build_pattern()
        self.nelem = conn.shape[0]
        self.bc_mask = np.zeros(self.ndof, dtype=np.uint8)
        if bc_nodes is not None and len(bc_nodes):
            em = self.ctx.get_dofmap()
            nv = conn.shape[1]
            node2dof = np.full(xyz.shape[0], -1, dtype=np.int64)
            node2dof[conn.reshape(-1).astype(np.int64)] = em[:, :nv].reshape(-1)
            dofs = np.unique(node2dof[np.asarray(bc_nodes, dtype=np.int64)])
            self.ctx.set_bc(dofs.astype(np.uint32), np.zeros(dofs.size), 1.0)
            self.bc_mask[dofs] = 1
        self.ut = torch.zeros(self.ndof, dtype=torch.float64, device=self.dev)
        self.ctx.interpolate(fn_target, 1.0, self.ut)
        self.rhs = rhs if rhs is not None else {"kind": 1, "fn": FN_CONST, "coef": 1.0}
        self.rtol, self.max_iter = rtol, max_iter
        self.u = torch.zeros(self.ndof, dtype=torch.float64, device=self.dev)
        self.iters = (0, 0)

    @classmethod
    def cube_q1(cls, n, alpha=0.2, seed=20261207, **kw):
        """The config-4 problem class: perturbed Q1 cube, Dirichlet on all six faces."""
        xyz, conn = meshgen.cube_hex(n)
        xyz = meshgen.perturb(xyz, n, alpha, seed)
        return cls(Q1HEX, xyz, conn, bc_nodes=meshgen.boundary_nodes(n), **kw)

    def loss(self, log_k):
        """J only (no gradient state is needed by the caller)."""
        return DiffusionLoss.apply(log_k, self)


class DiffusionLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, log_k, problem):
        k = torch.exp(log_k.detach()).contiguous()
        problem.ctx.set_coef(k)
        J, it = problem.ctx.adjoint_forward(problem.rhs, problem.ut, problem.rtol, problem.max_iter, u_out=problem.u)
        problem.iters = (it, 0)
        ctx.problem = problem
        return torch.tensor(J, dtype=torch.float64, device=log_k.device)

    @staticmethod
    def backward(ctx, grad_out):
        p = ctx.problem
        g = torch.empty(p.nelem, dtype=torch.float64, device=p.dev)
        it = p.ctx.adjoint_backward(g, dloss=float(grad_out))
        p.iters = (p.iters[0], it)
        return g, None
