"""Shared helpers of the tests: synthetic problems, the engine path through the C ABI,
the oracle path, and the comparison rules.

Tolerance (values), for every entry of a matrix or vector:
  - normwise: |v_gpu - v_oracle| <= 1e-12 * max|v_oracle|;
  - entrywise: |v_gpu - v_oracle| <= 1e-12 * |v_oracle| + floor.  For a matrix entry
    (r, c) the floor is 512 eps * max(max|row r|, max|row c|) of the oracle's matrix:
    the entry is a sum over elements and quadrature points whose terms, for the SPD
    element matrices of stiffness and mass, add up in absolute value to at most
    sqrt(K_rr K_cc) <= that maximum (Cauchy-Schwarz), and a sum of n terms evaluated in
    two different orders can differ by 2 gamma_n times that (Higham, Accuracy and
    Stability of Numerical Algorithms, 2nd ed., section 4.2), with n (elements times
    points times components) below 256.  Entries formed without cancellation are held
    to 1e-12 of themselves; entries formed by cancellation to the round-off of their
    terms.  For vectors the floor is 64 eps * max|v_oracle|.  The opt-in double-float
    kernels carry a 48-bit significand: their tests widen the floor by 2^5
    (eps 2^-47), which the parameter `eps` of the comparisons sets.
The oracle computes in FP64 in the reference's order; the engine in the context's
arithmetic (FP64 by default) with a different summation order.  The CSR pattern
(row_ptr, col_idx) and the DOF map must be identical.  The largest entrywise relative
error of each comparison, over the entries above 1e-3 and above 1e-8 of their row's
largest, is recorded in ERRORS and printed at the end of the run.
"""
import numpy as np

import oracle as O
from proxpde_gb300 import meshgen

TOL = 1e-12
EPS = 2.220446049250313e-16
EPS_DFL = 2.0 ** -47  # the double-float kernels' significand (48 bits), with a bit to spare
ROUNDOFF_BAND = 64 * EPS
# largest entrywise relative error per named comparison (printed by conftest): over the
# entries above 1e-3 and above 1e-8 of their row's (vector's) largest
ERRORS = {}


def record_error(what, err3, err8):
    if what:
        a, b = ERRORS.get(what, (0.0, 0.0))
        ERRORS[what] = (max(a, float(err3)), max(b, float(err8)))


GEN = {"hex": meshgen.cube_hex, "tet5": meshgen.cube_tet5, "tet6": meshgen.cube_tet6}


def problem(gen, n, alpha=0.0, seed=1, sigma=None):
    xyz, conn = GEN[gen](n)
    if alpha:
        xyz = meshgen.perturb(xyz, n, alpha, seed)
    k = meshgen.lognormal(seed + 1, conn.shape[0], sigma) if sigma else None
    return xyz, conn, k


def gpu_assemble(t, xyz, conn, ops, rhs=None, k=None, bc=None, device=0, field=None, scatter=None, threads=0,
                 arith=None):
    """Run the engine through the C ABI. ops: list of up to two lhs op dicts; scatter /
    threads select the scatter strategy and the block size (None: defaults); arith the
    arithmetic of the element kernels (None: the default, FP64).
    Returns dict(em, ndof, pattern, mats=[(rp, col, val)], b)."""
    import torch

    from proxpde_gb300 import Context

    ctx = Context(device)
    if arith is not None:
        ctx.set_arithmetic(arith)
    ctx.set_mesh(t, xyz, conn)
    ndof = ctx.build_dofmap()
    nnz = ctx.build_pattern()
    if scatter is not None:
        ctx.set_scatter(scatter, threads)
    if k is not None:
        ctx.set_coef(np.ascontiguousarray(k))
    if bc is not None:
        dofs, vals = bc
        ctx.set_bc(dofs, vals, 1.0)
    dev = f"cuda:{device}"
    vals = [torch.empty(nnz, dtype=torch.float64, device=dev) for _ in ops]
    b = torch.empty(ndof, dtype=torch.float64, device=dev)
    if rhs is not None and rhs.get("kind") in (2, 3):
        rhs = dict(rhs)
        rhs["field"] = torch.as_tensor(np.ascontiguousarray(field, dtype=np.float64)).to(dev)
    ctx.assemble(op0=ops[0] if ops else None, vals0=vals[0] if ops else None,
                 op1=ops[1] if len(ops) > 1 else None, vals1=vals[1] if len(ops) > 1 else None,
                 rhs=rhs, b=b)
    mats = []
    for v in vals:
        rp = torch.empty(ndof + 1, dtype=torch.int32, device=dev)
        ci = torch.empty(nnz, dtype=torch.int32, device=dev)
        vo = torch.empty(nnz, dtype=torch.float64, device=dev)
        m = ctx.close_matrix(v, rp, ci, vo)
        mats.append((rp.cpu().numpy(), ci[:m].cpu().numpy(), vo[:m].cpu().numpy()))
    torch.cuda.synchronize()
    out = dict(ndof=ndof, nnz=nnz, em=ctx.get_dofmap(), pattern=ctx.get_pattern(), mats=mats, b=b.cpu().numpy(),
               ctx=ctx, struct_vals=[v.cpu().numpy() for v in vals])
    return out


def oracle_lhs(op, k):
    d = {"stiff_kind": op.get("stiffness", 0), "stiff_c": op.get("stiff_coef", 1.0), "mass_kind": op.get("mass", 0),
         "mass_c": op.get("mass_coef", 1.0), "apply_bc": op.get("apply_bc", 0)}
    if d["stiff_kind"] == 2:
        d["k_e"] = np.asarray(k) * op.get("stiff_coef", 1.0)
    if d["mass_kind"] == 2:
        d["m_e"] = np.asarray(k) * op.get("mass_coef", 1.0)
    return d


def structural_pattern(em, ndof):
    keys = np.unique((em[:, :, None].astype(np.int64) * ndof + em[:, None, :]).reshape(-1))
    rows, cols = keys // ndof, keys % ndof
    rp = np.zeros(ndof + 1, dtype=np.int64)
    np.add.at(rp, rows + 1, 1)
    return np.cumsum(rp).astype(np.int32), cols.astype(np.int32)


def assert_close(a, b, tol=TOL, what="", eps=EPS):
    """Normwise and entrywise agreement of two vectors (b the oracle's); returns the
    largest entrywise relative error over entries above 1e-8 of max|b|."""
    scale = max(np.abs(b).max(), 1e-300) if b.size else 1.0
    d = np.abs(a - b)
    err = d.max() if a.size else 0.0
    assert err <= tol * scale, f"{what}: max|diff| {err:.3e} > {tol:g} * {scale:.3e}"
    bad = d > tol * np.abs(b) + 64 * eps * scale
    assert not bad.any(), (f"{what}: {bad.sum()} entries beyond 1e-12 relative + round-off floor, e.g. index "
                           f"{np.argmax(bad)}: {a[np.argmax(bad)]!r} vs {b[np.argmax(bad)]!r}")
    rel = [float((d[bg] / np.abs(b[bg])).max()) if bg.any() else 0.0
           for bg in (np.abs(b) > 1e-3 * scale, np.abs(b) > 1e-8 * scale)]
    record_error(what, *rel)
    return rel[1]


def _row_absmax(rp, v):
    """max |v| per CSR row (0 for an empty row)."""
    out = np.zeros(rp.size - 1)
    nz = np.diff(rp) > 0
    if nz.any():
        out[nz] = np.maximum.reduceat(np.abs(v), rp[:-1][nz])
    return out


def _entrywise(gv, ov, rows, cols, rowmax, tol, what, eps):
    """The entrywise bound on aligned value arrays, and the recorded error figures."""
    d = np.abs(gv - ov)
    bound = tol * np.abs(ov) + 512 * eps * np.maximum(rowmax[rows], rowmax[cols])
    bad = d > bound
    if bad.any():
        k = int(np.argmax(bad))
        raise AssertionError(f"{what}: {int(bad.sum())} entries beyond 1e-12 relative + round-off floor, e.g. "
                             f"({rows[k]},{cols[k]}): {gv[k]!r} vs {ov[k]!r}, row max {rowmax[rows[k]]:.3e}")
    rel = [float((d[bg] / np.abs(ov[bg])).max()) if bg.any() else 0.0
           for bg in (np.abs(ov) > 1e-3 * rowmax[rows], np.abs(ov) > 1e-8 * rowmax[rows])]
    record_error(what, *rel)


def compare_csr(g, o, ndof, tol=TOL, what="", eps=EPS):
    """Compare a pruned engine CSR with the oracle's.

    Values: normwise and entrywise (see the module docstring), on the union of the two
    patterns.  Pattern: identical, except entries that are present on one side only
    AND whose value there is round-off (|v| <= 64 eps * max|row|): such entries are
    mathematically zero, and whether they clear closeMatrix's 1e-16 prune threshold
    depends on evaluation order.  Returns the number of such round-off entries."""
    import scipy.sparse as sp

    scale = np.abs(o[2]).max() if o[2].size else 1.0
    if np.array_equal(g[0], o[0]) and np.array_equal(g[1], o[1]):
        # identical patterns: the value arrays are aligned
        err = np.abs(g[2] - o[2]).max() if o[2].size else 0.0
        assert err <= tol * scale, f"values: max|diff| {err:.3e} > {tol:g} * {scale:.3e}"
        rows = np.repeat(np.arange(ndof), np.diff(o[0]))
        rowmax = np.maximum(_row_absmax(g[0], g[2]), _row_absmax(o[0], o[2]))
        _entrywise(g[2], o[2], rows, o[1], rowmax, tol, what, eps)
        return 0
    A = sp.csr_matrix((g[2], g[1], g[0]), shape=(ndof, ndof))
    B = sp.csr_matrix((o[2], o[1], o[0]), shape=(ndof, ndof))
    D = (A - B).tocoo()
    err = np.abs(D.data).max() if D.nnz else 0.0
    assert err <= tol * scale, f"values: max|diff| {err:.3e} > {tol:g} * {scale:.3e}"
    rowmax = np.maximum(_row_absmax(g[0], g[2]), _row_absmax(o[0], o[2]))
    # the union of the patterns, with both sides' values (0 where an entry is absent)
    U = (abs(A) + abs(B)).tocoo()
    gv = np.asarray(A[U.row, U.col]).ravel()
    ov = np.asarray(B[U.row, U.col]).ravel()
    _entrywise(gv, ov, U.row, U.col, rowmax, tol, what, eps)
    Pa = sp.csr_matrix((np.ones(g[1].size), g[1], g[0]), shape=(ndof, ndof))
    Pb = sp.csr_matrix((np.ones(o[1].size), o[1], o[0]), shape=(ndof, ndof))
    only = (Pa - Pb).tocoo()
    n_band = 0
    for r, c, s in zip(only.row, only.col, only.data):
        v = A[r, c] if s > 0 else B[r, c]
        assert abs(v) <= ROUNDOFF_BAND * rowmax[r], f"pattern differs at ({r},{c}) with |v|={abs(v):.3e}"
        n_band += 1
    return n_band


# ---------------------------------------------------------------- full-size properties
def nnz_q1_cube(n):
    """Structural nnz of Q1 hexahedra on an n^3 cube: the 1D count 3n + 1, cubed."""
    return (3 * n + 1) ** 3


def nnz_p2_kuhn6(n):
    """Structural nnz of P2 tetrahedra on an n^3 cube split into 6 Kuhn tetrahedra per
    cell (a cubic in n, fitted to brute-force counts and checked against them)."""
    return 230 * n ** 3 + 138 * n ** 2 + 24 * n + 1


# Q1 reference element: node n sits at lattice position (x, y, z) with the vertex order
# of the hexahedron (bottom face counter-clockwise, then the top face)
_HEX_NODES = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])


def q1_quadrature(xyz, conn, k=None, chunk=131072):
    """Per-mesh sums by the 2x2x2 Gauss rule on the trilinear map, in numpy:
    (sum_e vol_e, sum_e k_e vol_e, sum_e sum_q |det J_q| f(x_q)) with
    f = sin(pi x) sin(pi y) sin(pi z) at the reference's quadrature point
    x_q = (vertex average) + J_q xi_q (curfe.hpp:92-94, geo.hpp:721-728)."""
    g = 1.0 / np.sqrt(3.0)
    s = 2 * _HEX_NODES - 1                          # node signs, (8, 3)
    xi = s * g                                      # Gauss points in the node order, (8, 3)
    # dN_n/dxi_c at xi_q: s_nc / 8 * prod_{d != c} (1 + s_nd xi_qd)
    f1 = 1.0 + xi[:, None, :] * s[None, :, :]       # (q, n, d)
    dN = np.empty((8, 8, 3))
    for c in range(3):
        others = [d for d in range(3) if d != c]
        dN[:, :, c] = s[None, :, c] / 8.0 * f1[:, :, others[0]] * f1[:, :, others[1]]
    dN2 = dN.transpose(1, 0, 2).reshape(8, 24)     # (n, q * 3 + c)
    vol = kvol = rhs = 0.0
    for e0 in range(0, conn.shape[0], chunk):
        X = xyz[conn[e0:e0 + chunk].astype(np.int64)]           # (e, n, 3)
        J = (X.transpose(0, 2, 1) @ dN2).reshape(-1, 3, 8, 3)  # J[e, r, q, c]
        det = np.abs(J[:, 0, :, 0] * (J[:, 1, :, 1] * J[:, 2, :, 2] - J[:, 1, :, 2] * J[:, 2, :, 1])
                     - J[:, 0, :, 1] * (J[:, 1, :, 0] * J[:, 2, :, 2] - J[:, 1, :, 2] * J[:, 2, :, 0])
                     + J[:, 0, :, 2] * (J[:, 1, :, 0] * J[:, 2, :, 1] - J[:, 1, :, 1] * J[:, 2, :, 0]))  # (e, q)
        org = X.mean(axis=1)                                    # (e, 3)
        xq = org[:, :, None] + np.einsum("erqc,qc->erq", J, xi)  # (e, r, q)
        fq = np.prod(np.sin(np.pi * xq), axis=1)                # (e, q)
        ve = det.sum(axis=1)
        vol += ve.sum()
        if k is not None:
            kvol += (k[e0:e0 + chunk] * ve).sum()
        rhs += (det * fq).sum()
    return vol, kvol, rhs


def vector_load_field(n):
    """The projected vector field of the vector-load case (the C++ test writes the same)."""
    k = np.arange(n, dtype=np.float64)
    return np.sin(0.37 * k) + 0.1 * (np.arange(n) % 7)


def vector_load_expect(elem, xyz, conn, field):
    """Expected b of the vector-load case, block by block from the oracle's scalar loads.

    The case: on the unit cube, a 3-component P2 / Q2 space and a P1 / Q1 space behind
    it (offset 3 * ndof); BCEss on the bottom (y = 0, every component) and on the left
    (x = 0, components 0 and 2); buildRhs of AssemblyRhsAnalytic with functions (sin3,
    const, poisson_rhs) and coefficients (1, 2, -0.5) on components 0 and 2, plus
    AssemblyS2SProjection(0.7, field) of field components (2, 0) into blocks (0, 1);
    and buildRhs of AssemblyRhsAnalytic(const, 3) on the scalar space without BCs.
    Returns (b, masks of the three blocks)."""
    tv = O.Q2HEX if elem == "hex" else O.P2TET
    tp = O.Q1HEX if elem == "hex" else O.P1TET
    em, nd = O.dofmap(tv, xyz.shape[0], conn)
    emp, ndp = O.dofmap(tp, xyz.shape[0], conn)
    dx = O.dof_coords(tv, xyz, conn, em, nd)
    on_y0, on_x0 = O.plane_bc_mask(dx, [("y", 0.0)]), O.plane_bc_mask(dx, [("x", 0.0)])
    masks = [on_y0 | on_x0, on_y0, on_y0 | on_x0]
    zero = np.zeros(nd)

    def load(c, rhs):
        return O.build(tv, xyz, conn, em, nd, rhs=dict(rhs, apply_bc=1), bc_mask=masks[c], bc_val=zero)[1]

    fc = [field[c * nd:(c + 1) * nd] for c in range(3)]
    blocks = [
        load(0, {"kind": 1, "fn": O.FN_SIN3, "c": 1.0}) + load(0, {"kind": 2, "c": 0.7, "field": fc[2]}),
        load(1, {"kind": 2, "c": 0.7, "field": fc[0]}),
        load(2, {"kind": 1, "fn": O.FN_POISSON_RHS, "c": -0.5}),
        O.build(tp, xyz, conn, emp, ndp, rhs={"kind": 1, "fn": O.FN_CONST, "c": 3.0})[1],
    ]
    return np.concatenate(blocks), masks
