"""CPU oracle for the proxpde assembly path (test infrastructure only).

This package wraps ``oracle/oracle.cpp`` (a plain C++ restatement of proxpde's
``Builder::buildLhs/buildRhs/closeMatrix`` element loop, see the header of that file
for the file:line of every restated piece) with ctypes.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` use it, to check
results and to time the CPU baseline.  The GPU engine in ``proxpde_gb300`` never
imports it.

The helpers ``poisson_*`` re-run the reference's own golden tests on the oracle:
build mesh -> DOF map -> BCs -> assemble -> direct solve -> ||u - I_h u||_2.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")

P1TET, P2TET, Q1HEX, Q2HEX = 0, 1, 2, 3
NAMES = {P1TET: "p1tet", P2TET: "p2tet", Q1HEX: "q1hex", Q2HEX: "q2hex"}

# analytic functions known to the oracle (and, by the same ids, to the engine)
FN_CONST, FN_SIN3, FN_POISSON_RHS, FN_POISSON_EXACT = 0, 1, 2, 3


class OrcLhs(C.Structure):
    _fields_ = [
        ("stiff_kind", C.c_int32),
        ("stiff_c", C.c_double),
        ("k_e", C.POINTER(C.c_double)),
        ("mass_kind", C.c_int32),
        ("mass_c", C.c_double),
        ("apply_bc", C.c_int32),
        ("m_e", C.POINTER(C.c_double)),
    ]


class OrcRhs(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("fn", C.c_int32),
        ("c", C.c_double),
        ("field", C.POINTER(C.c_double)),
        ("apply_bc", C.c_int32),
    ]


def build_lib(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile beside this file."""
    src = os.path.join(_HERE, "oracle.cpp")
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_lib()
        L = C.CDLL(_LIB)
        dp = C.POINTER(C.c_double)
        up = C.POINTER(C.c_uint32)
        i32p = C.POINTER(C.c_int32)
        u8p = C.POINTER(C.c_uint8)
        L.orc_num_dofs.argtypes = [C.c_int]
        L.orc_num_verts.argtypes = [C.c_int]
        L.orc_num_qpts.argtypes = [C.c_int]
        L.orc_quadrature.argtypes = [C.c_int, dp, dp]
        L.orc_shape.argtypes = [C.c_int, dp, dp, dp]
        L.orc_cube_hex.argtypes = [C.c_int, dp, up]
        L.orc_cube_hex.restype = C.c_int64
        L.orc_cube_tet5.argtypes = [C.c_int, dp, up]
        L.orc_cube_tet5.restype = C.c_int64
        L.orc_dofmap.argtypes = [C.c_int, C.c_int64, up, C.c_int64, up]
        L.orc_dofmap.restype = C.c_int64
        L.orc_dof_coords.argtypes = [C.c_int, dp, up, C.c_int64, up, dp]
        L.orc_interpolate.argtypes = [C.c_int, dp, up, C.c_int64, up, C.c_int, C.c_double, dp]
        L.orc_qpoints.argtypes = [C.c_int, dp, up, C.c_int64, dp]
        L.orc_element.argtypes = [C.c_int, dp, up, C.c_int64, C.POINTER(OrcLhs), C.POINTER(OrcRhs), up, dp, dp]
        L.orc_build.argtypes = [
            C.c_int, dp, up, C.c_int64, up, C.c_int64, C.POINTER(OrcLhs), C.POINTER(OrcRhs),
            u8p, dp, C.c_double, C.c_int, dp,
        ]
        L.orc_build.restype = C.c_void_p
        L.orc_csr_nnz.argtypes = [C.c_void_p]
        L.orc_csr_nnz.restype = C.c_int64
        L.orc_csr_copy.argtypes = [C.c_void_p, i32p, i32p, dp]
        L.orc_csr_free.argtypes = [C.c_void_p]
        L.orc_adjoint_grad.argtypes = [C.c_int, dp, up, C.c_int64, up, dp, u8p, dp, dp, C.c_int, dp]
        vp = C.c_void_p
        L.orc_system_call.argtypes = [vp, C.c_int, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, C.c_double, dp, up,
                                      C.c_int64, C.c_int, vp, vp, dp]
        L.orc_system_call.restype = vp
        L.orc_system_close.argtypes = [vp, C.c_int64]
        L.orc_system_close.restype = vp
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t)) if a is not None else None


def _dp(a):
    return _p(a, C.c_double)


def _up(a):
    return _p(a, C.c_uint32)


def num_dofs(t):
    return lib().orc_num_dofs(t)


def num_verts(t):
    return lib().orc_num_verts(t)


def quadrature(t):
    n = lib().orc_num_qpts(t)
    nodes = np.zeros((n, 3))
    w = np.zeros(n)
    lib().orc_quadrature(t, _dp(nodes), _dp(w))
    return nodes, w


def shape(t, p):
    N = num_dofs(t)
    phi = np.zeros(N)
    dphi = np.zeros((N, 3))
    lib().orc_shape(t, _dp(np.ascontiguousarray(p, dtype=np.float64)), _dp(phi), _dp(dphi))
    return phi, dphi


def cube_hex(n):
    xyz = np.zeros(((n + 1) ** 3, 3))
    conn = np.zeros((n ** 3, 8), dtype=np.uint32)
    lib().orc_cube_hex(n, _dp(xyz), _up(conn))
    return xyz, conn


def cube_tet5(n):
    xyz = np.zeros(((n + 1) ** 3, 3))
    conn = np.zeros((5 * n ** 3, 4), dtype=np.uint32)
    lib().orc_cube_tet5(n, _dp(xyz), _up(conn))
    return xyz, conn


def dofmap(t, nnodes, conn):
    conn = np.ascontiguousarray(conn, dtype=np.uint32)
    E = conn.shape[0]
    em = np.zeros((E, num_dofs(t)), dtype=np.uint32)
    ndof = lib().orc_dofmap(t, nnodes, _up(conn), E, _up(em))
    return em, int(ndof)


def dof_coords(t, xyz, conn, em, ndof):
    out = np.zeros((ndof, 3))
    lib().orc_dof_coords(t, _dp(np.ascontiguousarray(xyz)), _up(np.ascontiguousarray(conn, dtype=np.uint32)),
                         conn.shape[0], _up(np.ascontiguousarray(em, dtype=np.uint32)), _dp(out))
    return out


def qpoints(t, xyz, conn):
    """CurFE::qpoint of every element and quadrature point, (nelem, nq, 3)."""
    conn = np.ascontiguousarray(conn, dtype=np.uint32)
    nq = lib().orc_num_qpts(t)
    out = np.zeros((conn.shape[0], nq, 3))
    lib().orc_qpoints(t, _dp(np.ascontiguousarray(xyz)), _up(conn), conn.shape[0], _dp(out))
    return out


def interpolate(t, xyz, conn, em, ndof, fn, c=1.0):
    v = np.zeros(ndof)
    lib().orc_interpolate(t, _dp(np.ascontiguousarray(xyz)), _up(np.ascontiguousarray(conn, dtype=np.uint32)),
                          conn.shape[0], _up(np.ascontiguousarray(em, dtype=np.uint32)), fn, c, _dp(v))
    return v


def _lhs(lhs, keep):
    if lhs is None:
        return None
    k_e, m_e = lhs.get("k_e"), lhs.get("m_e")
    if k_e is not None:
        k_e = np.ascontiguousarray(k_e, dtype=np.float64)
        keep.append(k_e)
    if m_e is not None:
        m_e = np.ascontiguousarray(m_e, dtype=np.float64)
        keep.append(m_e)
    s = OrcLhs(int(lhs.get("stiff_kind", 0)), float(lhs.get("stiff_c", 0.0)), _dp(k_e),
               int(lhs.get("mass_kind", 0)), float(lhs.get("mass_c", 0.0)), int(lhs.get("apply_bc", 0)), _dp(m_e))
    return C.pointer(s)


def _rhs(rhs, keep):
    if rhs is None:
        return None
    f = rhs.get("field")
    if f is not None:
        f = np.ascontiguousarray(f, dtype=np.float64)
        keep.append(f)
    s = OrcRhs(int(rhs.get("kind", 0)), int(rhs.get("fn", 0)), float(rhs.get("c", 1.0)), _dp(f),
               int(rhs.get("apply_bc", 0)))
    return C.pointer(s)


def element(t, xyz, conn, e, lhs=None, rhs=None, em=None):
    N = num_dofs(t)
    keep = []
    Ke = np.zeros((N, N)) if lhs is not None else None
    Fe = np.zeros(N) if rhs is not None else None
    lib().orc_element(t, _dp(np.ascontiguousarray(xyz)), _up(np.ascontiguousarray(conn, dtype=np.uint32)), e,
                      _lhs(lhs, keep), _rhs(rhs, keep),
                      _up(np.ascontiguousarray(em, dtype=np.uint32)) if em is not None else None,
                      _dp(Ke), _dp(Fe))
    return Ke, Fe


def build(t, xyz, conn, em, ndof, lhs=None, rhs=None, bc_mask=None, bc_val=None, bc_diag=1.0,
          nthreads=1, b=None):
    """Builder::buildLhs(lhs) + buildRhs(rhs) + closeMatrix() on one matrix and one vector.

    Returns ((row_ptr, col, val) or None, b)."""
    keep = []
    if b is None:
        b = np.zeros(ndof)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.uint32)
    em = np.ascontiguousarray(em, dtype=np.uint32)
    m = None
    if bc_mask is not None:
        m = np.ascontiguousarray(bc_mask, dtype=np.uint8)
        bc_val = np.ascontiguousarray(bc_val if bc_val is not None else np.zeros(ndof), dtype=np.float64)
    h = lib().orc_build(t, _dp(xyz), _up(conn), conn.shape[0], _up(em), ndof, _lhs(lhs, keep), _rhs(rhs, keep),
                        _p(m, C.c_uint8), _dp(bc_val) if m is not None else None, bc_diag, nthreads, _dp(b))
    csr = None
    if h:
        nnz = lib().orc_csr_nnz(h)
        rp = np.zeros(ndof + 1, dtype=np.int32)
        col = np.zeros(nnz, dtype=np.int32)
        val = np.zeros(nnz)
        lib().orc_csr_copy(h, _p(rp, C.c_int32), _p(col, C.c_int32), _dp(val))
        lib().orc_csr_free(h)
        csr = (rp, col, val)
    return csr, b


def adjoint_grad(t, xyz, conn, em, k_e, bc_mask, u, lam, nthreads=1):
    E = conn.shape[0]
    g = np.zeros(E)
    m = np.ascontiguousarray(bc_mask, dtype=np.uint8) if bc_mask is not None else None
    lib().orc_adjoint_grad(t, _dp(np.ascontiguousarray(xyz)), _up(np.ascontiguousarray(conn, dtype=np.uint32)), E,
                           _up(np.ascontiguousarray(em, dtype=np.uint32)),
                           _dp(np.ascontiguousarray(k_e, dtype=np.float64)), _p(m, C.c_uint8),
                           _dp(np.ascontiguousarray(u)), _dp(np.ascontiguousarray(lam)), nthreads, _dp(g))
    return g


def csr_to_scipy(csr, n):
    import scipy.sparse as sp

    rp, col, val = csr
    return sp.csr_matrix((val, col, rp), shape=(n, n))


def facet_bc_mask(t, conn, em, ndof, facets, markers):
    """BCEss::setupDofMap (bc.hpp:252-295) for facets given by their vertex ids.

    ``facets`` is a list of (vertex-id tuple, marker).  For Lagrange elements the DOFs
    on a facet are its vertices plus, for P2, its edge midpoints: every DOF of an
    element that touches the facet and lies on it.  The facet's DOFs are found from
    the element that owns all its vertices (facingElem[0])."""
    N = num_dofs(t)
    mask = np.zeros(ndof, dtype=np.uint8)
    if t == P1TET:
        for verts, m in facets:
            if m in markers:
                # P1: DOF of vertex v is the one the DOF map gives at its local slot
                for v in verts:
                    mask[_vertex_dof(conn, em, v)] = 1
        return mask
    raise NotImplementedError("facet_bc_mask: P1 tetrahedra only")


_vdof_cache = {}


def _vertex_dof(conn, em, v):
    key = (id(conn), id(em))
    if key not in _vdof_cache:
        nv = conn.shape[1]
        d = {}
        flat_c = conn.reshape(-1)
        flat_e = em[:, :nv].reshape(-1)
        for a, b in zip(flat_c.tolist(), flat_e.tolist()):
            d.setdefault(a, b)
        _vdof_cache.clear()
        _vdof_cache[key] = d
    return _vdof_cache[key][v]


def plane_bc_mask(dofxyz, planes, tol=0.0):
    """Constrained DOFs of the structured unit cube: every DOF lying on one of the
    given planes, ('x', 0.0) etc.  markFacetsCube (mesh.hpp:442-498) marks exactly the
    boundary facets lying on each plane, and a Lagrange facet carries the DOFs that
    lie on it, so this equals BCEss{feSpace, side::...}'s DOF set."""
    mask = np.zeros(dofxyz.shape[0], dtype=np.uint8)
    ax = {"x": 0, "y": 1, "z": 2}
    for a, v in planes:
        mask |= (np.abs(dofxyz[:, ax[a]] - v) <= tol).astype(np.uint8)
    return mask


def poisson_golden(t, xyz, conn, bc_mask_fn, rhs_kind="analytic"):
    """The proxpde poisson3d tests: K u = b with BCs, return ||u - I_h u_exact||_2."""
    import scipy.sparse.linalg as spla

    em, ndof = dofmap(t, xyz.shape[0], conn)
    dx = dof_coords(t, xyz, conn, em, ndof)
    mask = bc_mask_fn(em, ndof, dx)
    val = np.zeros(ndof)
    lhs = {"stiff_kind": 1, "stiff_c": 1.0, "apply_bc": 1}
    if rhs_kind == "analytic":
        rhs = {"kind": 1, "fn": FN_POISSON_RHS, "c": 1.0, "apply_bc": 1}
    else:
        proj = interpolate(t, xyz, conn, em, ndof, FN_POISSON_RHS)
        rhs = {"kind": 2, "c": 1.0, "field": proj, "apply_bc": 1}
    csr, b = build(t, xyz, conn, em, ndof, lhs=lhs, rhs=None, bc_mask=mask, bc_val=val)
    _, b = build(t, xyz, conn, em, ndof, lhs=None, rhs=rhs, bc_mask=mask, bc_val=val, b=b)
    A = csr_to_scipy(csr, ndof).tocsc()
    u = spla.spsolve(A, b)
    ex = interpolate(t, xyz, conn, em, ndof, FN_POISSON_EXACT)
    return float(np.linalg.norm(u - ex))


# ------------------------------------------------------------ vector spaces / coupling
# Assembly kinds of orc_system_call (oracle.cpp): stiffness, tensor stiffness, mass,
# grad (rows: vector space, columns: scalar space), div (rows: scalar, columns: vector).
STIFF, TENSOR_STIFF, MASS, GRAD, DIV = 1, 2, 3, 4, 5


class System:
    """FE spaces on one mesh with offsets in one global system (FESpace<..., dim>,
    BLOCK ordering) and Builder calls over them (buildLhs / buildCoupling); close()
    is closeMatrix.  spaces: list of dict(t, qr, dim, offset, ndof, em)."""

    def __init__(self, xyz, conn, spaces, ntot):
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self.conn = np.ascontiguousarray(conn, dtype=np.uint32)
        self.spaces = spaces
        self.ntot = int(ntot)
        self.b = np.zeros(self.ntot)
        self._acc = None
        self.bc = [(None, None) for _ in spaces]
        self.diag = 1.0

    def set_bc(self, s, mask, vals, diag=1.0):
        """mask / vals over the space's ndof * dim component DOFs (id + d * ndof)."""
        self.bc[s] = (np.ascontiguousarray(mask, dtype=np.uint8), np.ascontiguousarray(vals, dtype=np.float64))
        self.diag = float(diag)

    def call(self, row, col, ops):
        sp = self.spaces
        n = len(sp)
        arr = lambda ty, xs: (ty * n)(*xs)
        ts = np.array([x["t"] for x in sp], dtype=np.int32)
        qs = np.array([x["qr"] for x in sp], dtype=np.int32)
        dims = np.array([x["dim"] for x in sp], dtype=np.int32)
        offs = np.array([x["offset"] for x in sp], dtype=np.int64)
        nd = np.array([x["ndof"] for x in sp], dtype=np.int64)
        ems = [np.ascontiguousarray(x["em"], dtype=np.uint32) for x in sp]
        em_p = arr(C.c_void_p, [e.ctypes.data for e in ems])
        mk_p = arr(C.c_void_p, [m.ctypes.data if m is not None else None for m, _ in self.bc])
        vl_p = arr(C.c_void_p, [v.ctypes.data if v is not None else None for _, v in self.bc])
        kinds = np.array([k for k, _ in ops], dtype=np.int32)
        coefs = np.array([c for _, c in ops], dtype=np.float64)
        acc = lib().orc_system_call(self._acc, int(row), int(col), ts.ctypes.data, qs.ctypes.data, dims.ctypes.data,
                                    offs.ctypes.data, nd.ctypes.data, em_p, mk_p, vl_p, self.diag, _dp(self.xyz),
                                    _up(self.conn), self.conn.shape[0], len(ops), kinds.ctypes.data,
                                    coefs.ctypes.data, _dp(self.b))
        if not acc:
            raise ValueError("orc_system_call: unknown assembly kind")
        self._acc = acc

    def close(self):
        h = lib().orc_system_close(self._acc, self.ntot)
        self._acc = None
        nnz = lib().orc_csr_nnz(h)
        rp = np.zeros(self.ntot + 1, dtype=np.int32)
        col = np.zeros(nnz, dtype=np.int32)
        val = np.zeros(nnz)
        lib().orc_csr_copy(h, _p(rp, C.c_int32), _p(col, C.c_int32), _dp(val))
        lib().orc_csr_free(h)
        return rp, col, val


def stokes_problem(elem, n=4, ly=2.0):
    """The mesh, spaces and Dirichlet data of proxpde's test/stokes3dhex.cpp and
    stokes3dtet.cpp: Taylor-Hood Q2-Q1 (P2-P1) on the box [0,1] x [0,ly] x [0,1] with
    n^3 cells; BCEss BOTTOM inlet (0, (1 - x^2) / 2, 0), RIGHT zero, TOP / LEFT zero on
    components 0, 2, BACK / FRONT zero on component 2 (the last value wins)."""
    if elem == "hex":
        xyz, conn = cube_hex(n)
        tv, tp = Q2HEX, Q1HEX
    else:
        xyz, conn = cube_tet5(n)
        tv, tp = P2TET, P1TET
    xyz = xyz.copy()
    xyz[:, 1] *= ly
    emv, ndv = dofmap(tv, xyz.shape[0], conn)
    emp, ndp = dofmap(tp, xyz.shape[0], conn)
    xv = dof_coords(tv, xyz, conn, emv, ndv)
    xp = dof_coords(tp, xyz, conn, emp, ndp)
    inlet = lambda X: np.stack([np.zeros(len(X)), 0.5 * (1.0 - X[:, 0] ** 2), np.zeros(len(X))], axis=1)
    zero = lambda X: np.zeros((len(X), 3))
    on = lambda a, v: np.abs(xv[:, a] - v) <= 1e-12
    bcs = [(on(1, 0.0), inlet, (0, 1, 2)), (on(0, 1.0), zero, (0, 1, 2)), (on(1, ly), zero, (0, 2)),
           (on(0, 0.0), zero, (0, 2)), (on(2, 0.0), zero, (2,)), (on(2, 1.0), zero, (2,))]
    mask = np.zeros(3 * ndv, dtype=np.uint8)
    vals = np.zeros(3 * ndv)
    for sel, f, comps in bcs:
        ids = np.nonzero(sel)[0]
        fv = f(xv[ids])
        for c in comps:
            mask[ids + c * ndv] = 1
            vals[ids + c * ndv] = fv[:, c]
    return dict(xyz=xyz, conn=conn, tv=tv, tp=tp, emv=emv, ndv=ndv, emp=emp, ndp=ndp, xv=xv, xp=xp,
                bc_mask=mask, bc_vals=vals, u_exact=inlet(xv), ly=ly)


def stokes_errors(P, sol, nu=0.1):
    """||u - u_ex||, ||v - v_ex||, ||w - w_ex||, ||p - p_ex|| (p_ex = nu (ly - y))."""
    ndv = P["ndv"]
    err = [float(np.linalg.norm(sol[c * ndv:(c + 1) * ndv] - P["u_exact"][:, c])) for c in range(3)]
    err.append(float(np.linalg.norm(sol[3 * ndv:] - nu * (P["ly"] - P["xp"][:, 1]))))
    return err


def stokes_golden(elem, n=4, ly=2.0, nu=0.1):
    """proxpde's test/stokes3dhex.cpp / stokes3dtet.cpp through the oracle: tensor
    stiffness on the velocity, grad / div couplings with the pressure, a direct solve;
    returns the four error norms (pinned at stokes3dhex.cpp:135-140,
    stokes3dtet.cpp:122-127), the closed matrix and b."""
    import scipy.sparse.linalg as spla

    P = stokes_problem(elem, n, ly)
    ndv, ndp = P["ndv"], P["ndp"]
    spaces = [dict(t=P["tv"], qr=P["tv"], dim=3, offset=0, ndof=ndv, em=P["emv"]),
              dict(t=P["tp"], qr=P["tv"], dim=1, offset=3 * ndv, ndof=ndp, em=P["emp"])]
    ntot = 3 * ndv + ndp
    S = System(P["xyz"], P["conn"], spaces, ntot)
    S.set_bc(0, P["bc_mask"], P["bc_vals"], 1.0)
    S.call(0, 0, [(TENSOR_STIFF, nu)])
    S.call(0, 1, [(GRAD, -1.0)])
    S.call(1, 0, [(DIV, -1.0)])
    rp, col, val = S.close()
    A = csr_to_scipy((rp, col, val), ntot).tocsc()
    sol = spla.spsolve(A, S.b)
    return stokes_errors(P, sol, nu), (rp, col, val), S.b
