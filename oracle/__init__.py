"""CPU oracle for the proxpde assembly path (test infrastructure only).

This package wraps ``oracle/oracle.cpp`` (a plain C++ restatement of proxpde's
``Builder::buildLhs/buildRhs/closeMatrix`` element loop, see the header of that file
for the file:line of every restated piece) with ctypes.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` use it, as the
checker.  The GPU engine in ``proxpde_gb300`` never imports it.

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


def interpolate(t, xyz, conn, em, ndof, fn, c=1.0):
    v = np.zeros(ndof)
    lib().orc_interpolate(t, _dp(np.ascontiguousarray(xyz)), _up(np.ascontiguousarray(conn, dtype=np.uint32)),
                          conn.shape[0], _up(np.ascontiguousarray(em, dtype=np.uint32)), fn, c, _dp(v))
    return v


def _lhs(lhs, keep):
    if lhs is None:
        return None
    k_e = lhs.get("k_e")
    if k_e is not None:
        k_e = np.ascontiguousarray(k_e, dtype=np.float64)
        keep.append(k_e)
    s = OrcLhs(int(lhs.get("stiff_kind", 0)), float(lhs.get("stiff_c", 0.0)), _dp(k_e),
               int(lhs.get("mass_kind", 0)), float(lhs.get("mass_c", 0.0)), int(lhs.get("apply_bc", 0)))
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
