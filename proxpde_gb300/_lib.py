"""ctypes binding of the engine's C ABI (include/pxg.h, library proxpde_gb300/libpxg.so).

There is no fallback: if the library is missing or no GPU is present the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpxg.so")

P1TET, P2TET, Q1HEX, Q2HEX = 0, 1, 2, 3
MEM_HOST, MEM_DEVICE = 0, 1
FN_CONST, FN_SIN3, FN_POISSON_RHS, FN_POISSON_EXACT = 0, 1, 2, 3
FN_COORD_X, FN_COORD_Y, FN_COORD_Z = 4, 5, 6
ACCUMULATE = 1

STATUS = {
    0: "ok", 1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "timeout",
    5: "not converged", 6: "unsupported", 7: "no CUDA device", 8: "numerical error",
}

# every symbol include/pxg.h declares (checked by the CPU tests)
EXPORTS = [
    "pxg_create", "pxg_destroy", "pxg_last_error", "pxg_status_string", "pxg_version",
    "pxg_set_mesh", "pxg_set_coords", "pxg_build_dofmap", "pxg_set_dofmap", "pxg_get_dofmap",
    "pxg_build_pattern", "pxg_get_pattern", "pxg_pattern_device", "pxg_set_coef", "pxg_set_bc",
    "pxg_assemble", "pxg_prune_count", "pxg_prune_count_device", "pxg_set_scatter", "pxg_colouring", "pxg_autotune",
    "pxg_build_facets", "pxg_get_facets", "pxg_set_facet_markers", "pxg_mark_facets_box", "pxg_set_bc_markers",
    "pxg_sys_create", "pxg_sys_destroy", "pxg_sys_get_pattern", "pxg_sys_pattern_device", "pxg_sys_set_bc",
    "pxg_sys_assemble",
    "pxg_close_matrix", "pxg_interpolate", "pxg_prune_csr_noalloc",
    "pxg_cg", "pxg_adjoint_grad", "pxg_adjoint_forward", "pxg_adjoint_backward",
    "pxg_batch_set", "pxg_batch_adjoint", "pxg_device_alloc", "pxg_device_free", "pxg_memcpy",
    "pxg_set_arithmetic", "pxg_fp64_rate", "pxg_red_rate", "pxg_sys_close_matrix", "pxg_get_qpoints",
]


class PxgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class LhsOp(C.Structure):
    _fields_ = [
        ("stiffness", C.c_int32),
        ("stiff_coef", C.c_double),
        ("mass", C.c_int32),
        ("mass_coef", C.c_double),
        ("apply_bc", C.c_int32),
    ]


class RhsOp(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("fn", C.c_int32),
        ("coef", C.c_double),
        ("field", C.c_void_p),
        ("apply_bc", C.c_int32),
    ]


class TuneReport(C.Structure):
    _fields_ = [
        ("threads", C.c_int),
        ("scatter", C.c_int),
        ("ncolours", C.c_int),
        ("ncand", C.c_int),
        ("cand_threads", C.c_int * 16),
        ("cand_scatter", C.c_int * 16),
        ("cand_ms", C.c_double * 16),
    ]


SCATTER_REDUCE, SCATTER_COLOUR = 0, 1
# arithmetic of the element kernels: IEEE binary64 (default) or double-float (opt-in)
ARITH_FP64, ARITH_DFL = 0, 1
SCATTER_NAMES = {SCATTER_REDUCE: "reduce", SCATTER_COLOUR: "colour"}

_lib = None


def load(path: str = LIB_PATH):
    """Load libpxg.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build the engine first (python -m proxpde_gb300.build)")
    L = C.CDLL(path)
    vp, i64, i64p = C.c_void_p, C.c_int64, C.POINTER(C.c_int64)
    sig = {
        "pxg_create": ([C.POINTER(vp), C.c_int], C.c_int),
        "pxg_destroy": ([vp], C.c_int),
        "pxg_last_error": ([vp], C.c_char_p),
        "pxg_status_string": ([C.c_int], C.c_char_p),
        "pxg_version": ([], C.c_int),
        "pxg_set_mesh": ([vp, C.c_int, vp, i64, vp, i64, C.c_int], C.c_int),
        "pxg_set_coords": ([vp, vp, C.c_int, vp], C.c_int),
        "pxg_build_dofmap": ([vp, i64p], C.c_int),
        "pxg_set_dofmap": ([vp, vp, i64, C.c_int], C.c_int),
        "pxg_get_dofmap": ([vp, vp, C.c_int], C.c_int),
        "pxg_build_pattern": ([vp, i64p], C.c_int),
        "pxg_get_pattern": ([vp, vp, vp, C.c_int], C.c_int),
        "pxg_pattern_device": ([vp, C.POINTER(vp), C.POINTER(vp)], C.c_int),
        "pxg_set_coef": ([vp, vp, C.c_int, vp], C.c_int),
        "pxg_set_bc": ([vp, vp, vp, i64, C.c_double, C.c_int], C.c_int),
        "pxg_assemble": ([vp, C.POINTER(LhsOp), vp, C.POINTER(LhsOp), vp, C.POINTER(RhsOp), vp, C.c_uint, vp],
                         C.c_int),
        "pxg_prune_count": ([vp, vp, i64p, vp], C.c_int),
        "pxg_prune_count_device": ([vp, vp, vp, vp], C.c_int),
        "pxg_set_scatter": ([vp, C.c_int, C.c_int], C.c_int),
        "pxg_set_arithmetic": ([vp, C.c_int], C.c_int),
        "pxg_fp64_rate": ([C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
        "pxg_red_rate": ([C.c_int, C.c_int, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
        "pxg_sys_create": ([C.POINTER(vp), vp, vp, vp, C.c_int, i64p, i64p], C.c_int),
        "pxg_sys_destroy": ([vp], C.c_int),
        "pxg_sys_get_pattern": ([vp, vp, vp], C.c_int),
        "pxg_sys_pattern_device": ([vp, C.POINTER(vp), C.POINTER(vp)], C.c_int),
        "pxg_sys_close_matrix": ([vp, vp, vp, vp, vp, i64p, vp], C.c_int),
        "pxg_sys_set_bc": ([vp, C.c_int, vp, vp, i64, C.c_double], C.c_int),
        "pxg_sys_assemble": ([vp, C.c_int, C.c_int, vp, vp, C.c_int, vp, vp, C.c_uint, vp], C.c_int),
        "pxg_build_facets": ([vp, i64p], C.c_int),
        "pxg_get_facets": ([vp, vp, vp], C.c_int),
        "pxg_set_facet_markers": ([vp, vp], C.c_int),
        "pxg_mark_facets_box": ([vp, vp, vp], C.c_int),
        "pxg_set_bc_markers": ([vp, vp, vp, vp, C.c_int, C.c_double], C.c_int),
        "pxg_colouring": ([vp, C.POINTER(C.c_int), vp, vp], C.c_int),
        "pxg_autotune": ([vp, C.POINTER(LhsOp), C.POINTER(LhsOp), C.POINTER(RhsOp), C.POINTER(TuneReport)], C.c_int),
        "pxg_close_matrix": ([vp, vp, vp, vp, vp, i64p, vp], C.c_int),
        "pxg_interpolate": ([vp, C.c_int, C.c_double, vp, vp], C.c_int),
        "pxg_get_qpoints": ([vp, vp, C.c_int, vp], C.c_int),
        "pxg_prune_csr_noalloc": ([vp, vp, vp, i64, vp, vp, vp, i64p, vp], C.c_int),
        "pxg_cg": ([vp, vp, vp, vp, i64, vp, vp, C.c_double, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), vp],
                   C.c_int),
        "pxg_adjoint_grad": ([vp, vp, vp, vp, vp], C.c_int),
        "pxg_adjoint_forward": ([vp, C.POINTER(RhsOp), vp, C.c_double, C.c_int, vp, C.POINTER(C.c_double),
                                 C.POINTER(C.c_int), vp], C.c_int),
        "pxg_adjoint_backward": ([vp, C.c_double, vp, vp, C.POINTER(C.c_int), vp], C.c_int),
        "pxg_batch_set": ([vp, C.POINTER(C.c_int64), i64], C.c_int),
        "pxg_device_alloc": ([vp, C.c_uint64, C.POINTER(vp)], C.c_int),
        "pxg_device_free": ([vp, vp], C.c_int),
        "pxg_memcpy": ([vp, vp, vp, C.c_uint64, C.c_int, vp], C.c_int),
        "pxg_batch_adjoint": ([C.POINTER(vp), C.c_int, C.POINTER(RhsOp), C.POINTER(vp), C.c_double, C.c_int,
                               C.POINTER(C.c_double), C.POINTER(vp), C.POINTER(C.c_int), C.c_int, vp], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def fp64_rate(device=0):
    """(FP64 FMAs per second, ms of the timed launch) measured on a device."""
    L = load()
    r, ms = C.c_double(), C.c_double()
    st = L.pxg_fp64_rate(int(device), C.byref(r), C.byref(ms))
    if st:
        raise PxgError(st, "fp64_rate")
    return r.value, ms.value


def red_rate(lanes_per_sector, nbytes=32 << 20, device=0):
    """(FP64 reductions per second, ms of the timed launch) measured on a device, with
    lanes_per_sector (1, 2, 4) lanes of a warp adding into one 32-byte sector, over an
    array of nbytes (a power of two)."""
    L = load()
    r, ms = C.c_double(), C.c_double()
    st = L.pxg_red_rate(int(device), int(lanes_per_sector), int(nbytes), C.byref(r), C.byref(ms))
    if st:
        raise PxgError(st, "red_rate")
    return r.value, ms.value


def _ptr(a):
    """Address of a numpy array (host) or a torch tensor (device or host)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"]
        return a.ctypes.data
    if isinstance(a, int):
        return a
    assert a.is_contiguous()
    return a.data_ptr()


def _mem(a):
    if isinstance(a, np.ndarray):
        return MEM_HOST
    if isinstance(a, int):
        return MEM_DEVICE
    return MEM_DEVICE if a.is_cuda else MEM_HOST


class Context:
    """One engine context (pxg_ctx) bound to a GPU."""

    def __init__(self, device: int = 0):
        self.L = load()
        h = C.c_void_p()
        st = self.L.pxg_create(C.byref(h), device)
        if st != 0:
            raise PxgError(st, "pxg_create")
        self.h = h
        self.device = device
        self.ndof = 0
        self.nnz = 0
        self.nelem = 0
        self.etype = None

    def _check(self, st, what):
        if st != 0:
            msg = self.L.pxg_last_error(self.h)
            raise PxgError(st, f"{what}: {msg.decode() if msg else ''}")

    def close(self):
        if getattr(self, "h", None):
            self.L.pxg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- inputs
    def set_mesh(self, etype, xyz, conn):
        nelem = int(conn.shape[0])
        self._check(self.L.pxg_set_mesh(self.h, etype, _ptr(xyz), int(xyz.shape[0]), _ptr(conn), nelem,
                                        _mem(xyz)), "set_mesh")
        # recorded once the library accepted the mesh
        self.etype = etype
        self.nelem = nelem

    def set_coords(self, xyz, stream=None):
        self._check(self.L.pxg_set_coords(self.h, _ptr(xyz), _mem(xyz), stream), "set_coords")

    def build_dofmap(self):
        n = C.c_int64()
        self._check(self.L.pxg_build_dofmap(self.h, C.byref(n)), "build_dofmap")
        self.ndof = n.value
        return self.ndof

    def set_dofmap(self, em, ndof):
        self._check(self.L.pxg_set_dofmap(self.h, _ptr(em), int(ndof), _mem(em)), "set_dofmap")
        self.ndof = int(ndof)

    def get_dofmap(self):
        N = {P1TET: 4, P2TET: 10, Q1HEX: 8, Q2HEX: 27}[self.etype]
        em = np.zeros((self.nelem, N), dtype=np.uint32)
        self._check(self.L.pxg_get_dofmap(self.h, _ptr(em), MEM_HOST), "get_dofmap")
        return em

    def build_pattern(self):
        n = C.c_int64()
        self._check(self.L.pxg_build_pattern(self.h, C.byref(n)), "build_pattern")
        self.nnz = n.value
        return self.nnz

    def get_pattern(self):
        rp = np.zeros(self.ndof + 1, dtype=np.int32)
        ci = np.zeros(self.nnz, dtype=np.int32)
        self._check(self.L.pxg_get_pattern(self.h, _ptr(rp), _ptr(ci), MEM_HOST), "get_pattern")
        return rp, ci

    def pattern_device(self):
        rp, ci = C.c_void_p(), C.c_void_p()
        self._check(self.L.pxg_pattern_device(self.h, C.byref(rp), C.byref(ci)), "pattern_device")
        return rp.value, ci.value

    def set_coef(self, k_e, stream=None):
        self._check(self.L.pxg_set_coef(self.h, _ptr(k_e), _mem(k_e), stream), "set_coef")

    def set_bc(self, dofs, vals, diag=1.0):
        dofs = np.ascontiguousarray(dofs, dtype=np.uint32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        self._check(self.L.pxg_set_bc(self.h, _ptr(dofs), _ptr(vals), int(dofs.size), float(diag), MEM_HOST),
                    "set_bc")

    # --- assembly
    @staticmethod
    def _lhs(o):
        if o is None:
            return None
        return C.pointer(LhsOp(int(o.get("stiffness", 0)), float(o.get("stiff_coef", 1.0)), int(o.get("mass", 0)),
                               float(o.get("mass_coef", 1.0)), int(o.get("apply_bc", 0))))

    @staticmethod
    def _rhs(rhs):
        if rhs is None:
            return None
        return C.pointer(RhsOp(int(rhs.get("kind", 0)), int(rhs.get("fn", 0)), float(rhs.get("coef", 1.0)),
                               _ptr(rhs.get("field")), int(rhs.get("apply_bc", 0))))

    def assemble(self, op0=None, vals0=None, op1=None, vals1=None, rhs=None, b=None, accumulate=False,
                 stream=None):
        self._check(self.L.pxg_assemble(self.h, self._lhs(op0), _ptr(vals0), self._lhs(op1), _ptr(vals1),
                                        self._rhs(rhs), _ptr(b), ACCUMULATE if accumulate else 0, stream), "assemble")

    def prune_count(self, vals, stream=None):
        n = C.c_int64()
        self._check(self.L.pxg_prune_count(self.h, _ptr(vals), C.byref(n), stream), "prune_count")
        return n.value

    def prune_count_device(self, vals, out, stream=None):
        """Asynchronous prune count into `out` (a one-element int64 device tensor)."""
        assert str(out.dtype) == "torch.int64" and out.is_cuda and out.numel() >= 1
        self._check(self.L.pxg_prune_count_device(self.h, _ptr(vals), _ptr(out), stream), "prune_count_device")

    # --- boundary facets and Dirichlet conditions from markers (on the device)
    def build_facets(self):
        n = C.c_int64()
        self._check(self.L.pxg_build_facets(self.h, C.byref(n)), "build_facets")
        self.nfacets = n.value
        return n.value

    def get_facets(self):
        """(faces: element * faces-per-element + local face, markers), in device order"""
        n = self.build_facets()
        faces = np.empty(n, dtype=np.uint32)
        markers = np.empty(n, dtype=np.int32)
        self._check(self.L.pxg_get_facets(self.h, faces.ctypes.data, markers.ctypes.data), "get_facets")
        return faces, markers

    def set_facet_markers(self, markers):
        markers = np.ascontiguousarray(markers, dtype=np.int32)
        self._check(self.L.pxg_set_facet_markers(self.h, markers.ctypes.data), "set_facet_markers")

    def mark_facets_box(self, origin=(0.0, 0.0, 0.0), length=(1.0, 1.0, 1.0)):
        o = np.ascontiguousarray(origin, dtype=np.float64)
        ln = np.ascontiguousarray(length, dtype=np.float64)
        self._check(self.L.pxg_mark_facets_box(self.h, o.ctypes.data, ln.ctypes.data), "mark_facets_box")

    def set_bc_markers(self, conditions, diag=1.0):
        """conditions: [(marker, fn id, coef)]; DOFs on the marked facets get coef * fn(x)."""
        m = np.ascontiguousarray([c[0] for c in conditions], dtype=np.int32)
        f = np.ascontiguousarray([c[1] for c in conditions], dtype=np.int32)
        v = np.ascontiguousarray([c[2] for c in conditions], dtype=np.float64)
        self._check(self.L.pxg_set_bc_markers(self.h, m.ctypes.data, f.ctypes.data, v.ctypes.data, len(conditions),
                                              float(diag)), "set_bc_markers")

    # --- scatter strategy and autotuning
    def set_scatter(self, scatter, threads=0):
        self._check(self.L.pxg_set_scatter(self.h, int(scatter), int(threads)), "set_scatter")

    def set_arithmetic(self, arith):
        """ARITH_FP64 (default) or ARITH_DFL for this context's element kernels."""
        self._check(self.L.pxg_set_arithmetic(self.h, int(arith)), "set_arithmetic")

    def colouring(self, with_order=False):
        """(number of colour classes, element order or None, class offsets or None)"""
        n = C.c_int()
        self._check(self.L.pxg_colouring(self.h, C.byref(n), None, None), "colouring")
        if not with_order:
            return n.value, None, None
        order = np.empty(self.nelem, dtype=np.uint32)
        offs = np.empty(n.value + 1, dtype=np.int64)
        self._check(self.L.pxg_colouring(self.h, C.byref(n), order.ctypes.data, offs.ctypes.data), "colouring")
        return n.value, order, offs

    def autotune(self, op0=None, op1=None, rhs=None):
        """Time every (threads, scatter) candidate on this mesh, keep the fastest; returns
        dict(threads, scatter, ncolours, candidates=[(threads, scatter, ms)])."""
        rep = TuneReport()
        self._check(self.L.pxg_autotune(self.h, self._lhs(op0), self._lhs(op1), self._rhs(rhs), C.byref(rep)),
                    "autotune")
        cands = [(rep.cand_threads[i], SCATTER_NAMES[rep.cand_scatter[i]], rep.cand_ms[i]) for i in range(rep.ncand)]
        return {"threads": rep.threads, "scatter": SCATTER_NAMES[rep.scatter], "ncolours": rep.ncolours,
                "candidates": cands}

    def close_matrix(self, vals, rp, ci, vout, stream=None):
        n = C.c_int64()
        self._check(self.L.pxg_close_matrix(self.h, _ptr(vals), _ptr(rp), _ptr(ci), _ptr(vout), C.byref(n), stream),
                    "close_matrix")
        return n.value

    def interpolate(self, fn, coef, v, stream=None):
        self._check(self.L.pxg_interpolate(self.h, int(fn), float(coef), _ptr(v), stream), "interpolate")

    def get_qpoints(self, out=None, stream=None):
        """CurFE::qpoint of every element and quadrature point: (nelem, nq, 3), into a
        host array (default) or a device tensor `out`."""
        nq = {P1TET: 4, P2TET: 11, Q1HEX: 8, Q2HEX: 27}[self.etype]
        if out is None:
            out = np.empty((self.nelem, nq, 3))
        self._check(self.L.pxg_get_qpoints(self.h, _ptr(out), _mem(out), stream), "get_qpoints")
        return out

    # --- solve and adjoint
    def cg(self, rp, ci, vals, b, x, rtol=1e-10, max_iter=10000, stream=None):
        it, rel = C.c_int(), C.c_double()
        self._check(self.L.pxg_cg(self.h, _ptr(rp), _ptr(ci), _ptr(vals), int(b.numel()), _ptr(b), _ptr(x),
                                  float(rtol), int(max_iter), C.byref(it), C.byref(rel), stream), "cg")
        return it.value, rel.value

    def adjoint_grad(self, u, lam, g, stream=None):
        self._check(self.L.pxg_adjoint_grad(self.h, _ptr(u), _ptr(lam), _ptr(g), stream), "adjoint_grad")

    def adjoint_forward(self, rhs, u_target, rtol=1e-10, max_iter=20000, u_out=None, stream=None):
        r = C.pointer(RhsOp(int(rhs.get("kind", 0)), int(rhs.get("fn", 0)), float(rhs.get("coef", 1.0)),
                            _ptr(rhs.get("field")), 1))
        loss, it = C.c_double(), C.c_int()
        self._check(self.L.pxg_adjoint_forward(self.h, r, _ptr(u_target), float(rtol), int(max_iter), _ptr(u_out),
                                               C.byref(loss), C.byref(it), stream), "adjoint_forward")
        return loss.value, it.value

    def adjoint_backward(self, grad, dloss=1.0, lam_out=None, stream=None):
        it = C.c_int()
        self._check(self.L.pxg_adjoint_backward(self.h, float(dloss), _ptr(grad), _ptr(lam_out), C.byref(it),
                                                stream), "adjoint_backward")
        return it.value


OP_STIFFNESS, OP_TENSOR_STIFFNESS, OP_MASS, OP_GRAD, OP_DIV = 1, 2, 3, 4, 5


class System:
    """pxg_sys: spaces (contexts on one mesh with DOF maps) with dims, offsets in BLOCK
    ordering, one pattern; assemble() is one Builder call over (row, col) spaces."""

    def __init__(self, spaces, dims, qr_types=None):
        self.L = load()
        self.spaces = list(spaces)
        self.dims = [int(d) for d in dims]
        n = len(self.spaces)
        ctxs = (C.c_void_p * n)(*[c.h.value for c in self.spaces])
        d = np.ascontiguousarray(self.dims, dtype=np.int32)
        q = None if qr_types is None else np.ascontiguousarray(qr_types, dtype=np.int32)
        self.h = C.c_void_p()
        nt, nz = C.c_int64(), C.c_int64()
        st = self.L.pxg_sys_create(C.byref(self.h), ctxs, d.ctypes.data, None if q is None else q.ctypes.data, n,
                                   C.byref(nt), C.byref(nz))
        if st != 0:
            raise PxgError(st, "pxg_sys_create: " + self.L.pxg_last_error(self.spaces[0].h).decode())
        self.ntot, self.nnz = nt.value, nz.value
        self.offsets = np.cumsum([0] + [c.ndof * dd for c, dd in zip(self.spaces, self.dims)])[:-1].tolist()

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.pxg_sys_destroy(self.h)
            self.h = C.c_void_p()

    def _check(self, st, what, space=0):
        if st != 0:
            raise PxgError(st, f"{what}: " + self.L.pxg_last_error(self.spaces[space].h).decode())

    def get_pattern(self):
        rp = np.zeros(self.ntot + 1, dtype=np.int32)
        ci = np.zeros(self.nnz, dtype=np.int32)
        self._check(self.L.pxg_sys_get_pattern(self.h, rp.ctypes.data, ci.ctypes.data), "sys_get_pattern")
        return rp, ci

    def pattern_device(self):
        rp, ci = C.c_void_p(), C.c_void_p()
        self._check(self.L.pxg_sys_pattern_device(self.h, C.byref(rp), C.byref(ci)), "sys_pattern_device")
        return rp.value, ci.value

    def close_matrix(self, vals, rp, ci, vout, stream=None):
        """closeMatrix on the system's pattern into device tensors; returns the kept count."""
        n = C.c_int64()
        self._check(self.L.pxg_sys_close_matrix(self.h, _ptr(vals), _ptr(rp), _ptr(ci), _ptr(vout), C.byref(n),
                                                stream), "sys_close_matrix")
        return n.value

    def set_bc(self, space, dofs, vals, diag=1.0):
        dofs = np.ascontiguousarray(dofs, dtype=np.uint32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        self._check(self.L.pxg_sys_set_bc(self.h, int(space), dofs.ctypes.data, vals.ctypes.data, dofs.size,
                                          float(diag)), "sys_set_bc", space)

    def assemble(self, row, col, ops, vals, b=None, accumulate=False, stream=None):
        """ops: [(kind, coef)]; vals (nnz) and b (ntot) device tensors."""
        k = np.ascontiguousarray([o[0] for o in ops], dtype=np.int32)
        c = np.ascontiguousarray([o[1] for o in ops], dtype=np.float64)
        self._check(self.L.pxg_sys_assemble(self.h, int(row), int(col), k.ctypes.data, c.ctypes.data, len(ops),
                                            _ptr(vals), _ptr(b), ACCUMULATE if accumulate else 0, stream),
                    "sys_assemble", row)
