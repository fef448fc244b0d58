"""proxpde_gb300 — GB300 finite-element assembly engine with proxpde's Builder interface.

The names below mirror proxpde's C++ API for the assembly path so that code (and the
parity tests) read like proxpde's own tests (e.g. test/poisson3dhex.cpp:46-74):

    mesh = buildHyperCube(Hexahedron, n)                    # include/mesh.hpp:385-421
    fe = FESpace(mesh, order=1)                             # include/fespace.hpp:27-193
    bcs = [BCEss(fe, side.LEFT), BCEss(fe, side.BOTTOM)]    # include/bc.hpp:32-306
    builder = Builder(fe)                                   # include/builder.hpp:12-391
    builder.buildLhs((AssemblyStiffness(1.0, fe),), bcs)
    builder.buildRhs((AssemblyRhsAnalytic(lambda p: np.sin(p[:, 0]), fe),), bcs)
    builder.closeMatrix()
    builder.A  (scipy CSR on the host) / builder.A_dev (device CSR)  builder.b

Every assembly runs on the GPU through libpxg.so (include/pxg.h); there is no CPU
path.  An analytic right-hand side is either any Python callable, evaluated on the
host at the quadrature points the device reports and integrated on the device, or one
of the device's function ids (FN_*), evaluated on the device.
"""
from __future__ import annotations

import numpy as np

from . import meshgen
from ._lib import (FN_CONST, FN_POISSON_EXACT, FN_POISSON_RHS, FN_SIN3, P1TET, P2TET, Q1HEX, Q2HEX,
                   SCATTER_COLOUR, SCATTER_REDUCE, Context, PxgError, load)

__all__ = [
    "Tetrahedron", "Hexahedron", "Mesh", "buildHyperCube", "FESpace", "BCEss", "side", "Builder",
    "AssemblyStiffness", "AssemblyStiffnessFE", "AssemblyScalarMass", "AssemblyMass", "AssemblyRhsAnalytic",
    "AssemblyS2SProjection", "AssemblyProjection", "interpolateAnalyticFunction", "Context", "PxgError",
    "AssemblyTensorStiffness", "AssemblyGrad", "AssemblyDiv",
    "FN_CONST", "FN_SIN3", "FN_POISSON_RHS", "FN_POISSON_EXACT", "P1TET", "P2TET", "Q1HEX", "Q2HEX", "meshgen",
    "load", "SCATTER_REDUCE", "SCATTER_COLOUR", "LUSolver",
]


class Tetrahedron:
    nv = 4


class Hexahedron:
    nv = 8


class side:
    """Boundary markers of the structured cube (include/mesh.hpp:178-188)."""
    NONE, BOTTOM, RIGHT, TOP, LEFT, BACK, FRONT = 0, 1, 2, 3, 4, 5, 6
    # plane of each marker as set by markFacetsCube (include/mesh.hpp:442-498)
    PLANE = {1: (1, 0.0), 2: (0, 1.0), 3: (1, 1.0), 4: (0, 0.0), 5: (2, 0.0), 6: (2, 1.0)}


class Mesh:
    """Mesh<Elem>{pointList, elementList} as arrays: xyz[nnodes,3], conn[nelem,nv]."""

    def __init__(self, elem, xyz, conn, facets=None):
        self.elem = elem
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self.conn = np.ascontiguousarray(conn, dtype=np.uint32)
        # optional tagged boundary facets: (vertex ids array [nf, k], markers [nf])
        self.facets = facets


def buildHyperCube(elem, n: int, origin=(0.0, 0.0, 0.0), length=(1.0, 1.0, 1.0)) -> Mesh:
    """buildCube on the box origin + [0, length] with n^3 cells (src/mesh.cpp:355-534):
    hexahedra, or 5 tetrahedra per cell."""
    if elem is Hexahedron:
        xyz, conn = meshgen.cube_hex(n)
    else:
        xyz, conn = meshgen.cube_tet5(n)
    xyz = np.asarray(origin, dtype=np.float64) + xyz * np.asarray(length, dtype=np.float64)
    m = Mesh(elem, xyz, conn)
    m.structured_n = n
    return m


def _etype(elem, order):
    if elem is Tetrahedron:
        return {1: P1TET, 2: P2TET}[order]
    return {1: Q1HEX, 2: Q2HEX}[order]


class _Dof:
    def __init__(self, fe):
        self._fe = fe
        self.size = fe.ctx.ndof
        self._em = None

    @property
    def elemMap(self):
        if self._em is None:
            self._em = self._fe.ctx.get_dofmap()
        return self._em

    def getId(self, e, i):
        return int(self.elemMap[e, i])


class FESpace:
    """FESpace<Mesh, LagrangeFE<Elem, order>::RefFE_T, RecommendedQR>: owns the device
    context with the mesh, the first-touch DOF map and the CSR pattern."""

    def __init__(self, mesh: Mesh, order: int = 1, device: int = 0, elem_map=None, ndof=None, dim: int = 1,
                 offset: int = 0, qr_order=None):
        self.mesh = mesh
        self.order = order
        self.etype = _etype(mesh.elem, order)
        # vector spaces (BLOCK ordering), the offset in a global system and the element
        # type whose quadrature rule the space uses (FESpace<Mesh, RefFE, QR, dim>)
        self.dim = int(dim)
        self.offset = int(offset)
        self.qr_type = _etype(mesh.elem, qr_order or order)
        self.ctx = Context(device)
        self.ctx.set_mesh(self.etype, mesh.xyz, mesh.conn)
        if elem_map is None:
            self.ctx.build_dofmap()
        else:
            self.ctx.set_dofmap(np.ascontiguousarray(elem_map, dtype=np.uint32), ndof)
        self.dof = _Dof(self)
        self._pattern = False
        self._bc_key = None
        self._marked = False

    def pattern(self):
        if not self._pattern:
            self.ctx.build_pattern()
            self._pattern = True
        return self.ctx.nnz

    def dofPts(self):
        """Coordinates of every DOF (RefFE::dofPts scattered by the DOF map)."""
        return np.stack([_interp_coord(self, d) for d in range(3)], axis=1)

    def set_coefficient(self, k_e):
        self.ctx.set_coef(np.ascontiguousarray(k_e, dtype=np.float64))

    def mark_facets(self):
        """Boundary facet markers on the device: the mesh's tagged facets, else the planes
        of its bounding box (markFacetsCube, include/mesh.hpp:443-481)."""
        if self._marked:
            return
        m = self.mesh
        if m.facets is None:
            lo, hi = m.xyz.min(axis=0), m.xyz.max(axis=0)
            self.ctx.mark_facets_box(lo, hi - lo)
        else:
            faces, _ = self.ctx.get_facets()
            hex_ = self.etype in (Q1HEX, Q2HEX)
            nf = 6 if hex_ else 4
            table = np.array(HEX_FACES if hex_ else [[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]])
            e, lf = faces // nf, faces % nf
            verts = np.sort(m.conn[e[:, None], table[lf]], axis=1)
            fverts, tags = m.facets
            lookup = {tuple(v[:3]): t for v, t in zip(np.sort(fverts, axis=1).tolist(), tags.tolist())}
            markers = np.array([lookup.get(tuple(v[:3]), 0) for v in verts.tolist()], dtype=np.int32)
            self.ctx.set_facet_markers(markers)
        self._marked = True

    def apply_bcs(self, bcs):
        key = tuple(id(b) for b in bcs)
        if key == self._bc_key:
            return
        if not bcs:
            self.ctx.set_bc(np.zeros(0, np.uint32), np.zeros(0), 1.0)
        elif all(b.device_setup for b in bcs):
            # marked facets -> constrained DOFs on the device (BCEss::setupDofMap)
            self.mark_facets()
            self.ctx.set_bc_markers([(b.marker, FN_CONST, b.value) for b in bcs], bcs[-1].diag)
        else:
            dofs = np.concatenate([b.dofs for b in bcs]).astype(np.uint32)
            vals = np.concatenate([b.values for b in bcs])
            self.ctx.set_bc(dofs, vals, bcs[-1].diag)
        self._bc_key = key


def _interp_coord(fe, d):
    # DOF coordinates from the mesh: vertices directly, higher-order DOFs as the
    # averages RefFE::dofPts forms (include/reffe.hpp:748-767, 960-988)
    em = fe.dof.elemMap
    X = fe.mesh.xyz[fe.mesh.conn.astype(np.int64)][:, :, d]
    cols = [X[:, a] for a in range(X.shape[1])]
    if fe.etype == P2TET:
        for a, b in ((0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3)):
            cols.append(.5 * (X[:, a] + X[:, b]))
    if fe.etype == Q2HEX:
        for a, b in ((0, 1), (1, 2), (2, 3), (3, 0), (0, 4), (1, 5), (2, 6), (3, 7), (4, 5), (5, 6), (6, 7), (7, 4)):
            cols.append(0.5 * (X[:, a] + X[:, b]))
        for f in ((0, 3, 2, 1), (3, 0, 4, 7), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (4, 5, 6, 7)):
            cols.append(0.25 * (X[:, f[0]] + X[:, f[1]] + X[:, f[2]] + X[:, f[3]]))
        s = X[:, 0]
        for a in range(1, 8):
            s = s + X[:, a]
        cols.append(.125 * s)
    P = np.stack(cols, axis=1)
    out = np.zeros(fe.dof.size)
    out[em.reshape(-1).astype(np.int64)] = P.reshape(-1)
    return out


def _component_bcs(fe, bcs, c):
    """Set the constrained DOFs of component c of a vector space on its scalar context
    (the context's DOF ids, values as given)."""
    nd = fe.dof.size
    dofs, vals = [np.zeros(0, np.int64)], [np.zeros(0)]
    for b in bcs:
        d, v = b.component_dofs()
        d = d.astype(np.int64)
        sel = (d >= c * nd) & (d < (c + 1) * nd)
        dofs.append(d[sel] - c * nd)
        vals.append(v[sel])
    fe.ctx.set_bc(np.concatenate(dofs).astype(np.uint32), np.concatenate(vals), bcs[-1].diag if bcs else 1.0)
    fe._bc_key = None


HEX_FACES = [[0, 3, 2, 1], [3, 0, 4, 7], [0, 1, 5, 4], [1, 2, 6, 5], [2, 3, 7, 6], [4, 5, 6, 7]]


class BCEss:
    """Essential BC on the DOFs of the boundary facets with a marker (bc.hpp:252-295),
    or on an explicit DOF list.  Marker form: ``value`` is a constant, or a function of
    the DOF points (n x 3 array) returning n values (scalar space) or n x dim values
    (vector space); ``comps`` restricts a vector BC to some components.  A scalar BC
    with a constant is set up on the device from the facet markers; the others are
    evaluated at the DOF points on the host (setup, off the assembly path)."""

    def __init__(self, fe: FESpace, marker=None, value=0.0, dofs=None, diag=1.0, comps=None):
        self.fe = fe
        self.diag = float(diag)
        self._dofs = None
        self.comps = list(range(fe.dim)) if comps is None else [int(c) for c in comps]
        self.func = value if callable(value) else None
        if dofs is None:
            if marker is None or (self.func is None and np.ndim(value) != 0):
                raise ValueError("BCEss: a marker with a constant or a function, or a DOF list")
            self.marker, self.value = int(marker), (0.0 if self.func else float(value))
        else:
            self.marker = None
            self._dofs = np.ascontiguousarray(dofs, dtype=np.uint32)
            v = np.asarray(value, dtype=np.float64)
            self.values = np.broadcast_to(v, self._dofs.shape).copy() if v.ndim == 0 else v.copy()

    @property
    def device_setup(self):
        """True when the constrained set is built on the device (scalar, constant)."""
        return self.marker is not None and self.func is None and self.fe.dim == 1

    def component_dofs(self):
        """(component DOF ids k + c * ndof, values) over the space's component DOFs."""
        if self.marker is None:
            return self.dofs, self.values
        ids = self._marker_dofs(self.fe, self.marker)
        nd = self.fe.dof.size
        if self.func is None:
            vals = np.full((ids.size, self.fe.dim), self.value)
        else:
            pts = self.fe.dofPts()[ids]
            vals = np.asarray(self.func(pts), dtype=np.float64).reshape(ids.size, -1)
        out_d = np.concatenate([ids + c * nd for c in self.comps]).astype(np.uint32)
        out_v = np.concatenate([vals[:, c if vals.shape[1] > 1 else 0] for c in self.comps])
        return out_d, out_v

    @property
    def dofs(self):
        """The constrained DOFs (host computation, for inspection)."""
        if self._dofs is None:
            self._dofs, self.values = self.component_dofs()
        return self._dofs

    @staticmethod
    def _marker_dofs(fe, marker):
        m = fe.mesh
        if m.facets is not None:
            # tagged facets: a Lagrange facet carries the DOFs of its vertices (P1/Q1)
            verts, tags = m.facets
            sel = np.unique(verts[tags == marker].reshape(-1))
            if fe.etype not in (P1TET, Q1HEX):
                raise NotImplementedError("tagged-facet BCs are provided for P1/Q1 spaces")
            em, conn = fe.dof.elemMap, m.conn
            nv = conn.shape[1]
            node2dof = np.full(m.xyz.shape[0], -1, dtype=np.int64)
            node2dof[conn.reshape(-1).astype(np.int64)] = em[:, :nv].reshape(-1)
            return node2dof[sel]
        # box: the facets markFacetsCube tags with `marker` lie on one plane of the box
        axis, upper = side.PLANE[marker]
        lo, hi = m.xyz[:, axis].min(), m.xyz[:, axis].max()
        val = hi if upper else lo
        x = _interp_coord(fe, axis)
        return np.nonzero(np.abs(x - val) <= 1e-6 * (hi - lo))[0]


# ----------------------------------------------------------------- assemblies
class AssemblyStiffness:
    """AssemblyStiffness(c, feSpace) (include/assembly_lhs.hpp:36-75)."""

    def __init__(self, coef, fe):
        self.fe, self.op = fe, {"stiffness": 1, "stiff_coef": float(coef)}


class AssemblyStiffnessFE:
    """AssemblyStiffnessFE(coefP0, feSpace) with a per-element (P0) coefficient
    (include/assembly_lhs.hpp:77-113)."""

    def __init__(self, k_e, fe, scale=1.0):
        self.k_e = np.ascontiguousarray(k_e, dtype=np.float64)
        fe.set_coefficient(self.k_e)
        self.fe, self.op = fe, {"stiffness": 2, "stiff_coef": float(scale)}


class AssemblyScalarMass:
    """AssemblyScalarMass / AssemblyMass(c, feSpace) (include/assembly_lhs.hpp:191-231, 347-365)."""

    def __init__(self, coef, fe):
        self.fe, self.op = fe, {"mass": 1, "mass_coef": float(coef)}


AssemblyMass = AssemblyScalarMass


class AssemblyMassFE:
    """AssemblyMassFE(coefP0, feSpace) with a per-element (P0) coefficient
    (include/assembly_lhs.hpp:234-277).  The space holds one per-element coefficient:
    with AssemblyStiffnessFE in the same call, both must be given the same values."""

    def __init__(self, k_e, fe, scale=1.0):
        self.k_e = np.ascontiguousarray(k_e, dtype=np.float64)
        fe.set_coefficient(self.k_e)
        self.fe, self.op = fe, {"mass": 2, "mass_coef": float(scale)}


class AssemblyTensorStiffness:
    """AssemblyTensorStiffness(c, feSpace) on a vector space (include/assembly_lhs.hpp:116-161)."""

    def __init__(self, coef, fe):
        self.fe, self.kind, self.coef = fe, 2, float(coef)


class AssemblyGrad:
    """AssemblyGrad(c, vector space, scalar space) (include/assembly_coupling.hpp:42-86)."""

    def __init__(self, coef, fe1, fe2):
        self.fe1, self.fe2, self.kind, self.coef = fe1, fe2, 4, float(coef)


class AssemblyDiv:
    """AssemblyDiv(c, scalar space, vector space) (include/assembly_coupling.hpp:89-132)."""

    def __init__(self, coef, fe1, fe2):
        self.fe1, self.fe2, self.kind, self.coef = fe1, fe2, 5, float(coef)


def _sys_op(a):
    """(space, kind, coef) of a square assembly in a system call."""
    if getattr(a, "kind", None) == 2:
        return a.fe, 2, a.coef
    o = getattr(a, "op", None) or {}
    if o.get("stiffness") == 1:
        return a.fe, 1, o["stiff_coef"]
    if o.get("mass") == 1:
        return a.fe, 3, o["mass_coef"]
    raise PxgError(6, f"{type(a).__name__} is not an assembly of the system path")


class AssemblyRhsAnalytic:
    """AssemblyRhsAnalytic(f, feSpace, comps) (include/assembly_rhs.hpp:34-91).

    f is any Python callable, as the reference takes any std::function: it gets the
    (n, 3) array of the space's quadrature points (CurFE::qpoint, from the device) and
    returns n values (a scalar space) or an (n, dim) array (a vector space); the values
    go to the device and are integrated there (rhs kind 3).  f may also be one of the
    device's function ids (pxg_fn, evaluated on the device: the fast path), one per
    component on a vector space.  coef scales f (one value or one per component), and
    only the components listed in ``comps`` (default: all) get a load: component c of
    the load goes to block c (assembly_rhs.hpp:66-73)."""

    def __init__(self, fn, fe, coef=1.0, comps=None):
        self.fe = fe
        coefs = np.broadcast_to(np.asarray(coef, dtype=np.float64), (fe.dim,))
        comps = list(range(fe.dim)) if comps is None else [int(c) for c in comps]
        if any(not 0 <= c < fe.dim for c in comps):
            raise ValueError("AssemblyRhsAnalytic: component out of range")
        if callable(fn):
            import torch

            qp = fe.ctx.get_qpoints().reshape(-1, 3)
            v = np.asarray(fn(qp), dtype=np.float64).reshape(qp.shape[0], -1)
            if v.shape[1] != fe.dim:
                raise ValueError(f"AssemblyRhsAnalytic: f returned {v.shape[1]} components, the space has {fe.dim}")
            dev = f"cuda:{fe.ctx.device}"
            self.values = [torch.as_tensor(np.ascontiguousarray(v[:, c])).to(dev) for c in range(fe.dim)]
            self.parts = [(c, {"kind": 3, "coef": float(coefs[c]), "field": self.values[c]}) for c in comps]
            self.rhs = self.parts[0][1]
            return
        if fe.dim == 1:
            if np.ndim(fn) != 0 or comps != [0]:
                raise ValueError("AssemblyRhsAnalytic: a scalar space takes one function id")
            self.rhs = {"kind": 1, "fn": int(fn), "coef": float(coef)}
            self.parts = [(0, self.rhs)]
            return
        fns = np.asarray(fn).reshape(-1)
        if fns.size != fe.dim:
            raise ValueError(f"AssemblyRhsAnalytic: a {fe.dim}-component space takes {fe.dim} function ids")
        self.parts = [(c, {"kind": 1, "fn": int(fns[c]), "coef": float(coefs[c])}) for c in comps]


class AssemblyS2SProjection:
    """AssemblyS2SProjection(c, field, feSpace, comps) (include/assembly_rhs.hpp:93-163).

    On a vector space the field holds every component (BLOCK ordering, component d of
    DOF k at k + d * ndof), and the j-th listed component of the field (default: all)
    is projected into block j, as the reference's running block index does
    (assembly_rhs.hpp:138-156)."""

    def __init__(self, coef, field, fe, comps=None):
        import torch

        self.field = torch.as_tensor(np.ascontiguousarray(field, dtype=np.float64)).to(f"cuda:{fe.ctx.device}")
        nd = fe.dof.size
        if self.field.numel() != nd * fe.dim:
            raise ValueError(f"AssemblyS2SProjection: the field has {self.field.numel()} values, "
                             f"the space {nd * fe.dim}")
        self.fe = fe
        self.rhs = {"kind": 2, "coef": float(coef), "field": self.field}
        comps = range(fe.dim) if comps is None else comps
        if any(not 0 <= int(c) < fe.dim for c in comps):
            raise ValueError("AssemblyS2SProjection: component out of range")
        self.parts = [(j, {"kind": 2, "coef": float(coef), "field": self.field[int(c) * nd:(int(c) + 1) * nd]})
                      for j, c in enumerate(comps)]


AssemblyProjection = AssemblyS2SProjection


def interpolateAnalyticFunction(fn, fe, coef=1.0):
    """interpolateAnalyticFunction (include/fespace.hpp:195-271) on the device."""
    import torch

    v = torch.zeros(fe.dof.size, dtype=torch.float64, device=f"cuda:{fe.ctx.device}")
    fe.ctx.interpolate(fn, coef, v)
    torch.cuda.synchronize()
    return v.cpu().numpy()


class Builder:
    """Builder (include/builder.hpp:12-391): buildLhs / buildRhs accumulate into a
    device value array on the structural pattern and into b; closeMatrix prunes
    |v| <= 1e-16 and exposes the CSR (A on the host as scipy, A_dev on the device)."""

    def __init__(self, fe):
        import torch

        if isinstance(fe, (int, np.integer)):
            # Builder{numDOFs} over spaces with offsets: the calls are recorded and run on
            # a device system (pxg_sys) by closeMatrix, when every space is known
            self.size, self.fe, self._calls, self._rhs = int(fe), None, [], []
            self.A = self.A_dev = None
            self._b = None
            return
        self.size = None
        self.fe = fe
        self.dev = f"cuda:{fe.ctx.device}"
        fe.pattern()
        self.vals = torch.zeros(fe.ctx.nnz, dtype=torch.float64, device=self.dev)
        self.b_dev = torch.zeros(fe.dof.size, dtype=torch.float64, device=self.dev)
        self.A = None
        self.A_dev = None

    def buildCoupling(self, assembly, bcsRow=(), bcsCol=()):
        """Builder::buildCoupling (include/builder.hpp:156-277)."""
        if self.size is None:
            raise PxgError(6, "buildCoupling needs Builder(numDOFs)")
        self._calls.append((assembly.fe1, assembly.fe2, [(assembly.kind, assembly.coef)], list(bcsRow), list(bcsCol)))

    def buildLhs(self, assemblies, bcs=()):
        if self.size is not None:
            ops = [_sys_op(a) for a in assemblies]
            fe = ops[0][0]
            if any(o[0] is not fe for o in ops):
                raise PxgError(6, "buildLhs: the assemblies of one call share one space")
            self._calls.append((fe, fe, [(k, c) for _, k, c in ops], list(bcs), list(bcs)))
            return
        op = {"stiffness": 0, "stiff_coef": 0.0, "mass": 0, "mass_coef": 0.0, "apply_bc": 1 if bcs else 0}
        if len(assemblies) == 0:
            raise ValueError("we need at least 1 assembly.")
        # the space holds one per-element coefficient: the call's P0 assemblies share it,
        # and it is set again here (another assembly may have been built since)
        coefs = [a.k_e for a in assemblies if getattr(a, "k_e", None) is not None]
        if any(not np.array_equal(c, coefs[0]) for c in coefs[1:]):
            raise PxgError(6, "the per-element coefficients of one buildLhs call must be the same")
        if coefs:
            self.fe.set_coefficient(coefs[0])
        for a in assemblies:
            o = getattr(a, "op", None)
            if o is None:
                raise PxgError(6, f"{type(a).__name__} is not a matrix assembly known to the engine")
            if "stiffness" in o:
                if op["stiffness"]:
                    raise PxgError(6, "one stiffness term per buildLhs call")
                op["stiffness"], op["stiff_coef"] = o["stiffness"], o["stiff_coef"]
            if "mass" in o:
                if op["mass"]:
                    raise PxgError(6, "one mass term per buildLhs call")
                op["mass"], op["mass_coef"] = o["mass"], o["mass_coef"]
        self.fe.apply_bcs(list(bcs))
        self.fe.ctx.assemble(op0=op, vals0=self.vals, b=self.b_dev if bcs else None, accumulate=True)

    def buildRhs(self, assemblies, bcs=()):
        if any(a.fe.qr_type != a.fe.etype for a in assemblies):
            # the element kernels integrate loads with the element's own rule
            raise PxgError(6, "buildRhs on a space with another quadrature rule is not provided")
        if self.size is not None:
            self._rhs.append((list(assemblies), list(bcs)))
            return
        if self.fe.dim != 1:
            raise PxgError(6, "a vector space needs Builder(numDOFs)")
        self.fe.apply_bcs(list(bcs))
        for a in assemblies:
            r = dict(a.rhs)
            r["apply_bc"] = 1 if bcs else 0
            self.fe.ctx.assemble(rhs=r, b=self.b_dev, accumulate=True)

    def _close_system(self):
        import scipy.sparse as sp
        import torch

        from ._lib import System

        spaces = []
        for fr, fc, _, _, _ in self._calls:
            for f in (fr, fc):
                if all(f is not g for g in spaces):
                    spaces.append(f)
        for a, _ in self._rhs:
            for x in a:
                if all(x.fe is not g for g in spaces):
                    spaces.append(x.fe)
        spaces.sort(key=lambda f: f.offset)
        off = 0
        for f in spaces:
            if f.offset != off:
                raise PxgError(1, f"space offsets: expected {off}, got {f.offset}")
            off += f.dof.size * f.dim
        if off != self.size:
            raise PxgError(1, f"Builder size {self.size} != sum of the spaces' DOFs {off}")
        S = System([f.ctx for f in spaces], [f.dim for f in spaces], [f.qr_type for f in spaces])
        index = {id(f): k for k, f in enumerate(spaces)}
        dev = f"cuda:{spaces[0].ctx.device}"
        vals = torch.zeros(S.nnz, dtype=torch.float64, device=dev)
        b = torch.zeros(S.ntot, dtype=torch.float64, device=dev)

        def set_bcs(f, bcs):
            if bcs:
                d, v = zip(*(x.component_dofs() for x in bcs))
                S.set_bc(index[id(f)], np.concatenate(d), np.concatenate(v), bcs[-1].diag)
            else:
                S.set_bc(index[id(f)], np.zeros(0, np.uint32), np.zeros(0))

        for fr, fc, ops, br, bc in self._calls:
            set_bcs(fr, br)
            if fc is not fr:
                set_bcs(fc, bc)
            S.assemble(index[id(fr)], index[id(fc)], ops, vals, b, accumulate=True)
        for assemblies, bcs in self._rhs:
            for a in assemblies:
                f = a.fe
                f.pattern()  # the element kernels scatter through the space's own pattern
                nd = f.dof.size
                for blk, part in a.parts:
                    # buildRhs zeroes the constrained rows of each block (C Fe,
                    # include/builder.hpp:322-343): block blk is condensed with the DOFs
                    # constrained in component blk
                    if f.dim == 1:
                        f.apply_bcs(bcs)
                    else:
                        _component_bcs(f, bcs, blk)
                    r = dict(part)
                    r["apply_bc"] = 1 if bcs else 0
                    lo = f.offset + blk * nd
                    f.ctx.assemble(rhs=r, b=b[lo:lo + nd], accumulate=True)
        rp, ci = S.get_pattern()
        torch.cuda.synchronize()
        A = sp.csr_matrix((vals.cpu().numpy(), ci, rp), shape=(S.ntot, S.ntot))
        A.data[np.abs(A.data) <= 1e-16] = 0.0  # closeMatrix: prune(1, 1e-16)
        A.eliminate_zeros()
        A.sort_indices()
        self.A = A
        self._b = b
        self._sys = S

    def closeMatrix(self):
        import scipy.sparse as sp
        import torch

        if self.size is not None:
            return self._close_system()
        ctx = self.fe.ctx
        rp_s, ci_s = ctx.pattern_device()
        n = self.fe.dof.size
        if ctx.prune_count(self.vals) == 0:
            rp = torch.empty(n + 1, dtype=torch.int32, device=self.dev)
            ci = torch.empty(ctx.nnz, dtype=torch.int32, device=self.dev)
            rph, cih = ctx.get_pattern()
            rp.copy_(torch.from_numpy(rph))
            ci.copy_(torch.from_numpy(cih))
            vals = self.vals.clone()
        else:
            rp = torch.empty(n + 1, dtype=torch.int32, device=self.dev)
            ci = torch.empty(ctx.nnz, dtype=torch.int32, device=self.dev)
            vals = torch.empty(ctx.nnz, dtype=torch.float64, device=self.dev)
            nnz = ctx.close_matrix(self.vals, rp, ci, vals)
            ci, vals = ci[:nnz], vals[:nnz]
        torch.cuda.synchronize()
        self.A_dev = (rp, ci, vals)
        self.A = sp.csr_matrix((vals.cpu().numpy(), ci.cpu().numpy(), rp.cpu().numpy()), shape=(n, n))
        self.vals.zero_()  # setFromTriplets consumed the triplets (builder.hpp:370)

    @property
    def b(self):
        import torch

        torch.cuda.synchronize()
        if self.size is not None:
            return self._b.cpu().numpy() if self._b is not None else np.zeros(self.size)
        return self.b_dev.cpu().numpy()

    def clearRhs(self):
        self.b_dev.zero_()

    def clearLhs(self):
        self.vals.zero_()

    def clear(self):
        self.clearLhs()
        self.clearRhs()


class LUSolver:
    """UmfPackLU's interface as proxpde's tests use it (include/sparse_matrix.hpp:44:
    analyzePattern, factorize, solve) over the engine's device Jacobi-preconditioned CG
    (pxg_cg) on a Builder's closed matrix: factorize keeps the device CSR
    (Builder.A_dev), each solve runs the CG from x = 0 to the relative residual rtol
    (1e-14 by default) and raises PxgError (not converged) at max_iter.  The CG needs a
    symmetric positive definite matrix, which a direct LU does not.  iterations and
    rel_res report the last solve."""

    def __init__(self, rtol=1e-14, max_iter=None):
        self.rtol, self.max_iter = float(rtol), max_iter
        self.builder = None
        self.iterations, self.rel_res = 0, 0.0

    def analyzePattern(self, builder):
        if getattr(builder, "A_dev", None) is None or builder.fe is None:
            raise PxgError(1, "LUSolver: a scalar Builder closed with closeMatrix is needed")
        self.builder = builder

    def factorize(self, builder):
        if builder is not self.builder:
            raise PxgError(1, "LUSolver: factorize the analysed Builder's matrix")
        rp, ci, v = builder.A_dev
        self.A = (rp, ci.contiguous(), v.contiguous())

    def compute(self, builder):
        self.analyzePattern(builder)
        self.factorize(builder)

    def solve(self, b):
        import torch

        rp, ci, v = self.A
        ctx = self.builder.fe.ctx
        bd = torch.as_tensor(np.ascontiguousarray(b, dtype=np.float64)).to(rp.device)
        x = torch.zeros_like(bd)
        n = bd.numel()
        mi = self.max_iter or 10 * n + 1000
        self.iterations, self.rel_res = ctx.cg(rp, ci, v, bd, x, rtol=self.rtol, max_iter=mi)
        torch.cuda.synchronize()
        return x.cpu().numpy()

