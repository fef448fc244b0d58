"""Host logic of the Python mirror that needs no GPU: how a load on a vector space is
split into per-block scalar loads (per-component function ids and coefficients, the
component list of assembly_rhs.hpp:34-91), and which constrained DOFs each block's
condensation gets (the component's DOFs, as the space's own ids)."""
import numpy as np
import pytest

import proxpde_gb300 as px
from proxpde_gb300 import _component_bcs


class FakeCtx:
    def __init__(self):
        self.calls = []

    def set_bc(self, dofs, vals, diag=1.0):
        self.calls.append((np.asarray(dofs).copy(), np.asarray(vals).copy(), diag))


class FakeSpace:
    def __init__(self, dim, nd=5):
        self.dim = dim
        self.dof = type("Dof", (), {"size": nd})()
        self.ctx = FakeCtx()
        self._bc_key = ("cached",)


class FakeBc:
    def __init__(self, dofs, vals, diag=1.0):
        self.d = np.asarray(dofs, dtype=np.uint32)
        self.v = np.asarray(vals, dtype=np.float64)
        self.diag = diag

    def component_dofs(self):
        return self.d, self.v


def test_vector_analytic_load_parts():
    vel = FakeSpace(3)
    a = px.AssemblyRhsAnalytic([px.FN_SIN3, px.FN_CONST, px.FN_POISSON_RHS], vel, coef=[1.0, 2.0, -0.5], comps=[2, 0])
    assert [(c, r["fn"], r["coef"], r["kind"]) for c, r in a.parts] == [
        (2, px.FN_POISSON_RHS, -0.5, 1), (0, px.FN_SIN3, 1.0, 1)]
    a = px.AssemblyRhsAnalytic([px.FN_CONST] * 3, vel, coef=4.0)
    assert [(c, r["coef"]) for c, r in a.parts] == [(0, 4.0), (1, 4.0), (2, 4.0)]
    s = px.AssemblyRhsAnalytic(px.FN_SIN3, FakeSpace(1), 2.0)
    assert s.parts == [(0, {"kind": 1, "fn": px.FN_SIN3, "coef": 2.0})] and s.rhs is s.parts[0][1]
    with pytest.raises(ValueError):
        px.AssemblyRhsAnalytic(px.FN_CONST, vel)  # one id per component
    with pytest.raises(ValueError):
        px.AssemblyRhsAnalytic([px.FN_CONST] * 2, vel)
    with pytest.raises(ValueError):
        px.AssemblyRhsAnalytic([px.FN_CONST] * 3, vel, comps=[3])
    with pytest.raises(ValueError):
        px.AssemblyRhsAnalytic([px.FN_CONST], FakeSpace(1))  # a scalar space takes one id


def test_component_dirichlet_sets():
    vel = FakeSpace(3, nd=5)
    # component DOF ids k + c * 5
    bcs = [FakeBc([0, 6, 12, 3], [1.0, 2.0, 3.0, 4.0]), FakeBc([14, 5], [5.0, 6.0], diag=2.5)]
    want = {0: ([0, 3], [1.0, 4.0]), 1: ([1, 0], [2.0, 6.0]), 2: ([2, 4], [3.0, 5.0])}
    for c in range(3):
        _component_bcs(vel, bcs, c)
        d, v, diag = vel.ctx.calls[-1]
        assert d.dtype == np.uint32 and d.tolist() == want[c][0] and v.tolist() == want[c][1] and diag == 2.5
        assert vel._bc_key is None  # the space's cached scalar BC set is invalidated
        vel._bc_key = ("cached",)
    _component_bcs(vel, [], 1)
    d, v, diag = vel.ctx.calls[-1]
    assert d.size == 0 and v.size == 0 and diag == 1.0
