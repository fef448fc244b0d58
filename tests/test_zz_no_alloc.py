"""The allocation-free prune entry point (pxg_prune_csr_noalloc) against the regular
closeMatrix entry point (pxg_close_matrix), through the C ABI.

The entry point exists for callers that cannot allocate GPU memory (for example a
host application that owns every device allocation, or code running in a host
callback); it keeps its intermediate data in a fixed device array instead.  Two
calls in a row must both reproduce the regular entry point exactly: the second call
finds the array holding the first call's data and must not depend on it.

This file is named to be collected last, so that a failure here does not hide the
results of the other tests in a run that stops at the first failure.
"""
import ctypes as C
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_prune_matches_close_matrix(engine):
    import torch

    from proxpde_gb300 import Context, _lib, meshgen

    # unperturbed P1 mesh with k = 1: many stiffness sums cancel and are pruned
    xyz, conn = meshgen.cube_tet6(10)
    ctx = Context(0)
    ctx.set_mesh(_lib.P1TET, xyz, conn)
    ndof = ctx.build_dofmap()
    nnz = ctx.build_pattern()
    vals = torch.empty(nnz, dtype=torch.float64, device="cuda")
    ctx.assemble(op0={"stiffness": 1, "stiff_coef": 1.0}, vals0=vals)

    # regular entry point
    rp = torch.empty(ndof + 1, dtype=torch.int32, device="cuda")
    ci = torch.empty(nnz, dtype=torch.int32, device="cuda")
    vo = torch.empty(nnz, dtype=torch.float64, device="cuda")
    m = ctx.close_matrix(vals, rp, ci, vo)
    assert 0 < m < nnz
    ref = (rp.cpu().numpy(), ci[:m].cpu().numpy(), vo[:m].cpu().numpy())

    L = _lib.load()
    srp, sci = ctx.pattern_device()
    for call in range(2):
        rp2 = torch.full((ndof + 1,), -7, dtype=torch.int32, device="cuda")
        ci2 = torch.full((nnz,), -7, dtype=torch.int32, device="cuda")
        vo2 = torch.full((nnz,), np.nan, dtype=torch.float64, device="cuda")
        n_out = C.c_int64(-1)
        st = L.pxg_prune_csr_noalloc(srp, sci, vals.data_ptr(), ndof, rp2.data_ptr(), ci2.data_ptr(),
                                     vo2.data_ptr(), C.byref(n_out), None)
        assert st == 0, f"call {call}: status {st}"
        assert n_out.value == m
        torch.cuda.synchronize()
        assert np.array_equal(rp2.cpu().numpy(), ref[0])
        assert np.array_equal(ci2[:m].cpu().numpy(), ref[1])
        assert np.array_equal(vo2[:m].cpu().numpy(), ref[2])  # a pure compaction: exact


def test_noalloc_rejects_oversize(engine):
    from proxpde_gb300 import _lib

    L = _lib.load()
    n_out = C.c_int64(-1)
    st = L.pxg_prune_csr_noalloc(1, 1, 1, (1 << 22) + 1, 1, 1, 1, C.byref(n_out), None)
    assert st == 1 and n_out.value == -1


@pytest.mark.parametrize("nrows", [5_000, 1 << 22], ids=["5k", "max"])
def test_noalloc_ragged_csr_and_no_allocation(engine, nrows):
    """A ragged synthetic CSR (empty rows included; values of both signs, exact zeros,
    1e-17, exactly 1e-16 and just above it) with more rows than one block-total scan
    thread covers, up to the 4,194,304-row maximum, against numpy's prune; and the
    call allocates no device memory: torch's allocator is unchanged across it and the
    device's free memory (cudaMemGetInfo) does not drop, after a first call that sets
    up the scratch address."""
    import torch

    from proxpde_gb300 import _lib

    rng = np.random.default_rng(nrows)
    lens = rng.integers(0, 5 if nrows > 100_000 else 17, nrows)
    lens[rng.random(nrows) < 0.05] = 0
    rp = np.zeros(nrows + 1, dtype=np.int32)
    np.cumsum(lens, out=rp[1:])
    nnz = int(rp[-1])
    ci = rng.integers(0, nrows, nnz).astype(np.int32)
    vals = rng.standard_normal(nnz)
    pick = rng.random(nnz)
    vals[pick < 0.2] = 0.0
    vals[(pick >= 0.2) & (pick < 0.25)] = 1e-17
    vals[(pick >= 0.25) & (pick < 0.28)] = -1e-16
    vals[(pick >= 0.28) & (pick < 0.31)] = 1.0000001e-16
    keep = ~(np.abs(vals) <= 1e-16)
    rows = np.repeat(np.arange(nrows), lens)
    kept_rows = np.bincount(rows[keep], minlength=nrows)
    rp_ref = np.zeros(nrows + 1, dtype=np.int32)
    np.cumsum(kept_rows, out=rp_ref[1:])
    m = int(keep.sum())

    d_rp, d_ci, d_v = (torch.as_tensor(x).cuda() for x in (rp, ci, vals))
    out_rp = torch.empty(nrows + 1, dtype=torch.int32, device="cuda")
    out_ci = torch.empty(nnz, dtype=torch.int32, device="cuda")
    out_v = torch.empty(nnz, dtype=torch.float64, device="cuda")
    L = _lib.load()

    def call():
        n_out = C.c_int64(-1)
        st = L.pxg_prune_csr_noalloc(d_rp.data_ptr(), d_ci.data_ptr(), d_v.data_ptr(), nrows, out_rp.data_ptr(),
                                     out_ci.data_ptr(), out_v.data_ptr(), C.byref(n_out), None)
        assert st == 0
        return n_out.value

    assert call() == m
    # objects of earlier tests that the garbage collector destroys during the window
    # would release device memory; an allocation by the call can only lower it
    gc.collect()
    gc.disable()
    try:
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        alloc0 = torch.cuda.memory_allocated()
        assert call() == m
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
    finally:
        gc.enable()
    assert torch.cuda.memory_allocated() == alloc0
    assert free1 >= free0, (free0, free1)
    assert np.array_equal(out_rp.cpu().numpy(), rp_ref)
    assert np.array_equal(out_ci[:m].cpu().numpy(), ci[keep])
    assert np.array_equal(out_v[:m].cpu().numpy(), vals[keep])
