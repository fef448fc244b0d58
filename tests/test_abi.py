"""The C ABI library: it builds here (nvcc cross-compiles for sm_103a), loads without
a GPU, and exports every function include/pxg.h declares.  No compute calls."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"^\s*(?:pxg_status|const char \*|int)\s+(pxg_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def lib():
    from proxpde_gb300 import build

    path = build.build()
    return ctypes.CDLL(path)


def test_exports_every_declared_symbol(lib):
    names = declared("pxg.h")
    assert len(names) >= 19
    for n in names:
        assert hasattr(lib, n), n


def test_python_binding_lists_every_symbol():
    from proxpde_gb300 import _lib

    assert sorted(_lib.EXPORTS) == declared("pxg.h")


def test_status_strings(lib):
    lib.pxg_status_string.restype = ctypes.c_char_p
    assert lib.pxg_status_string(0) == b"ok"
    assert lib.pxg_status_string(5) == b"not converged"
    lib.pxg_version.restype = ctypes.c_int
    assert lib.pxg_version() >= 10000


def test_no_device_and_null_context_are_reported(lib):
    """Without a GPU, pxg_create reports PXG_ERR_NO_DEVICE and leaves the context null;
    calls on a null context are rejected with PXG_ERR_INVALID_ARG before any CUDA call.
    (On a machine with a GPU only the null-context part runs.)"""
    import torch

    ctx = ctypes.c_void_p()
    if not torch.cuda.is_available():
        assert lib.pxg_create(ctypes.byref(ctx), 0) == 7
        assert ctx.value is None
        from proxpde_gb300 import Context, PxgError

        with pytest.raises(PxgError) as ei:
            Context(0)
        assert ei.value.status == 7
    n = ctypes.c_int64(-1)
    assert lib.pxg_build_dofmap(None, ctypes.byref(n)) == 1
    assert lib.pxg_build_pattern(None, ctypes.byref(n)) == 1
    assert lib.pxg_assemble(None, None, None, None, None, None, None, 0, None) == 1
    lib.pxg_last_error.restype = ctypes.c_char_p
    assert isinstance(lib.pxg_last_error(None), bytes)
