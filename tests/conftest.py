"""pytest configuration: the `gpu` marker and the repository root on sys.path.

Tests marked ``gpu`` need a CUDA device and the built engine library; the rest run
on any CPU (oracle, host logic, ABI exports).
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built engine library")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle

    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def engine():
    """Builds (if needed) and loads libpxg.so; GPU tests only."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    from proxpde_gb300 import build

    build.build()
    import proxpde_gb300 as px

    px.load()
    return px


def pytest_terminal_summary(terminalreporter):
    """The largest entrywise relative error of each named engine-vs-oracle comparison,
    over the entries above 1e-3 and above 1e-8 of their row's largest, one line each."""
    try:
        from helpers import ERRORS
    except ImportError:
        return
    if not ERRORS:
        return
    terminalreporter.write_sep("-", "entrywise relative error against the oracle (entries >= 1e-3 / >= 1e-8 "
                                    "of their row's largest)")
    for k in sorted(ERRORS):
        terminalreporter.write_line(f"{k}: {ERRORS[k][0]:.3e} / {ERRORS[k][1]:.3e}")
