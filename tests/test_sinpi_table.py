"""The table of the kernels' table-driven sin(pi x) (proxpde_gb300/csrc/pxg_sinpi_table.h):
entry k holds the doubles nearest to sin(pi k / 64) and cos(pi k / 64).  Checked against a
60-digit evaluation where mpmath is importable (exact equality), and against libm at
math.pi * k / 64 within 1e-15 (that argument is itself rounded, so libm's values are only
this close); the axes' zeros and ones are exact."""
import math
import os
import re

import pytest

HDR = os.path.join(os.path.dirname(__file__), "..", "proxpde_gb300", "csrc", "pxg_sinpi_table.h")


def table():
    txt = open(HDR).read()
    pairs = re.findall(r"\{(-?0x[0-9a-fp.+-]+), (-?0x[0-9a-fp.+-]+)\}", txt)
    return [(float.fromhex(s), float.fromhex(c)) for s, c in pairs]


def test_table_shape_and_axes():
    t = table()
    assert len(t) == 128
    for k in (0, 32, 64, 96):  # sin or cos exactly 0 and the other exactly +-1
        s, c = t[k]
        assert {abs(s), abs(c)} == {0.0, 1.0}
    assert t[0] == (0.0, 1.0) and t[32] == (1.0, 0.0) and t[64] == (0.0, -1.0) and t[96] == (-1.0, 0.0)


def test_table_against_libm():
    for k, (s, c) in enumerate(table()):
        a = math.pi * k / 64
        assert abs(s - math.sin(a)) <= 1e-15 and abs(c - math.cos(a)) <= 1e-15


def test_table_correctly_rounded():
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 60
    for k, (s, c) in enumerate(table()):
        x = mpmath.mpf(k) / 64
        assert s == float(mpmath.sinpi(x)) and c == float(mpmath.cospi(x))
