"""Writes pxg_sinpi_table.h: sin(pi k / 64) and cos(pi k / 64) for k = 0 .. 127, each
rounded to the nearest double from a 60-digit evaluation (mpmath's sinpi / cospi,
exact zeros on the axes), as C++17 hexadecimal
floating literals.  Run from this directory: python gen_sinpi_table.py"""
import os

import mpmath

mpmath.mp.dps = 60
lines = [
    "// Generated by gen_sinpi_table.py: {sin(pi k / 64), cos(pi k / 64)}, k = 0 .. 127, each the",
    "// double nearest to the exact value.",
    "#pragma once",
    "namespace pxg",
    "{",
    "__device__ __align__(16) double const kSinCosPi64[128][2] = {",
]
for k in range(128):
    a = mpmath.mpf(k) / 64  # exact
    s, c = float(mpmath.sinpi(a)), float(mpmath.cospi(a))  # exact zeros at the axes
    lines.append(f"    {{{s.hex()}, {c.hex()}}},")
lines += ["};", "} // namespace pxg", ""]
with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "pxg_sinpi_table.h"), "w") as f:
    f.write("\n".join(lines))
