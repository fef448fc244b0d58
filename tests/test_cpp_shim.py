"""The C++20 drop-in shim (include/proxgpu/builder.hpp): it compiles on any machine
(CPU test), and the C++ port of proxpde's poisson3dhex / poisson3dhex_q2 tests built
on it reproduces their golden error norms on the GPU (tolerance 1e-12)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "poisson3d.cpp")


def test_shim_compiles(tmp_path):
    r = subprocess.run(["g++", "-std=c++20", "-Wall", "-Wextra", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                        SRC], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("order,n,expected", [(1, 4, 0.1352139631934435),   # test/poisson3dhex.cpp:118
                                              (2, 4, 0.0070042836287997),   # test/poisson3dhex_q2.cpp:120
                                              (2, 8, 0.001164556821288369)])  # test/poisson3dhex_q2.cpp:126
def test_shim_reproduces_goldens(engine, tmp_path, order, n, expected):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    from proxpde_gb300 import build

    lib = build.build()
    exe = tmp_path / "poisson3d"
    r = subprocess.run(["g++", "-std=c++20", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", str(exe),
                        f"-L{os.path.dirname(lib)}", "-lpxg", f"-Wl,-rpath,{os.path.dirname(lib)}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(order), str(n), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = out.read_bytes()
    nrow, nnz = np.frombuffer(raw[:16], dtype=np.int64)
    off = 16
    rp = np.frombuffer(raw, np.int32, nrow + 1, off); off += 4 * (nrow + 1)
    ci = np.frombuffer(raw, np.int32, nnz, off); off += 4 * nnz
    va = np.frombuffer(raw, np.float64, nnz, off); off += 8 * nnz
    b = np.frombuffer(raw, np.float64, nrow, off); off += 8 * nrow
    ex = np.frombuffer(raw, np.float64, nrow, off)
    A = sp.csr_matrix((va, ci, rp), shape=(nrow, nrow)).tocsc()
    u = spla.spsolve(A, b)
    assert abs(np.linalg.norm(u - ex) - expected) < 1e-12
