"""The C++20 drop-in shim (include/proxgpu/builder.hpp): it compiles on any machine
(CPU test), and the C++ port of proxpde's poisson3dhex / poisson3dhex_q2 tests built
on it reproduces their golden error norms on the GPU (tolerance 1e-12)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "poisson3d.cpp")


STOKES = os.path.join(ROOT, "tests", "cpp", "stokes3d.cpp")
LOADS = os.path.join(ROOT, "tests", "cpp", "vector_loads.cpp")
PORT = os.path.join(ROOT, "tests", "cpp", "poisson3dhex_port.cpp")


@pytest.mark.parametrize("src", [SRC, STOKES, LOADS, PORT], ids=["poisson3d", "stokes3d", "vector_loads", "port"])
def test_shim_compiles(tmp_path, src):
    r = subprocess.run(["g++", "-std=c++20", "-Wall", "-Wextra", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                        src], capture_output=True, text=True)
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


@pytest.mark.gpu
@pytest.mark.parametrize("elem,expected", [
    # test/stokes3dhex.cpp:135-140
    ("hex", [1.309442419567852e-15, 1.021847252919293e-14, 1.800953966048908e-15, 1.097009563518918e-14]),
    # test/stokes3dtet.cpp:122-127
    ("tet", [1.191610761242353e-15, 4.347071660478249e-15, 1.168951507916659e-15, 5.36156027085171e-14]),
])
def test_shim_stokes_goldens(engine, tmp_path, elem, expected):
    """The C++ port of proxpde's Stokes tests on the shim (vector space, Builder{numDOFs},
    buildCoupling, component-wise BCEss with functions) reproduces their error norms."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    from proxpde_gb300 import build

    lib = build.build()
    exe = tmp_path / "stokes3d"
    r = subprocess.run(["g++", "-std=c++20", "-O2", "-I", os.path.join(ROOT, "include"), STOKES, "-o", str(exe),
                        f"-L{os.path.dirname(lib)}", "-lpxg", f"-Wl,-rpath,{os.path.dirname(lib)}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), elem, str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = out.read_bytes()
    nrow, nnz, ndu = np.frombuffer(raw[:24], dtype=np.int64)
    off = 24
    rp = np.frombuffer(raw, np.int32, nrow + 1, off); off += 4 * (nrow + 1)
    ci = np.frombuffer(raw, np.int32, nnz, off); off += 4 * nnz
    va = np.frombuffer(raw, np.float64, nnz, off); off += 8 * nnz
    b = np.frombuffer(raw, np.float64, nrow, off); off += 8 * nrow
    ex = np.frombuffer(raw, np.float64, nrow, off)
    u = spla.spsolve(sp.csr_matrix((va, ci, rp), shape=(nrow, nrow)).tocsc(), b)
    err = [np.linalg.norm(u[c * ndu:(c + 1) * ndu] - ex[c * ndu:(c + 1) * ndu]) for c in range(3)]
    err.append(np.linalg.norm(u[3 * ndu:] - ex[3 * ndu:]))
    for e, r_ in zip(err, expected):
        assert abs(e - r_) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("elem", ["hex", "tet"])
def test_shim_vector_loads(engine, tmp_path, elem):
    """buildRhs on a vector space through the shim's Builder{numDOFs} (per-component
    device functions, projection of reordered field components, component-wise BCEss)
    against the oracle's loads block by block (tests/helpers.py:vector_load_expect)."""
    from helpers import assert_close, vector_load_expect, vector_load_field
    from proxpde_gb300 import Hexahedron, Tetrahedron, build, buildHyperCube

    lib = build.build()
    exe = tmp_path / "vector_loads"
    r = subprocess.run(["g++", "-std=c++20", "-O2", "-I", os.path.join(ROOT, "include"), LOADS, "-o", str(exe),
                        f"-L{os.path.dirname(lib)}", "-lpxg", f"-Wl,-rpath,{os.path.dirname(lib)}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), elem, str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = out.read_bytes()
    ntot, ndu, ndp = np.frombuffer(raw[:24], dtype=np.int64)
    b = np.frombuffer(raw, np.float64, ntot, 24)
    assert ntot == 3 * ndu + ndp
    mesh = buildHyperCube(Hexahedron if elem == "hex" else Tetrahedron, 3)
    expect, _ = vector_load_expect(elem, mesh.xyz, mesh.conn, vector_load_field(3 * ndu))
    assert_close(b, expect, what="shim vector and scalar loads")


@pytest.mark.gpu
def test_shim_port_of_poisson3dhex(engine, tmp_path):
    """proxpde's test/poisson3dhex.cpp body on the shim with the namespace changed
    (buildHyperCube(mesh, origin, length, {n,n,n}), FESpace<Mesh_T, RefFE_T, QR_T>,
    BCEss << lambda, Builder{dof.size}, the rhs as a host lambda, LUSolver on the device
    CG, interpolateAnalyticFunction of a lambda, checkError): exit code 0 means the
    golden norm 0.1352139631934435 (test/poisson3dhex.cpp:118) is met to 1e-12, and the
    host residual builder.A * sol - builder.b (the Eigen-like interface of the closed
    matrix) is below 1e-12 of |b|."""
    from proxpde_gb300 import build

    lib = build.build()
    exe = tmp_path / "poisson3dhex_port"
    r = subprocess.run(["g++", "-std=c++20", "-O2", "-I", os.path.join(ROOT, "include"), PORT, "-o", str(exe),
                        f"-L{os.path.dirname(lib)}", "-lpxg", f"-Wl,-rpath,{os.path.dirname(lib)}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), "4", "0.1352139631934435"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
