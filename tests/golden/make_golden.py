"""Generates the committed golden fixtures under tests/golden/.

Run where a proxpde checkout is available, giving its path as the argument or in
the environment variable PROXPDE_SRC:

    python tests/golden/make_golden.py /path/to/proxpde

Fixtures written:
  cube_uns.npz  - the unstructured tetrahedral unit cube of proxpde's
                  data/cube_uns.msh (GMSH 2.2 ASCII): node coordinates, tetrahedra
                  and the tagged boundary triangles, converted the way readGMSH
                  (include/mesh.hpp:785-1057) reads them: 1-based ids made 0-based,
                  unused nodes dropped and the rest renumbered in file order.
                  Used by the P1-tet golden test (test/poisson3dtet.cpp with
                  data/poisson3dtet.yaml: expected error 0.88528925443).
"""
import os
import sys

import numpy as np


def read_gmsh22(path):
    with open(path) as f:
        tok = f.read().split()
    i = 0
    assert tok[i] == "$MeshFormat" and tok[i + 1] == "2.2" and tok[i + 2] == "0"
    i = tok.index("$Nodes") + 1
    nn = int(tok[i]); i += 1
    xyz = np.zeros((nn, 3))
    for n in range(nn):
        assert int(tok[i]) == n + 1
        xyz[n] = [float(tok[i + 1]), float(tok[i + 2]), float(tok[i + 3])]
        i += 4
    i = tok.index("$Elements") + 1
    ne = int(tok[i]); i += 1
    tets, tris, tri_tags = [], [], []
    for _ in range(ne):
        etype, ntags = int(tok[i + 1]), int(tok[i + 2])
        tags = [int(x) for x in tok[i + 3:i + 3 + ntags]]
        i += 3 + ntags
        npts = {4: 4, 2: 3, 1: 2, 15: 1}[etype]
        ids = [int(x) - 1 for x in tok[i:i + npts]]
        i += npts
        if etype == 4:
            tets.append(ids)
        elif etype == 2:
            tris.append(ids)
            tri_tags.append(tags[0])
    tets = np.array(tets, dtype=np.int64)
    used = np.zeros(nn, dtype=bool)
    used[tets.reshape(-1)] = True
    newid = -np.ones(nn, dtype=np.int64)
    newid[used] = np.arange(used.sum())
    return (xyz[used], newid[tets].astype(np.uint32), newid[np.array(tris)].astype(np.uint32),
            np.array(tri_tags, dtype=np.uint32))


def main():
    """python make_golden.py <proxpde checkout>, or with PROXPDE_SRC set to it."""
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PROXPDE_SRC")
    if not ref:
        sys.exit("usage: make_golden.py <proxpde checkout> (or set PROXPDE_SRC)")
    out = os.path.dirname(os.path.abspath(__file__))
    xyz, tets, tris, tags = read_gmsh22(os.path.join(ref, "data", "cube_uns.msh"))
    np.savez_compressed(os.path.join(out, "cube_uns.npz"), xyz=xyz, tets=tets, tris=tris, tri_tags=tags)
    print("cube_uns.npz:", xyz.shape, tets.shape, tris.shape, np.bincount(tags))


if __name__ == "__main__":
    main()
