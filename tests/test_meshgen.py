"""The seeded synthetic inputs (proxpde_gb300.meshgen, proxpde_gb300.batch) that the
oracle, the tests and the bench share: the SplitMix64 generator against its published
first outputs, the interior-only perturbation, the lognormal coefficients, the
boundary node sets and the ragged batch of problems."""
import numpy as np

from proxpde_gb300 import batch, meshgen


def test_splitmix64_known_answers():
    # SplitMix64 (Steele, Lea and Flood 2014) from state 0: its first three outputs
    got = [int(v) for v in meshgen.splitmix64(0, np.arange(3))]
    assert got == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]
    u = meshgen.uniform01(5, np.arange(100000))
    assert u.min() >= 0.0 and u.max() < 1.0 and abs(u.mean() - 0.5) < 0.01


def test_perturb_moves_interior_nodes_only():
    n, alpha = 6, 0.2
    xyz, _ = meshgen.cube_hex(n)
    p = meshgen.perturb(xyz, n, alpha, 11)
    bnd = meshgen.boundary_nodes(n)
    assert bnd.size == (n + 1) ** 3 - (n - 1) ** 3
    assert np.array_equal(p[bnd], xyz[bnd])  # boundary planes stay flat
    interior = np.setdiff1d(np.arange(xyz.shape[0]), bnd)
    d = p[interior] - xyz[interior]
    assert np.all(np.abs(d) <= alpha / n) and np.all(d != 0.0)
    assert np.array_equal(p, meshgen.perturb(xyz, n, alpha, 11))  # seeded
    assert not np.array_equal(p, meshgen.perturb(xyz, n, alpha, 12))


def test_lognormal_moments():
    k = meshgen.lognormal(20261206, 400000, 0.5)
    lk = np.log(k)
    assert abs(lk.mean()) < 0.005 and abs(lk.std() - 0.5) < 0.005
    assert np.array_equal(k, meshgen.lognormal(20261206, 400000, 0.5))


def test_tet_splits_cover_the_cube():
    for gen, per in ((meshgen.cube_tet5, 5), (meshgen.cube_tet6, 6)):
        xyz, conn = gen(3)
        assert conn.shape == (27 * per, 4)
        X = xyz[conn.astype(np.int64)]
        v = np.einsum("ij,ij->i", np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]), X[:, 3] - X[:, 0]) / 6
        assert abs(np.abs(v).sum() - 1.0) < 1e-14 and np.all(np.abs(v) > 0)


def test_ragged_batch_problems():
    probs = batch.make_problems(n_hex=5, n_tet=7, nmin=3, nmax=6)
    assert len(probs) == 12
    assert [p["etype"] for p in probs] == [2] * 5 + [0] * 7
    for p in probs:
        n = p["n"]
        assert 3 <= n <= 6
        assert p["conn"].shape[0] == n ** 3 * (1 if p["etype"] == 2 else 6)
        assert p["k"].shape[0] == p["conn"].shape[0] and np.all(p["k"] > 0)
        assert np.array_equal(p["bc_nodes"], meshgen.boundary_nodes(n))
    again = batch.make_problems(n_hex=5, n_tet=7, nmin=3, nmax=6)
    assert all(np.array_equal(a["xyz"], b["xyz"]) and np.array_equal(a["k"], b["k"]) for a, b in zip(probs, again))
