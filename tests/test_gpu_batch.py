"""Batched adjoint gradients (many ragged problems in one persistent, graph-captured
launch) against the same problems run one at a time through the plain path and
against the oracle's CPU gradient; the bounded grid-barrier wait of the persistent
kernel is made to run out from the host and must come back as PXG_ERR_TIMEOUT."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def small_problems():
    from proxpde_gb300 import batch

    return batch.make_problems(n_hex=5, n_tet=5, nmin=2, nmax=6, seed=77)


@pytest.mark.parametrize("use_graph", [True, False], ids=["graph", "stream"])
def test_batch_matches_plain_and_oracle(engine, use_graph):
    import torch

    from proxpde_gb300 import batch
    from proxpde_gb300.adjoint import DiffusionLoss, DiffusionProblem
    from test_gpu_adjoint import reference_gradient

    probs = small_problems()
    hexes = [p for p in probs if p["etype"] == O.Q1HEX]
    tets = [p for p in probs if p["etype"] == O.P1TET]
    B = [batch.Batch(hexes), batch.Batch(tets)]
    for _ in range(2):  # the second call replays the captured graph
        losses, iters = batch.batch_adjoint(B, rtol=1e-12, use_graph=use_graph)
    assert iters > 0
    p_glob = 0
    for b in B:
        for i, p in enumerate(b.problems):
            J_ref, g_ref, _ = reference_gradient(p["xyz"], p["conn"], p["k"], p["bc_nodes"], p["etype"])
            g = b.grad_of(i).cpu().numpy()
            assert abs(losses[p_glob] - J_ref) <= 1e-9 * abs(J_ref)
            assert np.linalg.norm(g - g_ref) <= 1e-8 * np.linalg.norm(g_ref)
            # the plain one-problem path gives the same gradient
            P = DiffusionProblem(p["etype"], p["xyz"], p["conn"], bc_nodes=p["bc_nodes"], rtol=1e-12)
            lk = torch.as_tensor(np.log(p["k"])).cuda().requires_grad_(True)
            DiffusionLoss.apply(lk, P).backward()
            assert np.linalg.norm(lk.grad.cpu().numpy() - g) <= 1e-8 * np.linalg.norm(g)
            p_glob += 1


def test_batch_barrier_timeout_is_reported(engine, monkeypatch):
    """Every grid barrier waits for one block more than the grid has: the bounded
    waits run out, the kernel returns, and the host gets PXG_ERR_TIMEOUT; the context
    then still works."""
    from proxpde_gb300 import PxgError, batch

    probs = batch.make_problems(n_hex=2, n_tet=0, nmin=2, nmax=3, seed=5)
    B = [batch.Batch(probs)]
    monkeypatch.setenv("PXG_TEST_BARRIER_SHORTFALL", "1")
    with pytest.raises(PxgError) as ei:
        batch.batch_adjoint(B, rtol=1e-10, use_graph=False)
    assert ei.value.status == 4
    monkeypatch.setenv("PXG_TEST_BARRIER_SHORTFALL", "0")
    losses, _ = batch.batch_adjoint(B, rtol=1e-10, use_graph=False)
    assert np.all(np.isfinite(losses))
