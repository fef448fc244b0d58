"""One named workload of the engine, timed with CUDA events: the small cases the ncu
summaries under profiles/ are captured on, runnable on their own.

    python -m proxpde_gb300.cases <case> [--n N] [--warmup W] [--reps R]

Cases (seeded synthetic inputs, the generators of proxpde_gb300.meshgen):
  q1hex  Q1 hexahedra n^3, interior nodes perturbed by U(-0.2h, 0.2h), k_e = exp(N(0,1));
         K(k_e) + M + sin(pi x) sin(pi y) sin(pi z) load in one call
  p2tet  P2 tetrahedra n^3 x 6 (Kuhn), vertices perturbed by 0.15h, k_e lognormal(0, 0.5);
         K(k_e) + M + unit load
  p1tet  P1 tetrahedra n^3 x 6 (Kuhn), unperturbed, k = 1; K + unit load
  q2hex  Q2 hexahedra n^3, perturbed by 0.2h, k_e = exp(N(0,1)); K(k_e) + M + sin load
  batch  n Q1 cubes + n P1 cubes with sizes U{8..28}: the batched adjoint gradient
         (assembly, forward and adjoint CG, gradient) in one persistent launch

Each warm-up and timed repetition is one engine call; the line printed is JSON with the
median event time of the repetitions.  The kernels' own names are in the output
(`kernel`), for `ncu -k regex:<name>`.  --arith dfl runs the opt-in double-float
kernels instead of the FP64 ones.
"""
from __future__ import annotations

import argparse
import json
import statistics

import numpy as np

from . import _lib as L
from . import meshgen

SEED = 20261211

ASSEMBLY = {
    # case: element type, mesh generator, perturbation, k_e sigma, mass, rhs function,
    # kernel (FP64), kernel (double-float)
    "q1hex": (L.Q1HEX, meshgen.cube_hex, 0.2, 1.0, True, L.FN_SIN3, "kAssembleQ1F64", "kAssembleQ1Group"),
    "p2tet": (L.P2TET, meshgen.cube_tet6, 0.15, 0.5, True, L.FN_CONST, "kAssembleTet64", "kAssembleTet"),
    "p1tet": (L.P1TET, meshgen.cube_tet6, 0.0, None, False, L.FN_CONST, "kAssembleTet64", "kAssembleTet"),
    "q2hex": (L.Q2HEX, meshgen.cube_hex, 0.2, 1.0, True, L.FN_SIN3, "kAssembleQ2F64", "kAssembleQ2"),
}


def _events(fn, warmup, reps):
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return statistics.median(ts)


def run_assembly(case, n, warmup, reps, arith="fp64"):
    import torch

    t, gen, alpha, sigma, mass, fn, k64, kdfl = ASSEMBLY[case]
    kernel = k64 if arith == "fp64" else kdfl
    xyz, conn = gen(n)
    if alpha:
        xyz = meshgen.perturb(xyz, n, alpha, SEED)
    ctx = L.Context(0)
    if arith == "dfl":
        ctx.set_arithmetic(L.ARITH_DFL)
    ctx.set_mesh(t, xyz, conn)
    ndof = ctx.build_dofmap()
    nnz = ctx.build_pattern()
    opK = {"stiffness": 1, "stiff_coef": 1.0}
    if sigma:
        ctx.set_coef(meshgen.lognormal(SEED + 1, conn.shape[0], sigma))
        opK = {"stiffness": 2, "stiff_coef": 1.0}
    K = torch.empty(nnz, dtype=torch.float64, device="cuda")
    M = torch.empty_like(K) if mass else None
    b = torch.empty(ndof, dtype=torch.float64, device="cuda")
    kw = dict(op0=opK, vals0=K, op1={"mass": 1, "mass_coef": 1.0} if mass else None, vals1=M,
              rhs={"kind": 1, "fn": fn, "coef": 1.0}, b=b)
    ms = _events(lambda: ctx.assemble(**kw), warmup, reps)
    return {"case": case, "n": n, "arith": arith, "elements": int(conn.shape[0]), "ndof": int(ndof), "nnz": int(nnz),
            "ms": ms, "kernel": kernel, "includes": "memset of the outputs + element kernel"}


def run_batch(n, warmup, reps):
    from . import batch

    probs = batch.make_problems(n_hex=n, n_tet=n, nmin=8, nmax=28)
    groups = [batch.Batch([p for p in probs if p["etype"] == L.Q1HEX]),
              batch.Batch([p for p in probs if p["etype"] == L.P1TET])]
    ms = _events(lambda: batch.batch_adjoint(groups), warmup, reps)
    return {"case": "batch", "problems": 2 * n, "elements": int(sum(p["conn"].shape[0] for p in probs)), "ms": ms,
            "kernel": "kBatchSolve", "includes": "assembly, forward and adjoint CG, loss and gradient of every problem"}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("case", choices=sorted(ASSEMBLY) + ["batch"])
    ap.add_argument("--n", type=int, default=32, help="cube size (batch: problems per element type)")
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--arith", choices=["fp64", "dfl"], default="fp64")
    a = ap.parse_args(argv)
    if a.case == "batch":
        out = run_batch(a.n, a.warmup, a.reps)
    else:
        out = run_assembly(a.case, a.n, a.warmup, a.reps, a.arith)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
