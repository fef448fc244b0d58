#!/usr/bin/env python3
"""Benchmark: elements/s assembled into CSR (K, M and the load vector), Q1 hexahedra.

Workload (one step): the perturbed 128^3 Q1-hex unit cube (2,097,152 elements,
2,146,689 nodes; interior nodes moved by a seeded U(-0.2h, 0.2h) per coordinate),
per-element diffusivity k_e = exp(N(0,1)), 2x2x2 Gauss quadrature, computed in FP64
arithmetic (IEEE binary64, as the reference): stiffness (AssemblyStiffnessFE with the
P0 coefficient) and mass (AssemblyMass(1)) CSR values plus the load vector of
f = sin(pi x) sin(pi y) sin(pi z), assembled in one fused pass on the device-resident
structural pattern, followed by closeMatrix's prune check of both matrices.  The mesh,
DOF map and pattern are built once (timed separately as `setup_s`).  Inputs are
synthetic (seeded), not a dataset.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 128]

Prints one JSON line.  Under torchrun (N > 1) every rank assembles its own replica
(weak scaling) and rank 0 prints the aggregate over ranks (max time over ranks).
Besides the contract's keys: `roofline.fp64` (the FP64 pipe, the bound the FP64
kernel meets: FP64 instructions per second against the FMA rate measured live by
pxg_fp64_rate), `dfl` (the same workload with the opt-in double-float kernels and
their largest entrywise deviation from the FP64 result), `e2e.host` (the GPU's NUMA
node and the CPUs the host-buffer leg ran on), `configs` (P1 16^3 x 6, P2 64^3 x 6,
Q2 48^3; with P2, the L2 reduction rate its scatter meets, live from pxg_red_rate),
`adjoint` (Q1 96^3 gradient), `batched` (256 ragged problems, batched vs
one at a time) and `widened` (Dirichlet setup from facet markers, Taylor-Hood Stokes
systems).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "elements/s assembled into CSR (frac. HBM peak); batched vs plain adjoint grads/s"
UNIT = "elements/s"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


PROFILE = "kAssembleQ1F64_q1hex96.md"


def profile_figure(key, name=PROFILE):
    """A per-element figure of the assembly kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(p):
            if line.startswith(key + ":"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def traffic_per_element():
    """DRAM bytes per element of the assembly kernel (ncu)."""
    return profile_figure("traffic_bytes_per_element")


def make_inputs(n, seed=20261205):
    from proxpde_gb300 import meshgen

    xyz, conn = meshgen.cube_hex(n)
    xyz = meshgen.perturb(xyz, n, 0.2, seed)
    k = meshgen.lognormal(seed + 1, conn.shape[0], 1.0)
    return xyz, conn, k


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, max clock, reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def gpu_local_cpus(dev):
    """(CPUs of this process that are local to the GPU, the GPU's NUMA node), from the
    PCI device's sysfs entries; (None, None) where they are not readable. Pinned host
    buffers are placed on the node of the thread that allocates them, and a host-device
    copy through a buffer on the far CPU's memory crosses the link between the CPUs."""
    import torch

    p = torch.cuda.get_device_properties(dev)
    base = f"/sys/bus/pci/devices/{p.pci_domain_id:04x}:{p.pci_bus_id:02x}:{p.pci_device_id:02x}.0"
    try:
        with open(base + "/local_cpulist") as f:
            spec = f.read().strip()
        with open(base + "/numa_node") as f:
            node = int(f.read().strip())
    except (OSError, ValueError):
        return None, None
    cpus = set()
    for part in spec.split(","):
        if part:
            lo, _, hi = part.partition("-")
            cpus.update(range(int(lo), int(hi or lo) + 1))
    return cpus & os.sched_getaffinity(0), node


def cpu_sample(n_sample, threads):
    """The oracle (restated reference loop: triplets + setFromTriplets + prune) on a
    bounded sample of the same workload; returns elements/s."""
    import oracle as O

    xyz, conn, k = make_inputs(n_sample)
    em, ndof = O.dofmap(O.Q1HEX, xyz.shape[0], conn)
    t0 = time.perf_counter()
    O.build(O.Q1HEX, xyz, conn, em, ndof, lhs={"stiff_kind": 2, "stiff_c": 1.0, "k_e": k}, nthreads=threads)
    O.build(O.Q1HEX, xyz, conn, em, ndof, lhs={"mass_kind": 1, "mass_c": 1.0},
            rhs={"kind": 1, "fn": O.FN_SIN3, "c": 1.0}, nthreads=threads)
    dt = time.perf_counter() - t0
    return conn.shape[0] / dt, dt


def measure_widened(xyz, conn, n_stokes=16):
    """The rows next to the assembly path: Dirichlet setup from facet markers on the
    headline mesh (own context), and Taylor-Hood Stokes systems (vector space, tensor
    stiffness, grad / div couplings) on n_stokes^3 boxes; device times of the calls."""
    import torch

    from proxpde_gb300 import _lib as L
    from proxpde_gb300 import meshgen
    from proxpde_gb300._lib import OP_DIV, OP_GRAD, OP_TENSOR_STIFFNESS, Context, System

    out = {}
    c = Context(0)
    c.set_mesh(L.Q1HEX, xyz, conn)
    c.build_dofmap()
    t0 = time.perf_counter()
    nf = c.build_facets()
    t1 = time.perf_counter()
    c.mark_facets_box()
    t2 = time.perf_counter()
    c.set_bc_markers([(m, L.FN_CONST, 0.0) for m in range(1, 7)])
    t3 = time.perf_counter()
    out["bc_setup_q1hex"] = {"elements": int(conn.shape[0]), "facets": nf, "build_facets_ms": 1e3 * (t1 - t0),
                             "mark_box_ms": 1e3 * (t2 - t1), "set_bc_markers_ms": 1e3 * (t3 - t2)}
    del c
    for name, gen, tv, tp in (("stokes_q2q1_hex", meshgen.cube_hex, L.Q2HEX, L.Q1HEX),
                              ("stokes_p2p1_tet", meshgen.cube_tet5, L.P2TET, L.P1TET)):
        X, E = gen(n_stokes)
        cv, cp = Context(0), Context(0)
        cv.set_mesh(tv, X, E)
        cp.set_mesh(tp, X, E)
        cv.build_dofmap()
        cp.build_dofmap()
        S = System([cv, cp], [3, 1], qr_types=[tv, tv])
        vals = torch.zeros(S.nnz, dtype=torch.float64, device="cuda")
        b = torch.zeros(S.ntot, dtype=torch.float64, device="cuda")

        def calls():
            S.assemble(0, 0, [(OP_TENSOR_STIFFNESS, 0.1)], vals, b)
            S.assemble(0, 1, [(OP_GRAD, -1.0)], vals, b, accumulate=True)
            S.assemble(1, 0, [(OP_DIV, -1.0)], vals, b, accumulate=True)

        calls()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        for _ in range(3):
            calls()
        ev1.record()
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / 3
        out[name] = {"n": n_stokes, "elements": int(E.shape[0]), "dofs": S.ntot, "nnz": S.nnz, "ms": ms,
                     "elements_per_s": E.shape[0] / (ms * 1e-3)}
    return out


def measure_configs(peak_gbs, reps=5):
    """The other element types on their own workloads: the P1 16^3 x 6 Poisson case
    (K + unit load, k = 1), the P2 64^3 x 6 case (perturbed 0.15 h, k_e lognormal(0, 0.5),
    K + M) and Q2 48^3 hexahedra (perturbed 0.2 h, K + M + sin3 load).  Best of `reps`
    event-timed assemblies each, with the algorithmic bytes of one assembly (vertex ids,
    DOF map, k_e, coordinates, value and load writes) against the HBM peak."""
    import torch

    from proxpde_gb300 import _lib as L
    from proxpde_gb300 import Context, meshgen

    out = {}
    cases = (("p1tet_16", L.P1TET, meshgen.cube_tet6, 16, 0.0, None, 1, {"kind": 1, "fn": L.FN_CONST, "coef": 1.0},
              "kAssembleTet64<P1>"),
             ("p2tet_64", L.P2TET, meshgen.cube_tet6, 64, 0.15, 0.5, 2, None, "kAssembleTet64<P2>"),
             ("q2hex_48", L.Q2HEX, meshgen.cube_hex, 48, 0.2, 1.0, 2, {"kind": 1, "fn": L.FN_SIN3, "coef": 1.0},
              "kAssembleQ2F64"))
    for name, t, gen, n, alpha, sigma, nmat, rhs, kern in cases:
        xyz, conn = gen(n)
        if alpha:
            xyz = meshgen.perturb(xyz, n, alpha, 20261211)
        E = conn.shape[0]
        ctx = Context(0)
        ctx.set_mesh(t, xyz, conn)
        ndof = ctx.build_dofmap()
        nnz = ctx.build_pattern()
        opK = {"stiffness": 1, "stiff_coef": 1.0}
        if sigma:
            ctx.set_coef(meshgen.lognormal(20261212, E, sigma))
            opK = {"stiffness": 2, "stiff_coef": 1.0}
        K = torch.empty(nnz, dtype=torch.float64, device="cuda")
        M = torch.empty_like(K) if nmat == 2 else None
        b = torch.empty(ndof, dtype=torch.float64, device="cuda") if rhs else None
        kw = dict(op0=opK, vals0=K, op1={"mass": 1, "mass_coef": 1.0} if M is not None else None, vals1=M, rhs=rhs, b=b)

        def best_ms():
            for _ in range(2):
                ctx.assemble(**kw)
            torch.cuda.synchronize()
            ts = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                ctx.assemble(**kw)
                e1.record()
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            return min(ts)

        ms = best_ms()
        ctx.set_arithmetic(L.ARITH_DFL)
        dms = best_ms()
        N = {L.P1TET: 4, L.P2TET: 10, L.Q1HEX: 8, L.Q2HEX: 27}[t]
        B = 4 * conn.shape[1] * E + 4 * N * E + (8 * E if sigma else 0) + 24 * xyz.shape[0] + 8 * nnz * nmat + \
            (8 * ndof if rhs else 0)
        gbs = B / (ms * 1e-3) / 1e9
        out[name] = {"elements": int(E), "ndof": int(ndof), "nnz": int(nnz), "ms": ms, "elements_per_s": E / (ms * 1e-3),
                     "kernel": kern, "dtype": "f64", "algorithmic_bytes": int(B), "achieved_gbs": gbs,
                     "frac_hbm": gbs / peak_gbs, "includes": "memset of the outputs + element kernel",
                     "dfl_ms": dms, "dfl_kernel": {L.P1TET: "kAssembleTet<P1>", L.P2TET: "kAssembleTet<P2>",
                                                   L.Q2HEX: "kAssembleQ2"}[t]}
        del ctx, K, M, b
        torch.cuda.empty_cache()
    # the L2 reduction rate the P2 scatter is bound by, live (pxg_red_rate, 32 MB array):
    # one lane per 32-byte sector, as element-by-element reductions land, and four, as
    # the warp-group scatter's sorted positions mostly do
    r1, _ = L.red_rate(1)
    r4, _ = L.red_rate(4)
    out["p2tet_64"]["l2_red_per_s"] = {"lanes_per_sector_1": r1, "lanes_per_sector_4": r4,
                                       "probe": "pxg_red_rate, 32 MB array"}
    return out


def measure_adjoint(n=96, reps=2):
    """Adjoint gradient dJ/dlog k_e on the perturbed Q1 96^3 cube (Dirichlet on all faces,
    f = 1, u_t = sin sin sin), device Jacobi-CG to 1e-10: forward + backward time."""
    import torch

    from proxpde_gb300.adjoint import DiffusionLoss, DiffusionProblem
    from proxpde_gb300 import meshgen

    P = DiffusionProblem.cube_q1(n, rtol=1e-10)
    k = meshgen.lognormal(20261208, P.nelem, 1.0)
    logk = torch.as_tensor(np.log(k)).cuda().requires_grad_(True)
    DiffusionLoss.apply(logk, P).backward()  # warm-up
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        logk.grad = None
        t0 = time.perf_counter()
        DiffusionLoss.apply(logk, P).backward()
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    t = min(ts)
    return {"workload": f"q1hex perturbed {n}^3, K(k)u=1, Dirichlet all faces, J=1/2|u-u_t|_M^2",
            "elements": P.nelem, "ndof": P.ndof, "grads_per_s": 1.0 / t, "ms_per_grad": 1e3 * t,
            "cg_iters": {"forward": P.iters[0], "adjoint": P.iters[1]}, "rtol": 1e-10}


def measure_batched(n_hex=128, n_tet=128, reps=3, tune=True, rank=0, world=1, dev="cuda"):
    """Batched adjoint gradients of 256 ragged problems (n ~ U{8..48}); batched persistent graph vs the
    same problems one at a time through the plain forward/backward pair.  On several ranks
    (one GPU each) the problems are split between them (batch.shard: independent problems,
    no exchange) and each time is the largest over the ranks."""
    import torch

    from proxpde_gb300 import batch
    from proxpde_gb300.adjoint import DiffusionLoss, DiffusionProblem

    sizes = batch.problem_sizes(n_hex=n_hex, n_tet=n_tet)
    mine = batch.shard(sizes, n_hex, rank, world)
    probs = batch.make_problems(n_hex=n_hex, n_tet=n_tet, only=mine)
    groups = [batch.Batch(ps) for ps in ([p for p in probs if p["etype"] == 2], [p for p in probs if p["etype"] == 0])
              if ps]

    def job_time(t):
        return max_over_ranks(t, world, dev)

    # the autotuner picks each batch's element kernel (elements per CTA, scatter)
    tuning = [g.ctx.autotune(op0={"stiffness": 2, "stiff_coef": 1.0, "apply_bc": 1}, op1={"mass": 1, "mass_coef": 1.0},
                             rhs={"kind": 1, "fn": 0, "coef": 1.0, "apply_bc": 1}) for g in groups] if tune else None
    batch.batch_adjoint(groups)  # builds and replays the graph
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        barrier(world)
        t0 = time.perf_counter()
        losses, iters = batch.batch_adjoint(groups)
        torch.cuda.synchronize()
        ts.append(job_time(time.perf_counter() - t0))
    tb = min(ts)
    # sequential plain launches
    plain = []
    for p in probs:
        P = DiffusionProblem(p["etype"], p["xyz"], p["conn"], bc_nodes=p["bc_nodes"], rtol=1e-10)
        lk = torch.as_tensor(np.log(p["k"])).cuda().requires_grad_(True)
        plain.append((P, lk))
    def seq_pass():
        out = []
        for P, lk in plain:
            lk.grad = None
            DiffusionLoss.apply(lk, P).backward()
            out.append(lk.grad)
        torch.cuda.synchronize()
        return out
    seq_pass()
    barrier(world)
    t0 = time.perf_counter()
    gs = seq_pass()
    ts_ = job_time(time.perf_counter() - t0)
    # batched vs plain gradients
    err = 0.0
    i = 0
    for g in groups:
        for q in range(g.nprob):
            a, b = g.grad_of(q), gs[i]
            err = max(err, float(torch.linalg.norm(a - b) / torch.linalg.norm(b)))
            i += 1
    err = job_time(err)
    E = int(job_sum(sum(g.nelem for g in groups), world, dev))
    iters = int(job_time(iters))
    return {"workload": f"{n_hex} Q1-hex + {n_tet} P1-tet cubes, n~U{{8..48}}, K+M assembly + adjoint gradient",
            "ranks": world, "partition": "problems split over the ranks (largest first to the least loaded), "
            "no exchange" if world > 1 else "one rank",
            "problems": n_hex + n_tet, "elements": E, "batched_grads_per_s": (n_hex + n_tet) / tb,
            "sequential_grads_per_s": (n_hex + n_tet) / ts_, "speedup": ts_ / tb, "batched_ms": 1e3 * tb,
            "sequential_ms": 1e3 * ts_, "max_cg_iters": iters,
            "grad_rel_err_vs_plain": err, "rtol": 1e-10, "tuning": tuning,
            "launch": "one CUDA graph: 2 assembly kernels, "
            "1 persistent cooperative solver (forward CG, loss, adjoint CG), 2 gradient kernels"}


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    return world, rank, local


def max_over_ranks(x, world, device):
    """The job's time: the largest of the ranks' values (no-op on one rank)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.item()


def job_sum(x, world, device):
    """The sum of the ranks' values (no-op on one rank)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.item()


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def run_reference(args, world, rank):
    if rank != 0:
        return
    import oracle as O

    O.lib()
    threads = os.cpu_count() or 1
    n_sample = args.cpu_n
    vals = []
    for s in range(args.warmup + args.steps):
        v, dt = cpu_sample(n_sample, threads)
        if s >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    E = n_sample ** 3
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * E / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": f"q1hex perturbed {args.n}^3 K+M+rhs (CPU sample {n_sample}^3)",
                   "elements": args.n ** 3, "sample_elements": E},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n_sample}^3 Q1 hexes (of the {args.n}^3 workload), oracle OpenMP"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--cpu-n", type=int, default=40)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (default kernels)")
    ap.add_argument("--no-widened", action="store_true", help="skip the Dirichlet-setup and Stokes measurements")
    ap.add_argument("--no-configs", action="store_true", help="skip the P1 / P2 / Q2 workload measurements")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-dfl", action="store_true", help="skip the double-float comparison leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint-gradient measurement")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-gradient measurement")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else max(args.warmup, 1)

    world, rank, local = dist_init(args)
    if args.impl == "reference":
        # the CPU reference arm: rank 0 times the oracle, the other ranks exit
        run_reference(args, world, rank)
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()
        return

    import torch

    from proxpde_gb300 import Context, build
    from proxpde_gb300 import _lib as L

    build.build()
    dev = local
    torch.cuda.set_device(dev)
    n = args.n
    xyz, conn, k = make_inputs(n)
    E, nn = conn.shape[0], xyz.shape[0]

    t0 = time.perf_counter()
    ctx = Context(dev)
    ctx.set_mesh(L.Q1HEX, xyz, conn)
    ndof = ctx.build_dofmap()
    nnz = ctx.build_pattern()
    ctx.set_coef(k)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0

    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream
    K = torch.empty(nnz, dtype=torch.float64, device=dev)
    M = torch.empty(nnz, dtype=torch.float64, device=dev)
    b = torch.empty(ndof, dtype=torch.float64, device=dev)
    opK = {"stiffness": 2, "stiff_coef": 1.0}
    opM = {"mass": 1, "mass_coef": 1.0}
    rhs = {"kind": 1, "fn": L.FN_SIN3, "coef": 1.0}
    # autotuner: elements per CTA x scatter strategy, timed on this mesh (setup, untimed)
    tuning = None if args.no_tune else ctx.autotune(op0=opK, op1=opM, rhs=rhs)

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]

    cnt = torch.zeros(2, dtype=torch.int64, device=dev)

    def step(i=None):
        if i is not None:
            ev[i][0].record(stream)
        ctx.assemble(op0=opK, vals0=K, op1=opM, vals1=M, rhs=rhs, b=b, stream=sp)
        if i is not None:
            ev[i][1].record(stream)
        # closeMatrix's prune check, stream-ordered (no host round trip inside a step)
        ctx.prune_count_device(K, cnt[0:1], stream=sp)
        ctx.prune_count_device(M, cnt[1:2], stream=sp)

    for _ in range(args.warmup):
        step()
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(dev)
    clk.start()
    time.sleep(0.3)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for i in range(args.steps):
        step(i)
    stop.record(stream)
    torch.cuda.synchronize()
    pruned = cnt.tolist()
    clocks = clk.stop()
    total_ms = max_over_ranks(start.elapsed_time(stop), world, dev)
    ms_step = total_ms / args.steps
    asm_ms = statistics.mean(a.elapsed_time(c) for a, c in ev)
    value = world * E / (ms_step * 1e-3)

    # algorithmic bytes of the fused assembly launch (conn, DOF map, k_e, xyz, two
    # value arrays written once, load vector)
    alg = 4 * 8 * E + 4 * 8 * E + 8 * E + 24 * nn + 8 * nnz * 2 + 8 * ndof
    hbm, which = peaks()
    achieved = alg / (asm_ms * 1e-3) / 1e9
    tpe = traffic_per_element()
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": tpe * E if tpe else None, "traffic_source": "ncu 96^3 capture scaled by elements",
            "peak_source": which, "kernel": "kAssembleQ1F64 (+memset of K, M, b)",
            "kernel_ms": asm_ms, "algorithmic_bytes": alg}
    # the bound the FP64 kernel meets: the FP64 pipe.  FP64 instructions per element from
    # ncu (96^3 capture: DFMA + DMUL + DADD thread instructions / elements) times the
    # elements over the event-timed launch, against the FMA rate measured now on this
    # GPU; the launch time includes the memsets, so the fraction is a lower bound
    from proxpde_gb300._lib import fp64_rate

    rate, rate_ms = fp64_rate(dev)
    fpe = profile_figure("fp64_instructions_per_element")
    roof["fp64"] = {"fp64_instructions_per_element": fpe, "peak": rate, "unit": "FP64 instructions/s",
                    "peak_source": f"pxg_fp64_rate: independent FMA chains, event-timed ({rate_ms:.2f} ms launch)"}
    if fpe:
        got = E * fpe / (asm_ms * 1e-3)
        roof["fp64"].update({"achieved": got, "frac": got / rate})

    # the opt-in double-float kernel on the same workload, and its largest entrywise
    # deviation from the FP64 result (entries above 1e-8 of the matrix's largest)
    dfl = None
    if not args.no_dfl:
        from proxpde_gb300._lib import ARITH_DFL

        cd = Context(dev)
        cd.set_arithmetic(ARITH_DFL)
        cd.set_mesh(L.Q1HEX, xyz, conn)
        cd.build_dofmap()
        cd.build_pattern()
        cd.set_coef(k)
        Kd, Md, bd = torch.empty_like(K), torch.empty_like(M), torch.empty_like(b)
        kw = dict(op0=opK, vals0=Kd, op1=opM, vals1=Md, rhs=rhs, b=bd, stream=sp)
        for _ in range(3):
            cd.assemble(**kw)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            cd.assemble(**kw)
        e1.record(stream)
        torch.cuda.synchronize()
        dms = e0.elapsed_time(e1) / args.steps
        ctx.assemble(op0=opK, vals0=K, op1=opM, vals1=M, rhs=rhs, b=b, stream=sp)
        torch.cuda.synchronize()

        def dev_rel(x, y):
            big = y.abs() > 1e-8 * y.abs().max()
            return float(((x - y).abs()[big] / y.abs()[big]).max())

        dfl = {"kernel": "kAssembleQ1Group<dfl> (+memset of K, M, b)", "ms": dms, "elements_per_s": E / (dms * 1e-3),
               "arithmetic": "double-float (unevaluated f32 pairs, ~48-bit significand) on the FP32 pipes; FP64 for "
                             "the coordinate differences, the final hi+lo sums and the reductions",
               "max_rel_dev_from_fp64": {"K": dev_rel(Kd, K), "M": dev_rel(Md, M), "b": dev_rel(bd, b)}}
        del cd, Kd, Md, bd
        torch.cuda.empty_cache()

    e2e = None
    if not args.no_e2e:
        # through the C ABI with host buffers: every step uploads the coordinates and
        # the coefficients from pinned memory and reads K, M, b and the two prune
        # counts back into pinned memory.  Two output sets alternate, so that the
        # read-back of step i (on a copy stream) overlaps the upload and the assembly
        # of step i + 1.
        # pinned buffers on the GPU's own CPU node: the allocating and launching thread
        # runs on the CPUs local to the GPU while they are allocated and used
        allowed = os.sched_getaffinity(0)
        local, node = gpu_local_cpus(dev)
        if local:
            os.sched_setaffinity(0, local)
        xyz_h = torch.from_numpy(xyz).pin_memory()
        k_h = torch.from_numpy(k).pin_memory()
        copy_stream = torch.cuda.Stream(dev)
        sets = []
        for j in range(2):
            sets.append({
                "K": K if j == 0 else torch.empty(nnz, dtype=torch.float64, device=dev),
                "M": M if j == 0 else torch.empty(nnz, dtype=torch.float64, device=dev),
                "b": b if j == 0 else torch.empty(ndof, dtype=torch.float64, device=dev),
                "cnt": torch.zeros(2, dtype=torch.int64, device=dev),
                "Kh": torch.empty(nnz, dtype=torch.float64).pin_memory(),
                "Mh": torch.empty(nnz, dtype=torch.float64).pin_memory(),
                "bh": torch.empty(ndof, dtype=torch.float64).pin_memory(),
                "cnth": torch.full((2,), -1, dtype=torch.int64).pin_memory(),
                "ready": torch.cuda.Event(), "done": torch.cuda.Event(), "used": False})

        def e2e_step(i):
            S = sets[i % 2]
            if S["used"]:
                stream.wait_event(S["done"])  # the set's previous read-back has finished
            ctx.set_coords(xyz_h, stream=sp)
            ctx.set_coef(k_h, stream=sp)
            ctx.assemble(op0=opK, vals0=S["K"], op1=opM, vals1=S["M"], rhs=rhs, b=S["b"], stream=sp)
            ctx.prune_count_device(S["K"], S["cnt"][0:1], stream=sp)
            ctx.prune_count_device(S["M"], S["cnt"][1:2], stream=sp)
            S["ready"].record(stream)
            copy_stream.wait_event(S["ready"])
            with torch.cuda.stream(copy_stream):
                S["Kh"].copy_(S["K"], non_blocking=True)
                S["Mh"].copy_(S["M"], non_blocking=True)
                S["bh"].copy_(S["b"], non_blocking=True)
                S["cnth"].copy_(S["cnt"], non_blocking=True)
            S["done"].record(copy_stream)
            S["used"] = True

        for i in range(2):
            e2e_step(i)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for i in range(args.steps):
            e2e_step(i)
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t1) / args.steps
        assert all(S["cnth"].tolist() == pruned for S in sets), "prune counts differ between the two legs"
        os.sched_setaffinity(0, allowed)
        e2e = {"value": world * E / e2e_s, "unit": UNIT, "h2d_bytes_per_step": xyz.nbytes + k.nbytes,
               "d2h_bytes_per_step": 2 * nnz * 8 + ndof * 8 + 16, "ms_per_step": e2e_s * 1e3,
               "overlap": "read-back of step i overlaps upload and assembly of step i + 1 (two output sets)",
               "host": {"gpu_numa_node": node, "cpus_allowed": len(allowed),
                        "cpus_used": len(local) if local else len(allowed),
                        "placement": "CPUs local to the GPU" if local else "process affinity unchanged"}}

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v_all, dt_all = cpu_sample(args.cpu_n, threads)
        v_one, dt_one = cpu_sample(min(args.cpu_n, 24), 1)
        cpu = {"value": v_all, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{args.cpu_n}^3 Q1 hexes of the same workload (K+M+rhs), oracle restatement with OpenMP",
               "value_1thread": v_one, "sample_1thread": f"{min(args.cpu_n, 24)}^3 hexes, 1 thread"}

    adjoint = batched = widened = configs = None
    if not args.no_batched:
        # every rank: the batch's problems are split over the ranks
        barrier(world)
        batched = measure_batched(tune=not args.no_tune, rank=rank, world=world, dev=dev)
    if rank == 0 and not args.no_widened:
        widened = measure_widened(xyz, conn)
    if rank == 0 and not args.no_configs:
        configs = measure_configs(hbm)
    if rank == 0 and not args.no_adjoint:
        adjoint = measure_adjoint()

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "arithmetic": "IEEE binary64 throughout (geometry, local matrices, sums, reductions); FP64-pipe bound",
            "data": "synthetic (seeded perturbed cube)",
            "config": {"workload": f"q1hex perturbed {n}^3: K(k_e)+M+rhs sin3, fused pass + prune check",
                       "elements": E, "nodes": nn, "ndof": ndof, "nnz": nnz, "pruned": list(pruned), "tuning": tuning,
                       "l2": "inputs larger than L2 (K+M values alone are %.0f MB)" % (2 * nnz * 8 / 1e6),
                       "setup_s": setup_s, "parallelism": f"replicas x{world}"},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks, "dfl": dfl, "widened": widened,
            "configs": configs,
            # per step: the zeroing of K, M and b (kZeroOutputs), the assembly (kAssembleQ1F64)
            # and the two prune counts (kPruneCount)
            "gpu_launches": 4 * args.steps, "adjoint": adjoint, "batched": batched,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
