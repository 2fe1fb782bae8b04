"""Benchmark of the lmgc hot path on GB300.

Workload (one step = one complete linear solve): 3D variable-coefficient
diffusion -div(k grad u) = f, P1 tetrahedra on the unit cube, six Kuhn
tetrahedra red-refined 6 times (65^3 = 274,625 unknowns, 4,018,753
nonzeros), k = exp(g) per element with g a seeded Gaussian field
(exponential covariance, correlation length 0.1, variance 1), seeded
uniform[-1,1] right-hand side; ls + lmgc V(2,2) with multicolour
Gauss-Seidel, base level 0, to 1e-8 relative defect.  Two precisions:
plain FP64 and the FP32 V-cycle inside FP64 iterative refinement (the
headline `value`).  Inputs are synthetic (seeded), generated on the host.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Multi-GPU: the path does not shard (a single solve has no partition), so N
ranks run independent replicas of the workload; value = all ranks' solves
divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solves/s to 1e-8 rel defect, mixed vs FP64 GPU; HBM GB/s; serve p50/p99 ms"
NREF, SEED, CORR, VAR = 6, 2026, 0.1, 1.0
RED = 1e-8
# the tetrahedra of the refined cube: "ug" = UG's red rules (shortest interior
# diagonal, UG's own mesh), "freudenthal" = the Freudenthal triangulation
MESH = "ug"
MESHES = {"ug": "UG red rules (shortest interior diagonal)", "freudenthal": "Freudenthal triangulation"}


# CUDA graphs for the ls iterations of every workload ($graph / $dloop);
# --no-graph turns them off so that profilers see every kernel launch
GRAPH = 1


class nvtx_range:
    """An NVTX range around one region (`ncu --nvtx --nvtx-include name/`
    then captures only its kernels); a no-op where NVTX is unavailable."""

    def __init__(self, name: str, on: bool = True):
        self.name, self.on = name, on

    def __enter__(self):
        if self.on:
            try:
                import torch
                torch.cuda.nvtx.range_push(self.name)
            except Exception:
                self.on = False
        return self

    def __exit__(self, *a):
        if self.on:
            import torch
            torch.cuda.nvtx.range_pop()


def gen_kind(G):
    return G.Generator.DIFFUSION3D_UG if MESH == "ug" else G.Generator.DIFFUSION3D


def workload_config(extra=None):
    c = {"workload": f"3D P1 diffusion k=exp(g) (corr 0.1, var 1), unit cube 6 Kuhn tets red x{NREF} "
                     f"({MESHES[MESH]}), 65^3=274625 unknowns, lmgc V(2,2) Gauss-Seidel, base level 0, "
                     "ls to 1e-8 rel defect",
         "mesh": MESH, "unknowns": 274625, "nnz": 4018753, "levels": NREF + 1, "smoother": "gs",
         "l2": "GPU arm: L2 flushed between timed steps (256 MB read); the hierarchy itself (~60 MB FP64) "
               "fits in L2"}
    if extra:
        c.update(extra)
    return c


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def reduce_over_ranks(x: float, op: str = "max") -> float:
    """max (times, latencies) or sum (throughputs) of a per-rank number over
    all ranks; identity without a process group.  Replicas never exchange
    data: this is the only collective of the benchmark."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def whole_job_rate(units_per_rank: float, ms_per_step_max: float, world: int) -> float:
    """Units per second of the whole job: every rank processes units_per_rank
    per step, the job takes the slowest rank's time."""
    return world * units_per_rank / (ms_per_step_max * 1e-3)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0])); mx.append(float(p[1]))
            except ValueError:
                continue
            for n, v in zip(names, p[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(kind="gs"):
    """DRAM bytes per launch of a roofline kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "roofline_traffic.txt")
    if not os.path.exists(p):
        return None
    key = f"{kind}_traffic_bytes_per_launch"
    with open(p) as f:
        for line in f:
            if line.startswith(key):
                return float(line.split("=")[1])
    return None


# ---------------------------------------------------------------- reference arm
def run_reference(args):
    """The reference's CPU implementation of the path on the host cores.

    UG itself cannot run on the GPU host (its sources are not there, and its
    build needs them), so the oracle port -- the C restatement of UG's ls +
    lmgc, pinned bit-for-bit to UG's kernels and solves -- solves the same
    workload.  The hierarchy comes from the oracle's own generator
    (oracle/cube_gen.c, bitwise equal to the one the GPU arm uses), so this
    process loads nothing but the oracle library.  Each step runs one
    complete solve to 1e-8 per host thread, all threads at once; the rate is
    the solves of a step over its wall time.  The oracle sweeps the rows in
    the generator's VECTOR-list order (UG's l_lgs), the GPU arm in
    multicolour order: the same smoother, a different order (the `ordering`
    key), both converging in 13 iterations."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    levels, rhs, _ = oracle.cube_levels(NREF, SEED, CORR, VAR, ug_rules=MESH == "ug")
    H = oracle.Hierarchy(levels)
    threads = max(1, min(os.cpu_count() or 1, 16))
    results = [None] * threads

    def solve(k):
        _, it, conv, hist = H.ls_solve(rhs, smoother="gs", baselevel=0, red=RED, abslimit=1e-50)
        results[k] = (it, conv, hist[-1, 0] / hist[0, 0])

    def step():
        th = [threading.Thread(target=solve, args=(k,)) for k in range(threads)]
        t0 = time.perf_counter()
        [t.start() for t in th]
        [t.join() for t in th]
        dt = time.perf_counter() - t0
        assert all(r is not None and r[1] for r in results), "an oracle solve did not converge"
        return dt

    for _ in range(args.warmup):
        step()
    times = [step() for _ in range(args.steps)]
    per_step = float(np.mean(times))
    value = threads / per_step
    iters = results[0][0]
    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
            "config": workload_config(),
            "ordering": "VECTOR-list order (lexicographic), as UG's l_lgs sweeps it",
            "iterations": iters, "final_rel_defect": float(results[0][2]),
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                             "sample": f"each step: {threads} complete FP64 solves to 1e-8 ({iters} iterations "
                                       f"each), one per host thread, run at once; {args.steps} steps timed"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- config 1
def run_c1(args, stream, flush_l2, world, rank):
    """The reference's CPU-runnable case: 2D Q1 Poisson on the unit square,
    257x257 nodes (66,049 unknowns; the 4x4 grid refined 6 times, i.e. one quad
    refined 8 times with base level 2), uniform[-1,1] right-hand side, plain
    FP64 lmgc V(2,2) with damped Jacobi (omega 0.8) to 1e-10 relative defect."""
    import torch
    import ug_gb300 as G
    gen = G.Generator(G.Generator.POISSON2D, 8, seed=SEED)
    mg = G.MultiGrid(gen, order=G.ORDER_COLOR, device=torch.cuda.current_device())
    G.lib().gmg_mg_set_stream(mg._h, stream.cuda_stream)
    G.setup_lmgc(mg, "jac", baselevel=2, damp=0.8, red=1e-10, abslimit=1e-50)
    b = np.ascontiguousarray(gen.rhs)
    x = np.empty_like(b)
    for _ in range(args.warmup):
        mg.solve_host("mgs", b, x)
    ts = []
    for _ in range(args.steps):
        flush_l2(); torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, lr = mg.solve_host("mgs", b, x)
        ts.append((time.perf_counter() - t0) * 1e3)
        assert lr.converged
    ms = reduce_over_ranks(float(np.mean(ts)))
    iters = lr.iters
    mg.close()
    out = {"workload": "2D Q1 Poisson 257x257 (66,049 unknowns), lmgc V(2,2) Jacobi omega 0.8, base 4x4 grid, "
                       "plain FP64, ls to 1e-10 rel defect",
           "value": whole_job_rate(1, ms, world), "unit": "solves/s (e2e, host b -> host x)", "ms_per_solve": ms,
           "iterations": iters}
    if rank == 0:
        try:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle
            oracle.build()
            H = oracle.Hierarchy(gen.levels())
            t0 = time.perf_counter()
            _, it, conv, _ = H.ls_solve(gen.rhs, smoother="jac", baselevel=2, damp=0.8, red=1e-10)
            dt = time.perf_counter() - t0
            out["cpu_baseline"] = {"value": 1.0 / dt, "unit": "solves/s", "cores": 1, "kind": "port",
                                   "sample": f"one FP64 solve, UG list order ({it} iterations, {dt:.2f} s)"}
        except Exception as e:  # reported, not fatal
            out["cpu_baseline"] = {"value": None, "sample": f"failed: {e}"}
    return out


# ---------------------------------------------------------------- locally refined workload
LOCAL_NUNI, LOCAL_NLOC = 7, 9


def run_local(args, stream, flush_l2, world, rank):
    """Plane-strain P1 elasticity (E=1, nu=0.3, 2x2 blocks) on the L-shaped
    domain: six coarse triangles refined 7 times uniformly, then 9 times toward
    the re-entrant corner (step k: leaf elements with a corner within 0.5^k,
    green closure, yellow copies; the hierarchy UG's grid manager builds,
    generated on the host), body force uniform[-1,1] per component.  Block
    ILU(0) V(2,2), level-scheduled triangular solves in subdomain order
    (a multicolour order stalls ILU(0) on this system), ls over UG's surface (FINE_GRID_DOF
    rows of every level) to 1e-8 relative defect, plain FP64 and FP32
    V-cycle in FP64 refinement."""
    import torch
    import ug_gb300 as G
    t0 = time.perf_counter()
    gen = G.LocalGenerator(LOCAL_NUNI, LOCAL_NLOC, seed=SEED)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    mg = G.MultiGrid(gen, order=G.ORDER_DOMAIN, fp32=True, autotune=True, device=torch.cuda.current_device())
    G.lib().gmg_mg_set_stream(mg._h, stream.cuda_stream)
    G.setup_lmgc(mg, "ilu", baselevel=0, red=RED, abslimit=1e-50, name="loc64", graph=GRAPH, dloop=GRAPH)
    mg.npcreate("loc32", "linear_solver.gls")
    mg.npinit("loc32", f"$A MAT $x sol $b rhs $red {RED} $abslimit 1e-50 $m 100 $I lmgc $mixed 1"
                       f" $graph {GRAPH} $dloop {GRAPH}")
    top = mg.top
    mg.createvector("b0")
    mg.upload_levels("b0", gen.rhs)
    mg.ls_preprocess("loc64", top, "sol", "rhs")  # ILU factors of every level (setup, not timed)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    surf = 0
    for l in range(mg.nlevels):
        d = gen.level(l)
        m = (d["vclass"] >= 2) if l == top else ((d["vclass"] >= 2) & (d["vnclass"] <= 1))
        surf += int(m.sum()) * (0 if l < mg.frl else 1)
    out = {"workload": f"2D plane-strain P1 elasticity on the L-shaped domain, 2x2 blocks, 6 coarse triangles "
                       f"refined {LOCAL_NUNI}x uniformly + {LOCAL_NLOC}x toward the re-entrant corner "
                       f"(UG's local refinement: green closure, yellow copies), block ILU(0) V(2,2) level-scheduled "
                       f"in subdomain order, ls over the surface to 1e-8 rel defect",
           "levels": mg.nlevels, "fullrefinelevel": mg.frl, "surface_dofs": 2 * surf,
           "vectors_all_levels": int(sum(mg.size(l)[0] for l in range(mg.nlevels))),
           "nnzb_all_levels": int(sum(mg.size(l)[2] for l in range(mg.nlevels))),
           "generate_s": gen_s, "setup_s": setup_s}

    def step(solver):
        lr = G.LResult()
        for l in range(mg.nlevels):
            mg.dcopy(l, "rhs", "b0")
            mg.dset(l, "sol", 0.0)
        mg.ls_defect(solver, top, "sol", "rhs")
        mg.ls_residuum(solver, 0, top, "sol", "rhs", lr)
        mg.ls_solver(solver, top, "sol", "rhs", lr)
        return lr

    res = {}
    for solver in ("loc64", "loc32"):
        for _ in range(args.warmup):
            step(solver)
        ms, launches = [], 0
        for k in range(args.steps):
            flush_l2()
            mg.launch_count(reset=True)
            a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with nvtx_range("c3_mixed_solve", solver == "loc32" and k == args.steps - 1):
                a.record(stream)
                lr = step(solver)
                e.record(stream)
                torch.cuda.synchronize()
            launches += mg.launch_count()
            assert lr.converged, f"{solver} did not converge"
            ms.append(a.elapsed_time(e))
        res[solver] = (reduce_over_ranks(float(np.mean(ms))), lr.iters, launches / args.steps)
    # one FP32 ILU solve (forward + backward sweep) of the finest level, HBM-cold
    # (the factors L, U and the inverse diagonal blocks stream once, t and b
    # are read / written): the smoother's kernel time against its bytes
    n_t, s_t, nnz_t = mg.size(top)
    mg.createvector("iv32", "id32", prec=G.FP32)
    lu_ms = []
    for k in range(args.warmup + 10):
        flush_l2()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        mg.l_luiter(top, "iv32", "id32")
        e.record(stream)
        torch.cuda.synchronize()
        if k >= args.warmup:
            lu_ms.append(a.elapsed_time(e))
    lu_ms = float(np.mean(lu_ms))
    # off-diagonal blocks of L and U (nnz - n) and the n inverse diagonal blocks
    lu_bytes = (nnz_t - n_t) * (s_t * s_t * 4 + 4) + n_t * s_t * s_t * 4 + 2 * (n_t + 1) * 4 + 3 * n_t * s_t * 4
    peak, peak_kind = measured_peak()
    dom = mg.domain_info(top)
    nc = dom["interface_colours"]
    out["ilu_sweep"] = {"kernel": f"l_luiter FP32 on the finest level ({dom['subdomains']} subdomain interiors, "
                                  f"{dom['interior_rows']} rows, + {nc}+{nc} interface colours), HBM-cold",
                        "launch_ms": lu_ms, "algorithmic_bytes": int(lu_bytes),
                        "achieved": lu_bytes / (lu_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": lu_bytes / (lu_ms * 1e-3) / 1e9 / peak, "peak_kind": peak_kind,
                        "note": f"latency-bound: ~18 interior wavefronts per subdomain block, {2 * nc} dependent "
                                "interface-colour launches"}
    b_host = np.ascontiguousarray(gen.rhs)
    x_host = np.empty_like(b_host)
    mg.solve_host("loc32", b_host, x_host)
    e2e = []
    for _ in range(args.steps):
        flush_l2(); torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, lr = mg.solve_host("loc32", b_host, x_host)
        e2e.append((time.perf_counter() - t0) * 1e3)
        assert lr.converged
    e2e_ms = reduce_over_ranks(float(np.mean(e2e)))
    mg.close()
    (ms64, it64, l64), (ms32, it32, l32) = res["loc64"], res["loc32"]
    out.update({"mixed": {"value": whole_job_rate(1, ms32, world), "unit": "solves/s", "ms_per_solve": ms32,
                          "iterations": it32, "launches_per_solve": l32},
                "fp64": {"value": whole_job_rate(1, ms64, world), "unit": "solves/s", "ms_per_solve": ms64,
                         "iterations": it64, "launches_per_solve": l64},
                "mixed_over_fp64": ms64 / ms32,
                "e2e": {"value": whole_job_rate(1, e2e_ms, world), "unit": "solves/s (mixed, host b -> host x)",
                        "h2d_bytes_per_step": int(b_host.size * 8), "d2h_bytes_per_step": int(b_host.size * 8),
                        "ms_per_step": e2e_ms}})
    if rank == 0:
        try:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle
            oracle.build()
            H = oracle.Hierarchy(gen.levels())
            t0 = time.perf_counter()
            _, it, conv, _ = H.ls_solve_surface(gen.rhs, smoother="ilu", baselevel=0, red=RED)
            dt = time.perf_counter() - t0
            out["cpu_baseline"] = {"value": 1.0 / dt, "unit": "solves/s", "cores": 1, "kind": "port",
                                   "sample": f"one full FP64 solve, list order ({it} iterations, {dt:.1f} s)"}
        except Exception as e:  # reported, not fatal
            out["cpu_baseline"] = {"value": None, "sample": f"failed: {e}"}
    return out


# ---------------------------------------------------------------- batched workload
BATCH_N = 512


def run_batched(args, stream, flush_l2, world, rank):
    """All instances in one batched hierarchy: FP32 Jacobi V(2,2) inside FP64
    iterative refinement to 1e-8 relative defect per instance (and the same
    batch in plain FP64), against the plain FP64 GPU path that solves one
    instance at a time (timed on a sample of instances)."""
    import torch
    import ug_gb300 as G
    from ug_gb300.workloads import batch_instances
    gens, nrefs = batch_instances(args.batch)
    mg = G.MultiGrid(gens, batched=True, order=G.ORDER_LIST, fp32=True, autotune=True,
                     device=torch.cuda.current_device())
    G.lib().gmg_mg_set_stream(mg._h, stream.cuda_stream)
    G.setup_lmgc(mg, "jac", baselevel=0, red=RED, abslimit=1e-50, name="bat64", graph=GRAPH, dloop=GRAPH)
    mg.npcreate("bat32", "linear_solver.gls")
    mg.npinit("bat32", f"$A MAT $x sol $b rhs $red {RED} $abslimit 1e-50 $m 100 $I lmgc $mixed 1"
                       f" $graph {GRAPH} $dloop {GRAPH}")
    b = mg.pack([g.rhs for g in gens])
    x = np.empty_like(b)
    unknowns = int(b.size)
    nnz = sum(mg.size(l)[2] for l in range(mg.nlevels))
    out = {"workload": f"{args.batch} x 2D Q1 Poisson, levels U{{3..7}} (81..16641 unknowns), k=exp(g) var 0.5, "
                       f"Jacobi V(2,2) omega 0.8, to 1e-8 rel defect per instance",
           "instances": args.batch, "unknowns": unknowns, "nnz_all_levels": int(nnz),
           "levels_histogram": {str(L): nrefs.count(L) for L in range(3, 8)}}

    def timed(solver):
        for _ in range(args.warmup):
            mg.solve_host(solver, b, x)
        ms, iters, launches = [], 0, 0
        with ClockSampler(torch.cuda.current_device()) as clk:
            for k in range(args.steps):
                flush_l2(); torch.cuda.synchronize()
                mg.launch_count(reset=True)
                t0 = time.perf_counter()
                with nvtx_range("c4_batch", solver == "bat32" and k == args.steps - 1):
                    _, lr = mg.solve_host(solver, b, x)
                ms.append((time.perf_counter() - t0) * 1e3)
                launches += mg.launch_count()
                assert lr.converged, f"batched {solver} did not converge"
                iters = lr.iters
        return float(np.mean(ms)), iters, launches / args.steps, clk.summary()

    ms32, it32, l32, clk32 = timed("bat32")
    ms64, it64, l64, _ = timed("bat64")
    ms32, ms64 = reduce_over_ranks(ms32), reduce_over_ranks(ms64)
    # device-only: one solve from resident data (b already on the device)
    top = mg.top
    mg.createvector("b0")
    mg.upload_packed("b0", b)
    dev_ms = []
    for k in range(args.warmup + args.steps):
        lr = G.LResult()
        flush_l2()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for l in range(mg.nlevels):
            mg.dcopy(l, "rhs", "b0")
            mg.dset(l, "sol", 0.0)
        mg.ls_defect("bat32", top, "sol", "rhs")
        mg.ls_residuum("bat32", 0, top, "sol", "rhs", lr)
        mg.ls_solver("bat32", top, "sol", "rhs", lr)
        e.record(stream)
        torch.cuda.synchronize()
        if k >= args.warmup:
            dev_ms.append(a.elapsed_time(e))
    # bandwidth of a large launch: FP32 dmatmul_minus on the deepest union
    # level (1.7M rows), HBM-cold, CUDA events on the launching stream
    nl, sl, nnzl = mg.size(top)
    mg.createvector("rx32", "ry32", prec=G.FP32)
    algo = nnzl * (4 + 4) + (nl + 1) * 4 + 3 * nl * 4
    kts = []
    for k in range(args.warmup + 10):
        flush_l2()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        mg.dmatmul_minus(top, "rx32", "ry32")
        e.record(stream)
        torch.cuda.synchronize()
        if k >= args.warmup:
            kts.append(a.elapsed_time(e))
    peak, peak_kind = measured_peak()
    kms = float(np.mean(kts))
    roof_large = {"bound": "hbm", "kernel": f"sell_spmv_kernel<float> on the deepest union level ({nl} rows, "
                                            f"{nnzl} stored entries), HBM-cold",
                  "achieved": algo / (kms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                  "frac": algo / (kms * 1e-3) / 1e9 / peak, "peak_kind": peak_kind, "algorithmic_bytes": int(algo),
                  "launch_ms": kms}
    mg.close()
    dev_ms_max = reduce_over_ranks(float(np.mean(dev_ms)))
    # plain FP64 GPU path: one instance at a time, on a sample
    rng = np.random.default_rng(1)
    sample = sorted(rng.choice(args.batch, size=min(32, args.batch), replace=False).tolist())
    solos = []
    for k in sample:
        m1 = G.MultiGrid(gens[k], order=G.ORDER_COLOR, fp32=False, device=torch.cuda.current_device())
        G.lib().gmg_mg_set_stream(m1._h, stream.cuda_stream)
        G.setup_lmgc(m1, "jac", baselevel=0, red=RED, abslimit=1e-50)
        m1.solve_host("mgs", gens[k].rhs)
        solos.append(m1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k, m1 in zip(sample, solos):
        m1.solve_host("mgs", gens[k].rhs)
    solo_s = time.perf_counter() - t0
    for m1 in solos:
        m1.close()
    # the sample's share of the batch's work (unknowns) scales it to the whole batch
    frac = sum(len(gens[k].rhs) for k in sample) / unknowns
    solo_per_s = len(sample) / solo_s
    solo_batch_s = solo_s / frac  # time to solve all instances one at a time
    out.update({
        "mixed": {"value": whole_job_rate(args.batch, ms32, world), "unit": "solves/s (e2e, host b -> host x)",
                  "ms_per_batch": ms32, "iterations_max": it32, "launches_per_batch": l32, "clocks": clk32,
                  "device_ms_per_batch": dev_ms_max,
                  "device_value": whole_job_rate(args.batch, dev_ms_max, world)},
        "fp64_batched": {"value": whole_job_rate(args.batch, ms64, world), "ms_per_batch": ms64, "iterations_max": it64,
                         "launches_per_batch": l64},
        "fp64_one_at_a_time": {"value": world * args.batch / solo_batch_s, "unit": "solves/s",
                               "sample": f"{len(sample)} instances solved one after another "
                                         f"({solo_per_s:.0f} instance solves/s), scaled to the batch by unknowns"},
        # batching and precision together (the plain FP64 path, one instance at
        # a time) / precision alone (both arms batched)
        "mixed_batched_over_fp64_one_at_a_time": solo_batch_s / (ms32 * 1e-3),
        "mixed_over_fp64_batched": ms64 / ms32,
        "roofline_large_launch": roof_large,
        "h2d_bytes_per_batch": int(unknowns * 8), "d2h_bytes_per_batch": int(unknowns * 8),
    })
    if rank == 0:
        try:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle
            oracle.build()
            cs = sample
            t0 = time.perf_counter()
            for k in cs:
                oracle.Hierarchy(gens[k].levels()).ls_solve(gens[k].rhs, smoother="jac", baselevel=0, damp=0.8,
                                                            red=RED)
            dt = time.perf_counter() - t0
            cfrac = sum(len(gens[k].rhs) for k in cs) / unknowns
            out["cpu_baseline"] = {"value": args.batch / (dt / cfrac), "unit": "solves/s", "cores": 1,
                                   "kind": "port", "sample": f"{len(cs)} instances, FP64, one core ({dt:.1f} s), "
                                                             f"scaled to the batch by unknowns"}
            # the embarrassingly parallel CPU figure: the same sample spread over
            # the host's threads (one instance per thread at a time; the oracle's
            # C calls release the GIL)
            threads = max(1, min(16, os.cpu_count() or 1))
            parts = [cs[i::threads] for i in range(threads)]

            def solve_part(part):
                for k in part:
                    oracle.Hierarchy(gens[k].levels()).ls_solve(gens[k].rhs, smoother="jac", baselevel=0,
                                                                damp=0.8, red=RED)

            t0 = time.perf_counter()
            th = [threading.Thread(target=solve_part, args=(pt,)) for pt in parts if pt]
            [t.start() for t in th]
            [t.join() for t in th]
            dtp = time.perf_counter() - t0
            out["cpu_baseline_parallel"] = {"value": args.batch / (dtp / cfrac), "unit": "solves/s",
                                            "cores": len(th), "kind": "port",
                                            "sample": f"the same {len(cs)} instances on {len(th)} threads "
                                                      f"({dtp:.2f} s), scaled to the batch by unknowns"}
        except Exception as e:  # reported, not fatal
            out["cpu_baseline"] = {"value": None, "sample": f"failed: {e}"}
    return out


# ---------------------------------------------------------------- serving workload
SERVE_RATE, SERVE_LEVELS = 200.0, (2, 7)


def run_serving(args, rank, mixed=(), extras=True):
    """The request loop: a seeded Poisson stream (mean 200 req/s) of 3D P1
    diffusion solves, depths U{2..7} (125 .. 2,146,689 unknowns), log-normal
    k (corr 0.1, var 1), FP32 multicolour-GS V(2,2) in FP64 refinement to
    1e-8, admitted into resident pools by free device memory.  mixed: groups
    of depths that share mixed pools (their V-cycles batched level by level
    across mesh sizes); extras: also time admissions, sample the served
    results' accuracy and time the CPU baseline."""
    import torch
    import ug_gb300 as G
    from ug_gb300.serve import Server, poisson_stream
    t0 = time.perf_counter()
    srv = Server(depths=range(SERVE_LEVELS[0], SERVE_LEVELS[1] + 1), device=torch.cuda.current_device(),
                 mixed=mixed, grow_after_ms=None, mesh=gen_kind(G))
    srv.warm()  # every pool's temporaries and CUDA graph
    setup_s = time.perf_counter() - t0
    srv.run(poisson_stream(max(24, args.warmup * 12), SERVE_RATE, SERVE_LEVELS, seed=77))
    reqs = poisson_stream(args.serve_requests, SERVE_RATE, SERVE_LEVELS, seed=2026 + rank)
    with ClockSampler(torch.cuda.current_device()) as clk:
        st = srv.run(reqs)
    if not extras:
        srv.close()
        st.p50_ms, st.p99_ms, st.mean_ms = (reduce_over_ranks(v) for v in (st.p50_ms, st.p99_ms, st.mean_ms))
        st.throughput = reduce_over_ranks(st.throughput, "sum")
        return {"workload": "the stream of `serving` (same requests)", "mixed_pools": [list(g) for g in mixed],
                "requests": st.completed, "p50_ms": st.p50_ms, "p99_ms": st.p99_ms, "mean_ms": st.mean_ms,
                "throughput_req_s": st.throughput, "all_converged": st.all_converged,
                "per_depth": {str(k): v for k, v in st.per_depth.items()},
                "queue_wait_ms": st.breakdown["queue_wait_ms"], "service_ms": st.breakdown["service_ms"],
                "setup_s": setup_s, "clocks": clk.summary()}
    # the admission's device work per depth (field, assembly of every level,
    # right-hand side, first norm), timed alone after the stream, with the
    # stream's FP32 field and with the FP64 field
    admit_ms = {"fp32_field": {}, "fp64_field": {}}
    for L, pools in srv.pools.items():
        p = pools[0]
        for key, prec in (("fp32_field", 1), ("fp64_field", 0)):
            G.lib().gmg_pool_set_field_precision(p._h, prec)
            ts = []
            for rep in range(3):
                slot = p.free_slot(L)
                torch.cuda.synchronize()
                t1 = time.perf_counter()
                p.admit(slot, 999 + rep, srv.corr, srv.var)
                torch.cuda.synchronize()
                ts.append((time.perf_counter() - t1) * 1e3)
                while True:  # iterate the request to its end, which frees the slot
                    p.launch()
                    while (done := p.poll()) is None:
                        pass
                    if slot in done:
                        break
                p.fetch(slot, False)
            admit_ms[key][str(L)] = float(np.median(ts))
        G.lib().gmg_pool_set_field_precision(p._h, 0 if srv.field_fp64 else 1)
    # accuracy of served results: a sample of the stream's requests solved again
    # alone in a pool of their depth (bitwise the result they had in the mix,
    # tests/test_serve.py), against FP64 oracle solutions converged to 1e-12 of
    # (a) the problem the slot held (its matrices read back from the device)
    # and (b) the host-assembled FP64 problem (depths up to 6 on the CPU)
    served_err = {}
    if rank == 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        oracle.build()
        for L in range(SERVE_LEVELS[0], min(SERVE_LEVELS[1], 6) + 1):
            sample = [r for r in reqs if r.nref == L][: (2 if L <= 5 else 1)]
            e_slot, e_host, same_iters = [], [], True
            p = srv.pools[L][0]
            for r in sample:
                slot = p.free_slot(L)
                x, lr = p.solve(r.seed, srv.corr, srv.var, slot=slot)
                same_iters = same_iters and lr.iters == r.iters
                levels, rhs, _ = oracle.cube_levels(L, r.seed, CORR, VAR, ug_rules=MESH == "ug")
                xo, _, conv, _ = oracle.Hierarchy(levels).ls_solve(rhs, smoother="gs", baselevel=0, red=1e-12,
                                                                   abslimit=1e-50, base_abslimit=1e-30)
                e_host.append(float(np.max(np.abs(x - xo)) / np.max(np.abs(xo))) if conv else float("nan"))
                held = [dict(d, val=p.slot_matrix(slot, l, d["val"].size)) for l, d in enumerate(levels)]
                xs, _, conv, _ = oracle.Hierarchy(held).ls_solve(rhs, smoother="gs", baselevel=0, red=1e-12,
                                                                 abslimit=1e-50, base_abslimit=1e-30)
                e_slot.append(float(np.max(np.abs(x - xs)) / np.max(np.abs(xs))) if conv else float("nan"))
            served_err[str(L)] = {"requests": len(sample), "same_iterations_as_served": same_iters,
                                  "max_rel_error_vs_fp64_oracle_of_served_problem": max(e_slot),
                                  "max_rel_error_vs_fp64_oracle_of_host_problem": max(e_host)}
    srv.close()
    # replicas: latencies of the slowest rank, throughput of all ranks
    st.p50_ms, st.p99_ms, st.mean_ms = (reduce_over_ranks(v) for v in (st.p50_ms, st.p99_ms, st.mean_ms))
    st.throughput = reduce_over_ranks(st.throughput, "sum")
    out = {"workload": f"{args.serve_requests} requests, Poisson arrivals mean {SERVE_RATE:.0f}/s, 3D P1 cube "
                       f"levels U{{{SERVE_LEVELS[0]}..{SERVE_LEVELS[1]}}} (125..2146689 unknowns, {MESHES[MESH]}), "
                       f"k=exp(g) corr 0.1 var 1, FP32 GS V(2,2) in FP64 refinement to 1e-8",
           "requests": st.completed, "p50_ms": st.p50_ms, "p99_ms": st.p99_ms, "mean_ms": st.mean_ms,
           "throughput_req_s": st.throughput, "offered_req_s": SERVE_RATE, "makespan_s": st.makespan_s,
           "iterations_mean": st.iterations_mean, "all_converged": st.all_converged,
           "per_depth": {str(k): v for k, v in st.per_depth.items()},
           "breakdown": st.breakdown, "admission_device_ms": admit_ms,
           "field": "FP64" if srv.field_fp64 else "FP32 (fixed-point phases, FP32 cosines: k within ~1e-6 of the "
                                                 "host generator's; the FP64 field is the pools' option)",
           "accuracy_sample": served_err,
           "pools": {str(L): {"pools": n, "slots_each": m} for L, (n, m) in srv.layout.items()},
           "mixed_pools": [list(g) for g in mixed],
           "setup_s": setup_s, "clocks": clk.summary(),
           "pools_grown_while_serving": [[round(t, 3), L] for t, L in srv.grown],
           "note": "latency = completion - arrival (queueing, on-device assembly, all iterations, "
                   "solution not copied back); the published stream has 20k requests"}
    if rank == 0:
        try:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle
            oracle.build()
            per = {}
            for L in range(SERVE_LEVELS[0], min(SERVE_LEVELS[1], 6) + 1):
                gen = G.Generator(gen_kind(G), L, seed=31 + L, corr=CORR, var=VAR)
                H = oracle.Hierarchy(gen.levels())
                t1 = time.perf_counter()
                H.ls_solve(gen.rhs, smoother="gs", baselevel=0, red=RED)
                per[L] = time.perf_counter() - t1
            for L in range(7, SERVE_LEVELS[1] + 1):
                per[L] = per[L - 1] * 8.0  # 8x the unknowns per refinement
            mean_s = float(np.mean(list(per.values())))
            out["cpu_baseline"] = {"value": 1.0 / mean_s, "unit": "req/s", "cores": 1, "kind": "port",
                                   "sample": "one FP64 solve per depth 2..6 (UG list-order GS), depth 7 taken as 8x "
                                             "depth 6; value = 1 / mean solve time over the uniform depth mix",
                                   "solve_s": {str(k): v for k, v in per.items()}}
        except Exception as e:  # reported, not fatal
            out["cpu_baseline"] = {"value": None, "sample": f"failed: {e}"}
    return out


# ---------------------------------------------------------------- roofline kernels of the C2 solve
def c2_roofline(G, mg, stream, flush_l2, reps=20, skip=3):
    """Roofline of the dominant streaming kernels of the C2 solve, each timed
    HBM-cold (L2 flushed before every repetition) with CUDA events on the
    launching stream:
    * the finest level's smoothing as lmgc runs it (gmg_iter_smooth, 2 FP32
      Gauss-Seidel steps): per colour one sell_gs_chain_kernel launch per
      step, then one sell_upper_defect_kernel launch; algorithmic bytes per
      smoothing = 2 (M + 6 V), M = nnz (4 + 4) + 4 (n + 1) the FP32 matrix
      stream, V = 4 n a vector (the GS step with fused defect update);
    * the finest level's dmatmul_minus (sell_spmv_kernel) in FP32 and FP64:
      nnz (p + 4) + 4 (n + 1) + 3 n q."""
    import torch
    top = mg.top
    n, s, nnz = mg.size(top)
    nwaves = mg.num_waves(top)
    for v in ("ry", "rx"):
        try:
            mg.vec(v)
        except G.GmgError:
            mg.createvector(v)
    for v in ("ry32", "rx32", "st32", "sb32", "sc32"):
        try:
            mg.vec(v)
        except G.GmgError:
            mg.createvector(v, prec=G.FP32)
    b0 = np.linspace(-1.0, 1.0, n * s)
    mg.upload("sb32", top, b0)
    mg.dset(top, "sc32", 0.0)
    algo_smooth = 2 * ((nnz * (4 + 4) + 4 * (n + 1)) + 6 * n * s * 4)
    launches_smooth = 2 * nwaves + 1
    algo = {64: nnz * (8 + 4) + (n + 1) * 4 + 3 * n * 8, 32: nnz * (4 + 4) + (n + 1) * 4 + 3 * n * 4}

    def event_ms(fn, name):
        ts = []
        for k in range(reps):
            if k % 5 == 0:
                mg.upload("sb32", top, b0)  # keep the defect away from denormals
            flush_l2()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with nvtx_range(name, k == reps - 1):
                a.record(stream)
                fn()
                b.record(stream)
                torch.cuda.synchronize()
            if k >= skip:
                ts.append(a.elapsed_time(b))
        return float(np.mean(ts))

    sm_ms = event_ms(lambda: mg.iter_smooth("smooth", top, "st32", "sb32", "sc32", 2), "c2_smooth")
    kms = {64: event_ms(lambda: mg.dmatmul_minus(top, "rx", "ry"), "c2_spmv64"),
           32: event_ms(lambda: mg.dmatmul_minus(top, "rx32", "ry32"), "c2_spmv32")}
    peak, peak_kind = measured_peak()
    ach = algo_smooth / (sm_ms * 1e-3) / 1e9
    ach32 = algo[32] / (kms[32] * 1e-3) / 1e9
    ach64 = algo[64] / (kms[64] * 1e-3) / 1e9
    tr = profiled_traffic("smooth")
    return {"bound": "hbm",
            "kernel": f"sell_gs_chain_kernel<float> + sell_upper_defect_kernel<float>: the finest level's "
                      f"2 Gauss-Seidel smoothing steps as lmgc runs them ({launches_smooth} launches: "
                      f"{nwaves} colours x 2 steps + 1 defect pass), HBM-cold; per launch",
            "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "peak_kind": peak_kind,
            "traffic": tr, "algorithmic_bytes": algo_smooth / launches_smooth,
            "launch_ms": sm_ms / launches_smooth, "smoothing_ms": sm_ms,
            "note": "each colour wave is a dependent gather chain of a few us (latency-bound launches); rows "
                    "store their lower entries first, so a forward wave streams only those",
            "spmv_fp32": {"kernel": "sell_spmv_kernel<float> (finest-level dmatmul_minus)",
                          "achieved": ach32, "frac": ach32 / peak, "algorithmic_bytes": algo[32],
                          "launch_ms": kms[32], "traffic": profiled_traffic("spmv")},
            "spmv_fp64": {"achieved": ach64, "frac": ach64 / peak, "algorithmic_bytes": algo[64],
                          "launch_ms": kms[64]}}


# ---------------------------------------------------------------- our arm
def mesh_comparison(args, stream, flush_l2, world):
    """The same mixed solve on the Freudenthal triangulation of the cube (same
    nodes, same edge count, 4 colours on every level where UG's red rules
    need up to 9): what the colour count costs.  Device-timed like `value`."""
    import torch
    import ug_gb300 as G
    gen = G.Generator(G.Generator.DIFFUSION3D, NREF, seed=SEED, corr=CORR, var=VAR)
    mg = G.MultiGrid(gen, order=G.ORDER_COLOR, fp32=True, autotune=True)
    G.lib().gmg_mg_set_stream(mg._h, stream.cuda_stream)
    mg.createvector("sol", "rhs", "rhs0")
    G.setup_lmgc(mg, "gs", baselevel=0, red=RED, abslimit=1e-50, name="mgs64")
    mg.npcreate("mgs32", "linear_solver.gls")
    mg.npinit("mgs32", f"$A MAT $x sol $b rhs $red {RED} $abslimit 1e-50 $m 100 $I lmgc $mixed 1 $graph 1 $dloop 1")
    top = mg.top
    mg.upload("rhs0", top, gen.rhs)
    mg.ls_preprocess("mgs32", top, "sol", "rhs")
    ms, it = [], 0
    for k in range(args.warmup + args.steps):
        flush_l2()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        lr = G.LResult()
        e0.record(stream)
        mg.dcopy(top, "rhs", "rhs0")
        mg.dset(top, "sol", 0.0)
        mg.ls_defect("mgs32", top, "sol", "rhs")
        mg.ls_residuum("mgs32", 0, top, "sol", "rhs", lr)
        mg.ls_solver("mgs32", top, "sol", "rhs", lr)
        e1.record(stream)
        torch.cuda.synchronize()
        assert lr.converged
        it = lr.iters
        if k >= args.warmup:
            ms.append(e0.elapsed_time(e1))
    waves = [mg.num_waves(l) for l in range(mg.nlevels)]
    mg.close()
    ms_step = reduce_over_ranks(float(np.mean(ms)), "max")
    return {"value": whole_job_rate(1, ms_step, world), "unit": "solves/s", "ms_per_step": ms_step,
            "iterations": it, "gs_waves_per_level": waves,
            "note": "mixed solve of the same problem on the Freudenthal triangulation (not UG's mesh)"}


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    import ug_gb300 as G

    # L2 flush between timed steps: READ 256 MB (twice the L2), which leaves
    # only clean lines behind (a write would leave dirty lines whose
    # write-back the next timed kernel would pay for)
    flush = torch.ones(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    sink = torch.empty((), dtype=torch.float32, device="cuda")

    def flush_l2():
        torch.sum(flush, dim=0, out=sink)

    single = {"c1": lambda: run_c1(args, stream, flush_l2, world, rank),
              "serving_mixed": lambda: run_serving(args, rank, mixed=[(2, 3, 4, 5)], extras=False),
              "local": lambda: run_local(args, stream, flush_l2, world, rank),
              "batched": lambda: run_batched(args, stream, flush_l2, world, rank),
              "serving": lambda: run_serving(args, rank)}
    if args.only in single:  # one workload alone (profiling runs)
        out = single[args.only]()
        if rank == 0:
            print(json.dumps({"only": args.only, args.only: out}), flush=True)
        return

    gen = G.Generator(gen_kind(G), NREF, seed=SEED, corr=CORR, var=VAR)
    mg = G.MultiGrid(gen, order=G.ORDER_COLOR, fp32=True, autotune=True, device=local)
    G.lib().gmg_mg_set_stream(mg._h, stream.cuda_stream)
    mg.createvector("sol", "rhs", "rhs0")
    graph = bool(GRAPH)
    G.setup_lmgc(mg, "gs", baselevel=0, red=RED, abslimit=1e-50, name="mgs64", graph=graph, dloop=graph)
    mg.npcreate("mgs32", "linear_solver.gls")
    mg.npinit("mgs32", f"$A MAT $x sol $b rhs $red {RED} $abslimit 1e-50 $m 100 $I lmgc $mixed 1"
                       f" $graph {int(graph)} $dloop {int(graph)}")
    top = mg.top
    mg.upload("rhs0", top, gen.rhs)
    mg.ls_preprocess("mgs64", top, "sol", "rhs")

    def step(solver):
        lr = G.LResult()
        mg.dcopy(top, "rhs", "rhs0")
        mg.dset(top, "sol", 0.0)
        mg.ls_defect(solver, top, "sol", "rhs")
        mg.ls_residuum(solver, 0, top, "sol", "rhs", lr)
        mg.ls_solver(solver, top, "sol", "rhs", lr)
        return lr

    if args.only == "c2mixed":  # the headline mixed solve alone (profiling runs)
        ms = []
        mg.launch_count(reset=True)
        for k in range(args.warmup + args.steps):
            flush_l2()
            a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with nvtx_range("c2_mixed_solve", k == args.warmup + args.steps - 1):
                a.record(stream)
                lr = step("mgs32")
                e.record(stream)
                torch.cuda.synchronize()
            assert lr.converged
            if k >= args.warmup:
                ms.append(a.elapsed_time(e))
        out = {"ms_per_step": float(np.mean(ms)), "iterations": lr.iters,
               "launches_per_solve": mg.launch_count() / (args.warmup + args.steps), "graph": graph,
               "mesh": MESH, "gs_waves_per_level": [mg.num_waves(l) for l in range(mg.nlevels)],
               "variants": [mg.level_variant(l) for l in range(mg.nlevels)]}
        mg.close()
        if rank == 0:
            print(json.dumps({"only": "c2mixed", "c2mixed": out}), flush=True)
        return
    if args.only == "roofline":  # the roofline kernels alone (profiling runs)
        roof = c2_roofline(G, mg, stream, flush_l2, reps=args.warmup + args.steps, skip=args.warmup)
        mg.close()
        if rank == 0:
            print(json.dumps({"only": "roofline", "roofline": roof}), flush=True)
        return

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    results, xs = {}, {}
    for solver in ("mgs64", "mgs32"):
        for _ in range(args.warmup):
            step(solver)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        launches = 0
        iters = []
        with ClockSampler(local) as clk:
            barrier(); torch.cuda.synchronize()
            t0 = time.perf_counter()
            for k in range(args.steps):
                flush_l2()
                mg.launch_count(reset=True)
                ev[k][0].record(stream)
                lr = step(solver)
                ev[k][1].record(stream)
                launches += mg.launch_count()
                iters.append(lr.iters)
                assert lr.converged, f"{solver} did not converge"
            torch.cuda.synchronize(); barrier()
            wall = time.perf_counter() - t0
        ms = [a.elapsed_time(b) for a, b in ev]
        xs[solver] = mg.download("sol", top)  # the last timed solve's solution (list order)
        ms_step = reduce_over_ranks(float(np.mean(ms)), "max")
        results[solver] = {"ms_per_step": ms_step, "iters": iters[-1], "launches_per_step": launches / args.steps,
                           "clocks": clk.summary(), "wall_s": wall}

    # end to end through the C ABI: host b -> solve -> host x, mixed precision
    b_host = np.ascontiguousarray(gen.rhs)
    x_host = np.empty_like(b_host)
    lr = G.LResult()
    mg.solve_host("mgs32", b_host, x_host)  # warm
    torch.cuda.synchronize()
    e2e_t = []
    for _ in range(args.steps):
        flush_l2(); torch.cuda.synchronize()
        t0 = time.perf_counter()
        mg.solve_host("mgs32", b_host, x_host)
        e2e_t.append(time.perf_counter() - t0)
    e2e_ms = reduce_over_ranks(float(np.mean(e2e_t)) * 1e3)

    n, s, nnz = mg.size(top)
    roof = c2_roofline(G, mg, stream, flush_l2)

    # CPU baseline: the oracle port, one FP64 solve on one core, bounded sample
    cpu, accuracy = None, None
    if rank == 0:
        try:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle
            oracle.build()
            H = oracle.Hierarchy(gen.levels())
            t0 = time.perf_counter()
            _, it_cpu, conv, _ = H.ls_solve(gen.rhs, smoother="gs", baselevel=0, red=RED)
            dt = time.perf_counter() - t0
            cpu = {"value": 1.0 / dt, "unit": "solves/s", "cores": 1, "kind": "port",
                   "sample": f"one full FP64 solve of the workload in UG's list order ({it_cpu} iterations, {dt:.1f} s)"}
            # the timed solutions against FP64: their defect computed by the
            # oracle in FP64, and their distance to the FP64 solution converged
            # to 1e-12 (the discrete solution up to 1e-12 of the defect)
            xt, it_t, conv_t, _ = H.ls_solve(gen.rhs, smoother="gs", baselevel=0, red=1e-12, abslimit=1e-50,
                                             base_abslimit=1e-30)
            nb = float(H.nrm2x(top, gen.rhs)[0])
            accuracy = {"reference": f"oracle FP64 solve to 1e-12 rel defect ({it_t} iterations, converged "
                                     f"{conv_t}); defects computed by the oracle in FP64"}
            for key, solver in (("mixed", "mgs32"), ("fp64", "mgs64")):
                d = H.matmul_minus(top, gen.rhs, xs[solver])
                accuracy[key] = {"rel_defect_fp64": float(H.nrm2x(top, d)[0]) / nb,
                                 "rel_error_vs_fp64_solution": float(np.max(np.abs(xs[solver] - xt)) /
                                                                     np.max(np.abs(xt)))}
            accuracy["mixed_vs_fp64_gpu"] = float(np.max(np.abs(xs["mgs32"] - xs["mgs64"])) /
                                                  np.max(np.abs(xs["mgs64"])))
        except Exception as e:  # reported, not fatal
            cpu = {"value": None, "unit": "solves/s", "cores": 1, "kind": "port", "sample": f"failed: {e}"}

    waves = [mg.num_waves(l) for l in range(mg.nlevels)]
    variants = [mg.level_variant(l) for l in range(mg.nlevels)]
    mg.close()
    other_mesh = mesh_comparison(args, stream, flush_l2, world) if MESH == "ug" else None
    rest = args.only != "c2"
    c1 = run_c1(args, stream, flush_l2, world, rank) if rest else None
    local_c3 = run_local(args, stream, flush_l2, world, rank) if rest and not args.no_local else None
    batched = run_batched(args, stream, flush_l2, world, rank) if rest and not args.no_batched else None
    serving = run_serving(args, rank) if rest and not args.no_serving else None
    serving_mixed = run_serving(args, rank, mixed=[(2, 3, 4, 5)], extras=False) if rest and not args.no_serving \
        else None

    if rank == 0:
        r32, r64 = results["mgs32"], results["mgs64"]
        value = whole_job_rate(1, r32["ms_per_step"], world)
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r32["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32-in-f64 (mixed); f64 reported beside",
            "data": "synthetic (seeded)",
            "config": workload_config(),
            "ordering": "multicolour (DSATUR colouring of every level)",
            "run": {"iterations_mixed": r32["iters"], "iterations_fp64": r64["iters"],
                    "parallelism": "replicas" if world > 1 else "1 GPU",
                    "gs_waves_per_level": waves,
                    "kernel_variants_per_level (autotuned)": variants,
                    "launches_per_solve": r32["launches_per_step"]},
            "fp64": {"value": whole_job_rate(1, r64["ms_per_step"], world), "unit": "solves/s",
                     "ms_per_step": r64["ms_per_step"],
                     "iterations": r64["iters"]},
            "mixed_over_fp64": r64["ms_per_step"] / r32["ms_per_step"],
            "e2e": {"value": whole_job_rate(1, e2e_ms, world), "unit": "solves/s", "h2d_bytes_per_step": int(n * s * 8),
                    "d2h_bytes_per_step": int(n * s * 8), "ms_per_step": e2e_ms},
            "roofline": roof,
            "gpu_launches": int(r32["launches_per_step"] * args.steps),
            "clocks": r32["clocks"],
            "cpu_baseline": cpu,
            "accuracy": accuracy,
            "freudenthal_mesh": other_mesh,
            "config1": c1,
            "local_refinement": local_c3,
            "batched": batched,
            "serving": serving,
            "serving_mixed_pools": serving_mixed,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    global MESH, GRAPH
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-instances workload")
    ap.add_argument("--no-local", action="store_true", help="skip the locally refined workload")
    ap.add_argument("--batch", type=int, default=BATCH_N, help="instances of the batched workload")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving workload")
    ap.add_argument("--serve-requests", type=int, default=2000, help="requests of the serving stream")
    ap.add_argument("--no-graph", action="store_true",
                    help="ls solvers without CUDA graphs ($graph 0 $dloop 0): every kernel an individual launch, "
                         "for profilers that do not see inside conditional graphs; not a benchmark setting")
    ap.add_argument("--only", default="all", choices=["all", "c2", "c2mixed", "roofline", "c1", "local", "batched",
                                                      "serving", "serving_mixed"],
                    help="run one workload alone and print its JSON (profiling runs); c2: the headline solve "
                         "without the other workloads; roofline: the C2 roofline kernels only, warmup + steps "
                         "repetitions each")
    ap.add_argument("--mesh", default=MESH, choices=sorted(MESHES),
                    help="tetrahedra of the headline workload (both arms): ug = UG's red rules, UG's own mesh; "
                         "freudenthal = the Freudenthal triangulation (same nodes and edge counts)")
    args = ap.parse_args()
    MESH = args.mesh
    GRAPH = 0 if args.no_graph else 1
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
