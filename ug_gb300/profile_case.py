"""Small driver for profiling the lmgc path with Nsight Compute.

One solve of the 3D P1 diffusion workload (unit cube, six Kuhn tetrahedra
refined --nref times, k = exp(g), multicolour Gauss-Seidel V(2,2)), limited
to --cycles ls iterations, with CUDA graphs off so that every kernel is an
individual launch in the profiler's launch list.

    python -m ug_gb300.profile_case --cycles 2 [--fp64] [--nref 6] [--fuse 40000]

With --batched N: N instances of the batched workload (2D Q1 Poisson,
levels 3..7, Jacobi V(2,2)) in one batched hierarchy instead.
With --spmv / --lgs: only the finest level's dmatmul_minus / Gauss-Seidel
sweep (l_lgs, one launch per colour) in FP32, --cycles times.
With --local NUNI: the locally refined L-shaped elasticity workload (NUNI
uniform + --nloc local refinements, block ILU(0) V(2,2)) instead.
With --coarse L: only the fused coarse cycle (one launch of one CTA), lmgc
Iter on levels 1..L of the 3D hierarchy, --cycles times each, FP32.
"""
import argparse

import numpy as np

import ug_gb300 as G


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cycles", type=int, default=2)
    ap.add_argument("--nref", type=int, default=6)
    ap.add_argument("--fp64", action="store_true")
    ap.add_argument("--fuse", type=int, default=40000)
    ap.add_argument("--batched", type=int, default=0)
    ap.add_argument("--order", default="color", choices=["color", "list"])
    ap.add_argument("--bsmem", type=int, default=None)
    ap.add_argument("--spmv", action="store_true")
    ap.add_argument("--lgs", action="store_true", help="only the finest level's FP32 Gauss-Seidel sweep (l_lgs)")
    ap.add_argument("--pool", type=int, default=0, help="one request in a one-slot serving pool of this depth")
    ap.add_argument("--local", type=int, default=0, help="uniform refinements of the locally refined workload")
    ap.add_argument("--nloc", type=int, default=9)
    ap.add_argument("--coarse", type=int, default=0,
                    help="only the fused coarse cycle: lmgc Iter on levels 1..COARSE, --cycles times each (FP32)")
    ap.add_argument("--narrow", type=int, default=1, help="$narrow of lmgc (0: the whole block on every level)")
    a = ap.parse_args()
    if a.local:
        gen = G.LocalGenerator(a.local, a.nloc, seed=2026)
        mg = G.MultiGrid(gen, order=G.ORDER_DOMAIN, fp32=True)
        G.setup_lmgc(mg, "ilu", baselevel=0, red=1e-8, maxit=a.cycles, mixed=not a.fp64, graph=False)
        mg.launch_count(reset=True)
        x, lr = mg.solve_host("mgs", gen.rhs)
        print(f"cycles={lr.iters} defect {lr.first_defect[0]:.3e} -> {lr.last_defect[0]:.3e}, "
              f"{mg.launch_count()} kernel launches")
        mg.close()
        return
    if a.pool:
        from ug_gb300.serve import Pool
        p = Pool(a.pool, 1)
        p.free.remove(0)
        p.admit(0, 2026, 0.1, 1.0)
        for _ in range(a.cycles):
            p.launch()
            while p.poll() is None:
                pass
        print(f"{a.cycles} pool iterations, depth {a.pool}")
        p.close()
        return
    if a.coarse:
        gen = G.Generator(G.Generator.DIFFUSION3D, a.nref, seed=2026, corr=0.1, var=1.0)
        mg = G.MultiGrid(gen, order=G.ORDER_COLOR, fp32=True)
        G.setup_lmgc(mg, "gs", baselevel=0, red=1e-8, mixed=True, graph=False, narrow=bool(a.narrow))
        mg.createvector("cc", "bb", prec=G.FP32)
        mg.iter_preprocess("lmgc", mg.top, "sol", "rhs")
        for lev in range(1, a.coarse + 1):
            mg.upload("bb", lev, np.linspace(-1.0, 1.0, mg.size(lev)[0] * mg.size(lev)[1]))
            mg.dset(lev, "cc", 0.0)
            for _ in range(a.cycles):
                mg.iter_iter("lmgc", lev, "cc", "bb")
        mg.sync()
        print(f"fused coarse cycles on levels 1..{a.coarse}, {a.cycles} each, narrow={a.narrow}")
        mg.close()
        return
    if a.spmv or a.lgs:
        gen = G.Generator(G.Generator.DIFFUSION3D, a.nref, seed=2026, corr=0.1, var=1.0)
        mg = G.MultiGrid(gen, order=G.ORDER_COLOR, fp32=True)
        mg.createvector("x32", "y32", prec=G.FP32)
        for _ in range(a.cycles):
            if a.lgs:
                mg.l_lgs(mg.top, "x32", "y32")
            else:
                mg.dmatmul_minus(mg.top, "x32", "y32")
        mg.sync()
        print(f"{a.cycles} {'l_lgs sweeps' if a.lgs else 'dmatmul_minus launches'} on {mg.size(mg.top)}")
        mg.close()
        return
    if a.batched:
        from ug_gb300.workloads import batch_instances
        gens, _ = batch_instances(a.batched)
        order = G.ORDER_COLOR if a.order == "color" else G.ORDER_LIST
        mg = G.MultiGrid(gens, batched=True, order=order, fp32=True)
        G.setup_lmgc(mg, "jac", baselevel=0, red=1e-8, maxit=a.cycles, mixed=not a.fp64, graph=False,
                     bsmem=a.bsmem)
        mg.launch_count(reset=True)
        x, lr = mg.solve_host("mgs", mg.pack([g.rhs for g in gens]))
        print(f"cycles={lr.iters} max defect {lr.first_defect[0]:.3e} -> {lr.last_defect[0]:.3e}, "
              f"{mg.launch_count()} kernel launches")
        mg.close()
        return
    gen = G.Generator(G.Generator.DIFFUSION3D, a.nref, seed=2026, corr=0.1, var=1.0)
    mg = G.MultiGrid(gen, order=G.ORDER_COLOR, fp32=True)
    G.setup_lmgc(mg, "gs", baselevel=0, red=1e-8, maxit=a.cycles, mixed=not a.fp64, graph=False, fuse=a.fuse)
    mg.launch_count(reset=True)
    x, lr = mg.solve_host("mgs", gen.rhs)
    print(f"cycles={lr.iters} defect {lr.first_defect[0]:.3e} -> {lr.last_defect[0]:.3e}, "
          f"{mg.launch_count()} kernel launches")
    mg.close()


if __name__ == "__main__":
    main()
