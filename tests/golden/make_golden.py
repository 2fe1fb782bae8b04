"""Regenerate the golden fixtures in this directory from the UG reference.

Builds the reference with oracle/Makefile (needs the UG 3.12.1 sources: set
the environment variable REF to that tree), runs oracle/_ref/ug_export{2d,3d} for each
case below and stores every record as a compressed .npz.  Each fixture holds
the hierarchy exactly as UG's grid manager and assembly produced it, the
known-answer vectors of UG's kernels on the finest level, and UG's own ls +
lmgc solve (iteration count, defect history, solution) and its cg + lmgc and
bcgs + lmgc solves (iteration count, defects, solution).  The ``ls_*`` cases
are locally refined: the L-shaped elasticity problem, uniformly refined
``nref`` times and then ``nloc`` times toward the re-entrant corner, with the
surface flags (FINE_GRID_DOF, NEW_DEFECT, FULLREFINELEVEL) and the solution on
every level.

    python tests/golden/make_golden.py [name ...]

The ``*bw*`` / ``*lex*`` cases repeat a case above after one of UG's order
numprocs renumbered every level (its GS / ILU then sweep in the new order).
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402

# name: (dimension, problem, nref, baselevel, smoother, seed[, nloc[, order[, imat]]]);
# order = one of UG's order numprocs run on every level after the assembly
# ("bw" = order.bw, "lex:<config>" = order.lex $config <config>); imat =
# "block": interpolation matrices and the transfer's matrix mode
CASES = {
    "q1_jac": (2, "poisson", 5, 2, "jac", 11),
    "q1_gs": (2, "poisson", 5, 2, "gs", 11),
    "q1_ilu": (2, "poisson", 5, 2, "ilu", 11),
    "p1_gs": (3, "poisson", 3, 0, "gs", 12),
    "p1k_jac": (3, "diffusion", 3, 0, "jac", 13),
    "p1k_gs": (3, "diffusion", 3, 0, "gs", 13),
    "p1k_ilu": (3, "diffusion", 3, 0, "ilu", 13),
    "el_jac": (2, "elasticity", 4, 1, "jac", 14),
    "el_gs": (2, "elasticity", 4, 1, "gs", 14),
    "el_ilu": (2, "elasticity", 4, 1, "ilu", 14),
    "ls_jac": (2, "lshape", 2, 0, "jac", 22, 6),
    "ls_gs": (2, "lshape", 2, 0, "gs", 22, 6),
    "ls_ilu": (2, "lshape", 2, 0, "ilu", 22, 6),
    "q1bw_gs": (2, "poisson", 5, 2, "gs", 11, 0, "bw"),
    "q1lex_ilu": (2, "poisson", 5, 2, "ilu", 11, 0, "lex:ur"),
    "p1lex_gs": (3, "poisson", 3, 0, "gs", 12, 0, "lex:dfl"),
    "elbw_ilu": (2, "elasticity", 4, 1, "ilu", 14, 0, "bw"),
    "ls_bw_gs": (2, "lshape", 2, 0, "gs", 22, 6, "bw"),
    # the transfer in UG's matrix mode (`$M`) on seeded block interpolation
    # matrices (IMATRIX) near the standard transfer
    "im_q1_gs": (2, "poisson", 5, 2, "gs", 11, 0, "none", "block"),
    "im_el_ilu": (2, "elasticity", 4, 1, "ilu", 14, 0, "none", "block"),
    "im_p1k_jac": (3, "diffusion", 3, 0, "jac", 13, 0, "none", "block"),
    "im_ls_gs": (2, "lshape", 2, 0, "gs", 22, 6, "none", "block"),
}


def main():
    env = dict(os.environ)
    if not env.get("REF"):
        raise SystemExit("set REF to the UG 3.12.1 source tree")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-j8", "ref"], check=True, env=env)
    only = set(sys.argv[1:])  # optional: the names to regenerate
    with tempfile.TemporaryDirectory() as tmp:
        for name, (dim, problem, nref, base, sm, seed, *rest) in CASES.items():
            if only and name not in only:
                continue
            exe = os.path.join(ROOT, "oracle", "_ref", f"ug_export{dim}d")
            raw = os.path.join(tmp, name + ".bin")
            nloc = rest[0] if rest else 0
            order = rest[1] if len(rest) > 1 else "none"
            imat = rest[2] if len(rest) > 2 else "none"
            subprocess.run([exe, problem, str(nref), str(base), sm, str(seed), raw, "100", str(nloc), order, imat],
                           check=True, stdout=subprocess.DEVNULL)
            fx = oracle.read_ugfx(raw)
            arrays = {k: (np.array(v) if not isinstance(v, str) else np.array(v)) for k, v in fx.items()}
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
            print(f"{name}: levels={int(fx['nlevels'][0])} n_top={int(fx['L%d_n' % (int(fx['nlevels'][0]) - 1)][0])}"
                  f" ug_iters={int(fx['ls_iters'][0])}")


if __name__ == "__main__":
    main()
