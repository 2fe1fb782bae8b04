"""The synthetic workloads of the benchmark, as hierarchy generators.

batched: `count` independent 2D Q1 Poisson instances on the unit square,
instance k refined L_k ~ U{3..7} times ((2^L+1)^2 = 81 .. 16,641 unknowns),
k = exp(g) with its own seeded field (correlation 0.1, variance 0.5) and its
own seeded uniform[-1,1] right-hand side."""
from __future__ import annotations

import numpy as np

BATCH_SEED, BATCH_CORR, BATCH_VAR = 4242, 0.1, 0.5


def batch_instances(count: int, seed: int = BATCH_SEED, levels=(3, 7)):
    """(generators, refinement counts) of the batched workload."""
    import ug_gb300 as G
    rng = np.random.default_rng(seed)
    nrefs = [int(L) for L in rng.integers(levels[0], levels[1] + 1, size=count)]
    gens = [G.Generator(G.Generator.POISSON2D, L, seed=seed + k, corr=BATCH_CORR, var=BATCH_VAR)
            for k, L in enumerate(nrefs)]
    return gens, nrefs
