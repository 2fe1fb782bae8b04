"""The oracle's own generator of the 3D diffusion hierarchy (oracle/cube_gen.c)
against the product's (ug_gb300/csrc/meshgen.cpp): bitwise the same levels,
transfers, coordinates and right-hand side.  The CPU reference arm of
bench.py builds its workload with the oracle's generator, so it loads no
ug_gb300 library; the second test runs that arm (on a smaller hierarchy) and
checks exactly that, the complete solves it times and its config."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("ug_rules", [False, True], ids=["freudenthal", "ug_red_rules"])
@pytest.mark.parametrize("nref,var,seed", [(2, 1.0, 7), (3, 1.0, 2026), (3, 0.0, 12), (4, 0.5, 5)])
def test_oracle_generator_equals_product_generator(oracle_mod, nref, var, seed, ug_rules):
    import ug_gb300 as G
    levels, rhs, xyz = oracle_mod.cube_levels(nref, seed, 0.1, var, threads=3, ug_rules=ug_rules)
    kind = G.Generator.DIFFUSION3D_UG if ug_rules else G.Generator.DIFFUSION3D
    gen = G.Generator(kind, nref, seed=seed, corr=0.1, var=var)
    assert gen.nlevels == len(levels) == nref + 1
    for l in range(nref + 1):
        g, o = gen.level(l), levels[l]
        keys = ["rowptr", "col", "val", "vclass", "vnclass", "skip"] + (["prowptr", "pcol", "pw"] if l else [])
        for k in keys:
            assert np.array_equal(np.asarray(g[k]), o[k]), (l, k)
        assert np.array_equal(np.asarray(g["xyz"]).reshape(-1, 3), xyz[l])
    assert np.array_equal(gen.rhs, rhs)


def test_reference_arm_loads_only_the_oracle():
    code = (
        "import sys, json\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '2', '--warmup', '1']\n"
        "import bench\n"
        "bench.NREF = 3\n"
        "bench.main()\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'ug_lib': 'libug_gb300' in maps, 'oracle_lib': 'liblmgc_oracle' in maps,\n"
        "                  'modules': sorted(m for m in sys.modules if m.startswith('ug_gb300'))}))\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    line, probe = lines[0], lines[1]
    assert not probe["ug_lib"] and probe["oracle_lib"] and probe["modules"] == []
    sys.path.insert(0, ROOT)
    import bench
    nref = bench.NREF
    try:
        bench.NREF = 3
        assert line["impl"] == "reference" and line["config"] == bench.workload_config()
    finally:
        bench.NREF = nref
    assert line["steps"] == 2 and line["warmup"] == 1 and line["iterations"] > 0
    assert line["final_rel_defect"] < 1e-8
    assert line["value"] == pytest.approx(line["cpu_baseline"]["cores"] / (line["ms_per_step"] * 1e-3))
