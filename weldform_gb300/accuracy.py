"""Error of the mixed FP32/FP64 form against FP64 after a fixed number of steps.

    python -m weldform_gb300.accuracy [--steps 1000] [--dx-mm 0.3353,0.2112,0.1331] [--v-top -1]

For each lattice spacing (defaults: 240,300 / 982,072 / 3,939,300 particles)
the cylinder-upsetting workload (R = 10 mm, L = 30 mm) is built twice from the same start and
stepped in the mixed and in the plain FP64 form; one JSON line per size gives
the relative L2 errors of displacement, stress, equivalent plastic strain and
density.  The plain FP64 form matches the CPU restatement of the reference to
~1e-9 (the GPU parity tests), so it is the FP64 reference at sizes a CPU run
cannot reach in minutes.
"""
import argparse
import json
import time

import numpy as np

from . import Domain, PRECISION_FP64, PRECISION_MIXED
from . import configs

FIELDS = ("Displacement", "Sigma", "pl_strain", "Density")


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b))


def run(make, dx, steps, v_top):
    d = make()
    case = configs.cylinder_upsetting(d, R=0.010, L=0.030, dx=dx, v_top=v_top)
    d.prepare(case.dt)
    t = time.perf_counter()
    d.step(steps)
    el = time.perf_counter() - t
    out = {f: d.get_array(f) for f in FIELDS}
    out["n"] = case.n
    out["s"] = el
    d.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--dx-mm", default="0.3353,0.2112,0.1331")
    ap.add_argument("--v-top", type=float, default=-1.0)
    a = ap.parse_args()
    for dx in [float(s) * 1e-3 for s in a.dx_mm.split(",")]:

        def gpu(prec):
            def mk():
                d = Domain()
                d.set("precision", prec)
                return d
            return mk

        m = run(gpu(PRECISION_MIXED), dx, a.steps, a.v_top)
        f = run(gpu(PRECISION_FP64), dx, a.steps, a.v_top)
        line = {"particles": m["n"], "dx_mm": dx * 1e3, "steps": a.steps, "v_top": a.v_top,
                "max_pl_strain": float(f["pl_strain"].max()),
                "mixed_vs_fp64": {k: rel_l2(m[k], f[k]) for k in FIELDS},
                "seconds": {"mixed": m["s"], "fp64": f["s"]}}
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
