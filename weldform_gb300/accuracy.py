"""Error of the mixed FP32/FP64 form against FP64 after a fixed number of steps.

    python -m weldform_gb300.accuracy [--steps 1000] [--dx-mm 0.3353,0.2112,0.1331] [--v-top -1]
    python -m weldform_gb300.accuracy --contact [--steps 1000] [--dx-mm 0.2] [--v-top -1]

For each lattice spacing (defaults: 240,300 / 982,072 / 3,939,300 particles)
the cylinder-upsetting workload (R = 10 mm, L = 30 mm) is built twice from the same start and
stepped in the mixed and in the plain FP64 form; one JSON line per size gives
the relative L2 errors of displacement, stress, equivalent plastic strain and
density.  The plain FP64 form matches the CPU restatement of the reference to
~1e-9 (the GPU parity tests), so it is the FP64 reference at sizes a CPU run
cannot reach in minutes.

With --contact the workload is the penalty-contact cylinder (Johnson-Cook,
conduction with plastic-work heating, rigid plane with stiffness 0.1 E/h and
friction 0.2; dx = 0.2 mm gives 1,150,200 particles) pressed by the plane at
--v-top, and the line adds the relative L2 error of the plane's reaction
force F_z sampled every steps / 10 steps and of the temperature rise.
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


def run_contact(make, dx, steps, v_punch):
    d = make()
    case = configs.contact_upsetting(d, R=0.010, L=0.030, dx=dx, v_punch=v_punch, stiffness="area")
    d.prepare(case.dt)
    every = max(steps // 10, 1)
    fz = []
    t = time.perf_counter()
    for _ in range(steps // every):
        d.step(every)
        fz.append(d.contact_force(case.mesh)[2])
    el = time.perf_counter() - t
    out = {f: d.get_array(f) for f in FIELDS}
    out["T_rise"] = d.get_array("T") - configs.Steel().T0
    out["reaction_force"] = np.array(fz)
    out["n"] = case.n
    out["s"] = el
    d.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--dx-mm", default="0.3353,0.2112,0.1331")
    ap.add_argument("--v-top", type=float, default=-1.0)
    ap.add_argument("--contact", action="store_true", help="penalty-contact JC + thermal workload")
    a = ap.parse_args()
    if a.contact and a.dx_mm == ap.get_default("dx_mm"):
        a.dx_mm = "0.2"
    for dx in [float(s) * 1e-3 for s in a.dx_mm.split(",")]:

        def gpu(prec):
            def mk():
                d = Domain()
                d.set("precision", prec)
                return d
            return mk

        go = run_contact if a.contact else run
        m = go(gpu(PRECISION_MIXED), dx, a.steps, a.v_top)
        f = go(gpu(PRECISION_FP64), dx, a.steps, a.v_top)
        keys = FIELDS + (("reaction_force", "T_rise") if a.contact else ())
        line = {"particles": m["n"], "dx_mm": dx * 1e3, "steps": a.steps, "v_top": a.v_top,
                "contact": a.contact, "max_pl_strain": float(f["pl_strain"].max()),
                "mixed_vs_fp64": {k: rel_l2(m[k], f[k]) for k in keys},
                "seconds": {"mixed": m["s"], "fp64": f["s"]}}
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
