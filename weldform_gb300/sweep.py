"""Batched parameter sweep against the same specimens run one at a time.

    python -m weldform_gb300.sweep [--specimens 256] [--steps 500] [--sequential 32]
                                   [--precision 1] [--autotune]

Builds `--specimens` seeded specimens (radius 4-12 mm, L/D 1-2, dx = 0.5 mm,
Johnson-Cook constants within +-20 %, punch speed 0.5-5 m/s) into one domain
and times `--steps` steps of all of them together; then times the first
`--sequential` specimens each in its own domain for the same steps and
extrapolates the one-at-a-time cost to the whole sweep by particle count.
Prints one JSON line: aggregate particle-steps/s of both ways and the ratio,
plus the relative L2 difference of the displacement of specimen 0 between the
two runs.
"""
import argparse
import json
import time

import numpy as np

from . import Domain, PRECISION_MIXED
from . import batch


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--specimens", type=int, default=256)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--sequential", type=int, default=32)
    ap.add_argument("--precision", type=int, default=PRECISION_MIXED)
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--dx", type=float, default=0.0005)
    a = ap.parse_args()
    specs = batch.random_specimens(a.specimens)

    d = Domain()
    d.set("precision", a.precision)
    t0 = time.perf_counter()
    sw = batch.build_sweep(d, specs, dx=a.dx)
    d.prepare(sw.dt)
    setup = time.perf_counter() - t0
    block = d.autotune(3) if a.autotune else 256
    d.step(2)
    ms, launches = d.step_timed(a.steps)
    together = sw.n * a.steps / (ms * 1e-3)
    a0, b0 = sw.ranges[0]
    u_together = d.get_array("Displacement")[a0:b0]
    d.close()

    seq_ms, seq_particles = 0.0, 0
    u_alone = None
    for k, s in enumerate(specs[: a.sequential]):
        e = Domain()
        e.set("precision", a.precision)
        one = batch.build_single(e, s, k, dx=a.dx)
        e.prepare(one.dt)
        ms1, _ = e.step_timed(a.steps + 2)
        seq_ms += ms1 * a.steps / (a.steps + 2)
        seq_particles += one.n
        if k == 0:
            u_alone = e.get_array("Displacement")
        e.close()
    alone = seq_particles * a.steps / (seq_ms * 1e-3)
    du = float(np.linalg.norm(u_together - u_alone) / max(np.linalg.norm(u_alone), 1e-300))
    print(json.dumps({
        "specimens": a.specimens, "particles": sw.n, "steps": a.steps, "precision": a.precision,
        "gather_block": block, "setup_s": setup,
        "batched_particle_steps_per_s": together, "batched_ms_per_step": ms / a.steps, "launches": launches,
        "sequential_specimens_timed": a.sequential, "sequential_particle_steps_per_s": alone,
        "batched_over_sequential": together / alone,
        "specimen0_displacement_rel_l2_batched_vs_alone": du}))


if __name__ == "__main__":
    main()
