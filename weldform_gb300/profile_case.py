"""A fixed-size run of the kick-drift step for profilers (ncu) and timing.

    python -m weldform_gb300.profile_case --n 250000 --steps 3 [--precision 0|1]

Builds the bench's cylinder-upsetting workload scaled to about n particles
(R = 10 mm, L = 30 mm, dx chosen for the count), prepares it and runs the
given number of steps; prints the particle count and the step time.
"""
import argparse
import time

from . import Domain
from . import configs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=250000)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--precision", type=int, default=0)
    ap.add_argument("--v-top", type=float, default=-1.0)
    ap.add_argument("--kernels", action="store_true", help="print per-kernel CUDA-event times of the steps")
    ap.add_argument("--gather-block", type=int, default=None, help="mixed gathers: threads per block")
    ap.add_argument("--particle-block", type=int, default=None, help="per-particle kernels: threads per block")
    a = ap.parse_args()
    dx = configs.dx_for_count(0.010, 0.030, a.n)
    d = Domain()
    d.set("precision", a.precision)
    case = configs.cylinder_upsetting(d, R=0.010, L=0.030, dx=dx, v_top=a.v_top)
    d.prepare(case.dt)
    if a.gather_block is not None:
        d.set("gather_block", a.gather_block)
    if a.particle_block is not None:
        d.set("particle_block", a.particle_block)
    t = time.perf_counter()
    d.step(a.steps)
    el = time.perf_counter() - t
    print(f"n={case.n} dx={dx:.6e} steps={a.steps} s/step={el / max(a.steps, 1):.4e} "
          f"searches={d.geti('nb_searches')} max_pl={d.get('max_pl_strain'):.3e}")
    if a.kernels:
        prof = d.profile_steps(a.steps)
        tot = sum(v[0] for v in prof.values())
        for k, (ms, n) in sorted(prof.items(), key=lambda kv: -kv[1][0]):
            print(f"  {k:24s} {n:4d} launches {ms:9.3f} ms  {100 * ms / tot:5.1f} %")
    d.close()


if __name__ == "__main__":
    main()
