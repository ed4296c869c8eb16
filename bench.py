"""Throughput of the GB300 kick-drift SPH step (particle-steps/s) at ~1M particles.

Workload (one "step" = one kick-drift step of the whole domain): elastoplastic
cylinder upsetting, R = 10 mm, L = 30 mm, dx = 0.2112 mm (982,072 particles),
h = 1.2 dx cubic spline, steel E = 200 GPa, bilinear sigma_y = 300 MPa,
Et = 1.5 GPa, bottom two layers fixed, top two layers at -1 m/s, Monaghan
viscosity alpha = 1, dt = 0.4 h / Cs, seeded +-1e-3 dx position jitter.  The
state (~1 GB) is far larger than the 129 MB L2, so no flush is needed between
steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

The default arm runs the CUDA library; ``--impl reference`` times the CPU
restatement of the reference's OpenMP structure (per-thread pair lists and the
Nishimura gather, built from oracle/) on all host cores, on the same workload.
N > 1 runs N independent replicas (the path does not shard across GPUs).

Measurement modes (each prints its own output instead of the bench line):

    python bench.py --config-table
        every synthetic configuration on both GPU forms and the CPU restatement
    python bench.py --case [--n 250000] [--steps 3] [--precision 0|1] [--v-top -1]
                    [--kernels] [--gather-block B] [--particle-block B] [--gather-lanes L]
        a fixed-size run of the bench cylinder scaled to about n particles, for
        ncu captures and per-kernel CUDA-event times (--kernels)
    python bench.py --accuracy [--steps 1000] [--dx-mm 0.3353,0.2112,0.1331]
                    [--v-top -1] [--contact]
        the mixed form against the plain FP64 form from the same start
    python bench.py --pipe-rates
        FP64/FP32 arithmetic and copy rates of the GPU (roofline ceilings)
    python bench.py --sweep [--specimens 256] [--steps 500] [--precision 1] [--autotune]
        the batched parameter sweep (uneven specimens in one domain, each with
        its own rebuild schedule) against every specimen run alone
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "particle-steps/s @1M: mixed vs FP64 on GB300 at ≤1e-4 err; adjoint/fwd time"
R, L = 0.010, 0.030
DX_1M = 0.2112e-3

# Compulsory HBM bytes per particle of each gather kernel (fields read once
# per pass, state read + written once, 4-byte neighbour index per entry and a
# 4-byte row length), at each form's storage widths: FP64 state; the mixed
# form's gathers read FP32 float-float shadows (x, v: 24 B each) and FP32
# Sigma/rho^2, m, rho, h.  The comment of each entry names its fields.
ALG_BYTES = {
    "k_accel": lambda nnz: 144 + 4 * nnz + 4,             # x,v,rho,m,h,Sigma(6) -> a
    "k_density_drift": lambda nnz: 272 + 4 * nnz + 4,     # x,v,a,rho,m,h -> v,rho ; x,v,a -> x,v
    "k_rate_stress": lambda nnz: 456 + 4 * nnz + 4,       # x,v,rho,m,h,p,tau,eps,eps_p,pl,sy -> tau,Sigma,..,dkin,dint
    "k_accel_mx": lambda nnz: 96 + 4 * nnz + 4,           # four f32 groups (ff x, v; Sigma/rho^2; m/rho), f64 rho -> a
    "k_density_drift_mx": lambda nnz: 336 + 4 * nnz + 4,  # f64 integration; next-step record written
    "k_rate_mx": lambda nnz: 72 + 4 * nnz + 4,            # next record -> 9 rates, dkin, conduction
    "k_stress_mx": lambda nnz: 440,                       # f64 stress state read + written
    # the two above in one kernel: the nine f32 rates are neither stored nor reloaded (2 x 36 B)
    "k_rate_stress_mx": lambda nnz: 72 + 4 * nnz + 4 + 440 - 72,
}
# FP64 operations per neighbour entry / per particle (plain form).
ALG_FLOPS = {"k_accel": (95, 10), "k_density_drift": (40, 20), "k_rate_stress": (70, 270)}
# The step kernels of each form: their algorithmic bytes summed give the
# step's compulsory traffic per particle-step (state read and written once
# per pass, neighbour re-reads from cache, 4 B per row entry per gather).
STEP_KERNELS = {"mixed": ("k_accel_mx", "k_density_drift_mx", "k_rate_mx", "k_stress_mx"),
                "mixed_fused": ("k_accel_mx", "k_density_drift_mx", "k_rate_stress_mx"),
                "fp64": ("k_accel", "k_density_drift", "k_rate_stress")}
# FP64 fused multiply-add rate of the GB300 (`python bench.py --pipe-rates`:
# 503 G FMA/s), the plain form's secondary ceiling.
FP64_PEAK_TFLOPS = 1.006


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            j = json.load(open(p))
            return float(j["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms in a thread."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.rows.append([c.strip() for c in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.05)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in self.rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in self.rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


V_TOP = -1.0          # the literal configuration: elastic, no rebuild after the first step
V_TOP_YIELD = -20.0   # the yielding variant: plastic from the first steps, rebuilds every 5 steps


def build_domain(dom, dx=DX_1M, v_top=V_TOP):
    from weldform_gb300 import configs
    return configs.cylinder_upsetting(dom, R=R, L=L, dx=dx, v_top=v_top)


def _workload(n, precision, v_top=V_TOP):
    return {"workload": f"cylinder upsetting R=10mm L=30mm dx={DX_1M * 1e3:.4f}mm N={n}, bilinear steel, "
                        f"v_top={v_top:g} m/s, alpha=1, dt=0.4h/Cs",
            "particles": n, "form": precision, "l2": "state > 129 MB L2 (no flush needed)",
            "parallelism": "replicas"}


def time_form(wfmod, precision, steps, warmup, gpu, v_top=V_TOP):
    """Headline timing of one precision form: graph-replayed steps between CUDA events."""
    d = wfmod.Domain()
    d.set("device", gpu)
    d.set("precision", precision)
    case = build_domain(d, v_top=v_top)
    d.prepare(case.dt)
    d.step(max(warmup, 3))
    ms, launches = d.step_timed(steps)
    nnz = 2.0 * d.geti("pair_count") / case.n
    return d, case, ms, launches, nnz


def roofline(d, case, nnz, steps, peak_gbs, peak_kind):
    prof = d.profile_steps(max(2, min(steps, 10)))
    kernels = {k: v for k, v in prof.items() if k in ALG_BYTES}
    tot = sum(v[0] for v in prof.values())
    top = max(kernels.items(), key=lambda kv: kv[1][0])
    name, (ms_tot, cnt) = top
    ms = ms_tot / cnt
    alg = ALG_BYTES[name](nnz) * case.n
    achieved = alg / (ms * 1e-3) / 1e9
    per_nb, per_p = ALG_FLOPS.get(name, (0, 0))
    flops = (per_nb * nnz + per_p) * case.n
    shares = {k: round(v[0] / tot, 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])[:8]}
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic_per_launch.txt")
    if os.path.exists(tp):
        for line in open(tp):
            parts = line.split()
            if len(parts) >= 2 and parts[0] == name:
                try:
                    traffic = float(parts[1]) * case.n
                except ValueError:
                    pass
    return {"kernel": name, "bound": "hbm", "achieved": round(achieved, 2), "peak": peak_gbs, "unit": "GB/s",
            "frac": round(achieved / peak_gbs, 4), "peak_source": peak_kind, "traffic": traffic,
            "alg_bytes_per_launch": alg, "ms_per_launch": round(ms, 4),
            "fp64_tflops": round(flops / (ms * 1e-3) / 1e12, 4) if flops else None,
            "kernel_time_shares": shares}


def step_roofline(form, nnz, particle_steps_per_s, peak_gbs, fused=False):
    """The whole step against HBM: the step kernels' algorithmic bytes per
    particle-step times the particle-steps/s; for the plain form also the
    algorithmic FP64 flops against the FP64 pipe.  fused: the mixed step runs
    the rate gather and the stress update as one kernel."""
    ks = STEP_KERNELS["fp64" if form == "fp64" else ("mixed_fused" if fused else "mixed")]
    b = sum(ALG_BYTES[k](nnz) for k in ks)
    gbs = b * particle_steps_per_s / 1e9
    out = {"bytes_per_particle_step": round(b, 1), "achieved_gbs": round(gbs, 1), "frac_hbm": round(gbs / peak_gbs, 4)}
    if form == "fp64":
        fl = sum(ALG_FLOPS[k][0] * nnz + ALG_FLOPS[k][1] for k in ks)
        tf = fl * particle_steps_per_s / 1e12
        out.update({"flops_per_particle_step": round(fl), "fp64_tflops": round(tf, 3),
                    "frac_fp64": round(tf / FP64_PEAK_TFLOPS, 4)})
    return out


E2E_OUT_EVERY = 20


def e2e(wfmod, precision, steps, gpu, pinned):
    """Through the C ABI with host buffers, the way a caller of the solve uses
    it: x and v uploaded from pinned host memory, then K steps with x and Sigma
    read back into pinned host memory every E2E_OUT_EVERY steps (and after the
    last).  20 steps is the dense end of the reference inputs' output
    intervals (1e-6 s at ~5.7e-8 s steps in the impact input; up to ~2000
    steps in the compression inputs), so the read-back cost per step does not
    shrink with K.  The reads are the asynchronous form
    (wf_get_particle_array_f64_async): each output is snapshotted on the
    device between steps and copied to the host while the next steps run;
    the timed region ends after wf_synchronize, with every copy landed."""
    d = wfmod.Domain()
    d.set("device", gpu)
    d.set("precision", precision)
    case = build_domain(d)
    d.prepare(case.dt)
    d.step(3)
    x = pinned(d.get_array("x"))
    v = pinned(d.get_array("v"))
    xo = pinned(np.empty_like(x))
    so = pinned(d.get_array("Sigma"))
    reads = 0
    t0 = time.perf_counter()
    d.set_array("x", x)
    d.set_array("v", v)
    done = 0
    while done < steps:
        k = min(E2E_OUT_EVERY, steps - done)
        d.step(k)
        done += k
        d.get_array_async("x", xo)
        d.get_array_async("Sigma", so)
        reads += 1
    d.synchronize()
    el = time.perf_counter() - t0
    h2d = (x.nbytes + v.nbytes) / steps
    d2h = reads * (xo.nbytes + so.nbytes) / steps
    d.close()
    return {"value": case.n * steps / el, "unit": "particle-steps/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "output_every": E2E_OUT_EVERY}


def cpu_baseline(steps=2):
    """The reference-structured CPU restatement on all host threads, 1M workload."""
    import ctypes
    import __graft_entry__ as ge
    import weldform_gb300 as wf
    path = os.path.join(ge.ORACLE_BUILD, "libwf_oracle.so")
    if not os.path.exists(path):
        ge.build_oracle()
    lib = wf.bind(ctypes.CDLL(path), "wfo_")
    threads = os.cpu_count() or 1
    d = wf.Domain(lib=lib, prefix="wfo_")
    d.set("cpu_mode", 1)
    d.set("cpu_threads", threads)
    case = build_domain(d)
    d.prepare(case.dt)
    d.step(1)  # first step carries the neighbour search
    ms, _ = d.step_timed(steps)
    d.close()
    return {"value": case.n * steps / (ms * 1e-3), "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} steady kick-drift steps of the {case.n}-particle workload after the first "
                      f"(search) step, reference-structured OpenMP restatement, {threads} threads"}


def _oracle_lib():
    import ctypes
    import __graft_entry__ as ge
    import weldform_gb300 as wf
    path = os.path.join(ge.ORACLE_BUILD, "libwf_oracle.so")
    if not os.path.exists(path):
        ge.build_oracle()
    return wf.bind(ctypes.CDLL(path), "wfo_")


def config_table(gpu=0):
    """Throughput of every synthetic configuration of the path: the plain FP64
    and mixed GPU forms (CUDA-graph steps between CUDA events, after the
    first step's search) and the reference-structured CPU restatement on all
    host threads and on one thread (bounded samples of steady steps).  One
    JSON object; rows in the order of the configurations."""
    import weldform_gb300 as wfmod
    from weldform_gb300 import configs
    lib = _oracle_lib()
    threads = os.cpu_count() or 1

    def cyl(dx):
        return lambda d: configs.cylinder_upsetting(d, R=R, L=L, dx=dx, v_top=-1.0)

    def contact(d):
        return configs.contact_upsetting(d, R=R, L=L, dx=0.2e-3, v_punch=-1.0, stiffness="area")

    # (name, builder, GPU FP64 steps, GPU mixed steps, CPU all-thread steps, CPU one-thread steps)
    rows_in = [
        ("1: elastoplastic cylinder dx=1mm, bilinear", cyl(1e-3), 1000, 1000, 200, 20),
        ("2: JC + conduction + penalty-contact plane (0.1E/h) dx=0.2mm, mu=0.2", contact, 50, 200, 2, 1),
        ("3: cylinder dx=0.3353mm", cyl(0.3353e-3), 50, 200, 4, 1),
        ("3: cylinder dx=0.2112mm", cyl(0.2112e-3), 20, 100, 2, 1),
        ("3: cylinder dx=0.1331mm", cyl(0.1331e-3), 10, 50, 1, 0),
    ]
    out = []
    for name, build, s64, smx, scpu, s1 in rows_in:
        row = {"config": name}
        for form, prec, steps in (("gpu_fp64", wfmod.PRECISION_FP64, s64), ("gpu_mixed", wfmod.PRECISION_MIXED, smx)):
            d = wfmod.Domain()
            d.set("device", gpu)
            d.set("precision", prec)
            case = build(d)
            d.prepare(case.dt)
            d.step(3)
            ms, _ = d.step_timed(steps)
            row["particles"] = case.n
            row[form] = {"particle_steps_s": case.n * steps / (ms * 1e-3), "ms_per_step": ms / steps,
                         "steps": steps}
            d.close()
        for form, nthr, steps in (("cpu_all_threads", threads, scpu), ("cpu_one_thread", 1, s1)):
            if steps <= 0:
                continue
            d = wfmod.Domain(lib=lib, prefix="wfo_")
            d.set("cpu_mode", 1)
            d.set("cpu_threads", nthr)
            case = build(d)
            d.prepare(case.dt)
            d.step(1)
            ms, _ = d.step_timed(steps)
            row[form] = {"particle_steps_s": case.n * steps / (ms * 1e-3), "ms_per_step": ms / steps,
                         "steps": steps, "threads": nthr}
            d.close()
        row["mixed_over_fp64"] = row["gpu_mixed"]["particle_steps_s"] / row["gpu_fp64"]["particle_steps_s"]
        out.append(row)
        print(json.dumps(row), file=sys.stderr, flush=True)
    return {"table": out, "cpu_kind": "port (reference-structured OpenMP restatement)", "cpu_threads": threads}


def adjoint_leg(wfmod, steps=400, every=10, k=20):
    """Reaction-force adjoint on the 53,352-particle penalty-contact workload
    (R = 10 mm, L = 30 mm, dx = 0.55 mm, JC + conduction + plastic heating,
    rigid plane at -20 m/s, friction 0.2, PFAC = 0.1 E / h), 400 steps, loss
    over 40 samples against the curve of JC constants perturbed by N(0, 5%):
    wall time of the adjoint (forward with checkpoints, reverse sweep) over a
    plain FP64 forward run of the same steps (CUDA graph)."""
    from weldform_gb300 import adjoint as adj
    case = adj.ContactCase()
    target = adj.perturbed_jc_target(case, steps, every)
    d = wfmod.Domain()
    mesh = adj.build(d, case, case.nominal())
    d.prepare(case.dt)
    d.checkpoint_save(0)
    d.step(1)
    d.checkpoint_restore(0)
    fwd_ms, _ = d.step_timed(steps)
    d.checkpoint_restore(0)
    r = d.adjoint_reaction_loss(steps, every, target, mesh=mesh, checkpoint_every=k)
    n = d.particle_count
    d.close()
    return {"workload": "penalty-contact cylinder R=10mm L=30mm dx=0.55mm, JC+thermal, plane -20 m/s",
            "particles": n, "steps": steps, "samples": steps // every, "checkpoint_every": k, "form": "fp64",
            "forward_ms": fwd_ms, "adjoint_forward_ms": r["fwd_ms"], "reverse_ms": r["adj_ms"],
            "adjoint_over_forward": r["adj_ms"] / fwd_ms,
            "gradient_over_forward": (r["fwd_ms"] + r["adj_ms"]) / fwd_ms,
            "loss": r["loss"], "grad": dict(zip(wfmod.PARAMS, r["grad"].tolist()))}


# ---------------------------------------------------------------- measurement modes
def case_mode(a):
    """A fixed-size run of the bench cylinder (R = 10 mm, L = 30 mm, dx chosen
    for about --n particles) for profilers: prepares, runs --steps steps and
    prints the particle count and the step time; --kernels adds per-kernel
    CUDA-event times of the same number of steps.  --timed times the steps
    as the bench does (3 untimed steps, then CUDA events around the graph
    replays) and adds the full and filtered search counts of the timed span;
    --nb-skin sets the search reuse's skin before the prologue."""
    import weldform_gb300 as wfmod
    from weldform_gb300 import configs
    dx = configs.dx_for_count(R, L, a.n)
    d = wfmod.Domain()
    d.set("precision", a.precision)
    case = configs.cylinder_upsetting(d, R=R, L=L, dx=dx, v_top=a.v_top)
    if a.nb_skin is not None:
        d.set("nb_skin", a.nb_skin)
    d.prepare(case.dt)
    if a.fuse_rate_stress is not None:
        d.set("fuse_rate_stress", a.fuse_rate_stress)
    if a.timed:
        d.step(3)
        s0, f0 = d.geti("nb_searches"), d.geti("nb_full_searches")
        ms, launches = d.step_timed(a.steps)
        print(f"n={case.n} fuse={d.geti('fuse_rate_stress')} nb_skin={a.nb_skin} skin_reuse={d.geti('skin_reuse')} steps={a.steps} "
              f"ms/step={ms / max(a.steps, 1):.4f} launches={launches} "
              f"searches={d.geti('nb_searches') - s0} full={d.geti('nb_full_searches') - f0} "
              f"max_pl={d.get('max_pl_strain'):.3e}")
        d.close()
        return
    if a.gather_block is not None:
        d.set("gather_block", a.gather_block)
    if a.particle_block is not None:
        d.set("particle_block", a.particle_block)
    if a.gather_lanes is not None:
        d.set("gather_lanes", a.gather_lanes)
    if a.fuse_rate_stress is not None:
        d.set("fuse_rate_stress", a.fuse_rate_stress)
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


def accuracy_mode(a):
    """The mixed form against the plain FP64 form (itself within 1e-9 of the
    CPU oracle in the parity tests) from the same start after --steps steps,
    at each --dx-mm: one JSON line per size with the relative L2 errors of
    displacement, stress, plastic strain and density.  --contact runs the
    penalty-contact workload (JC, conduction, plastic heating, area penalty
    0.1 E / h, friction 0.2; dx = 0.2 mm gives 1,150,200 particles) pressed at
    --v-top and adds the reaction-force curve (every steps / 10 steps) and the
    temperature rise."""
    import weldform_gb300 as wfmod
    from weldform_gb300 import configs
    fields = ("Displacement", "Sigma", "pl_strain", "Density")
    dxs = a.dx_mm if a.dx_mm else ("0.2" if a.contact else "0.3353,0.2112,0.1331")

    def run(prec, dx):
        d = wfmod.Domain()
        d.set("precision", prec)
        if a.contact:
            case = configs.contact_upsetting(d, R=R, L=L, dx=dx, v_punch=a.v_top, stiffness="area")
        else:
            case = configs.cylinder_upsetting(d, R=R, L=L, dx=dx, v_top=a.v_top)
        d.prepare(case.dt)
        every = max(a.steps // 10, 1)
        fz = []
        t = time.perf_counter()
        for _ in range(a.steps // every):
            d.step(every)
            if a.contact:
                fz.append(d.contact_force(case.mesh)[2])
        d.step(a.steps - every * (a.steps // every))
        out = {f: d.get_array(f) for f in fields}
        out["s"] = time.perf_counter() - t
        out["n"] = case.n
        if a.contact:
            out["reaction_force"] = np.array(fz)
            out["T_rise"] = d.get_array("T") - configs.Steel().T0
        d.close()
        return out

    def rel(x, y):
        ny = np.linalg.norm(y)
        return float(np.linalg.norm(x - y) / ny) if ny > 0 else float(np.linalg.norm(x - y))

    for dx in [float(v) * 1e-3 for v in dxs.split(",")]:
        m = run(wfmod.PRECISION_MIXED, dx)
        f = run(wfmod.PRECISION_FP64, dx)
        keys = fields + (("reaction_force", "T_rise") if a.contact else ())
        print(json.dumps({"particles": m["n"], "dx_mm": dx * 1e3, "steps": a.steps, "v_top": a.v_top,
                          "contact": a.contact, "max_pl_strain": float(f["pl_strain"].max()),
                          "mixed_vs_fp64": {k: rel(m[k], f[k]) for k in keys},
                          "seconds": {"mixed": m["s"], "fp64": f["s"]}}), flush=True)


PIPE_RATES_CU = r"""
// Arithmetic and copy rates: FP64 and FP32 fused multiply-add, FP64 divide
// and square root, FP64 -> FP32 conversion, device-to-device copy.  Every
// loop is bounded and every buffer is written in range.
#include <cstdio>
#include <cuda_runtime.h>
#define ITERS 2048
__global__ void k_dfma(double* out, double a, double b) {
  double x[8];
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-9 + k;
  for (int i = 0; i < ITERS; ++i)
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  double s = 0; for (int k = 0; k < 8; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_ffma(float* out, float a, float b) {
  float x[8];
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-9f + k;
  for (int i = 0; i < ITERS; ++i)
    for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], a, b);
  float s = 0; for (int k = 0; k < 8; ++k) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void k_ddiv(double* out, double a) {
  double x[4];
  for (int k = 0; k < 4; ++k) x[k] = threadIdx.x + 1.5 + k;
  for (int i = 0; i < ITERS / 8; ++i)
    for (int k = 0; k < 4; ++k) x[k] = a / x[k] + 1.0;
  out[blockIdx.x * blockDim.x + threadIdx.x] = x[0] + x[1] + x[2] + x[3];
}
__global__ void k_dsqrt(double* out) {
  double x[4];
  for (int k = 0; k < 4; ++k) x[k] = threadIdx.x + 1.5 + k;
  for (int i = 0; i < ITERS / 8; ++i)
    for (int k = 0; k < 4; ++k) x[k] = sqrt(x[k]) + 1.0;
  out[blockIdx.x * blockDim.x + threadIdx.x] = x[0] + x[1] + x[2] + x[3];
}
__global__ void k_d2f(float* out, double a) {
  double x0 = threadIdx.x * 1e-3;
  float s0 = 0, s1 = 0, s2 = 0, s3 = 0;
  for (int i = 0; i < ITERS; ++i) {
    x0 += a;
    s0 += (float)x0; s1 += (float)(x0 * 2.0); s2 += (float)(x0 * 3.0); s3 += (float)(x0 * 5.0);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = s0 + s1 + s2 + s3;
}
__global__ void k_copy(const double4* __restrict__ a, double4* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) b[i] = a[i];
}
int main() {
  int nsm = 0; cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0);
  int clk = 0; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, 0);
  int blocks = nsm * 8, threads = 256;
  size_t nthreads = (size_t)blocks * threads;
  double* dout; float* fout;
  if (cudaMalloc(&dout, nthreads * sizeof(double)) != cudaSuccess) return 1;
  if (cudaMalloc(&fout, nthreads * sizeof(float)) != cudaSuccess) return 1;
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  float ms;
  auto timeit = [&](const char* name, double ops_per_thread, auto launch) {
    for (int w = 0; w < 3; ++w) launch();
    cudaEventRecord(e0);
    for (int r = 0; r < 5; ++r) launch();
    cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    printf("%-8s %10.3f Gop/s  (%.3f ms/launch)\n", name, ops_per_thread * nthreads * 5 / (ms * 1e-3) / 1e9, ms / 5);
  };
  timeit("dfma", 8.0 * ITERS, [&] { k_dfma<<<blocks, threads>>>(dout, 0.999999, 1e-7); });
  timeit("ffma", 8.0 * ITERS, [&] { k_ffma<<<blocks, threads>>>(fout, 0.999999f, 1e-7f); });
  timeit("ddiv", 4.0 * ITERS / 8, [&] { k_ddiv<<<blocks, threads>>>(dout, 3.0); });
  timeit("dsqrt", 4.0 * ITERS / 8, [&] { k_dsqrt<<<blocks, threads>>>(dout); });
  timeit("d2f", 4.0 * ITERS, [&] { k_d2f<<<blocks, threads>>>(fout, 1e-3); });
  size_t n4 = (size_t)1 << 27;  // 4 GiB per buffer of 32-byte elements
  double4 *a = nullptr, *b = nullptr;
  if (cudaMalloc(&a, n4 * 32) == cudaSuccess && cudaMalloc(&b, n4 * 32) == cudaSuccess) {
    cudaMemset(a, 0, n4 * 32);
    for (int w = 0; w < 3; ++w) k_copy<<<nsm * 4, 512>>>(a, b, n4);
    cudaEventRecord(e0);
    for (int r = 0; r < 5; ++r) k_copy<<<nsm * 4, 512>>>(a, b, n4);
    cudaEventRecord(e1); cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    printf("copy     %10.1f GB/s\n", 2.0 * n4 * 32 * 5 / (ms * 1e-3) / 1e9);
  }
  printf("SMs %d clock %d kHz; err=%s\n", nsm, clk, cudaGetErrorString(cudaDeviceSynchronize()));
  return 0;
}
"""


def pipe_rates_mode():
    """Compiles PIPE_RATES_CU for sm_103a in a temporary directory and runs it."""
    nvcc = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
    with tempfile.TemporaryDirectory() as tmp:
        src, exe = os.path.join(tmp, "rates.cu"), os.path.join(tmp, "rates")
        with open(src, "w") as f:
            f.write(PIPE_RATES_CU)
        subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", exe, src], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
        sys.stdout.write(r.stdout)
        sys.stderr.write(r.stderr)
        if r.returncode:
            sys.exit(r.returncode)


def sweep_mode(a):
    """Seeded specimens (radius 4-12 mm, L/D 1-2, dx = 0.5 mm, JC constants
    within +-20 %, punch speed 0.5-5 m/s) stepped together in one batched
    domain, then every specimen alone in its own domain for the same steps
    (CUDA-graph steps between CUDA events after 2 warm-up steps in both).
    One JSON line: aggregate particle-steps/s of both ways, their ratio, the
    per-specimen search counts compared with the solo runs', and specimen 0's
    displacement difference between the two."""
    import weldform_gb300 as wfmod
    from weldform_gb300 import batch
    specs = batch.random_specimens(a.specimens)
    d = wfmod.Domain()
    d.set("precision", a.precision)
    t0 = time.perf_counter()
    sw = batch.build_sweep(d, specs, dx=0.0005)
    d.prepare(sw.dt)
    setup = time.perf_counter() - t0
    block = d.autotune(3) if a.autotune else d.geti("gather_block")
    lanes = d.geti("gather_lanes")
    d.step(2)
    s0, f0 = d.geti("nb_searches"), d.geti("nb_full_searches")
    ms, launches = d.step_timed(a.steps)
    together = sw.n * a.steps / (ms * 1e-3)
    dom_searches, dom_full = d.geti("nb_searches") - s0, d.geti("nb_full_searches") - f0
    layout = {"uniform_layout": d.geti("uniform_layout"), "skin_reuse": d.geti("skin_reuse")}
    a0, b0 = sw.ranges[0]
    u_together = d.get_array("Displacement")[a0:b0]
    searches = [d.batch_get(k, "nb_searches") for k in range(len(specs))]
    # per-kernel event timing over 20 more (instrumented) steps: ms per step
    prof = d.profile_steps(20)
    layout["kernel_ms_per_step"] = {k: round(v[0] / 20, 3) for k, v in
                                    sorted(prof.items(), key=lambda kv: -kv[1][0])[:12]}
    d.close()
    seq_ms, seq_particles, solo_searches, u_alone = 0.0, 0, [], None
    t1 = time.perf_counter()
    for k, s in enumerate(specs):
        e = wfmod.Domain()
        e.set("precision", a.precision)
        one = batch.build_single(e, s, k, dx=0.0005)
        e.prepare(one.dt)
        e.step(2)
        ms1, _ = e.step_timed(a.steps)
        seq_ms += ms1
        seq_particles += one.n
        solo_searches.append(e.geti("nb_searches"))
        if k == 0:
            u_alone = e.get_array("Displacement")
        e.close()
    alone = seq_particles * a.steps / (seq_ms * 1e-3)
    du = float(np.linalg.norm(u_together - u_alone) / max(np.linalg.norm(u_alone), 1e-300))
    print(json.dumps({
        "specimens": len(specs), "particles": sw.n, "steps": a.steps, "precision": a.precision,
        "gather_block": block, "gather_lanes": lanes, "setup_s": setup,
        "batched_particle_steps_per_s": together, "batched_ms_per_step": ms / a.steps, "launches": launches,
        "batched_steps_with_a_search": dom_searches, "batched_full_searches": dom_full, **layout,
        "sequential_specimens_timed": len(specs), "sequential_particle_steps_per_s": alone,
        "sequential_wall_s": time.perf_counter() - t1,
        "batched_over_sequential": together / alone,
        "search_counts_equal_solo": searches == solo_searches,
        "searches_min_max": [min(searches), max(searches)],
        "specimen0_displacement_rel_l2_batched_vs_alone": du}))


def dist_setup(n):
    rank = _env_int("RANK", 0)
    world = _env_int("WORLD_SIZE", 1)
    local = _env_int("LOCAL_RANK", 0)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return rank, world, local, pg


def reduce_max(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def barrier(pg):
    if pg is not None:
        pg.barrier()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--config-table", action="store_true",
                    help="time every configuration (GPU forms and CPU restatement) and print one JSON table")
    ap.add_argument("--case", action="store_true", help="fixed-size run for profilers (see --n, --kernels)")
    ap.add_argument("--accuracy", action="store_true", help="mixed form against the plain FP64 form")
    ap.add_argument("--pipe-rates", action="store_true", help="arithmetic and copy rates of the GPU")
    ap.add_argument("--n", type=int, default=250000, help="--case: particle count")
    ap.add_argument("--precision", type=int, default=None,
                    help="--case (default 0) / --sweep (default 1): 0 plain FP64, 1 mixed")
    ap.add_argument("--v-top", type=float, default=-1.0, help="--case/--accuracy: top or punch velocity (m/s)")
    ap.add_argument("--kernels", action="store_true", help="--case: per-kernel CUDA-event times")
    ap.add_argument("--gather-block", type=int, default=None, help="--case: threads per mixed gather block")
    ap.add_argument("--particle-block", type=int, default=None, help="--case: threads per per-particle block")
    ap.add_argument("--gather-lanes", type=int, default=None, help="--case: lanes per particle, acceleration gather")
    ap.add_argument("--nb-skin", type=float, default=None,
                    help="--case: Verlet skin of the search reuse, relative to the pair radius (0: off)")
    ap.add_argument("--fuse-rate-stress", type=int, default=None, choices=[0, 1],
                    help="--case: mixed form's rate gather and stress update in one kernel (default 1)")
    ap.add_argument("--timed", action="store_true",
                    help="--case: 3 untimed steps, then --steps steps between CUDA events")
    ap.add_argument("--dx-mm", default=None, help="--accuracy: lattice spacings (mm, comma-separated)")
    ap.add_argument("--contact", action="store_true", help="--accuracy: penalty-contact workload")
    ap.add_argument("--sweep", action="store_true", help="batched sweep against every specimen alone")
    ap.add_argument("--specimens", type=int, default=256, help="--sweep: specimens")
    ap.add_argument("--autotune", action="store_true", help="--sweep: autotune the batched domain's gathers")
    a = ap.parse_args()
    if a.config_table:
        print(json.dumps(config_table()))
        return
    if a.case:
        a.precision = 0 if a.precision is None else a.precision
        return case_mode(a)
    if a.accuracy:
        if a.steps == ap.get_default("steps"):
            a.steps = 1000
        return accuracy_mode(a)
    if a.pipe_rates:
        return pipe_rates_mode()
    if a.sweep:
        if a.steps == ap.get_default("steps"):
            a.steps = 500
        a.precision = 1 if a.precision is None else a.precision
        return sweep_mode(a)
    warmup = max(a.warmup, 3)
    rank, world, local, pg = dist_setup(a.gpus)

    if a.impl == "reference":
        if rank != 0:
            return
        import ctypes
        import __graft_entry__ as ge
        import weldform_gb300 as wf
        path = os.path.join(ge.ORACLE_BUILD, "libwf_oracle.so")
        if not os.path.exists(path):
            ge.build_oracle()
        lib = wf.bind(ctypes.CDLL(path), "wfo_")
        threads = os.cpu_count() or 1
        d = wf.Domain(lib=lib, prefix="wfo_")
        d.set("cpu_mode", 1)
        d.set("cpu_threads", threads)
        case = build_domain(d)
        d.prepare(case.dt)
        d.step(1)
        steps = max(1, min(a.steps, 10))
        wsteps = max(0, min(warmup, 2))
        d.step(wsteps)
        ms, _ = d.step_timed(steps)
        val = case.n * steps / (ms * 1e-3)
        line = {"metric": METRIC, "value": val, "unit": "particle-steps/s", "n_gpus": a.gpus, "steps": steps,
                "warmup": wsteps + 1, "ms_per_step": ms / steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
                "config": _workload(case.n, "reference OpenMP structure (CPU)"),
                "cpu_baseline": {"value": val, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                                 "sample": f"{steps} steps of the full {case.n}-particle workload"},
                "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import weldform_gb300 as wfmod
    try:
        import torch  # noqa: F811
        def pinned(arr):
            t = torch.from_numpy(np.ascontiguousarray(arr)).pin_memory()
            return t.numpy()
        have_torch_cuda = torch.cuda.is_available()
    except Exception:
        torch = None
        have_torch_cuda = False
        def pinned(arr):
            return np.ascontiguousarray(arr)

    gpu = local if world > 1 else 0
    peak, peak_kind = measured_peaks()
    try:
        wfmod.Domain().close()
    except Exception as e:
        print(json.dumps({"metric": METRIC, "error": str(e)}))
        raise
    forms = {}
    head = None
    for name, prec, vt in (("mixed", wfmod.PRECISION_MIXED, V_TOP), ("fp64", wfmod.PRECISION_FP64, V_TOP),
                           ("mixed_yielding", wfmod.PRECISION_MIXED, V_TOP_YIELD)):
        d, case, _, _, nnz = time_form(wfmod, prec, 1, warmup, gpu, v_top=vt)
        steps = a.steps
        s0, f0 = d.geti("nb_searches"), d.geti("nb_full_searches")
        barrier(pg)
        if have_torch_cuda:
            torch.cuda.synchronize()
        with ClockSampler(gpu) as clk:
            ms, launches = d.step_timed(steps)
        if have_torch_cuda:
            torch.cuda.synchronize()
        barrier(pg)
        ms_max = reduce_max(pg, ms)
        val = world * case.n * steps / (ms_max * 1e-3)
        searches = d.geti("nb_searches") - s0
        full = d.geti("nb_full_searches") - f0
        rl = roofline(d, case, nnz, steps, peak, peak_kind)
        fused = name != "fp64" and d.geti("fuse_rate_stress") == 1 and d.geti("gather_lanes") == 1
        rl["step"] = step_roofline(name, nnz, val, peak, fused)
        forms[name] = {"value": val, "ms_per_step": ms_max / steps, "steps": steps, "roofline": rl,
                       "gpu_launches": launches, "clocks": clk.summary(), "v_top": vt,
                       "rebuilds_in_timed_steps": searches, "full_searches_in_timed_steps": full}
        if name == "mixed":
            head = (case, nnz)
            xm, sm = d.get_array("Displacement"), d.get_array("Sigma")
        elif name == "fp64":
            xf, sf = d.get_array("Displacement"), d.get_array("Sigma")
        d.close()
    case, nnz = head
    mixed = forms["mixed"]
    ee = e2e(wfmod, wfmod.PRECISION_MIXED, a.steps, gpu, pinned)
    ee["value"] *= world
    line = {"metric": METRIC, "value": mixed["value"], "unit": "particle-steps/s", "n_gpus": world,
            "steps": a.steps, "warmup": warmup, "ms_per_step": mixed["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 pair sums + f64 integration (mixed form)",
            "data": "synthetic (seeded lattice jitter)", "config": _workload(case.n, "mixed FP32/FP64"),
            "gpu_launches": mixed["gpu_launches"], "clocks": mixed["clocks"], "roofline": mixed["roofline"],
            "e2e": ee, "neighbours_per_particle": round(nnz, 3),
            "forms": {k: {kk: v for kk, v in f.items() if kk not in ("clocks",)} for k, f in forms.items()},
            "mixed_over_fp64": mixed["value"] / forms["fp64"]["value"]}
    # Same steps from the same start on both forms: the mixed form's drift from
    # the plain FP64 form (itself within 1e-9 of the CPU oracle).
    if forms["fp64"]["steps"] == mixed["steps"]:
        line["mixed_vs_fp64_rel_l2"] = {
            "Displacement": float(np.linalg.norm(xm - xf) / max(np.linalg.norm(xf), 1e-300)),
            "Sigma": float(np.linalg.norm(sm - sf) / max(np.linalg.norm(sf), 1e-300))}
    if rank == 0 and not a.no_adjoint:
        line["adjoint"] = adjoint_leg(wfmod)
    if rank == 0 and not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline()
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
