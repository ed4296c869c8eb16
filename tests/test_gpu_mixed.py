"""Mixed FP32/FP64 form against the FP64 oracle, through the C ABI.

Bar: relative L2 error <= 1e-4 in stress and reaction force
after the stated steps; the same bound is applied to displacement, plastic
strain, density and temperature.  Neighbour lists stay bit-exact (the search
is shared with the plain form and runs on FP64 positions).
"""
import os

import numpy as np
import pytest

from tests._support import gpu_domain, oracle_domain, rel_l2
from weldform_gb300 import configs, HOLLOMON, JOHNSON_COOK, PRECISION_MIXED

pytestmark = pytest.mark.gpu

TOL = 1e-4
THREADS = os.cpu_count() or 1


def _run(build, steps, fields, scalars=(), **kw):
    out = {}
    for name in ("mixed", "oracle"):
        d = gpu_domain() if name == "mixed" else oracle_domain()
        if name == "mixed":
            d.set("precision", PRECISION_MIXED)
        else:
            d.set("cpu_threads", THREADS)
        case = build(d, **kw)
        d.prepare(case.dt)
        d.step(steps)
        out[name] = {f: d.get_array(f) for f in fields}
        for s in scalars:
            out[name][s] = d.get(s)
        out[name]["nbr"] = d.neighbours()
        if case.mesh is not None:
            out[name]["cf"] = d.contact_force(case.mesh)
        d.close()
    return out["mixed"], out["oracle"]


def _check(m, o, fields, tol=TOL):
    errs = {f: rel_l2(m[f], o[f]) for f in fields}
    for f, e in errs.items():
        assert e <= tol, f"{f}: relative L2 {e:.3e} (all: {errs})"
    return errs


FIELDS = ("Displacement", "Sigma", "Density", "v")


def test_mixed_elastic_config1_1000_steps():
    m, o = _run(configs.cylinder_upsetting, 1000, FIELDS, ("int_energy_sum",))
    _check(m, o, FIELDS)
    assert abs(m["int_energy_sum"] - o["int_energy_sum"]) <= TOL * abs(o["int_energy_sum"])
    assert np.array_equal(m["nbr"][1], o["nbr"][1])


def test_mixed_yielding_bilinear():
    f = FIELDS + ("pl_strain", "Strain_pl")
    m, o = _run(configs.cylinder_upsetting, 200, f, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
    assert o["pl_strain"].max() > 1e-2
    _check(m, o, f)


def test_mixed_johnson_cook_thermal():
    f = FIELDS + ("pl_strain", "T")
    m, o = _run(configs.cylinder_upsetting, 200, f, ("plastic_work",), R=0.004, L=0.008, dx=0.0005, v_top=-30.0,
                model=JOHNSON_COOK, thermal=True)
    _check(m, o, f + ())
    dT_m = m["T"] - 300.0
    dT_o = o["T"] - 300.0
    assert rel_l2(dT_m, dT_o) <= TOL
    assert abs(m["plastic_work"] - o["plastic_work"]) <= TOL * abs(o["plastic_work"])


def test_mixed_contact_reaction_force():
    f = FIELDS + ("pl_strain",)
    m, o = _run(configs.contact_upsetting, 150, f, ("contact_force_sum",), R=0.003, L=0.006, dx=0.0003,
                v_punch=-10.0, gap=0.0)
    assert abs(o["cf"][2]) > 0
    assert abs(m["cf"][2] - o["cf"][2]) <= TOL * abs(o["cf"][2])
    _check(m, o, f)


def test_mixed_hollomon_yielding():
    """Hollomon with plateau past its end (Material.cpp:48-64): the mixed
    form's return evaluates K (eps_p + eps0)^m in FP32."""
    f = FIELDS + ("pl_strain", "Sigmay")
    m, o = _run(configs.cylinder_upsetting, 200, f, R=0.004, L=0.008, dx=0.0005, v_top=-20.0, model=HOLLOMON)
    assert o["pl_strain"].max() > 1e-2
    _check(m, o, f)


@pytest.mark.parametrize("stiffness,v_slide", [("penalty", 0.0), ("penalty", 5.0), ("wang", 5.0)],
                         ids=["penalty", "penalty_sliding", "wang_sliding"])
def test_mixed_contact_laws_and_sliding(stiffness, v_slide):
    """The Fraser law kij = PFAC cont_stiff (Contact.cpp:423) and a plane
    sliding along x, whose pairs take the dynamic-friction branch: the
    reaction force and the state within the mixed form's bound."""
    f = FIELDS + ("pl_strain", "T")
    m, o = _run(configs.contact_upsetting, 150, f, ("contact_force_sum",), R=0.003, L=0.006, dx=0.0003,
                v_punch=-10.0, gap=0.0, stiffness=stiffness, v_slide=v_slide)
    assert abs(o["cf"][2]) > 0
    assert abs(m["cf"][2] - o["cf"][2]) <= TOL * abs(o["cf"][2])
    if v_slide:
        assert abs(m["cf"][0] - o["cf"][0]) <= TOL * abs(o["cf"][0])
    _check(m, o, f)


@pytest.mark.parametrize("V", [(1.0, 1.0, 1.0), (-3.0, 0.5, 10.0)], ids=["1m", "10m"])
def test_mixed_domain_away_from_the_origin(V):
    """The yielding cylinder placed with its base centre at V (metres).  The
    mixed form forms x_i - x_j from float-float position records held
    relative to the cell grid's centre, so its accuracy does not depend on
    where the domain sits; displacement (not absolute position) and stress
    stay within the bound."""
    f = FIELDS + ("pl_strain",)
    m, o = _run(configs.cylinder_upsetting, 200, f, R=0.004, L=0.008, dx=0.0005, v_top=-20.0, V=V)
    assert o["pl_strain"].max() > 1e-2
    errs = _check(m, o, f)
    # the same case at the origin, for scale: the offset costs nothing
    m0, o0 = _run(configs.cylinder_upsetting, 200, f, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
    errs0 = _check(m0, o0, f)
    for k in ("Displacement", "Sigma"):
        assert errs[k] <= 3.0 * errs0[k] + 1e-7, (k, errs[k], errs0[k])


def test_mixed_convection_heat():
    from tests.test_gpu_parity import convection
    f = FIELDS + ("pl_strain", "T", "q_conv")
    m, o = _run(convection, 200, f, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
    _check(m, o, f)
    assert rel_l2(m["T"] - 300.0, o["T"] - 300.0) <= TOL


@pytest.mark.slow
def test_mixed_250k_1000_steps_against_oracle():
    """The 240,300-particle configuration of the mixed-precision study
    (dx = 0.3353 mm) after 1000 steps, against the FP64 oracle."""
    m, o = _run(configs.cylinder_upsetting, 1000, FIELDS, ("int_energy_sum",), dx=0.3353e-3)
    assert m["v"].shape[0] == 240300
    errs = _check(m, o, FIELDS)
    print("mixed vs oracle, 240300 particles, 1000 steps:", errs)


def test_mixed_tensile_instability():
    from tests.test_gpu_parity import _tensile
    m, o = _run(_tensile, 100, FIELDS, R=0.004, L=0.008, dx=0.0005, v_top=20.0)
    _check(m, o, FIELDS)


def test_mixed_leapfrog():
    from tests.test_gpu_parity import _leapfrog
    f = FIELDS + ("pl_strain",)
    m, o = _run(_leapfrog, 200, f, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
    _check(m, o, f)


def test_mixed_gather_block_sizes_agree_bitwise():
    """Every gather block size computes each particle's sums in the same
    order, so a yielding JC + thermal + contact run is bit-identical across
    them (which block handles a particle does not matter)."""
    res = []
    for block in (256, 64, 128, 512):
        d = gpu_domain()
        d.set("precision", PRECISION_MIXED)
        case = configs.contact_upsetting(d, R=0.003, L=0.006, dx=0.0003, v_punch=-10.0, gap=0.0)
        d.prepare(case.dt)
        d.set("gather_block", block)
        assert d.geti("gather_block") == block
        d.step(60)
        res.append({f: d.get_array(f) for f in ("x", "v", "Sigma", "pl_strain", "T")})
        d.close()
    for r in res[1:]:
        for f in r:
            assert np.array_equal(r[f], res[0][f]), f


@pytest.mark.parametrize("workload", ["wang_contact", "bilinear_yielding", "hollomon_grad_corr"])
def test_fused_rate_stress_kernel_is_bit_identical(workload):
    """The fused rate-stress kernel (the rates kept in registers) against
    k_rate_mx followed by k_stress_mx: same sums in the same order, same
    update, same block partials, so every field and every reduced scalar
    agrees bit for bit after a yielding run.  One lane per particle is forced
    and the thermal solver is off (the fused kernel serves that launch shape
    only); the workloads take contact with friction, the plain bilinear
    return and the corrected-gradient variant with Hollomon hardening."""
    fields = ("x", "v", "Sigma", "pl_strain", "T", "Density", "StrainRate", "RotationRate",
              "dint_energy_dt", "dkin_energy_dt", "Sigmay", "q_plheat")
    res = []
    for fuse in (0, 1):
        d = gpu_domain()
        d.set("precision", PRECISION_MIXED)
        if workload == "wang_contact":
            case = configs.contact_upsetting(d, R=0.003, L=0.006, dx=0.0003, v_punch=-10.0, gap=0.0,
                                             thermal=False)
        elif workload == "bilinear_yielding":
            case = configs.cylinder_upsetting(d, R=0.003, L=0.006, dx=0.0003, v_top=-20.0)
        else:
            case = configs.cylinder_upsetting(d, R=0.003, L=0.006, dx=0.0003, v_top=-20.0, model=HOLLOMON)
            d.set("gradKernelCorr", 1)
        d.prepare(case.dt)
        d.set("gather_lanes", 1)
        d.set("fuse_rate_stress", fuse)
        assert d.geti("fuse_rate_stress") == fuse
        d.step(60)
        out = {f: d.get_array(f) for f in fields}
        for k in ("int_energy_sum", "kin_energy_sum", "max_pl_strain", "Time"):
            out[k] = d.get(k)
        out["searches"] = d.geti("nb_searches")
        res.append(out)
        d.close()
    if workload != "wang_contact":
        assert res[0]["max_pl_strain"] > 0.0
    for f in res[0]:
        assert np.array_equal(res[0][f], res[1][f]), f


def test_mixed_particles_of_different_mass_and_smoothing_length():
    """Masses spread by +-5 % and two smoothing lengths: the gathers read
    the five-group records (h, mass and Cs per particle) instead of the
    uniform-particle layout, and stay within the bound; writing uniform
    masses and h back after the prologue switches to the uniform layout
    mid-run, still within the bound."""
    f = FIELDS + ("pl_strain",)

    def build(d, **kw):
        case = configs.cylinder_upsetting(d, **kw)
        n = d.particle_count
        rng = np.random.default_rng(5)
        d.set_array("Mass", d.get_array("Mass") * (1.0 + 0.05 * rng.uniform(-1, 1, n)))
        h = d.get_array("h")
        h[::7] *= 1.02
        d.set_array("h", h)
        return case
    m, o = _run(build, 100, f, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
    _check(m, o, f)
    out = {}
    for name in ("mixed", "oracle"):
        d = gpu_domain() if name == "mixed" else oracle_domain()
        if name == "mixed":
            d.set("precision", PRECISION_MIXED)
        case = build(d, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
        d.prepare(case.dt)
        d.step(20)
        n = d.particle_count
        d.set_array("Mass", np.full(n, d.get_array("Mass").mean()))
        d.set_array("h", np.full(n, 1.2 * 0.0005))
        d.step(40)
        out[name] = {k: d.get_array(k) for k in f}
        d.close()
    _check(out["mixed"], out["oracle"], f)


@pytest.mark.parametrize("lanes", [2, 4, 8])
def test_mixed_acceleration_gather_lanes(lanes):
    """The acceleration, density and rate gathers with `lanes` lanes per
    particle (per-lane Kahan sums combined in FP64 by warp shuffles): within
    the bound against the oracle, and bit-identical across block sizes at a
    fixed lane count."""
    f = FIELDS + ("pl_strain",)

    def build(d, **kw):
        d.set("gather_lanes", lanes)
        return configs.cylinder_upsetting(d, **kw)
    m, o = _run(build, 100, f, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
    _check(m, o, f)
    res = []
    for gb in (64, 256, 512):
        d = gpu_domain()
        d.set("precision", PRECISION_MIXED)
        d.set("gather_lanes", lanes)
        d.set("gather_block", gb)
        case = configs.cylinder_upsetting(d, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
        d.prepare(case.dt)
        d.step(30)
        res.append(np.concatenate([d.get_array(f).ravel() for f in ("a", "Density", "Sigma")]))
        d.close()
    for r in res[1:]:
        assert np.array_equal(r, res[0])


@pytest.mark.parametrize("integrator", [0, 1], ids=["kickdrift", "leapfrog"])
def test_mixed_kernel_gradient_correction(integrator):
    """gradKernelCorr in the mixed form: corrected FP32 gradients in the
    acceleration, density (locking form), rate and conduction gathers, the
    matrix formed in FP64 on the solver's schedule."""
    from tests.test_gpu_parity import _grad_corr, _grad_corr_leapfrog
    build = _grad_corr if integrator == 0 else _grad_corr_leapfrog
    f = FIELDS + ("pl_strain", "T")
    m, o = _run(build, 200, f, R=0.004, L=0.008, dx=0.0005, v_top=-20.0, model=JOHNSON_COOK, thermal=True)
    assert o["pl_strain"].max() > 1e-2
    _check(m, o, f)


def test_mixed_adaptive_time_step():
    """Velocity-criterion adaptive step in the mixed form: the step, Time and
    state stay within the mixed form's bar of the oracle."""
    from tests.test_gpu_parity import _auto_ts
    f = FIELDS + ("pl_strain",)
    m, o = _run(_auto_ts(1, 0, 0), 200, f, ("deltat", "Time"), R=0.004, L=0.008, dx=0.0005, v_top=-20.0, cfl=0.8)
    _check(m, o, f)
    assert abs(m["deltat"] - o["deltat"]) <= TOL * o["deltat"]
    assert abs(m["Time"] - o["Time"]) <= TOL * o["Time"]


def test_mixed_staged_acceleration_gather():
    """The shared-memory staged acceleration gather (two threads per
    particle, even and odd row entries, sums added in FP64) on a yielding
    JC + thermal + contact run with several searches, each rebuilding the
    block halos: bit-identical for every halo capacity (a block over the
    capacity runs the same split on global memory), and within FP32
    summation-order differences of the one-thread gather."""
    res = []
    for stage, cap in ((0, 896), (1, 896), (1, 400), (1, 64)):
        d = gpu_domain()
        d.set("precision", PRECISION_MIXED)
        d.set("gather_staging", stage)
        d.set("stage_cap", cap)
        case = configs.contact_upsetting(d, R=0.003, L=0.006, dx=0.0003, v_punch=-10.0, gap=0.0)
        d.prepare(case.dt)
        assert d.geti("gather_staging") == stage and d.geti("stage_cap") == cap
        d.step(60)
        assert d.geti("nb_searches") > 1
        names = d.profile_steps(2)
        assert ("k_accel_mx_staged" in names) == bool(stage), names
        res.append({f: d.get_array(f) for f in ("Displacement", "v", "Sigma", "pl_strain", "T")})
        d.close()
    for r in res[2:]:
        for f in r:
            assert np.array_equal(r[f], res[1][f]), f
    for f in res[0]:
        assert rel_l2(res[1][f], res[0][f]) <= 1e-5, f
