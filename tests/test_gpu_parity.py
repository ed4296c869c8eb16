"""GPU (sm_103a) kick-drift path against the CPU oracle, through the C ABI.

Bar: neighbour lists bit-exact (same sets, same canonical row order);
floating-point state within 1e-9 relative L2 (the plain FP64 form's
tolerance), after the stated number of steps.
"""
import os

import numpy as np
import pytest

from tests._support import gpu_domain, oracle_domain, rel_l2
from weldform_gb300 import configs, HOLLOMON, JOHNSON_COOK

pytestmark = pytest.mark.gpu

TOL = 1e-9
THREADS = os.cpu_count() or 1


def _pair(build, steps, fields, scalars=(), **kw):
    out = {}
    for name in ("gpu", "oracle"):
        d = gpu_domain() if name == "gpu" else oracle_domain()
        if name == "oracle":
            d.set("cpu_threads", THREADS)
        case = build(d, **kw)
        d.prepare(case.dt)
        d.step(steps)
        out[name] = {f: d.get_array(f) for f in fields}
        for s in scalars:
            out[name][s] = d.get(s)
        out[name]["searches"] = d.geti("nb_searches")
        out[name]["nbr"] = d.neighbours()
        if case.mesh is not None:
            out[name]["cf"] = d.contact_force(case.mesh)
            out[name]["cp"] = d.contact_pairs()
        d.close()
    return out["gpu"], out["oracle"]


def _check(g, o, fields, scalars=(), tol=TOL):
    for f in fields:
        e = rel_l2(g[f], o[f])
        assert e <= tol, f"{f}: relative L2 {e:.3e}"
    for s in scalars:
        e = abs(g[s] - o[s]) / max(abs(o[s]), 1e-300)
        assert e <= 1e-8, f"{s}: {g[s]!r} vs {o[s]!r}"
    assert g["searches"] == o["searches"]
    assert np.array_equal(g["nbr"][0], o["nbr"][0]) and np.array_equal(g["nbr"][1], o["nbr"][1])


def test_neighbour_search_bit_exact_cylinder():
    res = {}
    for name in ("gpu", "oracle"):
        d = gpu_domain() if name == "gpu" else oracle_domain()
        case = configs.cylinder_upsetting(d, R=0.004, L=0.010, dx=0.0004)
        d.prepare(case.dt)
        d.neighbour_search()
        res[name] = (d.neighbours(), d.get_array("Nb"))
    (go, gi), gnb = res["gpu"]
    (oo, oi), onb = res["oracle"]
    assert np.array_equal(go, oo)
    assert np.array_equal(gi, oi)
    assert np.array_equal(gnb, onb)


def test_neighbour_search_reference_table():
    """The 12,144-particle case of the reference's recorded table (particle 2000)."""
    import json
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reduction_particle2000.json")))
    c = g["case"]
    d = gpu_domain()
    d.Kernel_Set(0)
    d.AddCylinderLength(1, c["V"], c["R"], c["Lz"], c["dx"] / 2.0, c["rho"], c["dx"] * c["hfac"], False)
    d.set_f64("DomMax.x", c["DomMax.x"])
    d.set_f64("DomMin.x", c["DomMin.x"])
    d.set_particles("Cs", 1000.0)
    d.prepare(1e-7)
    d.neighbour_search()
    off, idx = d.neighbours()
    p = g["particle"]
    assert list(idx[off[p]:off[p + 1]]) == sorted(g["j_greater"]) + sorted(g["j_smaller"])
    o = oracle_domain()
    o.Kernel_Set(0)
    o.AddCylinderLength(1, c["V"], c["R"], c["Lz"], c["dx"] / 2.0, c["rho"], c["dx"] * c["hfac"], False)
    o.set_f64("DomMax.x", c["DomMax.x"])
    o.set_f64("DomMin.x", c["DomMin.x"])
    o.prepare(1e-7)
    o.neighbour_search()
    oo, oi = o.neighbours()
    assert np.array_equal(off, oo) and np.array_equal(idx, oi)


@pytest.mark.parametrize("packing,random", [(1, False), (1, True), (0, False)])
def test_neighbour_search_bit_exact_box(packing, random):
    res = {}
    for name in ("gpu", "oracle"):
        d = gpu_domain() if name == "gpu" else oracle_domain()
        d.Kernel_Set(0)
        d.AddBoxLength(0, (0.0, 0.0, 0.0), 0.006, 0.005, 0.004, 0.00025, 7850.0, 0.0006, packing, 0, random, False)
        d.set_particles("Cs", 4600.0)
        d.prepare(1e-8)
        d.neighbour_search()
        res[name] = (d.get_array("x"), d.neighbours())
    assert np.array_equal(res["gpu"][0], res["oracle"][0])
    assert np.array_equal(res["gpu"][1][0], res["oracle"][1][0])
    assert np.array_equal(res["gpu"][1][1], res["oracle"][1][1])


FIELDS = ("x", "v", "Density", "Sigma", "ShearStress", "pl_strain", "Sigmay", "Strain", "Displacement")
SCALARS = ("int_energy_sum",)


def test_elastic_cylinder_steps():
    g, o = _pair(configs.cylinder_upsetting, 60, FIELDS, SCALARS, R=0.005, L=0.010, dx=0.0005)
    _check(g, o, FIELDS, SCALARS)


@pytest.mark.parametrize("precision,tol", [(0, TOL), (1, 1e-4)], ids=["fp64", "mixed"])
def test_viscosity_constants_written_after_the_prologue(precision, tol):
    """Per-particle Alpha/Beta written after prepare: the gathers leave the
    uniform-constant fast path (the step is recaptured) and match the oracle
    stepped with the same values; writing uniform values back restores it."""
    out = {}
    for name in ("gpu", "oracle"):
        d = gpu_domain() if name == "gpu" else oracle_domain()
        if name == "oracle":
            d.set("cpu_threads", THREADS)
        else:
            d.set("precision", precision)
        case = configs.cylinder_upsetting(d, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
        d.prepare(case.dt)
        d.step(5)
        n = d.particle_count
        a = np.random.default_rng(11).uniform(0.5, 1.5, n)
        d.set_array("Alpha", a)
        d.set_array("Beta", 0.5 * a)
        d.step(20)
        out[name] = {f: d.get_array(f) for f in ("Displacement", "v", "Sigma")}
        d.set_array("Alpha", np.ones(n))
        d.set_array("Beta", np.zeros(n))
        d.step(10)
        out[name]["Displacement2"] = d.get_array("Displacement")
        out[name]["Sigma2"] = d.get_array("Sigma")
        d.close()
    for f in out["oracle"]:
        e = rel_l2(out["gpu"][f], out["oracle"][f])
        assert e <= tol, (f, e)


def test_tensor_fields_read_back_as_full_rows():
    """Symmetric tensors come back as 3x3 rows equal to their transpose,
    RotationRate antisymmetric with a zero diagonal (both expanded on the
    device); StrainRate and RotationRate match the oracle, RotationRate's
    error measured against the velocity gradient's scale (its entries nearly
    cancel in the upsetting cylinder)."""
    f = ("Sigma", "ShearStress", "Strain", "StrainRate", "RotationRate")
    g, o = _pair(configs.cylinder_upsetting, 20, f, R=0.004, L=0.008, dx=0.0005)
    for k in ("Sigma", "ShearStress", "Strain", "StrainRate"):
        t = g[k].reshape(-1, 3, 3)
        assert np.array_equal(t, t.transpose(0, 2, 1)), k
    w = g["RotationRate"].reshape(-1, 3, 3)
    assert np.array_equal(w, -w.transpose(0, 2, 1))
    assert not np.any(w[:, [0, 1, 2], [0, 1, 2]])
    assert rel_l2(g["StrainRate"], o["StrainRate"]) <= TOL
    scale = np.linalg.norm(o["StrainRate"]) + np.linalg.norm(o["RotationRate"])
    assert np.linalg.norm(g["RotationRate"] - o["RotationRate"]) <= TOL * scale


def test_yielding_bilinear_with_rebuilds():
    g, o = _pair(configs.cylinder_upsetting, 80, FIELDS + ("Strain_pl", "eff_strain_rate"), SCALARS,
                 R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
    assert o["pl_strain"].max() > 1e-3 and o["searches"] > 10
    _check(g, o, FIELDS + ("Strain_pl", "eff_strain_rate"), SCALARS)


def test_johnson_cook_thermal():
    f = FIELDS + ("T", "dTdt", "q_plheat")
    g, o = _pair(configs.cylinder_upsetting, 80, f, SCALARS + ("plastic_work",), R=0.004, L=0.008, dx=0.0005,
                 v_top=-30.0, model=JOHNSON_COOK, thermal=True)
    assert o["T"].max() > 300.0
    _check(g, o, f, SCALARS + ("plastic_work",))


def test_hollomon_yielding_past_the_plateau():
    """Hollomon flow stress with plateau (Material.cpp:48-64) under yielding:
    sigma_y = sy0 on the plateau, K (eps_p + eps0)^m once eps_p + eps0 > eps1,
    recomputed in every return with the previous step's sigma_y scaling back
    (Particle.cpp:995-1011) and Ep held at its initial 0 (quirk Q1).  Most
    particles pass the plateau end within the run, with rebuilds every 5
    steps."""
    mat = configs.Steel()
    K, m = mat.hollomon
    eps0, eps1 = mat.sy0 / mat.E, (mat.sy0 / K) ** (1.0 / m)
    f = FIELDS + ("Strain_pl", "eff_strain_rate")
    g, o = _pair(configs.cylinder_upsetting, 100, f, SCALARS, R=0.004, L=0.008, dx=0.0005, v_top=-20.0,
                 model=HOLLOMON)
    past = o["pl_strain"] + eps0 > eps1
    assert past.sum() > 0.5 * len(past) and o["searches"] > 10
    assert (o["Sigmay"] > mat.sy0).sum() > 0.5 * len(past)  # on the power law, above the plateau
    _check(g, o, f, SCALARS)


@pytest.mark.parametrize("stiffness", ["wang", "area", "penalty"])
def test_rigid_plane_contact(stiffness):
    """Rigid plane closing on the top face (zero initial gap), Johnson-Cook,
    conduction + plastic heating, friction 0.2.  The x/y totals of the
    contact force carry the reference's static-friction term tgforce/Mass
    (Contact_Wang.cpp:279); z is the physical punch reaction."""
    f = FIELDS + ("T",)
    sc = ("int_energy_sum", "contact_force_sum", "ext_forces_work", "plastic_work")
    g, o = _pair(configs.contact_upsetting, 100, f + ("contforce",), sc, R=0.003, L=0.006, dx=0.0003,
                 v_punch=-10.0, stiffness=stiffness, gap=0.0)
    assert np.array_equal(g["cp"][0], o["cp"][0]) and np.array_equal(g["cp"][1], o["cp"][1])
    assert len(o["cp"][1]) > 0
    assert abs(o["cf"][2]) > 0
    assert abs(g["cf"][2] - o["cf"][2]) <= 1e-8 * abs(o["cf"][2])
    assert rel_l2(g["cf"], o["cf"]) <= 1e-8
    _check(g, o, f, sc)
    # Per-particle contact force.  The normal part is k delta with the
    # penetration delta = h - dist a small difference of lengths, so it
    # carries the positions' rounding-level differences amplified: held to
    # 1e-8, the bar of the total reaction force above.  The tangential part is
    # tgforce/Mass of the static branch, formed from du = (x + v dt +
    # a dt^2/2) - x - v_mesh dt: the rounding of x + (a displacement ~1e-8 of
    # it) leaves du_t ~1e-8 relative error by itself, so those columns are
    # held to 1e-6.
    cg, co = g["contforce"], o["contforce"]
    assert rel_l2(cg[:, 2], co[:, 2]) <= 1e-8
    assert rel_l2(cg[:, :2], co[:, :2]) <= 1e-6


@pytest.mark.parametrize("stiffness", ["wang", "area", "penalty"])
def test_sliding_contact_dynamic_friction(stiffness):
    """The plane slides along x at 5 m/s while closing at 10 m/s: the
    tangential trial force exceeds mu |F_n| on many pairs, which then take
    the dynamic-friction branch F_t = mu_d |F_n| t / |t| (Contact_Wang.cpp:
    284-290).  Both sides count those pair evaluations; the counts and the
    state must agree."""
    f = FIELDS + ("T", "contforce")
    sc = ("int_energy_sum", "contact_force_sum", "ext_forces_work", "plastic_work")
    out = {}
    for name in ("gpu", "oracle"):
        d = gpu_domain() if name == "gpu" else oracle_domain()
        if name == "oracle":
            d.set("cpu_threads", THREADS)
        case = configs.contact_upsetting(d, R=0.003, L=0.006, dx=0.0003, v_punch=-10.0, stiffness=stiffness,
                                         gap=0.0, v_slide=5.0)
        d.prepare(case.dt)
        d.step(100)
        out[name] = {k: d.get_array(k) for k in f}
        out[name].update({k: d.get(k) for k in sc})
        out[name]["dyn"] = d.geti("dynamic_friction_count")
        out[name]["cf"] = d.contact_force(case.mesh)
        d.close()
    g, o = out["gpu"], out["oracle"]
    assert o["dyn"] > 100 and g["dyn"] == o["dyn"]
    for k in FIELDS + ("T",):
        assert rel_l2(g[k], o[k]) <= TOL, k
    for k in sc:
        assert abs(g[k] - o[k]) <= 1e-8 * abs(o[k]), (k, g[k], o[k])
    assert rel_l2(g["cf"], o["cf"]) <= 1e-8
    # the sliding force's x component is the dynamic friction of the pairs
    assert abs(o["cf"][0]) > 0
    assert rel_l2(g["contforce"], o["contforce"]) <= 1e-6


def _tight_cells(d):
    """x extent of the cell grid 1e-5 below 9 cells (DomMin.x / DomMax.x):
    CellInitiate rounds the count up (quirk Q9), so cells are narrower than
    the pair radius and a pair within the radius can sit two cells apart."""
    d.set_f64("DomMin.x", -0.005)
    d.set_f64("DomMax.x", -0.005 - 0.0003 + 0.0012 * (9 - 1e-5) - 0.0003)


@pytest.mark.parametrize("grid", [None, _tight_cells], ids=["cells_cover_radius", "tight_cells"])
def test_skin_reuse_gives_the_rows_of_a_full_search(grid):
    """The Verlet-skin reuse of the search (default nb_skin 0.1): most
    rebuilds of a yielding cylinder filter the skin lists instead of
    re-sorting, the rows equal the oracle's after every kind of rebuild, and
    the per-particle state is bit-identical to a run with the reuse off (the
    particles' memory order differs, a row's summation order does not).
    With cells narrower than the pair radius the filter also tests that the
    two cells are adjacent, as the full search's stencil does."""
    f = FIELDS + ("Strain_pl",)
    runs = {}
    for skin in (0.1, 0.0):
        d = gpu_domain()
        d.set_f64("nb_skin", skin)
        if grid:
            grid(d)
        case = configs.cylinder_upsetting(d, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
        d.prepare(case.dt)
        rows = []
        for _ in range(6):
            d.step(20)
            rows.append(d.neighbours())
        runs[skin] = {k: d.get_array(k) for k in f}
        runs[skin]["rows"] = rows
        runs[skin]["searches"] = d.geti("nb_searches")
        runs[skin]["full"] = d.geti("nb_full_searches")
        runs[skin]["ie"] = d.get("int_energy_sum")
        runs[skin]["cells_x"] = d.geti("CellNo.x")
        d.close()
    on, off = runs[0.1], runs[0.0]
    if grid:
        assert on["cells_x"] == 9
    assert on["searches"] == off["searches"] > 20
    assert off["full"] == off["searches"] and on["full"] < on["searches"] // 2
    for k in f:
        assert np.array_equal(on[k], off[k]), k
    for a, b in zip(on["rows"], off["rows"]):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert abs(on["ie"] - off["ie"]) <= 1e-12 * abs(off["ie"])
    o = oracle_domain()
    o.set("cpu_threads", THREADS)
    if grid:
        grid(o)
    case = configs.cylinder_upsetting(o, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
    o.prepare(case.dt)
    o.step(120)
    oo, oi = o.neighbours()
    assert np.array_equal(on["rows"][-1][0], oo) and np.array_equal(on["rows"][-1][1], oi)
    for k in f:
        assert rel_l2(on[k], o.get_array(k)) <= TOL, k
    o.close()


def test_solve_loop_matches_reference_loop_control():
    res = {}
    for name in ("gpu", "oracle"):
        d = gpu_domain() if name == "gpu" else oracle_domain()
        case = configs.cylinder_upsetting(d, R=0.003, L=0.006, dx=0.0005)
        d.SolveDiffUpdateKickDrift(25 * case.dt, case.dt, 5 * case.dt)
        res[name] = (d.geti("steps"), d.Time, d.get_array("x"))
    assert res["gpu"][0] == res["oracle"][0]
    assert res["gpu"][1] == res["oracle"][1]
    assert rel_l2(res["gpu"][2], res["oracle"][2]) <= TOL


@pytest.mark.slow
def test_config1_full_1000_steps():
    """8,004-particle elastic cylinder, 1000 steps (the small plain-FP64 case)."""
    g, o = _pair(configs.cylinder_upsetting, 1000, FIELDS, SCALARS)
    assert g["x"].shape[0] == 8004
    _check(g, o, FIELDS, SCALARS)


def convection(dom, h_conv=1e6, T_inf=1000.0, **kw):
    """Johnson-Cook cylinder with conduction and plastic heating whose
    lateral surface (the outer lattice ring) carries a convection boundary
    condition (Thermal_BC = 1, as the JSON driver's ConvectionBC sets it,
    WeldForm.cpp:793-807) toward a hot ambient."""
    case = configs.cylinder_upsetting(dom, model=JOHNSON_COOK, thermal=True, **kw)
    x = dom.get_array("x")
    R = kw.get("R", 0.010)
    ring = (np.hypot(x[:, 0], x[:, 1]) > R - 1.5 * case.dx).astype(np.int32)
    dom.set_array("Thermal_BC", ring)
    dom.set_particles("h_conv", h_conv)
    dom.set_particles("T_inf", T_inf)
    case.info["ring"] = ring
    return case


def test_convection_heat():
    """CalcConvHeat (Thermal.cpp:339-389): q_conv of the surface ring, the
    temperature it drives and the state, against the oracle."""
    f = FIELDS + ("T", "dTdt", "q_conv")
    g, o = _pair(convection, 100, f, SCALARS, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
    assert (o["q_conv"] > 0).sum() > 100 and o["T"].max() > 301.0
    _check(g, o, f, SCALARS)


def _tensile(dom, **kw):
    """Cylinder pulled at the top (tension), tensile-instability term on
    (TI = 0.3, TIInitDist = dx, TIn = 4: the JSON driver's defaults,
    WeldForm.cpp:368, 900-901)."""
    case = configs.cylinder_upsetting(dom, **kw)
    dom.set_particles("TI", 0.3)
    dom.set_particles("TIInitDist", case.dx)
    return case


def test_tensile_instability():
    f = FIELDS + ("TIR",)
    g, o = _pair(_tensile, 100, f, SCALARS, R=0.004, L=0.008, dx=0.0005, v_top=20.0)
    assert np.abs(o["TIR"]).max() > 0
    _check(g, o, f, SCALARS)


def _leapfrog(dom, **kw):
    dom.set("integrator", 1)
    return configs.cylinder_upsetting(dom, **kw)


def _leapfrog_contact(dom, **kw):
    dom.set("integrator", 1)
    return configs.contact_upsetting(dom, **kw)


def test_leapfrog_yielding():
    """SolveDiffUpdateLeapFrog's update (SolverLeapfrog.cpp:203-291) with
    rebuilds every 5 steps once yielding."""
    f = FIELDS + ("Strain_pl",)
    g, o = _pair(_leapfrog, 80, f, SCALARS, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
    assert o["pl_strain"].max() > 1e-3
    _check(g, o, f, SCALARS)


def test_leapfrog_contact_thermal():
    f = FIELDS + ("T",)
    g, o = _pair(_leapfrog_contact, 100, f, SCALARS, R=0.003, L=0.006, dx=0.0003, v_punch=-10.0, gap=0.0,
                 stiffness="area")
    _check(g, o, f, SCALARS)
    assert abs(g["cf"][2] - o["cf"][2]) <= 1e-9 * abs(o["cf"][2])


def _grad_corr(dom, **kw):
    dom.set("gradKernelCorr", 1)
    return configs.cylinder_upsetting(dom, **kw)


def _grad_corr_leapfrog(dom, **kw):
    dom.set("gradKernelCorr", 1)
    dom.set("integrator", 1)
    return configs.cylinder_upsetting(dom, **kw)


@pytest.mark.parametrize("build", [_grad_corr, _grad_corr_leapfrog], ids=["kickdrift", "leapfrog"])
def test_kernel_gradient_correction(build):
    """gradKernelCorr with the locking sums it forces: corrected gradients in
    the acceleration, density, rate and conduction pair terms; the matrix
    recomputed per the solver's schedule (rebuilds every 5 steps here)."""
    f = FIELDS + ("gradCorrM", "T")
    g, o = _pair(build, 60, f, SCALARS, R=0.004, L=0.008, dx=0.0005, v_top=-20.0, model=JOHNSON_COOK, thermal=True)
    assert o["pl_strain"].max() > 1e-3
    _check(g, o, f, SCALARS)


def _auto_ts(vel, acc, integrator):
    def build(dom, **kw):
        dom.set("auto_ts", vel)
        dom.set("auto_ts_acc", acc)
        dom.set("integrator", integrator)
        return configs.cylinder_upsetting(dom, **kw)
    return build


@pytest.mark.parametrize("vel,acc,integrator", [(1, 0, 0), (0, 1, 0), (1, 1, 0), (1, 0, 1)],
                         ids=["velocity", "acceleration", "both", "leapfrog_velocity"])
def test_adaptive_time_step(vel, acc, integrator):
    """CheckMinTSVel / CheckMinTSAccel / AdaptiveTimeStep on the device:
    with a step above the CFL bound (cfl 0.8) the step shrinks; the state,
    the step size and Time follow the oracle."""
    f = FIELDS
    g, o = _pair(_auto_ts(vel, acc, integrator), 60, f, SCALARS + ("deltat", "Time"), R=0.004, L=0.008,
                 dx=0.0005, v_top=-20.0, cfl=0.8)
    h = 1.2 * 0.0005
    assert o["deltat"] < 0.95 * 0.8 * h / configs.Steel().Cs
    _check(g, o, f, SCALARS + ("deltat", "Time"))


def test_adaptive_time_step_with_contact_leapfrog_and_solve_loop():
    """The leapfrog solver with penalty contact and all three autoTS flags
    (its min_force_ts is the initial dt, so the contact criterion is inert),
    run through SolveDiffUpdateLeapFrog's loop control with outputs: step
    count, Time and state follow the oracle."""
    res = {}
    for name in ("gpu", "oracle"):
        d = gpu_domain() if name == "gpu" else oracle_domain()
        if name == "oracle":
            d.set("cpu_threads", THREADS)
        for k in ("auto_ts", "auto_ts_acc", "auto_ts_cont"):
            d.set(k, 1)
        d.set("integrator", 1)
        case = configs.contact_upsetting(d, R=0.003, L=0.006, dx=0.0003, v_punch=-10.0, gap=0.0, stiffness="area")
        d.SolveDiffUpdateLeapFrog(20 * case.dt, case.dt, 5 * case.dt)
        res[name] = (d.geti("steps"), d.Time, d.get("deltat"), d.get_array("x"), d.contact_force(case.mesh))
        d.close()
    g, o = res["gpu"], res["oracle"]
    assert g[0] == o[0] and g[0] > 20
    assert abs(g[1] - o[1]) <= 1e-9 * o[1] and abs(g[2] - o[2]) <= 1e-8 * o[2]
    assert rel_l2(g[3], o[3]) <= TOL
    assert abs(g[4][2] - o[4][2]) <= 1e-8 * abs(o[4][2])


def test_kickdrift_contact_time_step_is_rejected():
    from weldform_gb300 import WFError
    d = gpu_domain()
    d.set("auto_ts_cont", 1)
    case = configs.contact_upsetting(d, R=0.003, L=0.006, dx=0.0005, v_punch=-10.0)
    with pytest.raises(WFError):
        d.prepare(case.dt)
    d.close()


def test_frozen_topology_searches_once():
    """freeze_neighbours (a library option for finite-difference checks of
    the adjoint): a yielding cylinder that rebuilds its rows every 5 steps
    searches only at the first step, keeps the first search's rows, and its
    state differs from the regular run only through the stale rows."""
    res = {}
    for freeze in (0, 1):
        d = gpu_domain()
        if freeze:
            d.set("freeze_neighbours", 1)
        case = configs.cylinder_upsetting(d, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
        d.prepare(case.dt)
        d.step(1)
        first = d.neighbours()
        d.step(59)
        res[freeze] = (d.geti("nb_searches"), first, d.neighbours(), d.get_array("Sigma"))
        d.close()
    assert res[0][0] > 2 and res[1][0] == 1
    for k in (0, 1):
        assert np.array_equal(res[1][1][k], res[1][2][k])
        assert np.array_equal(res[0][1][k], res[1][1][k])
    assert rel_l2(res[1][3], res[0][3]) < 1e-2
