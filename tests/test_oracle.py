"""CPU checks of the oracle and the host-side helpers (no GPU)."""
import numpy as np
import pytest

from tests._support import oracle_domain, rel_l2
from weldform_gb300 import configs


def test_cylinder_count_matches_generator():
    for R, L, dx in ((0.010, 0.030, 0.001), (0.004, 0.008, 0.0005), (0.003, 0.006, 0.0003)):
        d = oracle_domain()
        d.AddCylinderLength(0, (0, 0, 0), R, L, dx / 2, 7850.0, 1.2 * dx, False)
        assert d.particle_count == configs.cylinder_count(R, L, dx)
    # 276 particles per layer x 29 layers at dx = 1 mm (the 30th layer is lost to
    # the accumulated zp += 2r, Domain.cpp:749-752)
    assert configs.cylinder_count(0.010, 0.030, 0.001) == 8004


def test_jitter_is_deterministic_and_bounded():
    a = configs.jitter(1000, 0.001)
    b = configs.jitter(1000, 0.001)
    assert np.array_equal(a, b)
    assert np.abs(a).max() <= 1e-6 and np.abs(a).max() > 0.9e-6
    assert not np.array_equal(a, configs.jitter(1000, 0.001, seed=1))


def _run(mode, steps, **kw):
    d = oracle_domain()
    d.set("cpu_mode", mode)
    d.set("cpu_threads", 4)
    case = configs.cylinder_upsetting(d, **kw)
    d.prepare(case.dt)
    d.step(steps)
    return {f: d.get_array(f) for f in ("x", "Sigma", "pl_strain", "Density")}, d


def test_reference_structured_mode_agrees_with_canonical_mode():
    """Per-thread pair lists + Nishimura gather (the timed CPU baseline) against
    the canonical gather: only the summation order differs."""
    kw = dict(R=0.003, L=0.006, dx=0.0005, v_top=-20.0)
    a, _ = _run(0, 40, **kw)
    b, _ = _run(1, 40, **kw)
    assert a["pl_strain"].max() > 0
    for f in a:
        assert rel_l2(b[f], a[f]) < 1e-9, f


@pytest.mark.parametrize("stiffness,ti", [("wang", 0.3), ("area", 0.0)])
def test_reference_structured_mode_agrees_on_contact_and_heat(stiffness, ti):
    """The same agreement on the configuration-2 physics the CPU baseline also
    times: a rigid plane pressing at 20 m/s and sliding at 5 m/s on a
    Johnson-Cook cylinder with conduction and plastic heating (80 steps,
    plastic strain to 4e-2, dynamic friction reached), with the tensile-
    instability term on for the Wang law.  The search schedule and the
    dynamic-friction count are equal; the contact force agrees to the
    rounding of the penalty force it sums."""
    out = []
    for mode in (0, 1):
        d = oracle_domain()
        d.set("cpu_mode", mode)
        d.set("cpu_threads", 4)
        case = configs.contact_upsetting(d, R=0.003, L=0.006, dx=0.0005, v_punch=-20.0, stiffness=stiffness,
                                         v_slide=5.0)
        d.set_particles("TI", ti)
        d.prepare(case.dt)
        d.step(80)
        r = {f: d.get_array(f) for f in ("x", "Sigma", "pl_strain", "Density", "T")}
        r["F"] = d.contact_force(case.mesh)
        r["counts"] = (d.geti("nb_searches"), d.geti("dynamic_friction_count"))
        out.append(r)
        d.close()
    a, b = out
    assert a["pl_strain"].max() > 1e-2 and a["counts"][1] > 0 and np.ptp(a["T"]) > 1.0
    assert a["counts"] == b["counts"]
    for f in ("x", "Sigma", "pl_strain", "Density", "T"):
        assert rel_l2(b[f], a[f]) < 1e-9, f
    assert rel_l2(b["F"], a["F"]) < 1e-9


def test_kinetic_energy_rate_cancels_pairwise():
    """CalcKinEnergyEqn adds +temp / -temp to the two particles of every pair
    (Domain.cpp:1775-1791), so its global sum is zero up to rounding."""
    _, d = _run(0, 20, R=0.003, L=0.006, dx=0.0005, v_top=-5.0)
    assert abs(d.get("kin_energy_sum")) < 1e-9 * max(abs(d.get("int_energy_sum")), 1e-12)


def test_yield_triggers_rebuild_schedule():
    """First yield searches at once; afterwards every ts_nb_inc = 5 steps."""
    _, d = _run(0, 30, R=0.003, L=0.006, dx=0.0005, v_top=-20.0)
    n = d.geti("nb_searches")
    assert 5 <= n <= 8


def test_unsupported_features_are_rejected():
    d = oracle_domain()
    d.AddCylinderLength(0, (0, 0, 0), 0.003, 0.006, 0.00025, 7850.0, 0.0006, False)
    d.set_particles("PresEq", 1)
    with pytest.raises(Exception):
        d.prepare(1e-8)


def test_tensile_instability_stress_is_the_positive_spectral_part():
    """StartAcceleration's TIR (Domain.cpp:1557-1569) from the stress at the
    start of the step: -TI/rho^2 times the positive spectral part of Sigma,
    checked against numpy's symmetric eigen-decomposition."""
    d = oracle_domain()
    d.AddCylinderLength(0, (0, 0, 0), 0.002, 0.004, 0.00025, 7850.0, 0.0006, False)
    n = d.particle_count
    rng = np.random.default_rng(7)
    A = rng.normal(size=(n, 3, 3)) * 1e8
    S = A + A.transpose(0, 2, 1)
    S[::3] = np.diag([2e8, -1e8, 3e8])         # diagonal and
    S[1::5] = np.diag([1e8, 1e8, -2e8])        # repeated eigenvalues
    d.set_array("Sigma", S.reshape(n, 9))
    d.set_particles("G", 76.9e9)
    d.set_particles("Cs", 4607.8)
    d.set_particles("TI", 0.3)
    d.prepare(1e-9)
    d.step(1)
    tir = d.get_array("TIR").reshape(n, 3, 3)
    w, V = np.linalg.eigh(S)
    f = np.where(w > 0, -0.3 * w / 7850.0 ** 2, 0.0)
    ref = np.einsum("nij,nj,nkj->nik", V, f, V)
    assert np.abs(tir - ref).max() <= 1e-12 * np.abs(ref).max()


def test_leapfrog_first_step_matches_kickdrift_half_kick():
    """Both integrators start from v(1/2) = v(0) + a(0) dt/2; afterwards the
    leapfrog keeps velocities at half steps, so the states part."""
    out = {}
    for integ in (0, 1):
        d = oracle_domain()
        d.set("integrator", integ)
        case = configs.cylinder_upsetting(d, R=0.003, L=0.006, dx=0.0005, v_top=-5.0)
        d.prepare(case.dt)
        d.step(1)
        x1 = d.get_array("x")
        d.step(10)
        out[integ] = (x1, d.get_array("x"), d.get_array("v"))
        d.close()
    assert rel_l2(out[1][0], out[0][0]) <= 1e-15  # x(1) = x(0) + dt v(1/2) in both
    assert rel_l2(out[1][2], out[0][2]) > 1e-6    # v(n+1/2) against v(n+1)


@pytest.mark.parametrize("integrator", [0, 1], ids=["kickdrift", "leapfrog"])
def test_update_order_of_each_solver(integrator):
    """One step of a free, yielding cylinder, from the step's own a:
    kick-drift kicks by a dt/2 before the drift and again after it with the
    same acceleration (SolverKickDrift.cpp:226-227, 254-263), so
    x' = x + (v + a dt/2) dt and v' = v + a dt/2 + a dt/2; leapfrog kicks the
    half-step velocity by a (dt_prev + dt)/2 = a dt and drifts with it
    (SolverLeapfrog.cpp:269, 296-301).
    Bit for bit, with Displacement advancing by the same du as x."""
    from weldform_gb300 import BILINEAR
    dx, h = 0.0005, 0.0006
    d = oracle_domain()
    d.set("integrator", integrator)
    mat = configs.Steel()
    d.Kernel_Set(0)
    d.AddCylinderLength(0, (0.0, 0.0, 0.0), 0.003, 0.006, dx / 2, mat.rho, h, False)
    x = d.get_array("x") + configs.jitter(d.particle_count, dx)
    d.set_array("x", x)
    configs._material_setup(d, mat, BILINEAR)
    d.set_array("v", 50.0 * np.random.default_rng(3).standard_normal(x.shape))
    dt = 0.4 * h / mat.Cs
    d.prepare(dt)
    d.step(3)
    x0, v0, u0 = d.get_array("x"), d.get_array("v"), d.get_array("Displacement")
    d.step(1)
    a, x1, v1, u1 = d.get_array("a"), d.get_array("x"), d.get_array("v"), d.get_array("Displacement")
    d.close()
    if integrator == 0:
        vh = v0 + a * (0.5 * dt)
        xe, ve = x0 + vh * dt, vh + a * (dt / 2.0)
    else:
        ve = v0 + a * dt
        xe = x0 + ve * dt
    assert np.array_equal(x1, xe) and np.array_equal(v1, ve)
    assert np.abs((u1 - u0) - (x1 - x0)).max() <= 1e-12 * np.abs(x1 - x0).max()


@pytest.mark.parametrize("integrator", [0, 1], ids=["kickdrift", "leapfrog"])
def test_velocity_bc_zones_move_as_prescribed(integrator):
    """UserAcc (WeldForm.cpp:51-120) at its call sites: after every step the
    particles of a BC zone carry exactly the prescribed velocity and zero
    acceleration, and moved by that velocity times dt.  A constant BC holds
    v = value; an amplitude BC holds amp_factor * amplitude(t) * value at the
    step's start time t, since Time advances at the end of the step
    (SolverKickDrift.cpp:299, SolverLeapfrog.cpp:331)."""
    d = oracle_domain()
    d.set("integrator", integrator)
    case = configs.cylinder_upsetting(d, R=0.003, L=0.006, dx=0.0005, v_top=-20.0)
    d.add_amplitude(7, [0.0, 1e-5], [0.0, 1.0])
    d.AssignZone((-1.0, -1.0, 0.0025), (1.0, 1.0, 0.0035), 4)
    d.add_velocity_bc(4, (3.0, 0.0, 0.0), value_type=1, amp_id=7, amp_factor=2.0)
    ids = d.get_array("ID")
    assert all((ids == z).sum() > 100 for z in (2, 3, 4))
    d.prepare(case.dt)
    for _ in range(5):
        x0, t0 = d.get_array("x"), d.Time
        d.step(1)
        x1, v, a = d.get_array("x"), d.get_array("v"), d.get_array("a")
        for zone, value in ((2, (0.0, 0.0, 0.0)), (3, (0.0, 0.0, -20.0)), (4, (2.0 * 3.0 * t0 / 1e-5, 0.0, 0.0))):
            m = ids == zone
            assert np.abs(v[m] - value).max() <= 1e-15 * max(1.0, abs(max(value, key=abs))), zone
            assert np.abs(a[m]).max() == 0.0, zone
            assert np.abs((x1 - x0)[m] - np.asarray(value) * case.dt).max() <= 1e-15, zone
    assert d.Time > 4 * case.dt
    d.close()


def test_rigid_plane_moves_as_its_bc_prescribes():
    """The plane's zone BC sets the mesh velocity m_v (WeldForm.cpp:51-120),
    and TriMesh::Update (Mesh.cpp:82-293) moves its particles by m_v dt each
    step: exactly, while contact with friction runs under it."""
    d = oracle_domain()
    case = configs.contact_upsetting(d, R=0.003, L=0.006, dx=0.0005, v_punch=-20.0, v_slide=5.0)
    plane = d.get_array("ID") == 10
    assert plane.sum() > 100
    d.prepare(case.dt)
    for _ in range(4):
        x0 = d.get_array("x")
        d.step(1)
        x1, v = d.get_array("x"), d.get_array("v")
        assert np.abs(v[plane] - (5.0, 0.0, -20.0)).max() == 0.0
        assert np.abs((x1 - x0)[plane] - np.array([5.0, 0.0, -20.0]) * case.dt).max() <= 1e-15
    assert np.abs(d.contact_force(case.mesh)).max() > 0.0
    d.close()


@pytest.mark.parametrize("stiffness", ["wang", "penalty", "area"])
def test_frictionless_contact_pushes_along_the_plane_normal(stiffness):
    """With both friction coefficients 0 the friction block is skipped
    (Contact_Wang.cpp:263, `fr_sta > 0`), so every particle's contact force
    and the plane's summed force lie along the plane normal (z): their x and y
    components are exactly 0 while the plane presses ~1e4 N."""
    d = oracle_domain()
    case = configs.contact_upsetting(d, R=0.003, L=0.006, dx=0.0005, v_punch=-20.0, friction=0.0,
                                     stiffness=stiffness)
    d.prepare(case.dt)
    d.step(60)
    cf, F = d.get_array("contforce"), d.contact_force(case.mesh)
    touching = np.abs(cf).max(axis=1) > 0
    assert touching.sum() > 20 and abs(F[2]) > 1e3
    assert np.abs(cf[:, :2]).max() == 0.0 and F[0] == 0.0 and F[1] == 0.0
    assert d.geti("dynamic_friction_count") == 0
    d.close()


def test_kernel_gradient_correction_matrix():
    """CalcGradCorrMatrix (Domain.cpp:1832-1940): isotropic (c I, the same c)
    for interior particles of a regular lattice — at h = 1.2 dx the discrete
    first moment -sum_j V_j grad W_ij (x) x_ij is 1.376 I, so c = 0.727 —
    and anisotropic where the free surface truncates the neighbourhood; the
    corrected step differs from the uncorrected one."""
    out = {}
    for corr in (0, 1):
        d = oracle_domain()
        d.set("gradKernelCorr", corr)
        case = configs.cylinder_upsetting(d, R=0.003, L=0.006, dx=0.0005, v_top=-5.0, jitter_amp=0.0)
        d.prepare(case.dt)
        d.step(5)
        out[corr] = (d.get_array("gradCorrM").reshape(-1, 3, 3), d.get_array("Nb"), d.get_array("x"))
        d.close()
    M, nb, _ = out[1]
    c = M[:, 0, 0]
    aniso = np.abs(M - c[:, None, None] * np.eye(3)).max(axis=(1, 2)) / np.abs(c)
    full = nb == nb.max()
    assert aniso[full].max() < 1e-12 and np.ptp(c[full]) < 1e-12 * abs(c[full][0])
    assert 0.6 < c[full][0] < 0.8
    assert aniso[nb < 0.6 * nb.max()].min() > 0.05
    assert np.array_equal(out[0][0], np.broadcast_to(np.eye(3), out[0][0].shape))
    assert rel_l2(out[1][2], out[0][2]) > 1e-12


def test_smoothing_length_update_leaves_h_unchanged():
    """UpdateSmoothingLength (Domain.cpp:2493-2510) runs after each regular
    rebuild, but both solvers call it after StartAcceleration zeroed dDensity,
    so htent == h and h never leaves h0: a yielding run with the flag set is
    identical to one without, in both integrators."""
    import numpy as np
    from tests._support import oracle_domain
    from weldform_gb300 import configs
    for integ in (0, 1):
        out = []
        for flag in (0, 1):
            d = oracle_domain()
            d.set("integrator", integ)
            d.set("h_update", flag)
            case = configs.cylinder_upsetting(d, R=0.002, L=0.004, dx=0.0005, v_top=-20.0)
            d.prepare(case.dt)
            d.step(40)
            assert d.geti("nb_searches") > 2
            out.append((d.get_array("h"), d.get_array("x"), d.get_array("Sigma")))
            d.close()
        for a, b in zip(out[0], out[1]):
            assert np.array_equal(a, b)


def test_kickdrift_contact_time_step_is_rejected_by_the_oracle():
    """auto_ts_cont with contact in the kick-drift solver reads
    Domain::min_force_ts, which nothing on that path sets: rejected."""
    import pytest
    from tests._support import oracle_domain
    from weldform_gb300 import configs, WFError
    d = oracle_domain()
    d.set("auto_ts_cont", 1)
    case = configs.contact_upsetting(d, R=0.002, L=0.004, dx=0.0005, v_punch=-10.0)
    with pytest.raises(WFError):
        d.prepare(case.dt)
    d.close()


def test_oracle_convection_source_matches_its_formula():
    """CalcConvHeat (Thermal.cpp:339-389): after a step, a convection
    particle's q_conv equals rho h_conv (m/rho)^(2/3) (T_inf - T) / m at its
    updated density and temperature; other particles keep q_conv = 0."""
    import numpy as np
    from tests._support import oracle_domain
    from tests.test_gpu_parity import convection
    d = oracle_domain()
    case = convection(d, R=0.003, L=0.006, dx=0.0005, v_top=-5.0)
    d.prepare(case.dt)
    d.step(3)
    q, rho, m, T = (d.get_array(k) for k in ("q_conv", "Density", "Mass", "T"))
    ring = case.info["ring"].astype(bool)
    want = rho * 1e6 * (m / rho) ** (2.0 / 3.0) * (1000.0 - T) / m
    assert np.allclose(q[ring], want[ring], rtol=1e-13, atol=0)
    assert not q[~ring].any()
