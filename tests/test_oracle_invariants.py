"""Physical invariants of the CPU oracle's kick-drift step.

The parity tests hold the GPU forms to the oracle; these hold the oracle to
properties of the SPH equations themselves, which a misreading of the
reference's pair terms would break whatever the restatement says:

* the acceleration pair term m_i m_j (Sigma_i/rho_i^2 + Sigma_j/rho_j^2 +
  Pi_ij) GK x_ij is antisymmetric in (i, j), so with no boundary condition
  or contact the mass-weighted sum of accelerations vanishes and the total
  momentum stays put (CalcAccel, InteractionAlt.cpp:35-197);
* every pair term reads velocities only as v_ij, so a uniform velocity added
  to every particle shifts v and x and changes nothing else (Galilean
  invariance of CalcAccel, CalcDensInc and CalcRateTensors,
  InteractionAlt.cpp:12-640);
* with kernel-gradient correction (M_i = inverse of -sum_j V_j grad W_ij (x)
  x_ij, Domain.cpp:1832-1940) the corrected velocity gradient of a linear
  field v = G x is exactly G at every particle, the free surface included
  (the corrected rate sums, InteractionAlt.cpp:330-350, 425-450); without it
  the estimate is off by the lattice's first-moment error;
* conduction adds one pair value to the first particle's sum and subtracts
  it from the second's (Thermal.cpp:72-131), so sum_i rho_i cp_i dT_i/dt
  vanishes at every step; the weight m_j/rho_j of the pair's second particle
  is used at both ends, so sum_i m_i cp_i dT_i/dt vanishes only while the
  density is uniform;
* the flow stress after each step is the material law evaluated at the
  particle's plastic strain before the step, the step's effective strain
  rate and its temperature (Johnson-Cook with the rate factor cut at
  eps_0, Material.cpp:6-23; Hollomon's plateau, Material.cpp:48-64; called
  from Particle.cpp:997-1000), and the returned deviatoric stress never leaves
  the yield surface of the step before (the scale factor uses the previous
  Sigmay, Particle.cpp:995);
* an unjittered cylinder upset along z keeps the lattice's symmetries
  (mirrors x -> -x and y -> -y, the swap x <-> y): vectors and tensors at
  mirrored particles are the mirrored vectors and tensors, through yielding,
  rebuilds and contact with the plane;
* the stress rate is objective: a pre-stressed body spinning rigidly
  carries its stress round with it, dtau/dt = W tau - tau W (the Jaumann
  terms SRT + RS, Particle.cpp:968-981), which fixes the sign convention of
  RotationRate against the velocity gradient.
"""
import numpy as np
import pytest

from tests._support import oracle_domain
from weldform_gb300 import BILINEAR, HOLLOMON, JOHNSON_COOK, configs

DX = 0.0005
H = 1.2 * DX


def _run(v_of_x, steps, alpha=1.0, corr=0, fields=("x", "v", "a", "Sigma", "StrainRate", "Mass", "pl_strain")):
    """A free cylinder (R 3 mm, L 6 mm, dx 0.5 mm, 968 particles, jittered),
    bilinear steel, no BC and no contact, initial velocities v_of_x(x);
    returns the listed fields after each of `steps` steps and dt."""
    d = oracle_domain()
    d.set("gradKernelCorr", corr)
    mat = configs.Steel()
    d.Kernel_Set(0)
    d.AddCylinderLength(0, (0.0, 0.0, 0.0), 0.003, 0.006, DX / 2, mat.rho, H, False)
    n = d.particle_count
    x = d.get_array("x") + configs.jitter(n, DX)
    d.set_array("x", x)
    configs._material_setup(d, mat, BILINEAR)
    d.set_particles("Alpha", alpha)
    d.set_array("v", v_of_x(x))
    dt = 0.4 * H / mat.Cs
    d.prepare(dt)
    out = []
    for _ in range(steps):
        d.step(1)
        out.append({k: d.get_array(k) for k in fields})
    d.close()
    return out, dt


def _random_v(seed, shift=(0.0, 0.0, 0.0)):
    return lambda x: 50.0 * np.random.default_rng(seed).standard_normal(x.shape) + np.asarray(shift)


def test_free_body_conserves_linear_momentum():
    """Random velocities of 50 m/s: the body yields (plastic strain > 1e-2,
    which also triggers neighbour rebuilds), yet sum m a = 0 and sum m v stays
    at its initial value to rounding at every step."""
    res, _ = _run(_random_v(3), 20)
    m = res[0]["Mass"][:, None]
    v0 = _random_v(3)(np.zeros((len(m), 3)))
    p0 = (m * v0).sum(axis=0)
    for r in res:
        force, force_abs = (m * r["a"]).sum(axis=0), (m * np.abs(r["a"])).sum(axis=0)
        mom_abs = (m * np.abs(r["v"])).sum(axis=0)
        assert np.abs(force).max() <= 1e-14 * force_abs.max()
        assert np.abs((m * r["v"]).sum(axis=0) - p0).max() <= 1e-14 * mom_abs.max()
    assert res[-1]["pl_strain"].max() > 1e-2


def test_uniform_velocity_changes_nothing_but_v_and_x():
    """Adding u = (3, -2, 5) m/s to every initial velocity leaves a, Sigma and
    StrainRate of the fifth step unchanged to rounding; v is shifted by u and
    x by 5 dt u."""
    u = np.array([3.0, -2.0, 5.0])
    ra, dt = _run(_random_v(7), 5)
    rb, _ = _run(_random_v(7, u), 5)
    a, b = ra[-1], rb[-1]
    for k in ("a", "Sigma", "StrainRate"):
        assert np.abs(a[k] - b[k]).max() <= 1e-13 * np.abs(a[k]).max(), k
    assert np.abs((b["v"] - a["v"]) - u).max() <= 1e-12 * np.abs(u).max()
    assert np.abs((b["x"] - a["x"]) - 5 * dt * u).max() <= 1e-10 * 5 * dt * np.abs(u).max()


def test_corrected_gradient_of_a_linear_field_is_exact():
    """v = G x with no viscosity and zero initial stress: the first step's
    acceleration is 0, the drift keeps the field linear (v = G' x' with
    G' = G (I + dt G)^-1), and the step's StrainRate and RotationRate are the
    symmetric and antisymmetric parts of G' at every particle, while the
    density rate, taken before the drift, is the continuity equation
    -rho tr(G) (CalcDensInc's corrected locking sum, InteractionAlt.cpp:589-605)
    to rounding.  What remains in the rates
    comes from the density and position updates between the correction
    matrix and the rate sums (relative O(|G| dt)) and the float weights
    m_j/rho_j of the locking sums (1e-7).  Without correction interior
    particles read c G with c = 1.376, the lattice's first moment at
    h = 1.2 dx with the generator's particle volume m/rho = pi R^2 L / N
    (Domain.cpp:840-842; 1.40 dx^3 for this cylinder)."""
    G = 10.0 * np.random.default_rng(0).standard_normal((3, 3))
    tol = 20.0 * np.abs(G).max() * 0.4 * H / configs.Steel().Cs + 1e-6
    err = {}
    for corr in (0, 1):
        res, dt = _run(lambda x: x @ G.T, 1, alpha=0.0, corr=corr,
                       fields=("a", "StrainRate", "RotationRate", "dDensity", "Density"))
        r = res[0]
        assert np.abs(r["a"]).max() == 0.0
        rho0 = configs.Steel().rho
        cont = np.abs(r["dDensity"] + rho0 * np.trace(G)) / (rho0 * abs(np.trace(G)))
        if corr:  # the continuity equation, from the pre-drift state the correction matrix was built on
            assert cont.max() <= 1e-13
            assert np.abs(r["Density"] - (rho0 + dt * r["dDensity"])).max() <= 1e-15 * rho0
        else:
            assert np.median(cont) > 0.3
        Gp = G @ np.linalg.inv(np.eye(3) + dt * G)
        S, W = 0.5 * (Gp + Gp.T), 0.5 * (Gp - Gp.T)
        eS = np.abs(r["StrainRate"].reshape(-1, 3, 3) - S).max(axis=(1, 2)) / np.abs(S).max()
        eW = np.abs(r["RotationRate"].reshape(-1, 3, 3) - W).max(axis=(1, 2)) / np.abs(W).max()
        err[corr] = np.maximum(eS, eW)
    assert err[1].max() <= tol, (err[1].max(), tol)
    assert np.median(err[0]) > 0.3  # the uncorrected estimate is not exact: the check discriminates


def _heat_rates(v_of_x, steps):
    """Conduction only (no plastic heating): a cylinder with a temperature
    gradient along z and a ripple along x; returns (rho cp dTdt, m cp dTdt,
    the density's relative spread) after each step."""
    d = oracle_domain()
    mat = configs.Steel()
    d.Kernel_Set(0)
    d.AddCylinderLength(0, (0.0, 0.0, 0.0), 0.003, 0.006, DX / 2, mat.rho, H, False)
    n = d.particle_count
    x = d.get_array("x") + configs.jitter(n, DX)
    d.set_array("x", x)
    configs._material_setup(d, mat, BILINEAR)
    d.set("thermal_solver", 1)
    d.set_array("T", 300.0 + 1000.0 * x[:, 2] / 0.006 + 50.0 * np.sin(2000.0 * x[:, 0]))
    d.set_array("v", v_of_x(x))
    d.prepare(0.4 * H / mat.Cs)
    out = []
    for _ in range(steps):
        d.step(1)
        m, cp, rho, dT = (d.get_array(k) for k in ("Mass", "cp_T", "Density", "dTdt"))
        out.append((rho * cp * dT, m * cp * dT, np.ptp(rho) / rho.mean()))
    d.close()
    return out


def test_conduction_exchanges_heat_pairwise():
    """At rest (uniform density) both balances hold to rounding; with the
    random 50 m/s velocities the density spreads by a few percent and only the
    density-weighted balance still holds, the mass-weighted one drifting by
    more than 1e-6 of the exchanged heat."""
    for rq, mq, spread in _heat_rates(lambda x: np.zeros_like(x), 3):
        assert spread == 0.0
        assert abs(rq.sum()) <= 1e-14 * np.abs(rq).sum()
        assert abs(mq.sum()) <= 1e-14 * np.abs(mq).sum()
    moving = _heat_rates(_random_v(3), 6)
    for rq, _, _ in moving:
        assert abs(rq.sum()) <= 1e-14 * np.abs(rq).sum()
    rq, mq, spread = moving[-1]
    assert spread > 1e-2 and abs(mq.sum()) > 1e-6 * np.abs(mq).sum()


def _von_mises(tau):
    t = tau.reshape(-1, 3, 3)
    return np.sqrt(1.5 * np.einsum("nij,nij->n", t, t))


def test_flow_stress_follows_the_material_law():
    """A cylinder upset at 20 m/s for 40 steps (plastic strain to ~2e-2):
    Johnson-Cook at 600 K (temperature factor 0.8) and Hollomon, whose
    plateau end (plastic strain 9.3e-4) is passed by part of the particles
    while others stay on it."""
    mat = configs.Steel()
    for model in (JOHNSON_COOK, HOLLOMON):
        d = oracle_domain()
        case = configs.cylinder_upsetting(d, R=0.003, L=0.006, dx=0.0005, v_top=-20.0, model=model)
        if model == JOHNSON_COOK:
            d.set_particles("T", 600.0)
        d.prepare(case.dt)
        plateau = past = 0
        for _ in range(40):
            pl0, sy0 = d.get_array("pl_strain"), d.get_array("Sigmay")
            d.step(1)
            sy, esr, T = d.get_array("Sigmay"), d.get_array("eff_strain_rate"), d.get_array("T")
            if model == JOHNSON_COOK:
                A, B, n, C, eps_0, m, T_m, T_t = mat.jc
                f = np.where(esr > eps_0, 1.0 + C * np.log(np.maximum(esr, eps_0) / eps_0), 1.0)
                law = (A + B * pl0 ** n) * f * (1.0 - ((T - T_t) / (T_m - T_t)) ** m)
            else:
                K, m = mat.hollomon
                eps0, eps1 = mat.sy0 / mat.E, (mat.sy0 / K) ** (1.0 / m)
                on = pl0 + eps0 > eps1
                law = np.where(on, K * (pl0 + eps0) ** m, mat.sy0)
                past += int(on.sum())
                plateau += int(((pl0 > 0) & ~on).sum())
            assert np.abs(sy - law).max() <= 1e-14 * law.max()
            assert (_von_mises(d.get_array("ShearStress")) <= sy0 * (1.0 + 1e-12)).all()
        assert d.get_array("pl_strain").max() > 1e-2
        if model == HOLLOMON:
            assert past > 0 and plateau > 0
        d.close()


def test_spinning_body_carries_its_stress_round():
    """A 5,244-particle cylinder (R 5 mm, L 10 mm, no jitter) with a uniform
    deviatoric stress tau0 (106 MPa von Mises, below yield) spins rigidly,
    v = Omega x.  The unbalanced stress at the free surface accelerates the
    outer particles in the first step; particles whose neighbours and
    neighbours' neighbours were not accelerated (168 here) see only the
    spin, so their stress rate over the step is 2G dev(S') + W' tau0 -
    tau0 W' with G' = Omega (I + dt Omega)^-1 the velocity gradient at the
    drifted positions.  With correction that holds to rounding (measured
    8e-8); the opposite sign of the rotation terms is off by ~2.  Without
    correction the same particles read the lattice's first moment c times
    G', c = 1 / gradCorrM_00 of the corrected run."""
    tau0 = np.array([[60.0, 30.0, 0.0], [30.0, -20.0, 10.0], [0.0, 10.0, -40.0]]) * 1e6
    w = np.array([300.0, -500.0, 1000.0])
    Om = np.array([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]])
    mat = configs.Steel()
    rate, moment = {}, None
    for corr in (1, 0):
        d = oracle_domain()
        d.set("gradKernelCorr", corr)
        d.Kernel_Set(0)
        d.AddCylinderLength(0, (0.0, 0.0, 0.0), 0.005, 0.010, DX / 2, mat.rho, H, False)
        n = d.particle_count
        x = d.get_array("x")
        configs._material_setup(d, mat, BILINEAR)
        d.set_particles("Alpha", 0.0)
        d.set_array("v", x @ Om.T)
        d.set_array("ShearStress", np.tile(tau0.ravel(), (n, 1)))
        d.set_array("Sigma", np.tile(tau0.ravel(), (n, 1)))
        dt = 0.4 * H / mat.Cs
        d.prepare(dt)
        d.step(1)
        tau = d.get_array("ShearStress").reshape(-1, 3, 3)
        a = d.get_array("a")
        off, idx = d.neighbours()
        if corr:
            moment = 1.0 / d.get_array("gradCorrM").reshape(-1, 3, 3)[:, 0, 0]
        d.close()
        still = np.abs(a).max(axis=1) < 1e-4
        calm = still.copy()
        for _ in range(2):
            calm = np.array([calm[i] and calm[idx[off[i]:off[i + 1]]].all() for i in range(n)])
        rate[corr] = (tau - tau0) / dt
    assert 100 <= calm.sum() < n // 10
    Gp = Om @ np.linalg.inv(np.eye(3) + dt * Om)
    S, W = 0.5 * (Gp + Gp.T), 0.5 * (Gp - Gp.T)
    dev = 2.0 * mat.G * (S - np.trace(S) / 3.0 * np.eye(3))
    jaumann, opposite = dev + W @ tau0 - tau0 @ W, dev - W @ tau0 + tau0 @ W
    scale = np.abs(jaumann).max()
    err = np.abs(rate[1][calm] - jaumann).max(axis=(1, 2)) / scale
    assert err.max() <= 1e-6
    assert (np.abs(rate[1][calm] - opposite).max(axis=(1, 2)) / scale).min() > 1.0
    c = moment[calm]
    assert np.ptp(c) <= 1e-12 * c[0] and abs(c[0] - 1.0) > 0.1
    assert (np.abs(rate[0][calm] - c[:, None, None] * jaumann).max(axis=(1, 2)) / scale).max() <= 1e-6


def _mirror_partner(x, M):
    """Index of the particle at M x for every particle (-1 where none)."""
    q = np.round(x * 1e9).astype(np.int64)
    where = {tuple(p): i for i, p in enumerate(q)}
    return np.array([where.get(tuple(p), -1) for p in np.round((x @ M.T) * 1e9).astype(np.int64)])


@pytest.mark.parametrize("case_name", ["bilinear", "jc_thermal_ti_corr", "plane"])
def test_lattice_symmetries_are_kept(case_name):
    """40 steps at 20 m/s (plastic strain ~2e-2, rebuilds): v and Sigma at
    the mirror partner of every solid particle are M v and M Sigma M^T, to
    1e-12 of their largest values for the bilinear cylinder; to 1e-10 with
    Johnson-Cook, conduction and plastic heating, the tensile-instability
    term (TI = 0.3) and kernel-gradient correction, whose temperature rise
    agrees to 1e-6 of its range; and to 1e-10 under the plane (Wang contact,
    friction 0.2), whose triangles, and so the pairs' order, are not
    mirror-symmetric."""
    maps = {"mirror_x": np.diag([-1.0, 1.0, 1.0]), "mirror_y": np.diag([1.0, -1.0, 1.0]),
            "swap_xy": np.array([[0.0, 1.0, 0.0], [1.0, 0.0, 0.0], [0.0, 0.0, 1.0]])}
    d = oracle_domain()
    if case_name == "plane":
        case = configs.contact_upsetting(d, R=0.003, L=0.006, dx=0.0005, v_punch=-20.0, jitter_amp=0.0)
    elif case_name == "bilinear":
        case = configs.cylinder_upsetting(d, R=0.003, L=0.006, dx=0.0005, v_top=-20.0, jitter_amp=0.0)
    else:
        d.set("gradKernelCorr", 1)
        case = configs.cylinder_upsetting(d, R=0.003, L=0.006, dx=0.0005, v_top=-20.0, jitter_amp=0.0,
                                          model=JOHNSON_COOK, thermal=True)
        d.set_particles("TI", 0.3)
    x0 = d.get_array("x")
    solid = d.get_array("ID") != 10
    partners = {k: _mirror_partner(x0[solid], M) for k, M in maps.items()}
    d.prepare(case.dt)
    d.step(40)
    v, S = d.get_array("v")[solid], d.get_array("Sigma").reshape(-1, 3, 3)[solid]
    T = d.get_array("T")[solid]
    assert d.get_array("pl_strain").max() > 1e-2 and d.geti("nb_searches") > 2
    d.close()
    tol = 1e-12 if case_name == "bilinear" else 1e-10
    for k, M in maps.items():
        m = partners[k]
        assert (m >= 0).all(), k
        assert np.abs(v[m] - v @ M.T).max() <= tol * np.abs(v).max(), k
        assert np.abs(S[m] - M @ S @ M.T).max() <= tol * np.abs(S).max(), k
        if case_name == "jc_thermal_ti_corr":
            assert np.ptp(T) > 1.0 and np.abs(T[m] - T).max() <= 1e-6 * np.ptp(T), k
