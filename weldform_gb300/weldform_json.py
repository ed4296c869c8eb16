"""WeldForm's JSON input front-end and CSV output, on the GB300 library.

    python -m weldform_gb300.weldform_json input.json [--out DIR] [--precision 0|1]

Reads a WeldForm input file (the reference application's `WeldForm
input.json`, Source/WeldForm.cpp:147-940), builds the domain through the
Domain API exactly as that driver does, runs the solver it names and writes
`WriteCSV` files (Source/Output.cpp:521-552) at the output times, named
``test06_NNNN.csv`` as the reference's solver calls name them.

Supported input (everything the kick-drift / leapfrog path covers):
  Configuration  solver ("Mech", "Mech-Thermal", "Mech-LeapFrog",
                 "Mech-Thermal-LeapFrog" -> SolveDiffUpdateLeapFrog;
                 "Mech-KickDrift", "Mech-Thermal-KickDrift" -> SolveDiffUpdateKickDrift),
                 particleRadius, hFactor, cflMethod/timeStepSize/cflFactor,
                 outTime, simTime, autoTS (velocity / acceleration criteria;
                 the contact one with leapfrog), artifViscAlpha/Beta,
                 contAlgorithm ("Wang"; "Fraser" also selects Wang, as the
                 reference), tensileInstability (default 0.3), nbsearchFreq,
                 sumType "Nishimura" (an unknown value keeps it, as the reference
                 does), stressGradType 0
  Materials[0]   Bilinear (const[0] = Et), Hollomon (yieldStress0, const = K, m),
                 JohnsonCook (const = A, B, n, C, eps_0, m, T_m, T_t);
                 density0, youngsModulus, poissonsRatio, plasticHeat,
                 thermalCond, thermalHeatCap, thermalExp
  DomainBlocks[0] Box or Cylinder, Cartesian grid
  DomainZones, Amplitudes, velocity BoundaryConditions (constant or
  amplitude, valueAng for rigid bodies), InitialConditions (velocity,
  temperature), RigidBodies of type Plane with Contact[0] (friction
  coefficients, penaltyFactor).
  BoundaryConditions of type 3 (convection: convCoeff, infTemp on the zone).
"Mech-Fraser" / "Mech-Thermal-Fraser" (SolveDiffUpdateFraser) build for the
oracle only; the library rejects that integrator.
Anything else (Thermal-only solvers, GMT, damage, file or axisymmetric
domains and meshes, 2D, heat-conduction contact, temperature / force BCs)
raises WFError(WF_ERR_UNSUPPORTED) before any step runs.
kernelGradCorr is supported in both forms; smoothlenUpdate is accepted (it
cannot change h in these solvers).
"""
from __future__ import annotations

import argparse
import json
import math
import os
from dataclasses import dataclass
from typing import Callable, Optional

import numpy as np

from . import BILINEAR, CONTACT_WANG, HOLLOMON, JOHNSON_COOK, Domain, WFError

WF_ERR_UNSUPPORTED = 8
FILE_KEY = "test06"  # the key WeldForm.cpp passes to the solvers (:921-930)
CSV_HEADER = "X, Y, Z, ID, Sigma_eq, Pl_Strain, vx, vy, vz, ax, ay, az, CFx, CFy, CZFz, p, Temp"


def _unsupported(msg):
    raise WFError(WF_ERR_UNSUPPORTED, msg)


@dataclass
class Run:
    dom: object
    integrator: int      # 0 kick-drift, 1 leapfrog, 2 Fraser (oracle only)
    dt: float
    sim_time: float
    out_time: float
    thermal: bool
    adaptive: bool = False  # autoTS velocity or acceleration criterion on


def _vec(v, n=3, default=0.0):
    v = list(v) if isinstance(v, (list, tuple)) else [v]
    return [float(x) for x in v] + [default] * (n - len(v))


def build(inp, make: Callable[[], object] = Domain, precision: Optional[int] = None) -> Run:
    """Build the domain an input file describes (WeldForm.cpp:147-940).  A key
    the reference driver reads without a default (readValue leaves the
    variable as it was, uninitialized) raises WF_ERR_UNSUPPORTED."""
    try:
        return _build(inp, make, precision)
    except KeyError as e:
        raise WFError(WF_ERR_UNSUPPORTED,
                      f"input lacks {e.args[0]!r}, which the reference driver reads into an uninitialized "
                      f"variable") from None


def _build(inp, make: Callable[[], object] = Domain, precision: Optional[int] = None) -> Run:
    """Build the domain of a WeldForm JSON input (file path or parsed dict)."""
    j = inp if isinstance(inp, dict) else json.load(open(inp))
    config = j.get("Configuration", {})
    material = j.get("Materials", [{}])
    domblock = j.get("DomainBlocks", [{}])
    domzones = j.get("DomainZones", [])
    amplitudes = j.get("Amplitudes", [])
    rigbodies = j.get("RigidBodies", [])
    contact_ = j.get("Contact", [{}])
    bcs = j.get("BoundaryConditions", [])
    ics = j.get("InitialConditions", [])

    dom = make()
    if precision is not None:
        dom.set("precision", precision)
    # ---- Configuration (WeldForm.cpp:195-226, 345-393)
    # WeldForm.cpp:198-202: "Locking" clears nonlock_sum; any other value but
    # "Nishimura" only prints a notice and keeps the default (Nishimura,
    # Domain.cpp:159).
    if config.get("sumType", "Nishimura") == "Locking":
        _unsupported("sumType Locking: only the Nishimura sum")
    dom.Kernel_Set(0)
    solver = config.get("solver", "Mech")
    leapfrog = ("Mech", "Mech-Thermal", "Mech-LeapFrog", "Mech-Thermal-LeapFrog")
    kickdrift = ("Mech-KickDrift", "Mech-Thermal-KickDrift")
    # The Fraser solver (SolverFraser.cpp) runs in the oracle only, which
    # checks itself against the reference's run log of it; the library
    # rejects integrator 2.
    fraser = ("Mech-Fraser", "Mech-Thermal-Fraser")
    if solver not in leapfrog + kickdrift + fraser:
        _unsupported(f"solver {solver!r}")
    thermal = solver in ("Mech-Thermal", "Mech-Thermal-LeapFrog", "Mech-Thermal-KickDrift", "Mech-Thermal-Fraser")
    integrator = 1 if solver in leapfrog else (2 if solver in fraser else 0)
    dom.set("integrator", integrator)
    if thermal:
        dom.set("thermal_solver", 1)
    r = float(config["particleRadius"])
    hfactor = float(config["hFactor"])
    # ---- Material (WeldForm.cpp:229-343)
    m0 = material[0]
    mattype = m0.get("type", "Bilinear")
    rho = float(m0["density0"])
    E = float(m0["youngsModulus"])
    nu = float(m0["poissonsRatio"])
    Fy = float(m0.get("yieldStress0", -1.0))
    c = [float(x) for x in m0.get("const", [])] + [0.0] * 10
    if m0.get("plasticHeat", False):
        dom.set("pl_heating", 1)
    if m0.get("damageModel", ""):
        _unsupported("damage models")
    # uninitialized doubles in the driver when absent (WeldForm.cpp:326-328);
    # only the thermal solvers read them
    k_T = float(m0["thermalCond"]) if thermal else float(m0.get("thermalCond", 0.0))
    cp_T = float(m0["thermalHeatCap"]) if thermal else float(m0.get("thermalHeatCap", 0.0))
    th_ex = float(m0.get("thermalExp", 0.0))
    K = E / (3. * (1. - 2 * nu))
    G = E / (2. * (1. + nu))
    dx = 2. * r
    h = dx * hfactor
    Cs = math.sqrt(K / rho)
    if int(config["cflMethod"]) == 0:  # an uninitialized int in the driver when absent (WeldForm.cpp:346)
        timestep = float(config["timeStepSize"])
    else:
        timestep = float(config["cflFactor"]) * h / Cs
    output_time = float(config["outTime"])
    sim_time = float(config["simTime"])
    # autoTS = [velocity, acceleration, contact] criteria, default [true, false,
    # false] (WeldForm.cpp:350, 364, 379-381)
    auto_ts = config.get("autoTS", [True, False, False])
    auto_ts = auto_ts if isinstance(auto_ts, list) else [auto_ts]
    auto_ts = (list(auto_ts) + [False, False, False])[:3]
    for key, flag in zip(("auto_ts", "auto_ts_acc", "auto_ts_cont"), auto_ts):
        dom.set(key, 1 if flag else 0)
    alpha = float(config.get("artifViscAlpha", 1.0))
    beta = float(config.get("artifViscBeta", 0.0))
    cont_alg = config.get("contAlgorithm", "Wang")
    if cont_alg not in ("Wang", "Fraser"):
        _unsupported(f"contact algorithm {cont_alg!r}")
    if config.get("kernelGradCorr", False):  # the reference then sums with locks (SolverKickDrift.cpp:107-110)
        dom.set("gradKernelCorr", 1)
    if int(config.get("stressGradType", 0)) != 0:
        _unsupported("stressGradType != 0")
    if config.get("smoothlenUpdate", False):  # WeldForm.cpp:377-389 (no effect on h in these solvers)
        dom.set("h_update", 1)
    tensins = float(config.get("tensileInstability", 0.3))
    dom.set("ts_nb_inc", int(config.get("nbsearchFreq", 5)))
    # ---- Domain block (WeldForm.cpp:395-560)
    b0 = domblock[0]
    start = _vec(b0["start"])  # an uninitialized Vec3_t in the driver when absent (WeldForm.cpp:393, 401)
    L = _vec(b0["dim"])
    domtype = b0.get("type", "Box")
    if b0.get("gridCoordSys", "Cartesian") != "Cartesian":
        _unsupported("non-Cartesian domain grids")
    sym = list(b0.get("sym", [False, False, False])) + [False] * 3
    # The reference's loop sets DomMax(0)/DomMin(0) from every L[i]; the last wins.
    dom.set_f64("DomMax.x", L[2])
    dom.set_f64("DomMin.x", -L[2])
    if abs(L[2]) < h:
        _unsupported("2D domains")
    if domtype == "Box":
        # the block's id tags the particles; an uninitialized int when absent
        # (WeldForm.cpp:394, 400, 434); cylinders are tagged 0 whatever it is
        dom.AddBoxLength(int(b0["id"]), start, L[0], L[1], L[2], r, rho, h, 1, 0, False, False)
    elif domtype == "Cylinder":
        if (sym[0] and sym[1]) or sym[2]:
            _unsupported("symmetric / ghost cylinders")
        dom.AddCylinderLength(0, start, L[0] / 2., L[2], r, rho, h, False)
    else:
        _unsupported(f"domain type {domtype!r}")
    for zone in domzones:
        dom.AssignZone(_vec(zone["start"]), _vec(zone["end"]), int(zone["id"]))
    # ---- Rigid bodies and contact (WeldForm.cpp:583-733)
    meshes = []
    for rb in rigbodies:
        if "type" not in rb:
            continue
        if rb["type"] != "Plane":
            _unsupported(f"rigid body type {rb['type']!r}")
        # read into the block's Vec3_t start (WeldForm.cpp:393, 595): absent,
        # the plane starts where the block does
        rstart = _vec(rb["start"]) if "start" in rb else list(start)
        rdim = _vec(rb["dim"])
        if rdim[0] != 0. and rdim[1] != 0. and rdim[2] != 0.:
            raise WFError(1, "Contact Plane Surface should have one null dimension")
        if float(rb.get("scaleFactor", 1.0)) != 1.0:
            _unsupported("rigid-body scaling")
        t = _vec(rb.get("translation", [0, 0, 0]))
        if math.sqrt(sum(x * x for x in t)) <= 1.0e-6:
            t = [0.0, 0.0, 0.0]
        p1 = [rstart[0] + t[0], rstart[1] + t[1], rstart[2] + t[2]]
        p2 = [rstart[0] + rdim[0] + t[0], rstart[1] + rdim[1] + t[1], rstart[2] + t[2]]
        dom.set("contact", 1)
        meshes.append(dom.add_rigid_plane(2, bool(rb.get("flipNormals", False)), p1, p2,
                                          int(rb.get("partSide", 10)), int(rb["zoneId"]), hfac=1.1))
        c0 = contact_[0] if contact_ else {}
        if c0.get("heatConductance", False) or c0.get("heatFriction", False):
            _unsupported("contact heat conduction / friction heat")
        dom.set_f64("friction_sta", float(c0.get("fricCoeffStatic", 0.0)))
        dom.set_f64("friction_dyn", float(c0.get("fricCoeffDynamic", 0.0)))
        dom.set_f64("PFAC", float(c0.get("penaltyFactor", 0.5)))
        dom.set_f64("DFAC", 0.0)
        dom.set("contact_alg", CONTACT_WANG)
    # ---- Amplitudes, BCs, initial conditions (WeldForm.cpp:743-862)
    for ampl in amplitudes:
        dom.add_amplitude(int(ampl["id"]), [float(x) for x in ampl["time"]], [float(x) for x in ampl["value"]])
    for bc in bcs:
        btype = int(bc.get("type", 0))  # BC_TYPE, Domain.h:94
        if btype == 3:  # Convection_BC (WeldForm.cpp:793-807): fields only, GeneralAfter skips it
            zone = int(bc["zoneId"])
            dom.set_particles("Thermal_BC", 1, zone)
            dom.set_particles("T_inf", float(bc["infTemp"]), zone)
            dom.set_particles("h_conv", float(bc["convCoeff"]), zone)
            continue
        if btype != 0:
            _unsupported("temperature / force / symmetry boundary conditions")
        vt = int(bc.get("valueType", 0))
        # An absent "value" leaves the driver's Vec3_t uninitialized
        # (WeldForm.cpp:776-779) and UserAcc multiplies it (WeldForm.cpp:76-77);
        # the reference's Traction.json has such an amplitude BC.  Zero here:
        # its zone is held still.
        value = _vec(bc.get("value", [0, 0, 0]))
        ang = _vec(bc.get("valueAng", [0, 0, 0]))
        if vt == 0:
            dom.add_velocity_bc(int(bc["zoneId"]), value, ang)
        else:
            dom.add_velocity_bc(int(bc["zoneId"]), value, ang, value_type=1, amp_id=int(bc["amplitudeId"]),
                                amp_factor=float(bc.get("amplitudeFactor", 1.0)))
    n = dom.particle_count
    ids = dom.get_array("ID")
    T = np.zeros(n)
    v = np.zeros((n, 3))
    nsolid = int(dom.geti("solid_part_count"))
    # The driver keeps one IniTemp across the conditions (WeldForm.cpp:828-833):
    # a condition without "Temp" applies the previous one's.
    temp = 0.0
    for ic in ics:
        temp = float(ic.get("Temp", temp))
        value = _vec(ic.get("value", [0, 0, 0]))
        zoneid = int(ic.get("zoneId", -1))
        if zoneid == -1:
            v[:nsolid] = value
            if thermal:
                T[:nsolid] = temp
        elif thermal:
            T[ids == zoneid] = temp
    dom.set_array("v", v)
    # ---- per-particle fields (WeldForm.cpp:870-913)
    if mattype == "Bilinear":
        mid = dom.add_material(BILINEAR, [E, nu])
        dom.set_particles("Ep", E * c[0] / (E - c[0]))
        if Fy <= 0.0:
            raise WFError(1, "Invalid Initial Yield Stress.")
        sy = np.full(n, Fy)
    elif mattype == "Hollomon":
        mid = dom.add_material(HOLLOMON, [E, nu, Fy, c[0], c[1]])
        dom.set_particles("Material_model", HOLLOMON)
        sy = None
    elif mattype == "JohnsonCook":
        mid = dom.add_material(JOHNSON_COOK, [E, nu] + c[:8])
        dom.set_particles("Material_model", JOHNSON_COOK)
        sy = None
    else:
        _unsupported(f"material type {mattype!r}")
    dom.set_particles("G", G)
    dom.set_particles("Cs", Cs)
    dom.set_particles("mat", mid)
    dom.set_particles("Fail", 1)
    dom.set_particles("Alpha", alpha)
    dom.set_particles("Beta", beta)
    dom.set_particles("TI", tensins)
    dom.set_particles("TIInitDist", dx)
    dom.set_particles("k_T", k_T)
    dom.set_particles("cp_T", cp_T)
    dom.set_particles("th_exp", th_ex)
    dom.set_array("T", T)
    if sy is None:  # CalcYieldStress(0, 0, T) of the material
        sy = _initial_yield(mattype, c, Fy, T)
    dom.set_array("Sigmay", sy)
    return Run(dom=dom, integrator=integrator, dt=timestep, sim_time=sim_time, out_time=output_time, thermal=thermal,
               adaptive=bool(auto_ts[0] or auto_ts[1]))


def _initial_yield(mattype, c, Fy, T):
    """mat->CalcYieldStress(0.0, 0.0, T) as WeldForm.cpp:905-906 calls it.
    Hollomon does not override the three-argument form (Material.h:101, 219),
    so the base class's 0.0 is what its particles start with."""
    if mattype == "Hollomon":
        return np.zeros(T.shape)
    A, B, n, C, e0, m, Tm, Tt = c[:8]
    Th = (T - Tt) / (Tm - Tt)
    return (A + B * 0.0 ** n) * 1.0 * (1.0 - np.power(Th, m))


def sigma_eq(tau9: np.ndarray) -> np.ndarray:
    """Particle::CalculateEquivalentStress (Particle.cpp:623-633) from ShearStress."""
    S = tau9.reshape(-1, 3, 3)
    J2 = 0.5 * (S[:, 0, 0] * S[:, 0, 0] + 2.0 * S[:, 0, 1] * S[:, 1, 0] + 2.0 * S[:, 0, 2] * S[:, 2, 0] +
                S[:, 1, 1] * S[:, 1, 1] + 2.0 * S[:, 1, 2] * S[:, 2, 1] + S[:, 2, 2] * S[:, 2, 2])
    return np.sqrt(3.0 * J2)


def _g(x: float) -> str:
    """A double as std::ostream prints it by default (6 significant digits)."""
    s = "%g" % x
    return s


def write_csv(dom, path: str):
    """Domain::WriteCSV (Output.cpp:521-552): one row per particle."""
    x = dom.get_array("x")
    ids = dom.get_array("ID")
    seq = sigma_eq(dom.get_array("ShearStress"))
    pl = dom.get_array("pl_strain")
    v = dom.get_array("v")
    a = dom.get_array("a")
    cf = dom.get_array("contforce")
    p = dom.get_array("Pressure")
    T = dom.get_array("T")
    lines = [CSV_HEADER]
    for i in range(x.shape[0]):
        vals = [_g(x[i, 0]), _g(x[i, 1]), _g(x[i, 2]), "%d" % ids[i], _g(seq[i]), _g(pl[i]),
                _g(v[i, 0]), _g(v[i, 1]), _g(v[i, 2]), _g(a[i, 0]), _g(a[i, 1]), _g(a[i, 2]),
                _g(cf[i, 0]), _g(cf[i, 1]), _g(cf[i, 2]), _g(p[i]), _g(T[i])]
        lines.append(", ".join(vals))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def run(inp, out_dir: str = ".", make: Callable[[], object] = Domain, precision: Optional[int] = None,
        max_outputs: int = 1000000, key: str = FILE_KEY) -> list:
    """Build and solve; write key_NNNN.csv at each output time.  Returns the
    written paths.  The loop control is SolveDiffUpdate*'s
    (while Time <= tf && idx_out <= maxidx; output when Time >= tout), with
    Time accumulated as the device does (Time += dt per step).  With an
    adaptive time step, Time is read back: the step never exceeds the initial
    dt, so floor((limit - Time) / dt) - 1 steps at a time stay inside the next
    loop or output boundary, and single steps finish the approach."""
    r = build(inp, make, precision)
    d = r.dom
    d.prepare(r.dt)
    os.makedirs(out_dir, exist_ok=True)
    Time, tout, idx_out = 0.0, 0.0, 1
    written = []

    def output():
        path = os.path.join(out_dir, "%s_%04d.csv" % (key, idx_out))
        write_csv(d, path)
        written.append(path)

    if r.adaptive:
        Time = d.get("Time")
        while Time <= r.sim_time and idx_out <= max_outputs:
            lim = min(r.sim_time, tout)
            n = int((lim - Time) // r.dt) if Time < lim else 0
            if n > 1:
                d.step(n - 1)
                Time = d.get("Time")
                continue
            d.step(1)
            Time = d.get("Time")
            if Time >= tout:
                output()
                idx_out += 1
                tout += r.out_time
        return written
    pending = 0
    while Time <= r.sim_time and idx_out <= max_outputs:
        Time += r.dt
        pending += 1
        if Time >= tout:
            d.step(pending)
            pending = 0
            output()
            idx_out += 1
            tout += r.out_time
    if pending:
        d.step(pending)
    return written


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("input")
    ap.add_argument("--out", default=".")
    ap.add_argument("--precision", type=int, default=None)
    a = ap.parse_args()
    paths = run(a.input, a.out, precision=a.precision)
    print(json.dumps({"outputs": len(paths), "last": paths[-1] if paths else None}))


if __name__ == "__main__":
    main()
