"""WeldForm JSON front-end and WriteCSV output (weldform_gb300/weldform_json.py).

The inputs below are written for these tests in the reference's input schema
(Source/WeldForm.cpp:147-940).  CPU tests drive the oracle; the GPU test runs
the same input on the library and compares with the oracle."""
import copy
import math
import os

import numpy as np
import pytest

from tests._support import gpu_domain, oracle_domain, rel_l2
from weldform_gb300 import BILINEAR, PRECISION_MIXED, WFError
from weldform_gb300 import weldform_json as wj

R, L, r = 0.003, 0.006, 0.00025
E, nu, rho = 200e9, 0.3, 7850.0
CS = math.sqrt(E / (3 * (1 - 2 * nu)) / rho)
DT = 0.4 * (2 * r * 1.2) / CS

COMPRESSION = {
    "Configuration": {"Nproc": 4, "particleRadius": r, "hFactor": 1.2, "cflMethod": 1, "cflFactor": 0.4,
                      "outTime": 5 * DT, "simTime": 20 * DT, "autoTS": [False, False, False],
                      "solver": "Mech", "tensileInstability": 0.0},
    "Materials": [{"type": "Bilinear", "density0": rho, "youngsModulus": E, "poissonsRatio": nu,
                   "yieldStress0": 300e6, "const": [1.5e9]}],
    "DomainBlocks": [{"type": "Cylinder", "zoneId": 0, "start": [0, 0, 0], "dim": [2 * R, 2 * R, L]}],
    "DomainZones": [{"id": 2, "start": [-1, -1, -1], "end": [1, 1, 2 * r]},
                    {"id": 3, "start": [-1, -1, L - 4 * r], "end": [1, 1, 1]}],
    "BoundaryConditions": [{"zoneId": 2, "valueType": 0, "value": [0, 0, 0]},
                           {"zoneId": 3, "valueType": 0, "value": [0, 0, -20.0]}],
}

CONTACT = {
    "Configuration": {"particleRadius": r, "hFactor": 1.2, "cflMethod": 1, "cflFactor": 0.4,
                      "outTime": 10 * DT, "simTime": 30 * DT, "autoTS": [False, False, False],
                      "solver": "Mech-Thermal"},
    "Materials": [{"type": "JohnsonCook", "density0": rho, "youngsModulus": E, "poissonsRatio": nu,
                   "const": [350e6, 275e6, 0.36, 0.022, 1.0, 1.0, 1793.0, 300.0], "plasticHeat": True,
                   "thermalCond": 50.0, "thermalHeatCap": 460.0}],
    "DomainBlocks": [{"type": "Cylinder", "start": [0, 0, 0], "dim": [2 * R, 2 * R, L]}],
    "DomainZones": [{"id": 2, "start": [-1, -1, -1], "end": [1, 1, 2 * r]}],
    # the generator's top layer is at L - 3r (the z accumulation drops the last
    # layer); the plane starts one smoothing length above it
    "RigidBodies": [{"type": "Plane", "zoneId": 10, "start": [-R - 2 * r, -R - 2 * r, L - 3 * r + 2 * r * 1.2],
                     "dim": [2 * R + 4 * r, 2 * R + 4 * r, 0], "partSide": 14}],
    "Contact": [{"fricCoeffStatic": 0.2, "fricCoeffDynamic": 0.2}],
    "Amplitudes": [{"id": 1, "time": [0.0, 10 * DT, 1.0], "value": [0.0, 1.0, 1.0]}],
    "BoundaryConditions": [{"zoneId": 2, "valueType": 0, "value": [0, 0, 0]},
                           {"zoneId": 10, "valueType": 1, "amplitudeId": 1, "amplitudeFactor": 1.0,
                            "value": [0, 0, -10.0]}],
    "InitialConditions": [{"Temp": 300.0, "zoneId": -1}],
}


def _oracle():
    d = oracle_domain()
    d.set("cpu_threads", min(os.cpu_count() or 1, 8))
    return d


def _read_csv(path):
    lines = open(path).read().splitlines()
    return lines[0], np.array([[float(v) for v in ln.split(", ")] for ln in lines[1:]])


def test_csv_layout_and_output_schedule(tmp_path):
    paths = wj.run(COMPRESSION, str(tmp_path), make=_oracle)
    assert [os.path.basename(p) for p in paths][:2] == ["test06_0001.csv", "test06_0002.csv"]
    assert 4 <= len(paths) <= 6          # t = dt, then every 5 dt up to 20 dt
    head, rows = _read_csv(paths[-1])
    assert head == wj.CSV_HEADER
    assert rows.shape[1] == 17
    d = _oracle()
    d.AddCylinderLength(0, (0, 0, 0), R, L, r, rho, 2 * r * 1.2, False)
    assert rows.shape[0] == d.particle_count
    assert set(np.unique(rows[:, 3]).astype(int)) <= {0, 2, 3}


def test_json_build_equals_the_api_build():
    """The same case built by hand through the Domain API, as the driver
    would (G, Cs, Ep, Sigmay, Alpha/Beta, TIInitDist, DomMax/DomMin quirk)."""
    run = wj.build(COMPRESSION, make=_oracle)
    a = run.dom
    a.prepare(run.dt)
    a.step(15)
    b = _oracle()
    b.set("integrator", 1)
    b.Kernel_Set(0)
    b.set_f64("DomMax.x", L)
    b.set_f64("DomMin.x", -L)
    b.AddCylinderLength(0, (0, 0, 0), R, L, r, rho, 2 * r * 1.2, False)
    b.AssignZone((-1, -1, -1), (1, 1, 2 * r), 2)
    b.AssignZone((-1, -1, L - 4 * r), (1, 1, 1), 3)
    b.add_velocity_bc(2, (0, 0, 0))
    b.add_velocity_bc(3, (0, 0, -20.0))
    mid = b.add_material(BILINEAR, [E, nu])
    b.set_particles("mat", mid)
    b.set_particles("Ep", E * 1.5e9 / (E - 1.5e9))
    b.set_particles("Sigmay", 300e6)
    b.set_particles("G", E / (2 * (1 + nu)))
    b.set_particles("Cs", CS)
    b.set_particles("Fail", 1)
    b.set_particles("Alpha", 1.0)
    b.set_particles("Beta", 0.0)
    b.set_particles("TIInitDist", 2 * r)
    b.prepare(run.dt)
    b.step(15)
    for f in ("x", "v", "Sigma", "pl_strain"):
        assert np.array_equal(a.get_array(f), b.get_array(f)), f


def test_contact_thermal_input_runs_in_the_oracle(tmp_path):
    paths = wj.run(CONTACT, str(tmp_path), make=_oracle)
    head, rows = _read_csv(paths[-1])
    assert np.abs(rows[:, 14]).max() > 0      # CZFz: contact force on surface particles
    assert rows[:, 16].max() >= 300.0


def test_convection_boundary_condition():
    """A type-3 BC (WeldForm.cpp:793-807) marks its zone for CalcConvHeat with
    its convCoeff and infTemp; GeneralAfter leaves it alone.  The zone heats
    toward T_inf faster than the same run without it."""
    j = copy.deepcopy(CONTACT)
    j["BoundaryConditions"].append({"zoneId": 2, "type": 3, "convCoeff": 5e7, "infTemp": 900.0})
    runs = {}
    for name, deck in (("conv", j), ("plain", CONTACT)):
        run = wj.build(deck, make=_oracle)
        d = run.dom
        d.prepare(run.dt)
        d.step(10)
        runs[name] = (d.get_array("T"), d.get_array("Thermal_BC"), d.get_array("h_conv"), d.get_array("T_inf"),
                      d.get_array("ID"))
    T, tbc, hc, tinf, ids = runs["conv"]
    zone = ids == 2
    assert zone.sum() > 0
    assert (tbc[zone] == 1).all() and (tbc[~zone] == 0).all()
    assert np.allclose(hc[zone], 5e7) and np.allclose(tinf[zone], 900.0)
    assert (T[zone] > runs["plain"][0][zone] + 1e-3).all()
    with pytest.raises(WFError) as e:
        bad = copy.deepcopy(CONTACT)
        bad["BoundaryConditions"].append({"zoneId": 2, "type": 3, "convCoeff": 5e7})
        wj.build(bad, make=_oracle)
    assert e.value.code == 8


@pytest.mark.parametrize("base,section,key", [
    ("compression", "Configuration", "cflMethod"),   # int cflMethod (WeldForm.cpp:346-351)
    ("compression", "DomainBlocks", "start"),        # Vec3_t start (WeldForm.cpp:393, 401)
    ("box", "DomainBlocks", "id"),                   # int id, the box particles' tag (WeldForm.cpp:394, 434)
    ("contact", "Materials", "thermalCond"),         # double k_T under a thermal solver (WeldForm.cpp:326-327)
    ("contact", "Materials", "thermalHeatCap"),      # double cp_T (WeldForm.cpp:326, 328)
])
def test_input_without_a_key_the_driver_leaves_uninitialized_is_rejected(base, section, key):
    """Keys the driver reads into variables it never initialised: an input
    that omits one has no defined meaning, so the front-end refuses it."""
    j = copy.deepcopy(CONTACT if base == "contact" else COMPRESSION)
    if base == "box":
        j["DomainBlocks"] = [{"type": "Box", "id": 0, "start": [0, 0, 0], "dim": [2 * R, 2 * R, L]}]
        wj.build(copy.deepcopy(j), make=_oracle).dom.close()  # complete, it builds
    tgt = j[section][0] if isinstance(j[section], list) else j[section]
    del tgt[key]
    with pytest.raises(WFError) as e:
        wj.build(j, make=_oracle)
    assert e.value.code == 8 and key in str(e.value)


def test_plane_without_start_starts_at_the_block_start():
    """The driver reads a rigid body's "start" into the domain block's start
    vector (WeldForm.cpp:393, 595; the zones keep their own), so a plane that
    gives none is laid from the block's start."""
    j = copy.deepcopy(CONTACT)
    j["DomainBlocks"][0]["start"] = [-0.001, -0.002, 0.0075]
    del j["RigidBodies"][0]["start"]
    run = wj.build(j, make=_oracle)
    x, ids = run.dom.get_array("x"), run.dom.get_array("ID")
    plane = x[ids == 10]
    assert plane.shape[0] > 0
    assert np.all(plane[:, 2] == plane[0, 2]) and abs(plane[0, 2] - 0.0075) < 1e-12
    assert abs(plane[:, 0].min() - (-0.001)) < 2 * r and abs(plane[:, 1].min() - (-0.002)) < 2 * r
    run.dom.close()


def test_initial_temperature_carries_over_between_conditions():
    """The driver reads every initial condition's "Temp" into one IniTemp
    declared outside the loop (WeldForm.cpp:828-833), so a condition without
    "Temp" applies the previous condition's temperature to its zone."""
    j = copy.deepcopy(CONTACT)
    j["DomainZones"].append({"id": 4, "start": [-1, -1, L / 2], "end": [1, 1, 1]})
    j["InitialConditions"] = [{"Temp": 300.0, "zoneId": -1}, {"Temp": 450.0, "zoneId": 2}, {"zoneId": 4}]
    run = wj.build(j, make=_oracle)
    ids, T = run.dom.get_array("ID"), run.dom.get_array("T")
    assert (T[ids == 2] == 450.0).all() and (T[ids == 4] == 450.0).all()
    assert (T[ids == 0] == 300.0).all() and (ids == 4).sum() > 0
    run.dom.close()


@pytest.mark.parametrize("patch", [
    ("Materials", "type", "GMT"),
    ("Materials", "damageModel", "Rankine"),
    ("DomainBlocks", "gridCoordSys", "AxiSymmetric"),
])
def test_unsupported_inputs_are_rejected(patch):
    j = copy.deepcopy(COMPRESSION)
    sec, key, val = patch
    tgt = j[sec][0] if isinstance(j[sec], list) else j[sec]
    tgt[key] = val
    with pytest.raises(WFError) as e:
        wj.build(j, make=_oracle)
    assert e.value.code == 8


@pytest.mark.gpu
def test_fraser_solver_is_rejected_by_the_library():
    """"Mech-Fraser" (SolveDiffUpdateFraser) runs in the oracle, which checks
    itself against the reference's run log of that solver; the library builds
    the kick-drift and leapfrog orders only and says so."""
    j = copy.deepcopy(COMPRESSION)
    j["Configuration"]["solver"] = "Mech-Fraser"
    with pytest.raises(WFError) as e:
        wj.build(j)
    assert e.value.code == 8


def test_default_adaptive_time_step(tmp_path):
    """Without an autoTS key the driver runs the velocity criterion
    (WeldForm.cpp:350): with cflFactor 0.8 the CFL bound on the shortest
    neighbour distance is below the input step, so the step shrinks and the
    run needs more steps to reach simTime than the fixed-step loop."""
    j = copy.deepcopy(COMPRESSION)
    del j["Configuration"]["autoTS"]
    j["Configuration"]["cflFactor"] = 0.8
    j["Configuration"]["simTime"] = 10 * DT
    j["Configuration"]["outTime"] = 5 * DT
    r = wj.build(j, make=_oracle)
    assert r.adaptive
    r.dom.prepare(r.dt)
    r.dom.step(3)
    assert r.dom.get("deltat") < 0.9 * r.dt
    paths = wj.run(j, str(tmp_path), make=_oracle)
    assert len(paths) >= 2
    head, rows = _read_csv(paths[-1])
    assert head == wj.CSV_HEADER


@pytest.mark.gpu
def test_json_run_on_the_gpu_matches_the_oracle(tmp_path):
    out = {}
    for name, make in (("gpu", gpu_domain), ("oracle", _oracle)):
        paths = wj.run(CONTACT, str(tmp_path / name), make=make)
        out[name] = [_read_csv(p)[1] for p in paths]
    assert len(out["gpu"]) == len(out["oracle"])
    for g, o in zip(out["gpu"], out["oracle"]):
        assert g.shape == o.shape
        cols = [0, 1, 2, 4, 5, 6, 7, 8, 14, 15, 16]  # x, Sigma_eq, pl, v, CZFz, p, T
        assert np.array_equal(g[:, 3], o[:, 3])
        for c in cols:
            assert rel_l2(g[:, c], o[:, c]) <= 2e-6, c   # 6 printed digits


HOLLOMON = copy.deepcopy(COMPRESSION)
HOLLOMON["Materials"] = [{"type": "Hollomon", "density0": rho, "youngsModulus": E, "poissonsRatio": nu,
                          "yieldStress0": 260e6, "const": [718e6, 0.22]}]


def _first_step_sigma(make, precision=None):
    r = wj.build(HOLLOMON, make=make)
    if precision is not None:
        r.dom.set("precision", precision)
    r.dom.prepare(r.dt)
    r.dom.step(1)
    s = r.dom.get_array("Sigma")
    r.dom.close()
    return s


def test_hollomon_input_starts_with_zero_yield_stress():
    """The driver gives Hollomon particles mat->CalcYieldStress(0, 0, T)
    (WeldForm.cpp:912-913), the base class's 0.0 (Material.h:101).  In the
    first stress update every particle with zero trial stress then takes
    min(0/0, 1) (Particle.cpp:277), which is NaN: its shear stress becomes
    NaN.  Particles the moving zone strains have a positive trial stress and
    stay finite."""
    r = wj.build(HOLLOMON, make=_oracle)
    assert np.all(r.dom.get_array("Sigmay") == 0.0)
    r.dom.close()
    s = _first_step_sigma(_oracle)
    bad = ~np.isfinite(s).all(axis=1)
    assert 0 < bad.sum() < len(bad)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [None, PRECISION_MIXED], ids=["fp64", "mixed"])
def test_hollomon_nan_pattern_matches_the_oracle(precision):
    """The GPU stress update keeps std::min's NaN (a NaN ratio is not clamped
    to 1): the same particles turn NaN as in the oracle, the others agree."""
    o = _first_step_sigma(_oracle)
    g = _first_step_sigma(gpu_domain, precision)
    assert np.array_equal(np.isnan(g), np.isnan(o))
    ok = np.isfinite(o)
    tol = 1e-9 if precision is None else 1e-4
    assert rel_l2(g[ok], o[ok]) <= tol


# Keys of the accepted reference decks the front-end does not read, each one
# the reference's driver does not act on either (Source/WeldForm.cpp).
_IGNORED_DECK_KEYS = {
    "BoundaryConditions[].components": "never read",
    "BoundaryConditions[].free": "read into bcon.free (WeldForm.cpp:822), never used",
    "BoundaryConditions[].valuetype": "misspelt in the decks; the driver reads valueType (WeldForm.cpp:777)",
    "Configuration.Nproc": "OpenMP thread count (WeldForm.cpp:195)",
    "Contact[].heatCondCoeff": "used only with heatConductance (WeldForm.cpp:689, 714-718), rejected here",
    "DomainBlocks[].denseMode": "never read",
    "DomainBlocks[].matID": "read (WeldForm.cpp:404), never used",
    "DomainBlocks[].scale": "never read",
    "DomainZones[].denseMode": "never read",
    "Materials[].const1": "never read (the driver reads const, WeldForm.cpp:252)",
    "Materials[].const2": "never read (the driver reads const, WeldForm.cpp:252)",
    "RigidBodies[].scale": "never read",
}


def test_every_key_of_the_accepted_decks_is_read_or_inert():
    """A key of an accepted deck that the front-end never mentions would be a
    silent misreading unless the reference's driver ignores it as well."""
    import json
    import re
    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_decks.json")
    decks = json.load(open(golden))["decks"]
    keys = set()

    def walk(o, path):
        if isinstance(o, dict):
            for k, v in o.items():
                p = f"{path}.{k}" if path else k
                keys.add(p)
                walk(v, p)
        elif isinstance(o, list):
            for x in o:
                walk(x, path + "[]")

    for deck in decks.values():
        walk(deck, "")
    src = open(wj.__file__).read()
    unread = {k for k in keys if '"%s"' % re.sub(r"\[.*", "", k.split(".")[-1]) not in src}
    assert unread == set(_IGNORED_DECK_KEYS), sorted(unread ^ set(_IGNORED_DECK_KEYS))
