"""The reference's own example input decks through the JSON front-end.

tests/golden/reference_decks.json holds the decks of examples/input/*.json
that the front-end accepts (3D Cartesian domains, Nishimura sums, no damage,
no mesh files, no pure-thermal solver), extracted by
tests/golden/make_golden.py.  Every deck builds and steps in the oracle; the
decks of the kick-drift and leapfrog solvers also run on the GPU in both
forms and must match the oracle after 100 steps (the Fraser-solver decks run
in the oracle only, which checks itself against the reference's run log of
one of them in test_oracle_golden.py).

Two decks (Compression_fast_short, Traction: Hollomon with yieldStress0 = 0)
turn particles NaN within the first steps in the reference's arithmetic; the
forms must turn the same particles NaN and agree on the rest.
"""
import json
import os

import numpy as np
import pytest

from tests._support import gpu_domain, oracle_domain
from weldform_gb300 import PRECISION_FP64, PRECISION_MIXED
from weldform_gb300 import weldform_json as wj

FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "reference_decks.json")
DECKS = json.load(open(FIXTURE))["decks"]
FRASER = sorted(n for n, j in DECKS.items() if "Fraser" in j["Configuration"].get("solver", "Mech"))
ON_GPU = sorted(n for n in DECKS if n not in FRASER)
STEPS = 100
THREADS = os.cpu_count() or 1


def _oracle():
    d = oracle_domain()
    d.set("cpu_threads", THREADS)
    return d


def _run(make, name, steps):
    run = wj.build(DECKS[name], make, None)
    d = run.dom
    d.prepare(run.dt)
    d.step(steps)
    out = {f: d.get_array(f) for f in ("Displacement", "Sigma", "v")}
    out["Time"] = d.get("Time")
    out["searches"] = d.geti("nb_searches")
    out["n"] = d.particle_count
    d.close()
    return out


def test_the_fixture_holds_the_accepted_decks():
    assert len(DECKS) == 12 and len(FRASER) == 4 and len(ON_GPU) == 8


@pytest.mark.parametrize("name", sorted(DECKS))
def test_every_deck_builds_and_steps_in_the_oracle(name):
    r = _run(_oracle, name, 3)
    assert r["n"] > 1000 and r["Time"] > 0.0 and r["searches"] >= 1


_ORACLE = {}


def _oracle_run(name):
    if name not in _ORACLE:
        _ORACLE[name] = _run(_oracle, name, STEPS)
    return _ORACLE[name]


def _close(a, b, tol, what):
    a = a.reshape(len(a), -1)
    b = b.reshape(len(b), -1)
    na, nb = ~np.isfinite(a).all(axis=1), ~np.isfinite(b).all(axis=1)
    assert np.array_equal(na, nb), (what, int(na.sum()), int(nb.sum()))
    fa, fb = a[~na], b[~nb]
    if fb.size == 0:
        return
    den = np.linalg.norm(fb)
    err = np.linalg.norm(fa - fb) / den if den > 0 else np.linalg.norm(fa)
    assert err <= tol, (what, err)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("name", ON_GPU)
def test_deck_on_the_gpu_matches_the_oracle(name, precision):
    """100 steps of the deck as the reference driver builds it: plain FP64
    within 1e-9 of the oracle, mixed within 1e-4 (relative L2 over the
    particles that stay finite; the same particles must turn NaN)."""
    def make():
        d = gpu_domain()
        d.set("precision", precision)
        return d
    g = _run(make, name, STEPS)
    o = _oracle_run(name)
    assert g["n"] == o["n"] and g["searches"] == o["searches"]
    assert abs(g["Time"] - o["Time"]) <= 1e-12 * abs(o["Time"])
    tol = 1e-9 if precision == PRECISION_FP64 else 1e-4
    for f in ("Displacement", "Sigma", "v"):
        _close(g[f], o[f], tol, f)


LOG = os.path.join(os.path.dirname(__file__), "golden", "contact_compression_fraser.json")


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED], ids=["fp64", "mixed"])
def test_kick_drift_on_the_logged_deck_tracks_the_reference_log(precision):
    """The reference logged Contact_Compression.json with its Fraser solver
    (the oracle reproduces that log to 6 digits).  The library's kick-drift
    path on the same deck — same generator, contact plane, materials, BCs —
    at cflFactor 0.4 (at the deck's 0.7 the kick-drift update with Wang's
    stiffness 2 m / dt^2 is unstable, in the oracle as on the GPU) must
    follow the logged run over its whole 0.01 s: external work within 1 %
    and internal energy within 3 % from 0.5 ms on (two integrators at two
    time steps; measured 0.26 % and 2.0 %), and the maximum plastic strain
    within 5 % of the log's 2-digit value once it passes 0.005 (yield near
    2.2 ms, then 1,013 searches)."""
    fx = json.load(open(LOG))
    rows = fx["outputs"]
    dt_log = 2.7323318164706004e-06  # the deck's CFL step, as the oracle forms it
    tlog = np.array([r["step"] * dt_log for r in rows])
    deck = json.loads(json.dumps(fx["deck"]))
    deck["Configuration"]["solver"] = "Mech-KickDrift"
    deck["Configuration"]["cflFactor"] = 0.4
    run = wj.build(deck, gpu_domain, precision)
    d = run.dom
    d.prepare(run.dt)
    checked = 0
    for k in range(1, len(rows)):
        n = int(round((tlog[k] - d.get("Time")) / run.dt))
        if n > 0:
            d.step(n)
        t = d.get("Time")
        if t < 5e-4:
            continue
        ext = np.interp(t, tlog, [r["ext_forces_work"] for r in rows])
        ie = np.interp(t, tlog, [r["int_energy_sum"] for r in rows])
        assert abs(d.get("ext_forces_work") / ext - 1.0) <= 1e-2, (t, d.get("ext_forces_work"), ext)
        assert abs(d.get("int_energy_sum") / ie - 1.0) <= 3e-2, (t, d.get("int_energy_sum"), ie)
        pl = np.interp(t, tlog, [r["max_pl"] for r in rows])
        if pl > 5e-3:
            assert abs(d.get("max_pl_strain") / pl - 1.0) <= 5e-2, (t, d.get("max_pl_strain"), pl)
            checked += 1
    assert checked > 50 and d.geti("nb_searches") > 500
    d.close()
