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
