"""Batched sweeps: specimens stepped together in one domain match the same
specimens stepped alone (same per-specimen positions, materials and BCs)."""
import numpy as np
import pytest

from tests._support import gpu_domain, oracle_domain
from weldform_gb300 import batch

SPECS = batch.random_specimens(3, r_range=(0.0025, 0.004), v_range=(0.5, 2.0))
DX = 0.0005
STEPS = 30


def _fields(d, a, b):
    return {f: d.get_array(f)[a:b] for f in ("Displacement", "v", "Sigma", "Density")}


def _sweep_vs_single(make):
    d = make()
    sw = batch.build_sweep(d, SPECS, dx=DX)
    d.prepare(sw.dt)
    d.step(STEPS)
    together = [_fields(d, a, b) for a, b in sw.ranges]
    d.close()
    alone = []
    for k, s in enumerate(SPECS):
        e = make()
        one = batch.build_single(e, s, k, dx=DX)
        e.prepare(one.dt)
        e.step(STEPS)
        alone.append(_fields(e, 0, one.n))
        e.close()
    return sw, together, alone


def _check(tog, alo, tol):
    for t, a in zip(tog, alo):
        for f in t:
            err = np.linalg.norm(t[f] - a[f]) / max(np.linalg.norm(a[f]), 1e-300)
            assert err <= tol, (f, err)


def test_sweep_equals_single_runs_in_the_oracle():
    """Placement shifts coordinates by the specimen offset, so differences
    x_i - x_j agree to rounding only: FP64 results agree to ~1e-12."""
    sw, tog, alo = _sweep_vs_single(oracle_domain)
    assert len(sw.ranges) == 3 and sw.n == sum(b - a for a, b in sw.ranges)
    _check(tog, alo, 1e-9)


@pytest.mark.gpu
def test_sweep_equals_single_runs_on_the_gpu():
    sw, tog, alo = _sweep_vs_single(gpu_domain)
    _check(tog, alo, 1e-9)


# Specimens that yield at different times (20, 8 and 0.5 m/s punches): each
# keeps its own rebuild schedule, so a batched specimen searches exactly when
# it does alone and its state matches its solo run.
_JC = SPECS[0].jc
UNEVEN = [batch.Specimen(R=0.003, L=0.006, v_punch=-20.0, jc=_JC),
          batch.Specimen(R=0.0035, L=0.005, v_punch=-0.5, jc=_JC),
          batch.Specimen(R=0.0025, L=0.006, v_punch=-8.0, jc=_JC)]


def _uneven(make, steps=60):
    d = make()
    sw = batch.build_sweep(d, UNEVEN, dx=DX)
    d.prepare(sw.dt)
    d.step(steps)
    tog = [_fields(d, a, b) for a, b in sw.ranges]
    searches = [d.batch_get(k, "nb_searches") for k in range(len(UNEVEN))]
    d.close()
    alo, solo_searches = [], []
    for k, s in enumerate(UNEVEN):
        e = make()
        one = batch.build_single(e, s, k, dx=DX)
        e.prepare(one.dt)
        e.step(steps)
        alo.append(_fields(e, 0, one.n))
        solo_searches.append(e.geti("nb_searches"))
        e.close()
    return tog, alo, searches, solo_searches


def test_each_specimen_keeps_its_own_schedule_in_the_oracle():
    tog, alo, searches, solo = _uneven(oracle_domain)
    assert searches == solo
    assert len(set(searches)) > 1  # the specimens really rebuild at different steps
    _check(tog, alo, 1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_each_specimen_keeps_its_own_schedule_on_the_gpu(precision):
    """Per-specimen search counts equal the solo runs' and the oracle's batch;
    the batched state matches the solo runs (1e-9 plain; the mixed form's
    records are kept relative to each domain's own grid centre, so 1e-6) and
    the oracle's batch (1e-9 plain, 1e-4 mixed)."""
    def make():
        d = gpu_domain()
        d.set("precision", precision)
        return d
    tog, alo, searches, solo = _uneven(make)
    otog, _, osearches, _ = _uneven(oracle_domain)
    assert searches == solo == osearches
    _check(tog, alo, 1e-9 if precision == 0 else 1e-6)
    _check(tog, otog, 1e-9 if precision == 0 else 1e-4)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_batched_skin_reuse_rows_equal_the_oracle(precision):
    """A batched domain reuses the Verlet-skin lists: most searches filter the
    lists of the specimens that ask (no re-sort) while the others keep their
    rows.  The specimens' masses differ, and the mixed records still take the
    four-group uniform layout (equal masses within each specimen).  After 60
    steps the rows equal the oracle's batch exactly."""
    d = gpu_domain()
    d.set("precision", precision)
    sw = batch.build_sweep(d, UNEVEN, dx=DX)
    d.prepare(sw.dt)
    d.step(60)
    assert d.geti("skin_reuse") == 1
    assert d.geti("uniform_layout") == 1
    m = d.get_array("Mass")
    assert len({float(m[a]) for a, _ in sw.ranges}) == len(UNEVEN)
    full, total = d.geti("nb_full_searches"), d.geti("nb_searches")
    assert 1 <= full < total, (full, total)
    off, idx = d.neighbours()
    searches = [d.batch_get(k, "nb_searches") for k in range(len(UNEVEN))]
    o = oracle_domain()
    osw = batch.build_sweep(o, UNEVEN, dx=DX)
    o.prepare(osw.dt)
    o.step(60)
    ooff, oidx = o.neighbours()
    assert searches == [o.batch_get(k, "nb_searches") for k in range(len(UNEVEN))]
    assert np.array_equal(off, ooff) and np.array_equal(idx, oidx)


@pytest.mark.gpu
def test_specimens_that_touch_are_rejected():
    """Two specimens side by side, their outer particles about 1.5 dx apart, share
    neighbour pairs: the first search fails the step with WF_ERR_ARG instead
    of coupling them silently."""
    from weldform_gb300 import WFError
    d = gpu_domain()
    sw = batch.build_sweep(d, [batch.Specimen(R=0.003, L=0.006, v_punch=-1.0, jc=_JC)] * 2, dx=DX)
    (a0, b0), (a1, b1) = sw.ranges
    x = d.get_array("x")
    width = x[a0:b0, 0].max() - x[a0:b0, 0].min()
    x[a1:b1] = x[a0:b0] + np.array([width + 1.5 * DX, 0.0, 0.0])  # outer particles ~1.5 dx apart
    d.set_array("x", x)
    d.prepare(sw.dt)
    with pytest.raises(WFError) as e:
        d.step(1)
    assert e.value.code == 1  # WF_ERR_ARG
    d.close()
