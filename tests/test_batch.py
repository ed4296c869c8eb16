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
