"""The oracle's FP64 tangent-linear run (the reference for the GPU adjoint)
against the oracle's own central finite differences, on small contact cases.

The tangent run restates the step on dual numbers; its value parts must
reproduce the oracle's doubles exactly (tangent_mismatch == 0), and its
gradient must match central differences of the oracle's loss (relative step
1e-6, FP64) to 1e-4 on every parameter the loss depends on (the differences
themselves carry ~1e-5 of rounding noise on the smallest sensitivities)."""
import os

import numpy as np
import pytest

from tests._support import oracle_domain
from weldform_gb300 import BILINEAR, JOHNSON_COOK, PARAMS
from weldform_gb300 import adjoint as adj

THREADS = min(os.cpu_count() or 1, 8)


def _oracle():
    d = oracle_domain()
    d.set("cpu_threads", THREADS)
    return d


def _tangent(case, steps, every, target):
    d = _oracle()
    mesh = adj.build(d, case, case.nominal())
    d.prepare(case.dt)
    r = d.adjoint_reaction_loss(steps, every, target, mesh=mesh)
    mm = d.get("tangent_mismatch")
    d.close()
    return r, mm


def _check(case, steps, every, must):
    target = adj.perturbed_jc_target(case, steps, every, make=_oracle) * 0.9
    r, mm = _tangent(case, steps, every, target)
    assert mm == 0.0, f"tangent values differ from the oracle by {mm:.3e}"
    prob = adj.Problem(case, steps, every, target, make=_oracle)
    g = r["grad"] * prob.scl * prob.norm
    fd = adj.central_fd(prob)
    for p in must:
        k = PARAMS.index(p)
        assert abs(fd[k]) > 0, p
        assert abs(g[k] - fd[k]) <= 1e-4 * abs(fd[k]), (p, g[k], fd[k])
    scale = np.abs(fd).max()
    for k, p in enumerate(PARAMS):  # the rest (zero or tiny sensitivities) agree in absolute terms
        assert abs(g[k] - fd[k]) <= 1e-6 * scale, (p, g[k], fd[k])
    return g, fd


def test_tangent_matches_fd_johnson_cook_thermal_area_contact():
    case = adj.ContactCase(R=0.0025, L=0.005, dx=0.0005, v_punch=-20.0, model=JOHNSON_COOK, thermal=True,
                           stiffness="area")
    _check(case, 40, 5, ("E", "A", "B", "n", "C", "PFAC"))


def test_tangent_matches_fd_bilinear_wang_contact():
    case = adj.ContactCase(R=0.0025, L=0.005, dx=0.0005, v_punch=-20.0, model=BILINEAR, thermal=False,
                           stiffness="wang")
    _check(case, 40, 5, ("E", "sy0", "Ep"))


def test_tangent_rejects_reference_mode():
    case = adj.ContactCase(R=0.002, L=0.004, dx=0.0005)
    d = _oracle()
    d.set("cpu_mode", 1)
    mesh = adj.build(d, case, case.nominal())
    d.prepare(case.dt)
    with pytest.raises(Exception):
        d.adjoint_reaction_loss(10, 5, np.zeros(2), mesh=mesh)
    d.close()
