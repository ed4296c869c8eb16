"""Reaction-force loss and its gradient with respect to material and contact parameters.

A rigid plane (TriMesh::AxisPlaneMesh) presses a cylinder; the loss is the
mean squared difference between the plane's reaction force F_z, sampled every
``every`` steps, and a target curve.  ``Domain.adjoint_reaction_loss`` returns
its gradient with respect to ``PARAMS`` = (E, sy0, Ep, A, B, n, C, m, mu,
PFAC) from the library's reverse-mode adjoint of the plain FP64 step
(checkpoint and recompute every k steps).

``build`` makes the parameter dependence explicit, exactly as the adjoint
differentiates it: G = E / (2 (1 + nu)) and Cs = sqrt(E / (3 (1 - 2 nu) rho))
on every particle, the time step fixed by the nominal E, Ep and the initial
Sigmay (bilinear: sy0; Johnson-Cook: CalcYieldStress(0, 0, T0)) set from the
parameters, friction_sta = friction_dyn = mu, and the contact stiffness factor
PFAC (contact_alg 2: k = PFAC (m / rho)^(2/3), with the nominal
PFAC = 0.1 E / h of the penalty-contact workload; contact_alg 1, the Fraser
law: k = PFAC * 9 K G / (3 K + G) dS, nominal PFAC = 0.6).  ``v_slide`` moves
the plane along x as well, so sliding contact pairs take the dynamic-friction
branch, the only one through which the loss depends on mu.

``ReactionLoss`` wraps the loss and the adjoint gradient as a
``torch.autograd.Function`` of dimensionless offsets u (theta = theta0 +
u * scale) for checking with ``torch.autograd.gradcheck``.

    python -m weldform_gb300.adjoint [--dx-mm 0.55] [--steps 400] [--every 10]
        [--v-punch -20] [--k 10,20,50] [--fd] [--stencil E,A] [--stencil-points 8]
        [--scan E] [--freeze-topology]

prints one JSON line: loss, adjoint gradient for every k, the wall time of a
plain forward run and of the adjoint (forward with checkpoints, reverse
sweep), with --fd the central finite differences (relative step 1e-6), and
with --stencil the central differences of the named parameters beside the
mean of the adjoint derivative over the same stencil, and with --scan the loss
at 21 points across relative offsets [-1e-5, 1e-5] of one parameter with its
residual from the adjoint's linear model.  --freeze-topology runs every
forward pass with the neighbour rows, contact pairs and surface flags of the
first step's search (the topology the adjoint holds fixed within each step is
then also fixed across steps), so finite differences see no search decision.
"""
from __future__ import annotations

import argparse
import json
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import BILINEAR, CONTACT_AREA, CONTACT_PENALTY, CONTACT_WANG, JOHNSON_COOK, PARAMS, Domain, PRECISION_FP64
from .configs import SEED, Steel, jitter


@dataclass
class ContactCase:
    """Cylinder pressed by a rigid plane; the penalty-contact workload with
    JC hardening, conduction and plastic-work heating (R = 10 mm, L = 30 mm,
    dx = 0.55 mm gives 53,352 particles)."""
    R: float = 0.010
    L: float = 0.030
    dx: float = 0.00055
    v_punch: float = -20.0
    model: int = JOHNSON_COOK
    thermal: bool = True
    stiffness: str = "area"
    gap: float = 0.0
    mat: Steel = field(default_factory=Steel)
    friction: float = 0.2
    jitter_amp: float = 1e-3
    seed: int = SEED
    cfl: float = 0.4
    freeze: bool = False  # topology searched only at the first step (library option "freeze_neighbours")
    alpha: float = 1.0    # Monaghan viscosity Alpha of every particle
    v_slide: float = 0.0  # plane velocity along x: sliding pairs reach the dynamic-friction branch

    @property
    def h(self) -> float:
        return 1.2 * self.dx

    @property
    def dt(self) -> float:
        return self.cfl * self.h / self.mat.Cs

    def nominal(self) -> np.ndarray:
        m = self.mat
        A, B, n, C, e0, mm, Tm, Tt = m.jc
        Ep = m.E * m.Et / (m.E - m.Et) if self.model == BILINEAR else 0.0
        # PFAC: the Fraser law's dimensionless factor (0.6, the reference inputs'
        # penaltyFactor) or the area law's pressure per length 0.1 E / h
        pfac = 0.6 if self.stiffness == "penalty" else 0.1 * m.E / self.h
        return np.array([m.E, m.sy0, Ep, A, B, n, C, mm, self.friction, pfac])

    def scale(self) -> np.ndarray:
        """Step sizes for parameters whose nominal value is 0 (Ep of JC particles)."""
        th = self.nominal()
        s = np.abs(th)
        s[s == 0.0] = self.mat.E / (2.0 * (1.0 + self.mat.nu)) * 1e-3
        return s


def build(dom, case: ContactCase, theta) -> int:
    """Fill `dom` with the case at parameters theta (PARAMS order); returns the mesh id."""
    E, sy0, Ep, A, B, n, C, m, mu, pfac = [float(t) for t in theta]
    mat = case.mat
    h = case.h
    dom.Kernel_Set(0)
    dom.AddCylinderLength(0, (0.0, 0.0, 0.0), case.R, case.L, case.dx / 2, mat.rho, h, False)
    npart = dom.particle_count
    x = dom.get_array("x")
    if case.jitter_amp:
        x = x + jitter(npart, case.dx, case.jitter_amp, case.seed)
        dom.set_array("x", x)
    dom.AssignZone((-1.0, -1.0, -1.0), (1.0, 1.0, 2 * case.dx), 2)
    dom.add_velocity_bc(2, (0.0, 0.0, 0.0))
    _, _, _, _, e0, _, Tm, Tt = mat.jc
    if case.model == JOHNSON_COOK:
        mid = dom.add_material(JOHNSON_COOK, [E, mat.nu, A, B, n, C, e0, m, Tm, Tt])
        dom.set_particles("Material_model", JOHNSON_COOK)
        Th = (mat.T0 - Tt) / (Tm - Tt)
        dom.set_particles("Sigmay", (A + B * 0.0 ** n) * 1.0 * (1.0 - Th ** m))
    else:
        mid = dom.add_material(BILINEAR, [E, mat.nu])
        dom.set_particles("Sigmay", sy0)
    dom.set_particles("Ep", Ep)
    dom.set_particles("mat", mid)
    dom.set_particles("G", E / (2. * (1. + mat.nu)))
    dom.set_particles("Cs", math.sqrt(E / (3. * (1. - 2 * mat.nu)) / mat.rho))
    dom.set_particles("Fail", 1)
    dom.set_particles("Alpha", case.alpha)
    dom.set_particles("Beta", 0.0)
    dom.set_particles("k_T", mat.k_T)
    dom.set_particles("cp_T", mat.cp_T)
    dom.set_particles("T", mat.T0)
    z_top = float(x[:, 2].max())
    half = case.R + 2 * case.dx
    dens = int(round(2 * half / case.dx))
    zp = z_top + h + case.gap
    mesh = dom.add_rigid_plane(2, False, (-half, -half, zp), (half, half, zp), dens, 10)
    dom.add_velocity_bc(10, (case.v_slide, 0.0, case.v_punch))
    dom.set("contact", 1)
    dom.set_f64("friction_sta", mu)
    dom.set_f64("friction_dyn", mu)
    if case.stiffness == "wang":
        dom.set("contact_alg", CONTACT_WANG)
    elif case.stiffness == "penalty":
        dom.set("contact_alg", CONTACT_PENALTY)
        dom.set_f64("PFAC", pfac)
    elif case.stiffness == "area":
        dom.set("contact_alg", CONTACT_AREA)
        dom.set_f64("PFAC", pfac)
    else:
        raise ValueError(f"unknown contact stiffness law {case.stiffness!r}")
    if case.thermal:
        dom.set("thermal_solver", 1)
        dom.set("pl_heating", 1)
    if case.freeze:
        dom.set("freeze_neighbours", 1)
    return mesh


def reaction_curve(dom, steps: int, every: int, mesh: int = 0, axis: int = 2) -> np.ndarray:
    """Forward run: the reaction force after every `every` steps."""
    out = []
    for _ in range(steps // every):
        dom.step(every)
        out.append(dom.contact_force(mesh)[axis])
    return np.array(out)


def perturbed_jc_target(case: ContactCase, steps: int, every: int, make=None, sigma: float = 0.05,
                        seed: int = SEED) -> np.ndarray:
    """Target curve: the forward model at the JC constants A, B, n, C, m each
    scaled by (1 + N(0, sigma)) with a fixed seed."""
    rng = np.random.default_rng(seed)
    th = case.nominal().copy()
    th[3:8] *= 1.0 + rng.normal(0.0, sigma, size=5)
    d = (make or Domain)()
    mesh = build(d, case, th)
    d.prepare(case.dt)
    c = reaction_curve(d, steps, every, mesh)
    d.close()
    return c


class Problem:
    """A reaction-force loss at theta = theta0 + u * scale, for ReactionLoss."""

    def __init__(self, case: ContactCase, steps: int, every: int, target, checkpoint_every: int = 20,
                 make=None):
        self.case, self.steps, self.every = case, steps, every
        self.target = np.asarray(target, dtype=np.float64)
        self.k = checkpoint_every
        self.make = make or Domain
        self.theta0 = case.nominal()
        self.scl = case.scale()
        self.norm = 1.0 / max(float(np.mean(self.target ** 2)), 1e-300)

    def theta(self, u) -> np.ndarray:
        return self.theta0 + np.asarray(u, dtype=np.float64) * self.scl

    def loss_grad(self, u):
        d = self.make()
        d.set("precision", PRECISION_FP64)
        mesh = build(d, self.case, self.theta(u))
        d.prepare(self.case.dt)
        r = d.adjoint_reaction_loss(self.steps, self.every, self.target, mesh=mesh, checkpoint_every=self.k)
        d.close()
        return r["loss"] * self.norm, r["grad"] * self.scl * self.norm

    def loss(self, u) -> float:
        d = self.make()
        mesh = build(d, self.case, self.theta(u))
        d.prepare(self.case.dt)
        c = reaction_curve(d, self.steps, self.every, mesh)
        d.close()
        return float(np.mean((c - self.target) ** 2)) * self.norm


def _autograd_function():
    import torch

    class ReactionLoss(torch.autograd.Function):
        """loss(u) with the adjoint gradient; u: float64 tensor of len(PARAMS)."""

        @staticmethod
        def forward(ctx, u, problem):
            loss, grad = problem.loss_grad(u.detach().cpu().numpy())
            ctx.save_for_backward(torch.as_tensor(grad, dtype=u.dtype))
            return torch.tensor(loss, dtype=u.dtype)

        @staticmethod
        def backward(ctx, gout):
            (g,) = ctx.saved_tensors
            return gout * g, None

    return ReactionLoss


def __getattr__(name):
    if name == "ReactionLoss":
        return _autograd_function()
    raise AttributeError(name)


def central_fd(problem: Problem, rel: float = 1e-6, only=None) -> np.ndarray:
    """Central differences of the (scaled) loss in u, step rel * theta0 / scale.
    A parameter whose nominal value is 0 (Ep of Johnson-Cook particles) gets a
    forward difference: a negative Ep is replaced by E in the step
    (Particle.cpp:1012-1013), a jump no difference may straddle.  ``only``
    (parameter names) restricts the differences to those; the rest stay 0."""
    g = np.zeros(len(PARAMS))
    base = None
    for p in range(len(PARAMS)):
        if only is not None and PARAMS[p] not in only:
            continue
        du = np.zeros(len(PARAMS))
        if problem.theta0[p] != 0:
            step = rel * abs(problem.theta0[p]) / problem.scl[p]
            du[p] = step
            g[p] = (problem.loss(du) - problem.loss(-du)) / (2 * step)
        else:
            if base is None:
                base = problem.loss(du)
            du[p] = rel
            g[p] = (problem.loss(du) - base) / rel
    return g


def stencil_mean_adjoint(problem: Problem, p: int, rel: float = 1e-6, points: int = 8) -> float:
    """Mean of the adjoint derivative dL/du_p over the central-difference
    stencil of ``central_fd`` at the same relative step (midpoint rule over
    ``points`` nodes).

    The step is piecewise smooth in every parameter: each particle's
    elastic-plastic transition and each pair's viscosity switch is a kink.
    For a loss that is continuous and piecewise smooth in u_p,
    (L(+s) - L(-s)) / (2 s) is exactly the mean of dL/du_p over [-s, +s];
    a kink inside the stencil separates the central difference from the
    derivative at the centre, not from this mean.  Comparing the two checks
    the adjoint against finite differences without the kink error."""
    step = rel * abs(problem.theta0[p]) / problem.scl[p]
    acc = 0.0
    for k in range(points):
        du = np.zeros(len(PARAMS))
        du[p] = -step + (2 * k + 1) * step / points
        acc += problem.loss_grad(du)[1][p]
    return acc / points


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dx-mm", type=float, default=0.55)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--every", type=int, default=10)
    ap.add_argument("--v-punch", type=float, default=-20.0)
    ap.add_argument("--k", default="10,20,50")
    ap.add_argument("--fd", action="store_true")
    ap.add_argument("--jc-n", type=float, default=None, help="Johnson-Cook hardening exponent of the workload")
    ap.add_argument("--alpha", type=float, default=1.0, help="artificial viscosity Alpha of the workload")
    ap.add_argument("--friction", type=float, default=0.2, help="friction coefficient of the workload")
    ap.add_argument("--freeze-topology", action="store_true",
                    help="search neighbours and contact pairs only at the first step, for every run")
    ap.add_argument("--stencil", default="", help="parameters (e.g. E,A) whose stencil-mean adjoint is "
                    "compared with central differences at relative steps 1e-5 and 1e-6")
    ap.add_argument("--stencil-points", type=int, default=8)
    ap.add_argument("--scan", default="", help="parameter (e.g. E) whose loss is sampled at 21 points across "
                    "relative offsets [-1e-5, 1e-5], with the residual from the adjoint's linear model")
    a = ap.parse_args()
    case = ContactCase(dx=a.dx_mm * 1e-3, v_punch=a.v_punch, freeze=a.freeze_topology, alpha=a.alpha,
                       friction=a.friction)
    if a.jc_n is not None:
        jc = list(case.mat.jc)
        jc[2] = a.jc_n
        case.mat = Steel(jc=tuple(jc))
    target = perturbed_jc_target(case, a.steps, a.every)
    th0 = case.nominal()
    # plain forward time of the same run (FP64 form, CUDA graph)
    d = Domain()
    mesh = build(d, case, th0)
    d.prepare(case.dt)
    n = d.particle_count
    d.checkpoint_save(0)
    d.step(1)
    d.checkpoint_restore(0)
    fwd_plain_ms, _ = d.step_timed(a.steps)
    d.checkpoint_restore(0)
    runs = {}
    for k in [int(s) for s in a.k.split(",")]:
        t = time.perf_counter()
        r = d.adjoint_reaction_loss(a.steps, a.every, target, mesh=mesh, checkpoint_every=k)
        wall = (time.perf_counter() - t) * 1e3
        d.checkpoint_restore(0)
        runs[k] = {"loss": r["loss"], "grad": r["grad"].tolist(), "fwd_ms": r["fwd_ms"], "adj_ms": r["adj_ms"],
                   "wall_ms": wall, "adjoint_over_forward": r["adj_ms"] / fwd_plain_ms,
                   "gradient_over_forward": (r["fwd_ms"] + r["adj_ms"]) / fwd_plain_ms}
    d.close()
    out = {"particles": n, "steps": a.steps, "every": a.every, "v_punch": a.v_punch, "params": list(PARAMS),
           "theta0": th0.tolist(), "forward_ms": fwd_plain_ms, "adjoint": runs}
    if a.fd:
        prob = Problem(case, a.steps, a.every, target)
        fd = central_fd(prob)
        k0 = min(runs)
        adj = np.array(runs[k0]["grad"]) * prob.scl * prob.norm
        out["fd_scaled"] = fd.tolist()
        out["adjoint_scaled"] = adj.tolist()
        big = np.abs(fd) > 1e-6 * np.abs(fd).max()
        out["fd_rel_err"] = [float(abs(adj[p] - fd[p]) / abs(fd[p])) if big[p] else None for p in range(len(PARAMS))]
    if a.stencil:
        prob = Problem(case, a.steps, a.every, target)
        centre = prob.loss_grad(np.zeros(len(PARAMS)))[1]
        st = {}
        for name in a.stencil.split(","):
            p = PARAMS.index(name)
            for rel in (1e-5, 1e-6):
                step = rel * abs(prob.theta0[p]) / prob.scl[p]
                du = np.zeros(len(PARAMS))
                du[p] = step
                fd = (prob.loss(du) - prob.loss(-du)) / (2 * step)
                mean = stencil_mean_adjoint(prob, p, rel, a.stencil_points)
                st[f"{name}@{rel:g}"] = {"fd": fd, "adjoint_centre": float(centre[p]), "adjoint_stencil_mean": mean,
                                         "centre_rel_err": abs(centre[p] - fd) / abs(fd),
                                         "stencil_rel_err": abs(mean - fd) / abs(fd)}
        out["stencil"] = st
    if a.scan:
        prob = Problem(case, a.steps, a.every, target)
        p = PARAMS.index(a.scan)
        l0, g0 = prob.loss_grad(np.zeros(len(PARAMS)))
        pts = []
        for k in range(-10, 11):
            rel = k * 1e-6
            du = np.zeros(len(PARAMS))
            du[p] = rel * abs(prob.theta0[p]) / prob.scl[p]
            lk = prob.loss(du)
            pts.append({"rel": rel, "loss": lk, "residual": lk - l0 - g0[p] * du[p]})
        out["scan"] = {"param": a.scan, "loss0": l0, "adjoint": float(g0[p]), "points": pts}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
