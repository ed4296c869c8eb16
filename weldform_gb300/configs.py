"""Synthetic workloads of the kick-drift path, built through the Domain API.

The reference measures nothing for this path; these are the concrete cases
used for parity tests and throughput numbers:

* ``cylinder_upsetting`` — elastoplastic cylinder between a fixed bottom zone
  and a top zone driven at a prescribed velocity (the JSON driver's velocity
  BCs, Source/WeldForm.cpp:51-120), bilinear or Johnson-Cook material, cubic
  spline with h = 1.2 dx, Monaghan viscosity alpha = 1, dt = 0.4 h / Cs.
* ``contact_upsetting`` — the same cylinder pressed by a rigid plane
  (TriMesh::AxisPlaneMesh) moving down (optionally also sliding along x),
  penalty contact with Coulomb friction (Wang's 2 m / dt^2, the Fraser
  PFAC * cont_stiff law or an area penalty), Johnson-Cook flow stress,
  conduction and plastic-work heating.

Positions receive a seeded, counter-based jitter of +-1e-3 dx per coordinate
(splitmix64 of (seed, particle, axis)), identical for every implementation
that calls this module.  Every function takes the Domain to fill, so the same
case can be built on any library with this ABI.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import BILINEAR, HOLLOMON, JOHNSON_COOK, CONTACT_WANG, CONTACT_PENALTY, CONTACT_AREA

SEED = 20261203
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(z: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser on uint64 arrays (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        z = (z + np.uint64(0x9E3779B97F4A7C15)) & _M64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
        return z ^ (z >> np.uint64(31))


def jitter(n: int, dx: float, amplitude: float = 1e-3, seed: int = SEED) -> np.ndarray:
    """(n, 3) offsets U(-1, 1) * amplitude * dx from splitmix64(seed, particle, axis)."""
    idx = np.arange(3 * n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        key = (np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15)) & _M64
        z = splitmix64(key ^ idx)
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return ((2.0 * u - 1.0) * (amplitude * dx)).reshape(n, 3)


@dataclass
class Steel:
    rho: float = 7850.0
    E: float = 200e9
    nu: float = 0.3
    sy0: float = 300e6
    Et: float = 1.5e9
    # Johnson-Cook [A, B, n, C, eps_0, m, T_m, T_t]
    jc: tuple = (350e6, 275e6, 0.36, 0.022, 1.0, 1.0, 1793.0, 300.0)
    # Hollomon with plateau [K, m] (sigma_y = K (eps_p + eps0)^m past eps1,
    # eps0 = sy0 / E, eps1 = (sy0 / K)^(1/m); Material.cpp:48-64): with
    # sy0 = 300 MPa the plateau ends at eps_p = eps1 - eps0 = 9.3e-4
    hollomon: tuple = (1.0e9, 0.2)
    k_T: float = 50.0
    cp_T: float = 460.0
    T0: float = 300.0

    @property
    def K(self):
        return self.E / (3. * (1. - 2 * self.nu))

    @property
    def G(self):
        return self.E / (2. * (1. + self.nu))

    @property
    def Cs(self):
        return math.sqrt(self.K / self.rho)


@dataclass
class Case:
    dx: float
    h: float
    dt: float
    n: int
    z_top: float
    mesh: Optional[int] = None
    info: dict = field(default_factory=dict)


def cylinder_count(R: float, L: float, dx: float) -> int:
    """Particle count of AddCylinderLength (Domain.cpp:708-860) without building it."""
    r = dx / 2

    def half(xinc):
        c, yp, xp = 1, r, r + (xinc - 1) * 2. * r
        rad = math.sqrt(yp * yp + xp * xp)
        while rad <= R - r:
            yp += 2. * r
            rad = math.sqrt(yp * yp + xp * xp)
            c += 1
        return c - 1

    nxy = half(1)
    per_layer = 0
    yinc, s = nxy, -1
    for _ in range(2 * nxy):
        per_layer += 2 * half(yinc)
        yinc += s
        if yinc < 1:
            yinc, s = 1, 1
    layers, zp = 0, r
    while zp <= L - r:
        layers += 1
        zp += 2. * r
    return per_layer * layers


def dx_for_count(R: float, L: float, target: int) -> float:
    """Lattice spacing whose cylinder count is closest to target (R, L fixed)."""
    dx = (math.pi * R * R * L / target) ** (1. / 3.)
    best = (abs(cylinder_count(R, L, dx) - target), dx)
    for f in np.linspace(0.97, 1.03, 61):
        c = cylinder_count(R, L, dx * f)
        best = min(best, (abs(c - target), dx * f))
    return best[1]


def _material_setup(dom, mat: Steel, model: int):
    if model == BILINEAR:
        mid = dom.add_material(BILINEAR, [mat.E, mat.nu])
        Ep = mat.E * mat.Et / (mat.E - mat.Et)  # WeldForm.cpp:264
        dom.set_particles("Ep", Ep)
        dom.set_particles("Sigmay", mat.sy0)
    elif model == HOLLOMON:
        K, m = mat.hollomon
        mid = dom.add_material(HOLLOMON, [mat.E, mat.nu, mat.sy0, K, m])
        dom.set_particles("Material_model", HOLLOMON)
        dom.set_particles("Sigmay", mat.sy0)  # the plateau's flow stress; Ep stays 0 (Particle.cpp:78)
    else:
        A, B, n, C, e0, m, Tm, Tt = mat.jc
        mid = dom.add_material(JOHNSON_COOK, [mat.E, mat.nu, A, B, n, C, e0, m, Tm, Tt])
        dom.set_particles("Material_model", JOHNSON_COOK)
        # CalcYieldStress(0, 0, T0) as WeldForm.cpp:905-906
        Th = (mat.T0 - Tt) / (Tm - Tt)
        dom.set_particles("Sigmay", (A + B * 0.0 ** n) * 1.0 * (1.0 - Th ** m))
    dom.set_particles("mat", mid)
    dom.set_particles("G", mat.G)
    dom.set_particles("Cs", mat.Cs)
    dom.set_particles("Fail", 1)
    dom.set_particles("Alpha", 1.0)
    dom.set_particles("Beta", 0.0)
    dom.set_particles("TI", 0.0)
    dom.set_particles("k_T", mat.k_T)
    dom.set_particles("cp_T", mat.cp_T)
    dom.set_particles("T", mat.T0)


def cylinder_upsetting(dom, R: float = 0.010, L: float = 0.030, dx: float = 0.001, v_top: float = -1.0,
                       model: int = BILINEAR, mat: Optional[Steel] = None, jitter_amp: float = 1e-3,
                       seed: int = SEED, thermal: bool = False, cfl: float = 0.4,
                       V: tuple = (0.0, 0.0, 0.0)) -> Case:
    """Cylinder upsetting: bottom two layers fixed, top two layers at v_top (z).
    V is the cylinder's base centre (AddCylinderLength's V)."""
    mat = mat or Steel()
    h = 1.2 * dx
    dom.Kernel_Set(0)
    dom.AddCylinderLength(0, tuple(V), R, L, dx / 2, mat.rho, h, False)
    n = dom.particle_count
    x = dom.get_array("x")
    if jitter_amp:
        x = x + jitter(n, dx, jitter_amp, seed)
        dom.set_array("x", x)
    lo, hi = -1.0 + min(V), 1.0 + max(V)
    dom.AssignZone((lo, lo, lo), (hi, hi, V[2] + 2 * dx), 2)
    dom.AssignZone((lo, lo, V[2] + L - 3 * dx), (hi, hi, hi), 3)
    dom.add_velocity_bc(2, (0.0, 0.0, 0.0))
    dom.add_velocity_bc(3, (0.0, 0.0, v_top))
    _material_setup(dom, mat, model)
    if thermal:
        dom.set("thermal_solver", 1)
        dom.set("pl_heating", 1)
    dt = cfl * h / mat.Cs
    return Case(dx=dx, h=h, dt=dt, n=n, z_top=float(x[:, 2].max()))


def contact_upsetting(dom, R: float = 0.010, L: float = 0.030, dx: float = 0.0002, v_punch: float = -1.0,
                      mat: Optional[Steel] = None, friction: float = 0.2, stiffness: str = "wang",
                      jitter_amp: float = 1e-3, seed: int = SEED, thermal: bool = True, cfl: float = 0.4,
                      gap: float = 0.0, v_slide: float = 0.0, pfac: Optional[float] = None,
                      V: tuple = (0.0, 0.0, 0.0)) -> Case:
    """Rigid top plane pressing a Johnson-Cook cylinder with conduction and
    plastic-work heating; bottom two layers fixed.

    stiffness: "wang" (kij = 2 m / dt^2, Contact_Wang.cpp:187), "penalty"
    (kij = PFAC * cont_stiff, cont_stiff = 9 K G / (3 K + G) dS, Contact.cpp:423
    and SolverKickDrift.cpp:79-84; PFAC default 0.6, the penaltyFactor of the
    reference's contact inputs) or "area" (0.1 E / h read as a pressure per
    length times the contact area (m / rho)^(2/3)).  v_slide moves the plane
    along x as well, so the contact pairs slide and reach the dynamic-friction
    branch (Contact_Wang.cpp:284-290).  V is the cylinder's base centre."""
    mat = mat or Steel()
    h = 1.2 * dx
    dom.Kernel_Set(0)
    dom.AddCylinderLength(0, tuple(V), R, L, dx / 2, mat.rho, h, False)
    n = dom.particle_count
    x = dom.get_array("x")
    if jitter_amp:
        x = x + jitter(n, dx, jitter_amp, seed)
        dom.set_array("x", x)
    lo, hi = -1.0 + min(V), 1.0 + max(V)
    dom.AssignZone((lo, lo, lo), (hi, hi, V[2] + 2 * dx), 2)
    dom.add_velocity_bc(2, (0.0, 0.0, 0.0))
    _material_setup(dom, mat, JOHNSON_COOK)
    z_top = float(x[:, 2].max())
    half = R + 2 * dx
    dens = int(round(2 * half / dx))
    zp = z_top + h + gap  # contact engages as the plane closes the last h
    mesh = dom.add_rigid_plane(2, False, (V[0] - half, V[1] - half, zp), (V[0] + half, V[1] + half, zp), dens, 10)
    dom.add_velocity_bc(10, (v_slide, 0.0, v_punch))
    dom.set("contact", 1)
    dom.set_f64("friction_sta", friction)
    dom.set_f64("friction_dyn", friction)
    if stiffness == "wang":
        dom.set("contact_alg", CONTACT_WANG)
    elif stiffness == "penalty":
        dom.set("contact_alg", CONTACT_PENALTY)
        dom.set_f64("PFAC", 0.6 if pfac is None else pfac)
    elif stiffness == "area":  # 0.1 E / h read as a pressure per length, times the contact area
        dom.set("contact_alg", CONTACT_AREA)
        dom.set_f64("PFAC", 0.1 * mat.E / h if pfac is None else pfac)
    else:
        raise ValueError(f"unknown contact stiffness law {stiffness!r}")
    if thermal:
        dom.set("thermal_solver", 1)
        dom.set("pl_heating", 1)
    dt = cfl * h / mat.Cs
    return Case(dx=dx, h=h, dt=dt, n=n, z_top=z_top, mesh=mesh)
