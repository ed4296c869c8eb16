"""Parameter sweeps: many independent specimens stepped together in one domain.

Every specimen is an elastoplastic cylinder (AddCylinderLength) upset by a
prescribed top-zone velocity over a fixed bottom zone, with its own
Johnson-Cook constants and punch speed.  The specimens are laid out on a
plane grid with gaps wider than any kernel support, so no pair ever links two
specimens; one domain holds them all, so every kernel launch of a step
advances every specimen and the GPU load-balances across specimens of uneven
size for free (the unit of work is the particle, not the specimen).

Each specimen keeps the neighbour-rebuild schedule a run of it alone would
have (SolverKickDrift.cpp:153-186, 315-324): the domain is partitioned with
``Domain.batch_specimens`` (wf_batch_specimens), a search serves only the
specimens that ask for one, and the others keep their rows.  Masses are set
per specimen (AddCylinderLength, Domain.cpp:840-855, divides the last
cylinder's volume by the count of *all* particles and assigns it to every
particle; a multi-body domain needs per-body masses).  A specimen then evolves
as it does alone, up to the rounding of its coordinates' offset.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Sequence

import numpy as np

from . import JOHNSON_COOK
from .configs import Steel, SEED, jitter, cylinder_count


@dataclass
class Specimen:
    R: float
    L: float
    v_punch: float
    jc: tuple  # (A, B, n, C, eps_0, m, T_m, T_t)


@dataclass
class Sweep:
    specimens: List[Specimen]
    ranges: List[tuple]   # [first, last) particle of each specimen
    offsets: List[tuple]  # (ox, oy) of each specimen's axis
    dx: float
    h: float
    dt: float
    n: int


def random_specimens(count: int, seed: int = SEED, r_range=(0.004, 0.012), ld_range=(1.0, 2.0),
                     v_range=(0.5, 5.0), spread: float = 0.2, base: Steel = None) -> List[Specimen]:
    """Seeded specimens: radius and L/D uniform, JC constants A, B, n, C, m
    uniform within +-spread of the base material, punch speed uniform."""
    base = base or Steel()
    rng = np.random.default_rng(seed)
    out = []
    A, B, n, C, e0, m, Tm, Tt = base.jc
    for _ in range(count):
        R = float(rng.uniform(*r_range))
        L = float(2 * R * rng.uniform(*ld_range))
        f = rng.uniform(1 - spread, 1 + spread, size=5)
        v = float(rng.uniform(*v_range))
        out.append(Specimen(R=R, L=L, v_punch=-v, jc=(A * f[0], B * f[1], n * f[2], C * f[3], e0, m * f[4], Tm, Tt)))
    return out


def build_sweep(dom, specimens: Sequence[Specimen], dx: float = 0.0005, mat: Steel = None,
                jitter_amp: float = 1e-3, seed: int = SEED, cfl: float = 0.4, first_index: int = 0) -> Sweep:
    """Fill `dom` (a Domain of any library with this ABI) with the specimens.
    Specimen k's jitter is keyed by (seed + first_index + k, local particle
    index), so a specimen gets the same positions alone or inside a sweep."""
    mat = mat or Steel()
    h = 1.2 * dx
    dom.Kernel_Set(0)
    rmax = max(s.R for s in specimens)
    pitch = 2 * rmax + 6 * h
    cols = int(math.ceil(math.sqrt(len(specimens))))
    ranges, offsets = [], []
    for k, s in enumerate(specimens):
        ox, oy = (k % cols) * pitch, (k // cols) * pitch
        n0 = dom.particle_count
        dom.AddCylinderLength(0, (ox, oy, 0.0), s.R, s.L, dx / 2, mat.rho, h, False)
        ranges.append((n0, dom.particle_count))
        offsets.append((ox, oy))
    n = dom.particle_count
    x = dom.get_array("x")
    if jitter_amp:
        for k, (a, b) in enumerate(ranges):
            x[a:b] += jitter(b - a, dx, jitter_amp, seed + first_index + k)
        dom.set_array("x", x)
    mass = np.empty(n)
    ids = np.zeros(n, dtype=np.int32)
    mats = np.zeros(n, dtype=np.int32)
    nws = np.zeros(n, dtype=np.int32)
    sy = np.empty(n)
    for k, (s, (a, b)) in enumerate(zip(specimens, ranges)):
        mass[a:b] = math.pi * s.R * s.R * s.L * mat.rho / (b - a)
        A, B, nn, C, e0, m, Tm, Tt = s.jc
        mid = dom.add_material(JOHNSON_COOK, [mat.E, mat.nu, A, B, nn, C, e0, m, Tm, Tt])
        mats[a:b] = mid
        Th = (mat.T0 - Tt) / (Tm - Tt)
        sy[a:b] = (A + B * 0.0 ** nn) * (1.0 - Th ** m)  # CalcYieldStress(0, 0, T0)
        z = x[a:b, 2]
        bottom = z <= 2 * dx
        top = z >= s.L - 3 * dx
        ids[a:b][bottom] = 2
        ids[a:b][top] = 1000 + first_index + k
        nws[a:b][bottom | top] = 1
        dom.add_velocity_bc(1000 + first_index + k, (0.0, 0.0, s.v_punch))
    dom.add_velocity_bc(2, (0.0, 0.0, 0.0))
    dom.set_array("Mass", mass)
    dom.set_array("ID", ids)
    dom.set_array("not_write_surf_ID", nws)
    dom.set_array("mat", mats)
    dom.set_particles("Material_model", JOHNSON_COOK)
    dom.set_array("Sigmay", sy)
    dom.set_particles("G", mat.G)
    dom.set_particles("Cs", mat.Cs)
    dom.set_particles("Fail", 1)
    dom.set_particles("Alpha", 1.0)
    dom.set_particles("Beta", 0.0)
    dom.set_particles("T", mat.T0)
    dom.set_particles("k_T", mat.k_T)
    dom.set_particles("cp_T", mat.cp_T)
    if len(ranges) > 1:
        dom.batch_specimens(ranges)
    return Sweep(specimens=list(specimens), ranges=ranges, offsets=offsets, dx=dx, h=h, dt=cfl * h / mat.Cs, n=n)


def build_single(dom, s: Specimen, index: int, dx: float = 0.0005, mat: Steel = None, jitter_amp: float = 1e-3,
                 seed: int = SEED, cfl: float = 0.4) -> Sweep:
    """Specimen number `index` of a sweep, alone, built exactly as it appears
    inside the sweep (same positions, material, BC values)."""
    return build_sweep(dom, [s], dx=dx, mat=mat, jitter_amp=jitter_amp, seed=seed, cfl=cfl, first_index=index)


def sweep_particles(specimens: Sequence[Specimen], dx: float = 0.0005) -> int:
    return sum(cylinder_count(s.R, s.L, dx) for s in specimens)
