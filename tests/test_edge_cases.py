"""Edge cases of the search and the step: an empty domain, a smoothing length
that puts more than MAX_NB_PER_PART = 100 neighbours (Domain.h:49) in a row,
and a particle with no neighbours.  CPU tests drive the oracle; the GPU tests
run the same domains on the library and compare with the oracle."""
import numpy as np
import pytest

from tests._support import gpu_domain, oracle_domain
from weldform_gb300 import PRECISION_MIXED, WFError

E, nu, rho = 200e9, 0.3, 7850.0
G = E / (2 * (1 + nu))
CS = (E / (3 * (1 - 2 * nu)) / rho) ** 0.5
r = 0.00025


def _material(d):
    d.set_particles("G", G)
    d.set_particles("Cs", CS)
    d.set_particles("Sigmay", 300e6)
    d.set_particles("Ep", 0.0)
    d.set_particles("Fail", 1)
    d.set_particles("Alpha", 1.0)
    d.set_particles("TIInitDist", 2 * r)


def _box(d, L, h):
    d.Kernel_Set(0)
    d.AddBoxLength(0, (0.0, 0.0, 0.0), L, L, L, r, rho, h, 1, 0, False, False)
    _material(d)


def _empty(make):
    d = make()
    d.Kernel_Set(0)
    with pytest.raises(WFError) as e:
        d.prepare(1e-8)
    d.close()
    return e.value.code


def _overflow(make):
    """h = 6 r: the pair radius 2h = 12 r holds ~900 lattice neighbours."""
    d = make()
    _box(d, 0.004, 6 * r)
    with pytest.raises(WFError) as e:
        d.prepare(1e-8)
        d.neighbour_search()
        d.step(1)
    d.close()
    return e.value.code


def _isolated(make, precision=None):
    """A 4 x 4 x 4 lattice whose pair radius 2h = 0.8 x spacing holds no
    neighbour: every row is empty, so each particle keeps its velocity,
    density and zero stress.  (A lone particle is not a valid domain: its
    extent hmax gives CellNo = floor(0.5) = 0, Neighbour.cpp:75-87, which the
    library rejects with WF_ERR_ARG.)"""
    d = make()
    if precision is not None:
        d.set("precision", precision)
    _box(d, 8 * r, 0.4 * 2 * r)
    n = d.particle_count
    v = np.random.default_rng(7).uniform(-2.0, 2.0, (n, 3))
    d.set_array("v", v)
    d.prepare(1e-8)
    x0 = d.get_array("x")
    d.step(10)
    out = {f: d.get_array(f) for f in ("x", "v", "Density", "Sigma", "Nb")}
    out["x0"], out["v0"] = x0, v
    d.close()
    return out


def test_empty_domain_is_rejected_by_the_oracle():
    assert _empty(oracle_domain) == 6  # WF_ERR_STATE


def test_neighbour_cap_overflow_in_the_oracle():
    assert _overflow(oracle_domain) == 4  # WF_ERR_NBR_OVERFLOW


def test_lone_particle_is_rejected_by_the_oracle():
    d = oracle_domain()
    _box(d, 2 * r, 1.2 * 2 * r)
    assert d.particle_count == 1
    with pytest.raises(WFError) as e:
        d.prepare(1e-8)
    d.close()
    assert e.value.code == 1  # WF_ERR_ARG


def test_particles_without_neighbours_in_the_oracle():
    o = _isolated(oracle_domain)
    assert len(o["Nb"]) == 64 and not np.any(o["Nb"])
    assert np.array_equal(o["v"], o["v0"])
    assert np.allclose(o["x"] - o["x0"], 10 * 1e-8 * o["v0"], rtol=1e-9, atol=0)
    assert np.all(o["Density"] == rho)
    assert not np.any(o["Sigma"])


@pytest.mark.gpu
def test_empty_domain_is_rejected():
    assert _empty(gpu_domain) == 6


@pytest.mark.gpu
def test_neighbour_cap_overflow():
    assert _overflow(gpu_domain) == 4


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [None, PRECISION_MIXED], ids=["fp64", "mixed"])
def test_particles_without_neighbours(precision):
    o = _isolated(oracle_domain)
    g = _isolated(gpu_domain, precision)
    for f in ("x", "v", "Density", "Sigma", "Nb"):
        assert np.array_equal(g[f], o[f]), f


# ---- particles whose position is not finite --------------------------------
NAN_AT = {3: (0, np.nan), 100: (2, np.inf), 777: (1, -np.inf), 1500: (0, np.nan)}


def _nan_search(make, steps_after=0):
    """A yielding cylinder after 5 steps with four positions made non-finite
    from the host, then a neighbour search (and optionally more steps)."""
    from weldform_gb300 import configs
    d = make()
    case = configs.cylinder_upsetting(d, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
    d.prepare(case.dt)
    d.step(5)
    x = d.get_array("x")
    for p, (c, v) in NAN_AT.items():
        x[p, c] = v
    d.set_array("x", x)
    d.neighbour_search()
    out = {"nbr": d.neighbours(), "nan": d.geti("nan_particles")}
    if steps_after:
        d.step(steps_after)
        out["Sigma"] = d.get_array("Sigma")
        out["Displacement"] = d.get_array("Displacement")
        out["nbr_after"] = d.neighbours()
    d.close()
    return out


def test_oracle_nonfinite_positions_have_empty_rows():
    o = _nan_search(oracle_domain)
    off, idx = o["nbr"]
    assert o["nan"] == len(NAN_AT)
    for p in NAN_AT:
        assert off[p + 1] == off[p]
        assert not np.isin(list(NAN_AT), idx).any()


@pytest.mark.gpu
def test_nonfinite_positions_rows_match_the_oracle():
    """Rows of a search with non-finite positions equal the oracle's (the
    reference's clamped-cell binning, where CheckRadius rejects every pair
    with such a particle), and the other particles step on unaffected: their
    state after 10 more steps (two rebuilds) matches the oracle's."""
    g = _nan_search(gpu_domain, 10)
    o = _nan_search(oracle_domain, 10)
    assert g["nan"] == o["nan"] == len(NAN_AT)
    for k in ("nbr", "nbr_after"):
        assert np.array_equal(g[k][0], o[k][0]) and np.array_equal(g[k][1], o[k][1])
    keep = np.ones(len(g["Sigma"]), bool)
    keep[list(NAN_AT)] = False
    for f in ("Sigma", "Displacement"):
        a, b = g[f][keep], o[f][keep]
        assert np.isfinite(a).all()
        assert np.linalg.norm(a - b) <= 1e-9 * np.linalg.norm(b), f


@pytest.mark.gpu
def test_nan_check_raises_and_search_stays_linear():
    """With nan_check on, a non-finite position fails the next step with
    WF_ERR_NAN.  A search over a domain whose every position is NaN costs
    no more than a search of the finite domain (the reference's clamped cell
    would make it quadratic)."""
    import time
    from weldform_gb300 import configs
    d = gpu_domain()
    d.set("nan_check", 1)
    case = configs.cylinder_upsetting(d, R=0.004, L=0.008, dx=0.0005, v_top=-20.0)
    d.prepare(case.dt)
    d.step(2)
    x = d.get_array("x")
    x[10, 1] = np.nan
    d.set_array("x", x)
    with pytest.raises(WFError) as e:
        d.step(6)  # the step after the next rebuild
    assert e.value.code == 3  # WF_ERR_NAN
    d.close()

    def timed_search(all_nan):
        d = gpu_domain()
        case = configs.cylinder_upsetting(d, R=0.008, L=0.016, dx=0.0004)
        d.prepare(case.dt)
        if all_nan:
            d.set_array("x", np.full((d.particle_count, 3), np.nan))
        d.neighbour_search()
        t = time.perf_counter()
        for _ in range(3):
            d.neighbour_search()
        d.synchronize()
        dt = (time.perf_counter() - t) / 3
        n = d.geti("nan_particles")
        off, _ = d.neighbours()
        d.close()
        return dt, n, off
    t_fin, n_fin, _ = timed_search(False)
    t_nan, n_nan, off = timed_search(True)
    assert n_fin == 0 and n_nan == len(off) - 1 > 30000
    assert off[-1] == 0
    assert t_nan <= 3.0 * t_fin + 0.02, (t_nan, t_fin)
