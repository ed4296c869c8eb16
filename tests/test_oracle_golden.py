"""The oracle against the reference's own recorded neighbour table.

Docs/reduction.txt:28-37 lists the Nishimura neighbour tables of particle 2000
in the reference's CompressionVel-style cylinder (12,144 particles).  The
oracle's generator (AddCylinderLength) and linked-list cell search must
reproduce that set exactly: 28 neighbours with larger index, 27 with smaller.
"""
import json
import os

import pytest

from tests._support import oracle_domain

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reduction_particle2000.json")


@pytest.mark.parametrize("dom_override", [True, False])
def test_reference_neighbour_table_particle_2000(dom_override):
    g = json.load(open(GOLDEN))
    c = g["case"]
    d = oracle_domain()
    d.Kernel_Set(0)
    d.AddCylinderLength(1, c["V"], c["R"], c["Lz"], c["dx"] / 2.0, c["rho"], c["dx"] * c["hfac"], False)
    if dom_override:  # CompressionVel.cpp:117-118
        d.set_f64("DomMax.x", c["DomMax.x"])
        d.set_f64("DomMin.x", c["DomMin.x"])
    assert d.particle_count == 12144
    d.prepare(1e-7)
    d.neighbour_search()
    off, idx = d.neighbours()
    p = g["particle"]
    row = list(idx[off[p]:off[p + 1]])
    assert len(row) == g["Nb"]
    up = [j for j in row if j > p]
    dn = [j for j in row if j < p]
    assert len(up) == g["ipairs"] and len(dn) == g["jpairs"]
    assert sorted(up) == sorted(g["j_greater"])
    assert sorted(dn) == sorted(g["j_smaller"])
    # canonical row order: j > i ascending, then j < i ascending
    assert row == sorted(up) + sorted(dn)
    nb = d.get_array("Nb")
    assert nb[p] == 55
