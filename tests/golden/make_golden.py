"""Extract the reference's recorded neighbour table into a JSON fixture.

Docs/reduction.txt:28-37 of the WeldForm tree holds the Nishimura tables
(Anei) that the reference printed for particle 2000 of its cylinder
compression example (R = 0.15, L = 0.56, dx = 0.015, h = 1.2 dx, cylinder
shifted by -L/10 and lengthened by 2L/10, examples/CompressionVel.cpp:90-124).
Row entries 0..ipairs-1 are the j > i neighbours, entries 99..100-jpairs the
j < i neighbours.  Run in a tree where the reference is mounted:

    python tests/golden/make_golden.py /path/to/WeldForm
"""
import json
import os
import re
import sys


def main(ref_root: str):
    txt = open(os.path.join(ref_root, "Docs", "reduction.txt")).read()
    m = re.search(r"Particle i: (\d+)\s+Nb Count (\d+)\s+ipairs: (\d+)\s+jpairs: (\d+).*?Nb list\s+([\d,\s]+)Ref list", txt, re.S)
    pid, nb, ip, jp = (int(m.group(k)) for k in range(1, 5))
    row = [int(v) for v in m.group(5).replace("\n", " ").split(",") if v.strip()]
    assert len(row) == 100, len(row)
    jgt = row[:ip]
    jlt = [row[99 - n] for n in range(jp)]
    out = {
        "source": "Docs/reduction.txt:28-37 (WeldForm)",
        "case": {"R": 0.15, "L": 0.56, "dx": 0.015, "hfac": 1.2, "V": [0.0, 0.0, -0.056], "Lz": 0.672,
                 "DomMax.x": 0.56, "DomMin.x": -0.56, "rho": 2700.0},
        "particle": pid, "Nb": nb, "ipairs": ip, "jpairs": jp,
        "j_greater": jgt, "j_smaller": jlt,
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reduction_particle2000.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <WeldForm source tree>")
    main(sys.argv[1])
