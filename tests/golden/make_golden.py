"""Extract the reference's recorded outputs into JSON fixtures.

1. reduction_particle2000.json — Docs/reduction.txt:28-37 of the WeldForm tree holds the Nishimura tables
(Anei) that the reference printed for particle 2000 of its cylinder
compression example (R = 0.15, L = 0.56, dx = 0.015, h = 1.2 dx, cylinder
shifted by -L/10 and lengthened by 2L/10, examples/CompressionVel.cpp:90-124).
Row entries 0..ipairs-1 are the j > i neighbours, entries 99..100-jpairs the
j < i neighbours.

2. contact_compression_fraser.json — the input deck
examples/input/Contact_Compression.json (a 0.3 x 0.616 aluminium cylinder,
bilinear hardening, upset by a rigid plane at 1 m/s with Wang penalty
contact, solver "Mech-Fraser") and the integrals that WeldForm v0.4.2.4
(commit 331c3a8e) printed at each of its 101 outputs in
examples/input/Contact_Compression.out (SolverFraser.cpp:440-470): step,
time step, maximum plastic strain, maximum displacement per axis (taken
before that step's update, SolverFraser.cpp:151-159), contact force and
reaction sums, external work, internal and kinetic energy, each with the 6
significant digits of the log.

3. reference_decks.json — the reference's example input decks
(examples/input/*.json) that the JSON front-end accepts: 3D Cartesian
domains, Nishimura sums, no damage, no mesh files, no pure-thermal solver.

Run in a tree where the reference is mounted:

    python tests/golden/make_golden.py /path/to/WeldForm
"""
import json
import os
import re
import sys


def reduction_table(ref_root: str):
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


# A printed Vec3_t: each field %g with 6 significant digits, right-aligned in
# at least 10 characters, so neighbouring fields can touch
# ("0.000134010.000134010.00189624").  A token is a piece that %g prints back
# unchanged; the split into three must be unique.
def _splits(s: str):
    if not s:
        return [[]]
    out = []
    for i in range(1, len(s) + 1):
        t = s[:i]
        try:
            ok = "%g" % float(t) == t
        except ValueError:
            ok = False
        if ok:
            out += [[t] + rest for rest in _splits(s[i:])]
    return out


def _vec3(s: str):
    ways = [[]]
    for part in s.split():
        ways = [w + x for w in ways for x in _splits(part)]
    ways = [w for w in ways if len(w) == 3]
    assert len(ways) == 1, (s, ways)
    return [float(t) for t in ways[0]]


def fraser_log(ref_root: str):
    base = os.path.join(ref_root, "examples", "input", "Contact_Compression")
    deck = json.load(open(base + ".json"))
    log = open(base + ".out").read()
    head = re.search(r"v\. ([\d.]+) -+\s*\n-+ (\d+) -+\s*\n-- ([0-9a-f]+) --", log)
    rows = []
    for blk in log.split("step number: ")[1:]:
        row = {"step": int(blk.split("\n", 1)[0])}
        row["dt"] = float(re.search(r"Current Time Step = (\S+)", blk).group(1))
        m = re.search(r"Max plastic strain: (\S+?)in particle(\d+)", blk)
        row["max_pl"] = float(m.group(1))
        row["max_disp"] = _vec3(re.search(r"Max Displacements \(No Cont Surf\): 3 \[(.*?)\]", blk).group(1))
        m = re.search(r"Contact Force Sum (\S+), Reaction Sum (\S+)", blk)
        row["contact_force_sum"], row["contact_reaction_sum"] = float(m.group(1)), float(m.group(2))
        row["ext_forces_work"] = float(re.search(r"External Forces Work (\S+)", blk).group(1))
        m = re.search(r"Int Energy: (\S+), Kin Energy: (\S+)", blk)
        row["int_energy_sum"], row["kin_energy_sum"] = float(m.group(1)), float(m.group(2))
        assert row["max_disp"][0] == row["max_disp"][1], row
        rows.append(row)
    out = {
        "source": "examples/input/Contact_Compression.json and .out (WeldForm v%s, %s, commit %s)"
                  % (head.group(1), head.group(2), head.group(3)),
        "deck": deck,
        "outputs": rows,
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "contact_compression_fraser.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path, len(rows), "outputs")


DECKS = ("Cantilever", "Compression", "Compression_fast_short", "Compression_thermal", "Contact_Compression",
         "Contact_Compression_Fraser", "Contact_Compression_JC", "Contact_Compression_Rot",
         "Contact_Compression_Rot_JC", "Contact_Compression_Wang", "Impact_Campos", "Traction")


def decks(ref_root: str):
    out = {"source": "examples/input/<name>.json (WeldForm)",
           "decks": {n: json.load(open(os.path.join(ref_root, "examples", "input", n + ".json"))) for n in DECKS}}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_decks.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path, len(DECKS), "decks")


def main(ref_root: str):
    reduction_table(ref_root)
    fraser_log(ref_root)
    decks(ref_root)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <WeldForm source tree>")
    main(sys.argv[1])
