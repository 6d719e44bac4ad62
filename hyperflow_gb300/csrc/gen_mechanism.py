#!/usr/bin/env python3
"""Generate ``mech_h2li.h`` (constexpr mechanism tables) from a Cantera YAML file.

The reference loads ``HyperFlow_V3/H2_Li.yaml`` through Cantera at run time
(``src/BlockAMR.cpp:29``, ``src/chemistry_batch.cpp:36-37``).  The GPU kernels
need the same numbers at compile time, so this script reads the YAML text (no
PyYAML is installed) and writes them out as C++ tables.  It is run by hand
when the mechanism changes; the generated header is committed.

Units follow Cantera's defaults for a YAML file without a ``units`` block:
lengths in m, quantities in kmol, activation energies given explicitly in
cal/mol and converted here to Ea/R in K.  Molecular weights are summed from
Cantera's element weights (H 1.008, O 15.999, N 14.007, Ar 39.95).

Besides the nine species of the file, the table carries a tenth, inert ``AR``
(monatomic, cp/R = 2.5, h(298.15 K) = 0, third-body efficiency 1.0).  It is a
mechanism extension used only by workloads that ask for argon dilution; the
nine-species layout of the reference never sees it.

usage: python gen_mechanism.py PATH/TO/H2_Li.yaml > mech_h2li.h
"""
import re
import sys

ATOMIC_WEIGHT = {"H": 1.008, "O": 15.999, "N": 14.007, "Ar": 39.95}
CAL = 4.184                      # J per cal (Cantera)
GAS_CONSTANT = 8314.46261815324  # J/kmol/K (Cantera, CODATA 2018)


def parse_float_list(text):
    return [float(v) for v in re.findall(r"[-+]?\d+\.?\d*(?:[eE][-+]?\d+)?", text)]


def parse(path):
    lines = open(path).read().splitlines()
    species_order = None
    species = {}
    reactions = []
    section = None
    cur = None
    i = 0
    while i < len(lines):
        line = lines[i]
        if line.startswith("  species: [") and species_order is None:
            species_order = [s.strip() for s in line.split("[", 1)[1].rstrip("]").split(",")]
        if line.startswith("species:"):
            section = "species"
        elif line.startswith("reactions:"):
            section = "reactions"
        elif section == "species":
            m = re.match(r"- name: (\S+)", line)
            if m:
                cur = {"name": m.group(1)}
                species[cur["name"]] = cur
            elif line.strip().startswith("composition:"):
                comp = dict(re.findall(r"(\w+):\s*([\d.]+)", line.split(":", 1)[1]))
                cur["composition"] = {k: float(v) for k, v in comp.items()}
            elif line.strip().startswith("temperature-ranges:"):
                cur["ranges"] = parse_float_list(line.split(":", 1)[1])
            elif line.strip().startswith("data:"):
                # two 7-coefficient rows, each possibly wrapped over two lines
                block = ""
                j = i + 1
                while j < len(lines) and not re.match(r"\s*(transport|note|- name):?", lines[j]):
                    block += lines[j] + " "
                    j += 1
                rows = [parse_float_list(r) for r in block.split("- [")[1:]]
                cur["low"], cur["high"] = rows[0], rows[1]
                assert len(cur["low"]) == 7 and len(cur["high"]) == 7, cur["name"]
                i = j - 1
        elif section == "reactions":
            m = re.match(r"- equation: (.+)", line)
            if m:
                cur = {"equation": m.group(1).strip(), "type": "elementary", "duplicate": False}
                reactions.append(cur)
            elif line.strip().startswith("type:"):
                cur["type"] = line.split(":", 1)[1].strip()
            elif line.strip().startswith(("rate-constant:", "high-P-rate-constant:", "low-P-rate-constant:")):
                key = line.strip().split(":", 1)[0]
                body = line.split(":", 1)[1]
                A = float(re.search(r"A:\s*([-+\d.eE]+)", body).group(1))
                b = float(re.search(r"b:\s*([-+\d.eE]+)", body).group(1))
                ea = re.search(r"Ea:\s*([-+\d.eE]+)\s*(\S+?)}", body)
                assert ea.group(2) == "cal/mol", body
                cur[key] = (A, b, float(ea.group(1)) * CAL * 1000.0 / GAS_CONSTANT)
            elif line.strip().startswith("efficiencies:"):
                eff = dict(re.findall(r"(\w+):\s*([\d.eE+-]+)", line.split(":", 1)[1]))
                cur["efficiencies"] = {k: float(v) for k, v in eff.items()}
            elif line.strip().startswith("Troe:"):
                body = line.split(":", 1)[1]
                t = dict(re.findall(r"(\w+):\s*([-+\d.eE]+)", body))
                cur["troe"] = {k: float(v) for k, v in t.items()}
            elif line.strip().startswith("duplicate:"):
                cur["duplicate"] = True
        i += 1
    return species_order, species, reactions


def side(text, order):
    text = text.replace("(+ M)", "").strip()
    out = []
    third = False
    for tok in [t.strip() for t in text.split(" + ")]:
        if tok == "M":
            third = True
            continue
        m = re.match(r"(\d+)\s+(\S+)", tok)
        n, name = (int(m.group(1)), m.group(2)) if m else (1, tok)
        out += [order.index(name)] * n
    return out, third


def main():
    path = sys.argv[1]
    order, species, reactions = parse(path)
    assert order == ["H2", "O2", "H2O", "H", "O", "OH", "HO2", "H2O2", "N2"], order
    names = order + ["AR"]
    mw, low, high, tmid = [], [], [], []
    for name in order:
        s = species[name]
        mw.append(sum(ATOMIC_WEIGHT[e] * n for e, n in s["composition"].items()))
        low.append(s["low"])
        high.append(s["high"])
        tmid.append(s["ranges"][1])
    ar = [2.5, 0.0, 0.0, 0.0, 0.0, -745.375, 4.366]
    mw.append(ATOMIC_WEIGHT["Ar"])
    low.append(ar)
    high.append(ar)
    tmid.append(1000.0)

    def arr(v):
        return "{" + ", ".join(repr(float(x)) for x in v) + "}"

    out = []
    w = out.append
    w("// Generated by gen_mechanism.py from H2_Li.yaml; do not edit by hand.")
    w("// Species order and data follow HyperFlow_V3/H2_Li.yaml:9-185; reactions :187-249.")
    w("// Index 9 (AR) is an inert extension species, absent from the YAML file.")
    w("#pragma once")
    w("namespace hfmech {")
    w("constexpr int NS_FILE = 9;   // species in H2_Li.yaml")
    w("constexpr int NS_MAX = 10;   // with the inert AR extension")
    w("constexpr int NR = %d;" % len(reactions))
    w("constexpr double GAS_CONSTANT = %r;  // J/kmol/K" % GAS_CONSTANT)
    w("constexpr double ONE_ATM = 101325.0;  // Pa, NASA7 reference pressure")
    w("constexpr const char* SPECIES[NS_MAX] = {%s};" % ", ".join('"%s"' % n for n in names))
    w("constexpr double MW[NS_MAX] = %s;  // kg/kmol" % arr(mw))
    w("constexpr double T_MID[NS_MAX] = %s;" % arr(tmid))
    w("constexpr double NASA_LOW[NS_MAX][7] = {")
    for row in low:
        w("  %s," % arr(row))
    w("};")
    w("constexpr double NASA_HIGH[NS_MAX][7] = {")
    for row in high:
        w("  %s," % arr(row))
    w("};")
    w("enum : int { RXN_ELEMENTARY = 0, RXN_THREE_BODY = 1, RXN_FALLOFF = 2 };")
    w("struct Reaction {")
    w("  int type;")
    w("  int nreac, reac[3];   // reactant species, repeated by stoichiometric coefficient")
    w("  int nprod, prod[3];   // product species, repeated likewise")
    w("  double A, b, EaR;     // rate constant (high-pressure limit for falloff); Ea/R in K")
    w("  double A0, b0, Ea0R;  // low-pressure limit (falloff only)")
    w("  double troeA, troeT3, troeT1, troeT2;  // Troe parameters; troeT2 used only if hasT2")
    w("  int hasT2;")
    w("  double eff[NS_MAX];   // third-body efficiencies (1.0 where not listed)")
    w("};")
    w("constexpr Reaction RXN[NR] = {")
    for r in reactions:
        eq = r["equation"]
        assert "<=>" in eq, eq
        lhs, rhs = eq.split("<=>")
        reac, _ = side(lhs, order)
        prod, _ = side(rhs, order)
        typ = {"elementary": 0, "three-body": 1, "falloff": 2}[r["type"]]
        if typ == 2:
            A, b, EaR = r["high-P-rate-constant"]
            A0, b0, Ea0R = r["low-P-rate-constant"]
            troe = r["troe"]
        else:
            A, b, EaR = r["rate-constant"]
            A0 = b0 = Ea0R = 0.0
            troe = {"A": 0.0, "T3": 0.0, "T1": 0.0}
        eff = [1.0] * 10
        for k, v in r.get("efficiencies", {}).items():
            eff[names.index(k)] = v
        pad = lambda v: v + [0] * (3 - len(v))
        w("  // %s%s" % (eq, " (duplicate)" if r["duplicate"] else ""))
        w("  {%d, %d, {%s}, %d, {%s}, %r, %r, %r, %r, %r, %r, %r, %r, %r, %r, %d, %s}," % (
            typ, len(reac), ", ".join(map(str, pad(reac))), len(prod), ", ".join(map(str, pad(prod))),
            A, b, EaR, A0, b0, Ea0R, troe.get("A", 0.0), troe.get("T3", 0.0), troe.get("T1", 0.0),
            troe.get("T2", 0.0), int("T2" in troe), arr(eff)))
    w("};")
    w("}  // namespace hfmech")
    print("\n".join(out))


if __name__ == "__main__":
    main()
