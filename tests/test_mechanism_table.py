"""The kernels' compile-time mechanism table (hyperflow_gb300/csrc/mech_h2li.h, written by
gen_mechanism.py) against the numbers of the reference's mechanism file as a separate
parser read them (tests/golden/h2li_mechanism.json, from HyperFlow_V3/H2_Li.yaml by
make_reference_records.py).  The oracle and the GPU both include the generated table,
so this is the check that catches a generator error: species order, NASA7
coefficients, molecular weights from the compositions, each reaction's participants,
type, rate parameters, the cal/mol -> K conversion of the activation energies,
efficiencies and Troe parameters, and the inert AR extension."""
import json
import os
import re

import pytest

HERE = os.path.dirname(__file__)
HEADER = os.path.join(HERE, "..", "hyperflow_gb300", "csrc", "mech_h2li.h")
FIXTURE = os.path.join(HERE, "golden", "h2li_mechanism.json")

WEIGHT = {"H": 1.008, "O": 15.999, "N": 14.007, "Ar": 39.95}  # Cantera's element weights
CAL = 4.184                                                   # J per thermochemical cal
R_MOLAR = 8.31446261815324                                    # J/mol/K (CODATA 2018)


def _numbers(text):
    return [float(v) for v in re.findall(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?", text)]


def _block(text, name):
    start = text.index(name)
    body = text[text.index("{", start):]
    depth = 0
    for i, ch in enumerate(body):
        depth += ch == "{"
        depth -= ch == "}"
        if depth == 0:
            return body[:i + 1]
    raise ValueError(name)


@pytest.fixture(scope="module")
def table():
    text = open(HEADER).read()
    species = re.findall(r'"([A-Z0-9]+)"', _block(text, "SPECIES[NS_MAX]"))
    mw = _numbers(_block(text, "MW[NS_MAX]"))
    tmid = _numbers(_block(text, "T_MID[NS_MAX]"))
    low = _numbers(_block(text, "NASA_LOW[NS_MAX][7]"))
    high = _numbers(_block(text, "NASA_HIGH[NS_MAX][7]"))
    body = _block(text, "RXN[NR]")
    rows = []
    for line in body.splitlines():
        line = line.strip()
        if line.startswith("{") and len(_numbers(line)) >= 30:
            rows.append(_numbers(line))
    rxn = []
    for v in rows:
        # {type, nreac, {3}, nprod, {3}, A, b, EaR, A0, b0, Ea0R, troeA, T3, T1, T2, hasT2, {10 eff}}
        rxn.append({"type": int(v[0]), "reac": [int(x) for x in v[2:2 + int(v[1])]],
                    "prod": [int(x) for x in v[6:6 + int(v[5])]], "A": v[9], "b": v[10], "EaR": v[11],
                    "A0": v[12], "b0": v[13], "Ea0R": v[14], "troe": v[15:19], "hasT2": int(v[19]), "eff": v[20:30]})
    return {"species": species, "mw": mw, "tmid": tmid, "low": [low[7 * k:7 * k + 7] for k in range(10)],
            "high": [high[7 * k:7 * k + 7] for k in range(10)], "rxn": rxn}


@pytest.fixture(scope="module")
def yaml():
    return json.load(open(FIXTURE))


def test_species_thermo_and_weights(table, yaml):
    names = yaml["phase_species"]
    assert table["species"][:9] == names and table["species"][9] == "AR"
    by_name = {s["name"]: s for s in yaml["species"]}
    for k, name in enumerate(names):
        s = by_name[name]
        assert table["low"][k] == s["nasa7"][0] and table["high"][k] == s["nasa7"][1], name
        assert table["tmid"][k] == s["temperature_ranges"][1], name
        w = sum(n * WEIGHT[el] for el, n in s["composition"].items())
        assert table["mw"][k] == pytest.approx(w, rel=1e-14), name
    # the inert extension: monatomic argon, cp/R = 2.5 in both ranges, h(298.15 K) = 0
    assert table["mw"][9] == 39.95
    for coef in (table["low"][9], table["high"][9]):
        assert coef[:5] == [2.5, 0.0, 0.0, 0.0, 0.0]
        assert coef[5] + 2.5 * 298.15 == pytest.approx(0.0, abs=1e-9)


def _side(text, names):
    out = []
    for term in text.replace("(+ M)", "").split("+"):
        term = term.strip()
        if not term or term == "M":
            continue
        m = re.match(r"(\d+)\s*(\S+)", term)
        n, sp = (int(m.group(1)), m.group(2)) if m else (1, term)
        out += [names.index(sp)] * n
    return sorted(out)


def test_reactions(table, yaml):
    names = yaml["phase_species"]
    assert len(table["rxn"]) == len(yaml["reactions"]) == 21
    kinds = {"elementary": 0, "three-body": 1, "falloff": 2}
    for g, y in zip(table["rxn"], yaml["reactions"]):
        eq = y["equation"]
        lhs, rhs = eq.split("<=>")
        assert g["type"] == kinds[y["type"]], eq
        assert sorted(g["reac"]) == _side(lhs, names) and sorted(g["prod"]) == _side(rhs, names), eq
        k = y["rate-constant"] if y["type"] != "falloff" else y["high-P-rate-constant"]
        assert k["Ea_unit"] == "cal/mol"
        assert g["A"] == k["A"] and g["b"] == k["b"], eq  # SI (m, kmol, s): no unit block in the file
        assert g["EaR"] == pytest.approx(k["Ea"] * CAL / R_MOLAR, rel=1e-14, abs=1e-12), eq
        if y["type"] == "falloff":
            k0 = y["low-P-rate-constant"]
            assert g["A0"] == k0["A"] and g["b0"] == k0["b"], eq
            assert g["Ea0R"] == pytest.approx(k0["Ea"] * CAL / R_MOLAR, rel=1e-14, abs=1e-12), eq
            troe = y["Troe"]
            assert g["troe"][:3] == [troe["A"], troe["T3"], troe["T1"]], eq
            assert g["hasT2"] == (1 if "T2" in troe else 0), eq
        if y["type"] in ("three-body", "falloff"):
            eff = y.get("efficiencies", {})
            assert g["eff"][:9] == [eff.get(n, 1.0) for n in names], eq
            assert g["eff"][9] == 1.0, eq  # the inert extension collides like the default
