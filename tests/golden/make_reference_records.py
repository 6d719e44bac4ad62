"""Writes reference_records.json: the run outcomes that HyperFlow V3 records for its own
checks (HyperFlow_V3/docs/case_checks.json and docs/amr_checks.json), reduced to the
fields the oracle and GPU tests compare with; reference_cases.json: the keys of its
two smoke case configurations (cases/*/smoke.json) that the case loader reads; and
h2li_mechanism.json: the numbers of its mechanism file (H2_Li.yaml: species order,
compositions, NASA7 ranges and coefficients; each reaction's equation, type, rate
parameters as written, efficiencies, Troe parameters), read by a parser of its own so
that a test can check the generated kernel tables against them independently.  Run
where the reference tree is present, with its HyperFlow_V3 directory as the one required
argument:

    python tests/golden/make_reference_records.py <reference tree>/HyperFlow_V3
"""
import json
import os
import sys

FIELDS = {
    ("case_checks.json", "cases", "sun_cj"): ["final_time_s", "steps", "retries", "dx_min_m", "dy_min_m",
                                              "initial_hotspot_volume_m3", "mass_relative_change",
                                              "energy_relative_change"],
    ("case_checks.json", "cases", "teng_case1"): ["final_time_s", "steps", "retries", "dx_min_m", "dy_min_m"],
    ("amr_checks.json", "tests", "moving_refine_coarsen"): ["steps"],
    ("amr_checks.json", "tests", "uniform_local_amr"): ["leaf_cells"],
    ("amr_checks.json", "tests", "zero_dimensional_cvode"): ["chemistry_cell_calls", "expected_leaf_calls",
                                                             "relative_temperature_error", "max_absolute_Y_error"],
    ("amr_checks.json", "tests", "blast2d_inert"): ["steps", "transpose_pressure_error"],
    ("amr_checks.json", "tests", "blast2d_reacting"): ["peak_radical_mass_fraction", "steps", "retries",
                                                       "first_order_stages"],
}


# the keys of a case configuration that hyperflow_gb300.case reads
CASE_KEYS = {"problem", "T0", "P0", "u0", "v0", "hot_T", "hot_P", "hotspot_width", "inflow_speed", "wedge_angle_deg",
             "wedge_start", "base_cells", "length", "origin", "periodic", "boundary_lo", "boundary_hi", "cfl",
             "end_time", "output_times", "chemistry", "max_level", "tag_buffer", "regrid_interval", "max_grid_size",
             "pressure_tag", "temperature_tag", "fuel_rate_tag", "tag_box", "tag_mode", "tag_velocity", "adaptive",
             "center", "radius", "sigma", "amplitude", "initial_subsamples", "interface"}


def _flow_map(text):
    """'{A: 1.0, b: -0.5, Ea: 3.0 cal/mol}' -> {"A": 1.0, "b": -0.5, "Ea": 3.0, "Ea_unit": "cal/mol"}"""
    body = text.strip()
    assert body[0] == "{" and body[-1] == "}", text
    out = {}
    for item in body[1:-1].split(","):
        k, v = item.split(":", 1)
        parts = v.split()
        out[k.strip()] = float(parts[0])
        if len(parts) > 1:
            out[k.strip() + "_unit"] = " ".join(parts[1:])
    return out


def mechanism(path):
    text = open(path).read()
    lines = text.splitlines()
    phase_species = None
    species, reactions = [], []
    section = None
    i = 0
    while i < len(lines):
        line = lines[i]
        stripped = line.strip()
        if line.startswith("phases:"):
            section = "phases"
        elif line.startswith("species:"):
            section = "species"
        elif line.startswith("reactions:"):
            section = "reactions"
        elif section == "phases" and stripped.startswith("species:") and phase_species is None:
            phase_species = [t.strip() for t in stripped.split("[", 1)[1].rstrip("]").split(",")]
        elif section == "species" and line.startswith("- name:"):
            species.append({"name": stripped.split(":", 1)[1].strip(), "nasa7": []})
        elif section == "species" and stripped.startswith("composition:"):
            species[-1]["composition"] = _flow_map(stripped.split(":", 1)[1])
        elif section == "species" and stripped.startswith("temperature-ranges:"):
            species[-1]["temperature_ranges"] = [float(t) for t in stripped.split("[", 1)[1].rstrip("]").split(",")]
        elif section == "species" and stripped.startswith("- [") and "temperature_ranges" in species[-1]:
            buf = stripped[2:]
            while "]" not in buf:
                i += 1
                buf += " " + lines[i].strip()
            species[-1]["nasa7"].append([float(t) for t in buf.strip("[] ").split(",")])
        elif section == "reactions" and line.startswith("- equation:"):
            reactions.append({"equation": stripped.split(":", 1)[1].strip(), "type": "elementary"})
        elif section == "reactions" and reactions and ":" in stripped:
            key, val = stripped.split(":", 1)
            val = val.strip()
            if key in ("rate-constant", "high-P-rate-constant", "low-P-rate-constant", "efficiencies", "Troe"):
                reactions[-1][key] = _flow_map(val)
            elif key == "type":
                reactions[-1]["type"] = val
            elif key == "duplicate":
                reactions[-1]["duplicate"] = val == "true"
        i += 1
    return {"source": "HyperFlow_V3/H2_Li.yaml", "phase_species": phase_species, "species": species,
            "reactions": reactions}


def main(root):
    out = {}
    for (name, group, case), keys in FIELDS.items():
        with open(os.path.join(root, "docs", name)) as f:
            rec = json.load(f)[group][case]
        out[case] = {"source": "HyperFlow_V3/docs/" + name, **{k: rec[k] for k in keys}}
    here = os.path.dirname(os.path.abspath(__file__))
    path = os.path.join(here, "reference_records.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")
    print("wrote", path)
    cases = {}
    for case in ("sun_cj", "teng_case1"):
        with open(os.path.join(root, "cases", case, "smoke.json")) as f:
            c = json.load(f)
        cases[case] = {k: c[k] for k in sorted(c) if k in CASE_KEYS}
    path = os.path.join(here, "reference_cases.json")
    with open(path, "w") as f:
        json.dump(cases, f, indent=1, sort_keys=True)
        f.write("\n")
    print("wrote", path)
    path = os.path.join(here, "h2li_mechanism.json")
    with open(path, "w") as f:
        json.dump(mechanism(os.path.join(root, "H2_Li.yaml")), f, indent=1)
        f.write("\n")
    print("wrote", path)


if __name__ == "__main__":
    if len(sys.argv) != 2 or not os.path.isdir(os.path.join(sys.argv[1], "docs")):
        sys.exit("usage: python tests/golden/make_reference_records.py <HyperFlow_V3 directory of the reference tree>")
    main(sys.argv[1])
