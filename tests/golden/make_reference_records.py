"""Writes reference_records.json: the run outcomes that HyperFlow V3 records for its own
checks (HyperFlow_V3/docs/case_checks.json and docs/amr_checks.json), reduced to the
fields the oracle and GPU tests compare with; and reference_cases.json: the keys of its
two smoke case configurations (cases/*/smoke.json) that the case loader reads.  Run
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


if __name__ == "__main__":
    if len(sys.argv) != 2 or not os.path.isdir(os.path.join(sys.argv[1], "docs")):
        sys.exit("usage: python tests/golden/make_reference_records.py <HyperFlow_V3 directory of the reference tree>")
    main(sys.argv[1])
