"""Copies the golden results of OpenMOC's own regression tests for the
flat-source eigenvalue path into tests/golden/reference_results.json, and
those of its linear-source tests into tests/golden/reference_results_ls.json.

Source files (read from the reference tree named by the environment
variable REF):
  tests/test_forward_pin_cell/results_true.dat
  tests/test_forward_pin_cell_70g/results_true.dat
  tests/test_2d_gradient_linear_source/results_true.dat  (CPULSSolver)
  tests/test_fixed_linear_source/results_true.dat        (CPULSSolver)
Each holds the iteration count, keff (%12.5E, eigenvalue runs only) and the
FSR scalar fluxes (%12.6E), in the format written by tests/testing_harness.py.

Run from the repo root:  python tests/golden/import_reference_goldens.py
"""
import json
import os
import sys

REF = os.environ.get("REF", "")
HERE = os.path.dirname(os.path.abspath(__file__))
CASES = {"pin_c5g7": "test_forward_pin_cell",
         "pin_70g": "test_forward_pin_cell_70g"}
LS_CASES = {"grad2d_ls": "test_2d_gradient_linear_source",
            "fixls_c5g7": "test_fixed_linear_source"}


def parse(path):
    out = {"fluxes": []}
    with open(path) as f:
        lines = [l.strip() for l in f if l.strip()]
    for l in lines:
        if l.startswith("# Iterations:"):
            out["iterations"] = int(l.split(":")[1])
        elif l.startswith("keff:"):
            out["keff_text"] = l.split(":")[1].strip()
            out["keff"] = float(out["keff_text"])
        elif l == "fluxes:":
            continue
        else:
            out["fluxes"].append(float(l))
    return out


def main():
    if not REF:
        sys.exit("set REF to the OpenMOC source tree")
    for cases, name in ((CASES, "reference_results.json"),
                        (LS_CASES, "reference_results_ls.json")):
        res = {}
        for case, test in cases.items():
            p = os.path.join(REF, "tests", test, "results_true.dat")
            if not os.path.exists(p):
                sys.exit(f"missing {p}")
            d = parse(p)
            d["source"] = f"tests/{test}/results_true.dat"
            res[case] = d
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(res, f, indent=1)
        print("wrote", os.path.join(HERE, name))


if __name__ == "__main__":
    main()
