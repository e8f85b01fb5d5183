"""Generate the golden fixtures of this directory from the reference tree.

Run with the root of an AMPE source tree as the one argument:
    python tests/golden/make_golden.py <path-to-AMPE-sources>
It reads, as data only:
  - thermodynamic_data/calphadAuNi.dat       -> calphad_AuNi.json
  - tests/CALPHADbinaryEquilibrium/test.input (temperature, initial guess,
    ExpectedResults)                         -> kats.json["calphad_ceq"]
  - tests/CALPHADbinaryKKS/test.input        -> kats.json["calphad_kks"]
  - tests/KKSdiluteBinaryKKS/test.input      -> kats.json["dilute_kks"]
  - tests/KKSdiluteBinaryEquilibrium/test.input -> kats.json["dilute_ceq"]
and records, for each known-answer test, the tolerance the reference test
applies (tests/testCALPHADbinaryEquilibrium.cc:114-125,
tests/testCALPHADbinaryKKS.cc:150, tests/testKKSdiluteBinaryKKS.cc:101,
tests/testKKSdiluteBinaryEquilibrium.cc:91).
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from ampe_gb300.calphad_db import database_from_text, parse_input_text  # noqa: E402


def main(ref):
    with open(os.path.join(ref, "thermodynamic_data/calphadAuNi.dat")) as f:
        db = database_from_text(f.read())
    db["source"] = "thermodynamic_data/calphadAuNi.dat"
    with open(os.path.join(HERE, "calphad_AuNi.json"), "w") as f:
        json.dump(db, f, indent=1, sort_keys=True)

    def inp(rel):
        with open(os.path.join(ref, rel)) as f:
            return parse_input_text(f.read())

    kats = {}
    t = inp("tests/CALPHADbinaryEquilibrium/test.input")["ModelParameters"]
    e = inp("tests/CALPHADbinaryEquilibrium/test.input")["ExpectedResults"]
    kats["calphad_ceq"] = {
        "source": "tests/CALPHADbinaryEquilibrium/test.input",
        "T": t["Temperature"]["temperature"][0],
        "initial_guess": t["initial_guess"],
        "expected": e["concentrations"],
        "tol": 1.0e-6,
    }
    t = inp("tests/CALPHADbinaryKKS/test.input")["ModelParameters"]
    kats["calphad_kks"] = {
        "source": "tests/CALPHADbinaryKKS/test.input",
        "T": t["Temperature"]["temperature"][0],
        "c": t["concentration"][0],
        "phi": t["phi"][0],
        "conc_interp": "p",
        "initial_guess": [0.5, 0.5],
        "mu_tol": 1.0e-5,
    }
    for key, rel in (
        ("dilute_kks", "tests/KKSdiluteBinaryKKS/test.input"),
        ("dilute_ceq", "tests/KKSdiluteBinaryEquilibrium/test.input"),
    ):
        t = inp(rel)["ModelParameters"]
        cm = t["ConcentrationModel"]
        d = {
            "source": rel,
            "T": t["Temperature"]["temperature"][0],
            "liquidus_slope": cm["liquidus_slope"][0],
            "meltingT": cm["meltingT"][0],
            "keq": cm["keq"][0],
            "tol": 1.0e-5,
        }
        if "concentration" in t:
            d["c"] = t["concentration"][0]
            d["phi"] = t["phi"][0]
            d["conc_interp"] = "l"
            d["initial_guess"] = [0.5, 0.5]
        kats[key] = d
    with open(os.path.join(HERE, "kats.json"), "w") as f:
        json.dump(kats, f, indent=1, sort_keys=True)
    print("wrote calphad_AuNi.json and kats.json")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path-to-AMPE-sources>")
    main(sys.argv[1])
