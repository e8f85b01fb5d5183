"""Writes tests/golden/kkscomposition_oracle.json: the CPU oracle's run of
the reference's KKScomposition regression case (tests/kkscomposition.py)
to t = 0.3 -- solid fraction, mean composition and temperature at every
output time (0.03 apart, the deck's ScalarDiagnostics interval) and the
final phi and c as means over 8^3-cell blocks -- for the GPU regression
test to compare its own run with.

Run from the repository root (about 80 minutes on 8 cores):
    OMP_NUM_THREADS=8 python tests/golden/make_kkscomposition.py
With --mobility: the same run with the atomic-mobility diffusivities the
reference uses for this deck (kkscomposition.model(mobility=True)), written
to tests/golden/kkscomposition_mobility_oracle.json (about 140 minutes on
8 cores).
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

import kkscomposition as K  # noqa: E402
import oracle as O  # noqa: E402


def main():
    mobility = "--mobility" in sys.argv[1:]
    t0 = time.time()
    r = K.run(lambda m, p: O.OracleStepper(m, p), mobility=mobility)
    out = {
        "case": "tests/KKScomposition (64^3 periodic mirror of the 32^3 zero-slope box)",
        "diffusivities": "atomic mobilities" if mobility else "the deck's D_L, D_S",
        "integrator": "fixed-step BDF1, dt <= 2e-3 after a geometric start-up, atol 1e-6",
        "t": r["t"], "T": r["T"], "solid": r["solid"], "cmean": r["cmean"],
        "steps": r["steps"], "rejected": r["rejected"], "drift": r["drift"],
        "block": 8,
        "phi_blocks": K.block_means(r["phi"], 8).ravel().tolist(),
        "c_blocks": K.block_means(r["c"], 8).ravel().tolist(),
        "cpu_seconds": time.time() - t0,
    }
    with open(K.FIXTURE_MOBILITY if mobility else K.FIXTURE, "w") as f:
        json.dump(out, f, indent=1)
    print("solid fraction %.4f at t = %.3f, drift %.2e, %d steps (%d rejected), %.0f s"
          % (out["solid"][-1], out["t"][-1], out["drift"], out["steps"], out["rejected"],
             out["cpu_seconds"]))


if __name__ == "__main__":
    main()
