"""Writes tests/golden/singlegrain_oracle.json: the CPU oracle's run of the
reference's SingleGrainGrowthAuNi regression case (tests/singlegrain.py)
to t = 0.3 with the deck's variable-step integration -- step sizes, solid
fraction, mean composition and temperature at every output time (0.02
apart, the deck's ScalarDiagnostics interval) and the final phi and c as
means over 8^2-cell blocks -- for the GPU regression test to compare its
own run with.

Run from the repository root (about a minute on 8 cores):
    OMP_NUM_THREADS=8 python tests/golden/make_singlegrain.py
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

import oracle as O  # noqa: E402
import singlegrain as SG  # noqa: E402


def main():
    t0 = time.time()
    r = SG.run(lambda m, p: O.OracleStepper(m, p))
    out = {
        "case": "tests/SingleGrainGrowthAuNi (128^2 periodic mirror of the 64^2 zero-slope box)",
        "integrator": "variable-step BDF orders 1-2, atol 1e-5, rtol 1e-7, h0 1e-6",
        "t": r["t"], "T": r["T"], "solid": r["solid"], "cmean": r["cmean"],
        "h": r["h"], "steps": r["steps"], "rejected": r["rejected"],
        "newton_iters": r["newton_iters"], "drift": r["drift"],
        "block": 8,
        "phi_blocks": SG.block_means(r["phi"], 8).ravel().tolist(),
        "c_blocks": SG.block_means(r["c"], 8).ravel().tolist(),
        "cpu_seconds": time.time() - t0,
    }
    with open(SG.FIXTURE, "w") as f:
        json.dump(out, f, indent=1)
    print("solid fraction %.4f at t = %.3f, drift %.2e, %d steps (%d rejected), %.0f s"
          % (out["solid"][-1], out["t"][-1], out["drift"], out["steps"], out["rejected"],
             out["cpu_seconds"]))


if __name__ == "__main__":
    main()
