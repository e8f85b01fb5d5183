"""GPU stepper against the CPU oracle at the full sizes of the benchmark
configurations, on the bench's own seeded workloads and integrator
settings (dt 0.1, BDF <= 2, Newton-GMRES(5), multigrid-preconditioned FAC
blocks, atol 1e-6):

* 2D dilute 256^2, the whole 100-step run;
* 3D phi + c CALPHAD 256^3 (the headline level), 2 steps;
* 3D phi + q + c polycrystal 128^3 (8 grains), 2 steps, q compared too;
* 2D anisotropic dendrite 2048^2 (16 seeds), 2 steps.

Bars: the FP64 path within 1e-10 relative L2 per field of the oracle with
identical step, Newton, GMRES, f-evaluation, preconditioner and FAC-cycle
counts; the mixed path (FP32 kernels inside the FP64 Newton residual)
within 1e-6 per field of the same oracle run.  Each case prints one
"PARITY {...}" line with the measured errors."""
import json
import os

import numpy as np
import pytest

import oracle as O
from ampe_gb300 import configs
from ampe_gb300.stepper import ImplicitStepper

import bench

pytestmark = pytest.mark.gpu

COUNTS = ("steps", "newton_iters", "gmres_iters", "rhs_evals", "precond_solves", "fac_cycles")
CASES = {  # name: (workload, cells per side, steps)
    "dilute256": ("dilute", 256, 100),
    "calphad256": ("calphad", 256, 2),
    "poly128": ("poly", 128, 2),
    "dendrite2048": ("dendrite", 2048, 2),
}
FP64_TOL = 1e-10
MIXED_TOL = 1e-6


def params(precision):
    return configs.step_params(dt=0.1, precond=2, mg_levels=5, atol=bench.ATOL,
                               precision=precision)


def fields(s, quat):
    phi, c = s.get_state()[:2]
    out = {"phi": phi, "c": c}
    if quat:
        out["q"] = s.get_quat()
    return out


def report(name, rec):
    line = "PARITY " + json.dumps(dict(rec, case=name))
    print(line)
    path = os.environ.get("AMPE_PARITY_OUT")
    if path:
        with open(path, "a") as f:
            f.write(line + "\n")


@pytest.mark.parametrize("name", list(CASES))
def test_config_parity(cuda, name):
    kind, n, nsteps = CASES[name]
    m, st0 = bench.workload(n, kind)
    quat = st0.quat is not None
    o = O.OracleStepper(m, params(0))
    st0.load(o)
    rc, so = o.advance(nsteps)
    assert rc == 0
    fo = fields(o, quat)
    o.close()

    rec = {"cells": m.cells(), "steps": nsteps, "oracle_counts": {k: so[k] for k in COUNTS}}
    g = ImplicitStepper(m, params(0))
    st0.load(g)
    sg = g.advance(nsteps)
    fg = fields(g, quat)
    g.close()
    rec["fp64"] = {f: O.rel_l2(fg[f], fo[f]) for f in fo}
    rec["fp64_counts_equal"] = all(sg[k] == so[k] for k in COUNTS)

    gm = ImplicitStepper(m, params(1))
    st0.load(gm)
    sm = gm.advance(nsteps)
    fm = fields(gm, quat)
    gm.close()
    rec["mixed"] = {f: O.rel_l2(fm[f], fo[f]) for f in fo}
    rec["mixed_newton_iters"] = sm["newton_iters"]
    report(name, rec)

    for k in COUNTS:
        assert sg[k] == so[k], (k, sg[k], so[k])
    for f in fo:
        assert np.isfinite(fg[f]).all() and np.isfinite(fm[f]).all()
        assert rec["fp64"][f] <= FP64_TOL, (f, rec["fp64"][f])
        assert rec["mixed"][f] <= MIXED_TOL, (f, rec["mixed"][f])
