"""bench.py host logic on CPU: each arm describes the level it stepped
(the reference arm times a bounded sample of the workload and says so), every workload
builds its model, and the CPU sample sizes stay small."""
import argparse

import pytest

import bench


def _args(workload, n=0, path="mixed+surrogate"):
    a = argparse.Namespace(workload=workload, n=n, path=path, atol=bench.ATOL, cpu_n=80)
    if a.n <= 0:
        a.n = bench.default_n(workload)
    return a


@pytest.mark.parametrize("kind,cells", [("calphad", 256 ** 3), ("poly", 128 ** 3),
                                        ("dendrite", 2048 ** 2), ("dilute", 256 ** 2)])
def test_arm_config(kind, cells):
    a = _args(kind)
    cfg = bench.arm_config(a)
    assert cfg["cells"] == cells
    assert cfg["path"].startswith("mixed+surrogate")
    assert cfg["workload"] == bench.WORKLOAD_NAMES[kind] % (a.n, a.atol)
    # the reference arm reports the level it stepped: the full one, or a
    # sample of it named as such
    n = bench.cpu_sample_n(a)
    ref = bench.arm_config(a, n=n)
    m, _ = bench.workload(n, kind, state=False)
    assert ref["cells"] == m.cells()
    if n != a.n:
        assert "sample of the %d-cell level" % cells in ref["workload"]
    else:
        assert ref == cfg


@pytest.mark.parametrize("kind", ["calphad", "poly", "dendrite", "dilute"])
def test_cpu_sample_bounded(kind):
    a = _args(kind)
    n = bench.cpu_sample_n(a)
    m, _ = bench.workload(n, kind, state=False)
    assert 0 < m.cells() <= 600_000


def test_small_workload_states():
    for kind, n in (("calphad", 16), ("poly", 16), ("dendrite", 32), ("dilute", 32)):
        m, st = bench.workload(n, kind)
        assert st.phi.size == m.cells() and st.c.size == m.cells()


def test_l2_policy():
    """The 256^3 headline streams its state from HBM (twice the L2); levels
    whose state fits in L2 are flushed before every timed step."""
    for kind, n, flush in (("calphad", 256, False), ("poly", 512, False), ("poly", 128, True),
                           ("dendrite", 2048, True), ("dilute", 256, True)):
        a = _args(kind, n)
        m, _ = bench.workload(a.n, kind, state=False)
        assert bench.flushes_l2(a, m) == flush, (kind, n)
        assert ("flushed" in bench.arm_config(a)["l2"]) == flush


def test_kernel_rooflines():
    kt = {"kks_newton": {"ms": 2.0, "launches": 4}, "smooth_fine": {"ms": 1.0, "launches": 10},
          "mlp_infer_tc": {"ms": 0.0, "launches": 0}, "quat_rhs": {"ms": 0.0, "launches": 0},
          "precond_solve": {"ms": 5.0, "launches": 3}}
    per_cell = {"kks_newton": 36, "smooth_fine": 20}
    pk = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}
    r = bench.kernel_rooflines(kt, per_cell, 1000000, pk)
    assert set(r) == {"kks_newton", "smooth_fine"}
    assert abs(r["kks_newton"]["achieved"] - 36 * 1e6 * 4 / 2e-3 / 1e9) < 1e-9
    assert abs(r["smooth_fine"]["frac"] - (20 * 1e6 * 10 / 1e-3 / 1e9) / 6800.0) < 1e-12
