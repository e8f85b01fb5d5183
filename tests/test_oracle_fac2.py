"""Two-level composite FAC in the oracle (FACPreconditioner.cc:267-683,
EllipticFACOps.cc:948-2029, 3d/ellipticfacops.m4 efo_* routines): the
composite operator conserves flux across the coarse-fine boundary (with
C = 0 and M = 1 the volume-weighted sum of A u over the composite grid is
zero, for the reference's spacing rule and the per-level one), and FAC
cycles converge on random variable-coefficient problems, the box away from
and across the periodic boundary."""
import ctypes as C

import numpy as np
import pytest

import fac2_case
import oracle as O


def interior(a, m):
    g = m.ng
    return a[g:-g, g:-g, g:-g]


@pytest.mark.parametrize("level_dx", [0, 1])
@pytest.mark.parametrize("lo", [(4, 3, 2), (13, 10, 8)])
def test_composite_flux_conservation(orc, level_dx, lo):
    p, m, mf, lev = fac2_case.make(lo=lo, level_dx=level_dx, seed=2)
    p.c_const = 0.0
    rng = np.random.default_rng(9)
    for name, mm in (("c", m), ("f", mf)):
        lev[name]["C"] = None
        lev[name]["M"] = None
        lev[name]["f"] = np.zeros(mm.ghost_shape())
        lev[name]["u"] = rng.standard_normal(mm.ghost_shape())
    rc = np.zeros(m.ghost_shape())
    rf = np.zeros(mf.ghost_shape())
    sc = fac2_case.level_struct(lev["c"], O.ptr)
    sf = fac2_case.level_struct(lev["f"], O.ptr)
    norm = orc.orc_fac2_composite_residual(C.byref(p), C.byref(sc), C.byref(sf),
                                           O.ptr(lev["c"]["f"]), O.ptr(lev["f"]["f"]),
                                           O.ptr(lev["c"]["u"]), O.ptr(lev["f"]["u"]),
                                           O.ptr(rc), O.ptr(rf))
    assert norm > 0
    dvc = np.prod(list(m.dx))
    dvf = dvc / 8
    out = ~fac2_case.under_box(p, m)
    tot = dvc * interior(rc, m)[out].sum() + dvf * interior(rf, mf).sum()
    scale = dvc * np.abs(interior(rc, m)[out]).sum() + dvf * np.abs(interior(rf, mf)).sum()
    assert abs(tot) <= 1e-13 * scale
    # the coarse cells under the box hold the restricted fine residual
    rfi = interior(rf, mf)
    R = rfi.reshape(rfi.shape[0] // 2, 2, rfi.shape[1] // 2, 2, rfi.shape[2] // 2, 2)
    R = R.mean(axis=(1, 3, 5))
    idx = [((p.lo[d] + np.arange(p.nbox[d])) % m.n[d]) for d in range(3)]
    assert np.allclose(interior(rc, m)[np.ix_(idx[2], idx[1], idx[0])], R, atol=1e-13)


@pytest.mark.parametrize("level_dx", [0, 1])
@pytest.mark.parametrize("lo", [(4, 3, 2), (13, 10, 8)])
def test_fac_cycles_converge(orc, level_dx, lo):
    p, m, mf, lev = fac2_case.make(lo=lo, level_dx=level_dx, seed=3)
    sc = fac2_case.level_struct(lev["c"], O.ptr)
    sf = fac2_case.level_struct(lev["f"], O.ptr)
    norms = np.zeros(31)
    it = orc.orc_fac2_solve(C.byref(p), C.byref(sc), C.byref(sf), O.ptr(lev["c"]["f"]),
                            O.ptr(lev["f"]["f"]), O.ptr(lev["c"]["u"]), O.ptr(lev["f"]["u"]),
                            30, 1e-10, O.ptr(norms))
    h = norms[:it + 1]
    print("level_dx %d lo %s: %d cycles, norms %s" % (level_dx, lo, it, h[[0, 1, 2, -1]]))
    assert np.all(np.diff(h) < 0)
    assert h[-1] <= 1e-10 * max(1.0, h[0]) or h[-1] <= 1e-10
    assert it < 30
