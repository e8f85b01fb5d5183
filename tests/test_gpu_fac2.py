"""Two-level composite FAC on the GPU (ampe_fac2_composite_residual,
ampe_fac2_solve; FACPreconditioner.cc:267-683, EllipticFACOps.cc:948-2029)
against the oracle: the composite residual on random data (relative L2
<= 1e-13 per level, the norm within 1e-13), and whole solves (the same
cycle count, the residual norm after every cycle within 1e-8 relative or
1e-13 of the initial norm, the solutions within 1e-11), with the
reference's spacing rule and the per-level one, variable and constant
coefficients, the box inside the domain and across its periodic
boundary."""
import ctypes as C

import numpy as np
import pytest

import fac2_case
import oracle as O

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch

    return None if a is None else torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _P(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _level(d, keep):
    t = {"D": [_dev(x) for x in d["D"]], "C": _dev(d["C"]), "M": _dev(d["M"])}
    keep.append(t)
    return fac2_case.level_struct(t, lambda x: _P(x).value)


def interior(a, m):
    g = m.ng
    return a[g:-g, g:-g, g:-g]


@pytest.mark.parametrize("level_dx", [0, 1])
@pytest.mark.parametrize("lo,variable", [((4, 3, 2), True), ((13, 10, 8), True),
                                         ((5, 2, 3), False)])
def test_fac2_against_oracle(cuda, orc, level_dx, lo, variable):
    import torch

    p, m, mf, lev = fac2_case.make(lo=lo, level_dx=level_dx, seed=4, variable=variable)
    L = cuda.lib
    keep = []
    gc, gf = _level(lev["c"], keep), _level(lev["f"], keep)
    sc = fac2_case.level_struct(lev["c"], O.ptr)
    sf = fac2_case.level_struct(lev["f"], O.ptr)
    nw = L.ampe_fac2_work_doubles(C.byref(p))
    assert nw > 0
    work = torch.zeros(nw, dtype=torch.float64, device="cuda")
    fc, ff = _dev(lev["c"]["f"]), _dev(lev["f"]["f"])
    # composite residual on random u
    rng = np.random.default_rng(5)
    uc0 = rng.standard_normal(m.ghost_shape())
    uf0 = rng.standard_normal(mf.ghost_shape())
    rc_o, rf_o = np.zeros(m.ghost_shape()), np.zeros(mf.ghost_shape())
    uc_o, uf_o = uc0.copy(), uf0.copy()
    n_o = orc.orc_fac2_composite_residual(C.byref(p), C.byref(sc), C.byref(sf),
                                          O.ptr(lev["c"]["f"]), O.ptr(lev["f"]["f"]),
                                          O.ptr(uc_o), O.ptr(uf_o), O.ptr(rc_o), O.ptr(rf_o))
    uc, uf = _dev(uc0), _dev(uf0)
    rc, rf = _dev(np.zeros(m.ghost_shape())), _dev(np.zeros(mf.ghost_shape()))
    nrm = C.c_double()
    assert L.ampe_fac2_composite_residual(C.byref(p), C.byref(gc), C.byref(gf), _P(fc), _P(ff),
                                          _P(uc), _P(uf), _P(rc), _P(rf), _P(work),
                                          C.byref(nrm), None) == 0
    torch.cuda.synchronize()
    assert O.rel_l2(interior(rc.cpu().numpy(), m), interior(rc_o, m)) <= 1e-13
    assert O.rel_l2(interior(rf.cpu().numpy(), mf), interior(rf_o, mf)) <= 1e-13
    assert abs(nrm.value - n_o) <= 1e-13 * n_o
    # whole solves from zero
    no = np.zeros(41)
    uc_o, uf_o = np.zeros(m.ghost_shape()), np.zeros(mf.ghost_shape())
    it_o = orc.orc_fac2_solve(C.byref(p), C.byref(sc), C.byref(sf), O.ptr(lev["c"]["f"]),
                              O.ptr(lev["f"]["f"]), O.ptr(uc_o), O.ptr(uf_o), 40, 1e-10,
                              O.ptr(no))
    ng = np.zeros(41)
    uc, uf = _dev(np.zeros(m.ghost_shape())), _dev(np.zeros(mf.ghost_shape()))
    it_g = L.ampe_fac2_solve(C.byref(p), C.byref(gc), C.byref(gf), _P(fc), _P(ff), _P(uc),
                             _P(uf), 40, 1e-10, _P(work), ng.ctypes.data, None)
    torch.cuda.synchronize()
    dn = np.max(np.abs(ng[:it_g + 1] - no[:it_o + 1]) / no[:it_o + 1])
    print("level_dx %d lo %s variable %s: %d cycles, %.3e -> %.3e, norms max rel diff %.2e"
          % (level_dx, lo, variable, it_g, ng[0], ng[it_g], dn))
    assert it_g == it_o and 0 < it_g < 40
    # the norms fall 1e10-fold: rounding differences of the O(1) solution
    # (fused multiply-adds on the GPU) set their agreement once they are small
    assert np.allclose(ng[:it_g + 1], no[:it_o + 1], rtol=1e-8, atol=1e-13 * no[0])
    assert O.rel_l2(interior(uc.cpu().numpy(), m), interior(uc_o, m)) <= 1e-11
    assert O.rel_l2(interior(uf.cpu().numpy(), mf), interior(uf_o, mf)) <= 1e-11


def test_fac2_refusals(cuda):
    p, m, mf, lev = fac2_case.make()
    L = cuda.lib
    q = type(p).from_buffer_copy(p)
    q.nbox[0] = 1
    assert L.ampe_fac2_work_doubles(C.byref(q)) < 0
    q = type(p).from_buffer_copy(p)
    q.coarse.dim = 2
    assert L.ampe_fac2_work_doubles(C.byref(q)) < 0
