"""The "kks" composition flux form (AMPE's default rhs_form,
KKSCompositionRHSStrategy.cc:98-441): flux = D0 grad c + D0 h'(phibar)
(cLbar - cSbar) grad phi, coefficients lagged in finite-difference
evaluations.  Leaf kernel relative L2 <= 1e-12 against the oracle; FP64
steps <= 1e-10 with identical solver counts; the mixed path's analytic
product within 1e-5 of the oracle's analytic product and its steps within
2e-6 of the FP64 oracle; mass conserved."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from ampe_gb300 import abi, configs, initial
from ampe_gb300.stepper import ImplicitStepper

pytestmark = pytest.mark.gpu

_KEEP = []


@pytest.fixture(autouse=True)
def _keep_alive():
    yield
    _KEEP.clear()


def dev(a):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    _KEEP.append(t)
    return t


def host(t):
    import torch

    torch.cuda.synchronize()
    return t.cpu().numpy()


def P(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def case(name):
    if name == "dilute2d":
        m = configs.dilute2d(64)
        st = initial.dilute2d_state(64, seed=1, radius=12)
    else:
        m = configs.calphad3d(16, seed=3, T_run=1500.0)
        st = initial.calphad3d_state(16, seed=2, nseeds=2, radius=4.5)
    m.conc_form = abi.CONC_KKS
    return m, st


@pytest.mark.parametrize("name", ["dilute2d", "calphad3d"])
def test_flux_leaf(cuda, orc, name):
    m, _ = case(name)
    rng = np.random.default_rng(3)
    shp = m.interior_shape()
    phi = O.ghosted(m, rng.uniform(0, 1, shp))
    conc = O.ghosted(m, rng.uniform(0.2, 0.5, shp))
    cl = O.ghosted(m, rng.uniform(0.2, 0.5, shp))
    cs = O.ghosted(m, rng.uniform(0.2, 0.5, shp))
    fo = [np.zeros(int(np.prod(s))) for s in m.face_shapes()]
    orc.orc_conc_flux_kks(C.byref(m), *[O.ptr(a) for a in (phi, cl, cs)], None, O.ptr(phi),
                          O.ptr(conc), *[O.ptr(f) for f in fo])
    fg = [dev(np.zeros_like(f)) for f in fo]
    assert cuda.lib.ampe_conc_flux_kks(C.byref(m), P(dev(phi)), None, P(dev(conc)), P(dev(cl)),
                                       P(dev(cs)), *[P(f) for f in fg], None) == 0
    for d in range(m.dim):
        assert O.rel_l2(host(fg[d]), fo[d]) <= 1e-12


@pytest.mark.parametrize("name", ["dilute2d", "calphad3d"])
@pytest.mark.parametrize("precond", [0, 2])
def test_fp64_steps(cuda, name, precond):
    m, (phi, c) = case(name)
    p = configs.step_params(dt=0.1, precond=precond, mg_levels=3, atol=1e-6)
    o = O.OracleStepper(m, p)
    o.set_state(phi, c)
    rc, so = o.advance(4)
    assert rc == 0
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    sg = g.advance(4)
    for k in ("steps", "newton_iters", "gmres_iters", "rhs_evals", "precond_solves",
              "fac_cycles"):
        assert sg[k] == so[k], (k, sg[k], so[k])
    xg, xo = g.get_state(), o.get_state()
    for a, b in zip(xg, xo):
        assert O.rel_l2(a, b) <= 1e-10
    assert abs(xg[1].mean() - c.mean()) < 1e-9


@pytest.mark.parametrize("name", ["dilute2d", "calphad3d"])
def test_mixed(cuda, name):
    m, (phi, c) = case(name)
    p64 = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6)
    o = O.OracleStepper(m, p64)
    o.set_state(phi, c)
    o.advance(2)
    ph, cc, cl, cs = o.get_state()
    o.set_state(ph, cc, cl, cs)
    pm = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6, precision=1)
    gm = ImplicitStepper(m, pm)
    gm.set_state(ph, cc, cl, cs)
    v = np.random.default_rng(9).standard_normal(2 * m.cells()) * 1e-3
    an = o.jv(v, 0.1, 1)
    out = gm.jv(v, 0.1)
    assert O.rel_l2(out - v, an - v) <= 1e-5
    # steps from the initial state
    o2 = O.OracleStepper(m, p64)
    o2.set_state(phi, c)
    rc, so = o2.advance(6)
    assert rc == 0
    g = ImplicitStepper(m, pm)
    g.set_state(phi, c)
    sg = g.advance(6)
    assert sg["steps"] == 6
    errs = [O.rel_l2(a, b) for a, b in zip(g.get_state()[:2], o2.get_state()[:2])]
    print(name, "kks form mixed vs FP64 oracle rel L2 (phi, c):", errs)
    assert max(errs) <= 2e-6
