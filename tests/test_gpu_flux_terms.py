"""GPU leaf kernels of the thermal-diffusion (grad T) and antitrapping
composition fluxes (ampe_add_flux_from_grad_t,
ampe_add_flux_from_antitrapping; reference: addconcentrationfluxfromgradt
and addconcentrationfluxfromantitrapping, 3d/concentrationrhs.m4:460-700,
called from QuatIntegrator.cc:2604-2612) against the oracle, 2D and 3D,
side arrays without ghosts and with one ghost (the faces outside the
interior untouched).  Bar: relative L2 <= 1e-12 (FP64)."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from ampe_gb300 import abi, configs

pytestmark = pytest.mark.gpu
TOL = 1e-12
SENTINEL = 7.0


def _model(dim):
    if dim == 2:
        m = configs.dilute2d(24)
        m.n[1] = 20
        m.dx[1] = 0.7
    else:
        m = configs.calphad3d(12, seed=3, T_run=1500.0)
        m.n[1], m.n[2] = 10, 8
        m.dx[2] = 1.3
    return m


def _dev(a, keep):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    keep.append(t)
    return C.c_void_p(t.data_ptr()), t


def _embed(ms, plain, d):
    g = ms.ng_side
    gz = g if ms.dim == 3 else 0
    out = np.full(ms.face_shapes()[d], SENTINEL)
    out[gz:out.shape[0] - gz, g:out.shape[1] - g, g:out.shape[2] - g] = plain
    return out


def _interior(ms, a):
    g = ms.ng_side
    gz = g if ms.dim == 3 else 0
    return a[gz:a.shape[0] - gz, g:a.shape[1] - g, g:a.shape[2] - g]


def _sides(m, ms, arrays, keep):
    out = []
    for d in range(3):
        if d < m.dim:
            out.append(_dev(_embed(ms, arrays[d], d), keep))
        else:
            out.append(_dev(np.zeros((1, 1, 1)), keep))
    return out


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("ng_side", [0, 1])
def test_flux_terms(cuda, orc, dim, ng_side):
    import torch

    keep = []
    m = _model(dim)
    m.avg_type = b"h"
    ms = abi.Model.from_buffer_copy(m)
    ms.ng_side = ng_side
    rng = np.random.default_rng(7)
    shp = m.interior_shape()
    T = O.ghosted(m, rng.uniform(1400, 1600, shp))
    q = [rng.uniform(0.5, 2.0, s) for s in m.face_shapes()]
    f = [rng.standard_normal(s) for s in m.face_shapes()]
    fo = [x.copy() for x in f]
    orc.orc_add_flux_from_grad_t(C.byref(m), O.ptr(T), *[O.ptr(x) for x in q],
                                 *[O.ptr(x) for x in fo])
    qd = _sides(m, ms, q, keep)
    fd = _sides(m, ms, f, keep)
    assert cuda.lib.ampe_add_flux_from_grad_t(C.byref(ms), _dev(T, keep)[0],
                                              *[p for p, _ in qd], *[p for p, _ in fd],
                                              None) == 0
    torch.cuda.synchronize()
    for d in range(dim):
        a = fd[d][1].cpu().numpy()
        assert O.rel_l2(_interior(ms, a), fo[d]) <= TOL
        if ng_side:
            b = a.copy()
            b[tuple(slice(ng_side, s - ng_side) if (ax > 0 or dim == 3) else slice(None)
                    for ax, s in enumerate(b.shape))] = SENTINEL
            assert np.all(b == SENTINEL)
    P = rng.uniform(0, 1, shp)
    P[..., :3] = 0.5
    P = O.ghosted(m, P)
    cl = O.ghosted(m, rng.uniform(0.1, 0.2, shp))
    cs = O.ghosted(m, rng.uniform(0.0, 0.1, shp))
    dp = O.ghosted(m, rng.standard_normal(shp))
    f = [rng.standard_normal(s) for s in m.face_shapes()]
    fo = [x.copy() for x in f]
    orc.orc_add_flux_from_antitrapping(C.byref(m), O.ptr(P), O.ptr(cl), O.ptr(cs), O.ptr(dp),
                                       0.35, *[O.ptr(x) for x in fo])
    fd = _sides(m, ms, f, keep)
    assert cuda.lib.ampe_add_flux_from_antitrapping(
        C.byref(ms), _dev(P, keep)[0], _dev(cl, keep)[0], _dev(cs, keep)[0], _dev(dp, keep)[0],
        0.35, *[p for p, _ in fd], None) == 0
    torch.cuda.synchronize()
    for d in range(dim):
        a = _interior(ms, fd[d][1].cpu().numpy())
        assert O.rel_l2(a, fo[d]) <= TOL
        assert not np.array_equal(a, f[d])


@pytest.mark.parametrize("interp", [b"p", b"h"])
def test_kim_mobility(cuda, orc, interp):
    """Kim phase mobility (ampe_kim_mobility; KimMobilityStrategyInfMob.cc:
    49-80) over the ghost box against the oracle, 3D CALPHAD with the x
    temperature gradient."""
    import torch

    keep = []
    m = _model(3)
    m.energy_interp = interp
    rng = np.random.default_rng(9)
    shp = m.interior_shape()
    cl = O.ghosted(m, rng.uniform(0.3, 0.5, shp))
    cs = O.ghosted(m, rng.uniform(0.1, 0.25, shp))
    a2 = 47.0 / 60.0 if interp == b"p" else 0.5
    factor = 16 * m.phase_well_scale / (3 * m.epsilon_phi ** 2 * a2)
    mo = np.zeros_like(cl)
    orc.orc_kim_mobility(C.byref(m), None, O.ptr(cl), O.ptr(cs), factor, 2.5, 4.0e4, 7.68e-6,
                         O.ptr(mo))
    pm, tm = _dev(np.zeros_like(cl), keep)
    assert cuda.lib.ampe_kim_mobility(C.byref(m), None, _dev(cl, keep)[0], _dev(cs, keep)[0],
                                      2.5, 4.0e4, 7.68e-6, pm, None) == 0
    torch.cuda.synchronize()
    assert O.rel_l2(tm.cpu().numpy(), mo) <= TOL
    m.energy_interp = b"l"
    assert cuda.lib.ampe_kim_mobility(C.byref(m), None, _dev(cl, keep)[0], _dev(cs, keep)[0],
                                      2.5, 4.0e4, 7.68e-6, pm, None) == abi.AMPE_ERR_INVALID


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("ng_side", [0, 1])
def test_mobility_diffusion(cuda, orc, dim, ng_side):
    """Composition-dependent diffusion from the AuNi atomic mobilities
    (ampe_conc_diffusion_mobility; MobilityCompositionDiffusionStrategy.cc:
    180-611) against the oracle: the weighted face coefficients and the
    per-phase ones, side arrays with 0 and 1 ghost (ghost faces untouched)."""
    import json
    import os

    import torch

    from ampe_gb300 import calphad_db

    keep = []
    m = _model(dim)
    with open(os.path.join(os.path.dirname(__file__), "golden", "calphad_AuNi.json")) as f:
        db = json.load(f)
    calphad_db.apply_database(m, db)
    m.T0, m.gradT = 1450.0, 5.0
    m.temp_mode = abi.TEMP_GRADIENT
    mb = calphad_db.mobility_struct(db["mobility"])
    ms = abi.Model.from_buffer_copy(m)
    ms.ng_side = ng_side
    rng = np.random.default_rng(12)
    shp = m.interior_shape()
    phi = O.ghosted(m, rng.uniform(0, 1, shp))
    cl = O.ghosted(m, rng.uniform(0.05, 0.5, shp))
    cs = O.ghosted(m, rng.uniform(0.02, 0.3, shp))
    faces = m.face_shapes()
    zero = [np.zeros(faces[d]) if d < dim else np.zeros((1, 1, 1)) for d in range(3)]
    out = [[x.copy() for x in zero] for _ in range(4)]
    orc.orc_conc_diffusion_mobility(C.byref(m), C.byref(mb), O.ptr(phi), None, O.ptr(cl),
                                    O.ptr(cs), *[O.ptr(a) for grp in out for a in grp])
    # interiors start at the sentinel too, so every face written is checked
    plain = [np.full(faces[d], SENTINEL) if d < dim else None for d in range(3)]
    dev = [_sides(m, ms, plain, keep) for _ in range(4)]
    assert cuda.lib.ampe_conc_diffusion_mobility(
        C.byref(ms), C.byref(mb), _dev(phi, keep)[0], None, _dev(cl, keep)[0],
        _dev(cs, keep)[0], *[p for grp in dev for p, _ in grp], None) == 0
    torch.cuda.synchronize()
    for q in range(4):
        for d in range(dim):
            a = dev[q][d][1].cpu().numpy()
            assert O.rel_l2(_interior(ms, a), out[q][d]) <= TOL
            if ng_side:
                b = a.copy()
                gz = ng_side if dim == 3 else 0
                b[gz:b.shape[0] - gz, ng_side:b.shape[1] - ng_side,
                  ng_side:b.shape[2] - ng_side] = SENTINEL
                assert np.all(b == SENTINEL)
    bad = abi.Mobility.from_buffer_copy(mb)
    bad.qq[0][0][2][1] = 0.0  # ln(0): refused
    assert cuda.lib.ampe_conc_diffusion_mobility(
        C.byref(ms), C.byref(bad), _dev(phi, keep)[0], None, _dev(cl, keep)[0],
        _dev(cs, keep)[0], *[p for grp in dev for p, _ in grp], None) == abi.AMPE_ERR_INVALID
