"""The oracle's thermal-diffusion (grad T) and antitrapping composition
fluxes against a second, vectorised numpy restatement of the reference's
loops (addconcentrationfluxfromgradt, 3d/concentrationrhs.m4:460-535,
2d:369-437; addconcentrationfluxfromantitrapping, 3d:537-700, 2d:439-527).
Bar: relative L2 <= 1e-13 (only the evaluation order of sums may differ)."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from ampe_gb300 import configs


def _model(dim):
    if dim == 2:
        m = configs.dilute2d(12)
        m.n[1] = 10
        m.dx[1] = 0.7
    else:
        m = configs.calphad3d(8, seed=3, T_run=1500.0)
        m.n[1], m.n[2] = 7, 6
        m.dx[2] = 1.3
    return m


def _sl(m, axis, lo):
    """Slices of a ghosted (z, y, x) array selecting, for the faces of normal
    `axis` (numpy axis 2 - axis), the cells on the face's lower side (lo) or
    upper side, over the face index range."""
    g = m.ng
    gz = g if m.dim == 3 else 0
    n = [m.n[0], m.n[1], m.n[2] if m.dim == 3 else 1]
    start = [g, g, gz]
    stop = [g + n[0], g + n[1], gz + n[2]]
    start[axis] -= 1 if lo else 0
    stop[axis] += 0 if lo else 1
    return (slice(start[2], stop[2]), slice(start[1], stop[1]), slice(start[0], stop[0]))


def _shift(m, axis, lo, d, s):
    """As _sl, moved by s cells along direction d (0 x, 1 y, 2 z)."""
    sl = list(_sl(m, axis, lo))
    ax = 2 - d
    sl[ax] = slice(sl[ax].start + s, sl[ax].stop + s)
    return tuple(sl)


def _avg(a, b, t):
    return 0.5 * (a + b) if t == b"a" else 2.0 * a * b / (a + b)


def gradt_np(m, T, q, f):
    out = [x.copy() for x in f]
    for d in range(m.dim):
        lo, up = T[_sl(m, d, True)], T[_sl(m, d, False)]
        side = _avg(lo, up, m.avg_type)
        out[d] = out[d] - (1.0 / m.dx[d]) * q[d] * ((up - lo) / side)
    return out


def antitrapping_np(m, P, cl, cs, dp, alpha, f):
    tol2 = float(np.float32(1e-8)) ** 2
    out = [x.copy() for x in f]
    for d in range(m.dim):
        comp = []
        for e in range(m.dim):
            if e == d:
                comp.append((P[_sl(m, d, False)] - P[_sl(m, d, True)]) / m.dx[d])
            else:
                a = P[_shift(m, d, False, e, 1)] - P[_shift(m, d, False, e, -1)]
                b = P[_shift(m, d, True, e, 1)] - P[_shift(m, d, True, e, -1)]
                comp.append(0.25 * (a + b) / m.dx[e])
        g2 = sum(c * c for c in comp)
        mask = np.abs(g2) > tol2
        gn = np.sqrt(np.where(mask, g2, 1.0))
        term = alpha * (comp[d] / gn) * (0.5 * (cl[_sl(m, d, True)] + cl[_sl(m, d, False)])
                                         - 0.5 * (cs[_sl(m, d, True)] + cs[_sl(m, d, False)])) \
            * 0.5 * (dp[_sl(m, d, True)] + dp[_sl(m, d, False)])
        out[d] = out[d] + np.where(mask, term, 0.0)
    return out


@pytest.mark.parametrize("dim", [2, 3])
def test_grad_t_flux(orc, dim):
    m = _model(dim)
    m.avg_type = b"h"
    rng = np.random.default_rng(3)
    T = O.ghosted(m, rng.uniform(1400, 1600, m.interior_shape()))
    q = [rng.uniform(0.5, 2.0, s) for s in m.face_shapes()]
    f = [rng.standard_normal(s) for s in m.face_shapes()]
    fo = [x.copy() for x in f]
    orc.orc_add_flux_from_grad_t(C.byref(m), O.ptr(T), *[O.ptr(x) for x in q],
                                 *[O.ptr(x) for x in fo])
    ref = gradt_np(m, T, q, f)
    for d in range(dim):
        assert O.rel_l2(fo[d], ref[d]) <= 1e-13


@pytest.mark.parametrize("dim", [2, 3])
def test_antitrapping_flux(orc, dim):
    m = _model(dim)
    rng = np.random.default_rng(4)
    shp = m.interior_shape()
    P = rng.uniform(0, 1, shp)
    P[..., :3] = 0.5  # flat patch: |grad phi| below the threshold on some faces
    P = O.ghosted(m, P)
    cl = O.ghosted(m, rng.uniform(0.1, 0.2, shp))
    cs = O.ghosted(m, rng.uniform(0.0, 0.1, shp))
    dp = O.ghosted(m, rng.standard_normal(shp))
    f = [rng.standard_normal(s) for s in m.face_shapes()]
    fo = [x.copy() for x in f]
    orc.orc_add_flux_from_antitrapping(C.byref(m), O.ptr(P), O.ptr(cl), O.ptr(cs), O.ptr(dp),
                                       0.35, *[O.ptr(x) for x in fo])
    ref = antitrapping_np(m, P, cl, cs, dp, 0.35, f)
    for d in range(dim):
        assert O.rel_l2(fo[d], ref[d]) <= 1e-13
        assert not np.array_equal(fo[d], f[d])
