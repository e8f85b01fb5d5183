"""The oracle's composition-dependent diffusion from CALPHAD atomic
mobilities (MobilityCompositionDiffusionStrategy.cc:180-611,
CALPHADMobility.cc:152-215, CALPHADMobility.h:70-115) against a numpy
restatement on the AuNi database's MobilityParameters
(thermodynamic_data/calphadAuNi.dat:66-112, read into
tests/golden/calphad_AuNi.json), 2D and 3D, with the model's temperature
gradient and with a temperature field.  The free-energy curvature comes
from the oracle's second derivative (checked against finite differences of
the free energy in test_oracle_kats).  Bar: relative L2 <= 1e-13."""
import ctypes as C
import json
import os

import numpy as np
import pytest

import oracle as O
from ampe_gb300 import abi, calphad_db, configs

R = 8.314472
HERE = os.path.dirname(os.path.abspath(__file__))


def _db():
    with open(os.path.join(HERE, "golden", "calphad_AuNi.json")) as f:
        return json.load(f)


def _model(dim, field):
    if dim == 2:
        m = configs.dilute2d(12)
        m.n[1] = 10
    else:
        m = configs.calphad3d(6, seed=3, T_run=1450.0)
        m.n[1], m.n[2] = 5, 4
    calphad_db.apply_database(m, _db())
    m.T0, m.gradT = 1450.0, 20.0
    m.temp_mode = abi.TEMP_FIELD if field else abi.TEMP_GRADIENT
    m.avg_type = b"a"
    m.diff_interp = b"p"
    return m


def _q(a, T):
    a = list(a) + [0.0] * (4 - len(a))
    return a[0] + R * T * np.log(a[1]) + a[2] * T * np.log(T) + a[3] / T


def _qq(d, n, T):
    a = d.get("q%dAB" % n, [0.0, 1.0])
    return a[0] + R * T * np.log(a[1])


def _diffusion(orc, m, mob, ph, c, T):
    """D_p(c, T) = c(1-c)(c M_B + (1-c) M_A) 1e12 f_p''(c)."""
    c1 = 1.0 - c
    ms = []
    for s in ("0", "1"):
        d = mob[s][ph]
        dc = c - c1
        dG = (c * _q(d["qA"], T) + c1 * _q(d["qB"], T) +
              c * c1 * (_qq(d, 0, T) + dc * (_qq(d, 1, T) + dc * (_qq(d, 2, T) +
                                                                dc * _qq(d, 3, T)))))
        ms.append(np.exp(dG / (R * T)) / (R * T))
    mm = c * ms[1] + c1 * ms[0]
    p = 0 if ph == "L" else 1
    d2 = np.vectorize(lambda cc, tt: orc.orc_d2fdc2(C.byref(m), tt, cc, p))(c, T)
    return c * c1 * mm * 1e12 * d2


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("field", [False, True])
def test_mobility_diffusion(orc, dim, field):
    m = _model(dim, field)
    db = _db()
    mob = db["mobility"]
    mb = calphad_db.mobility_struct(mob)
    rng = np.random.default_rng(31 + dim)
    shp = m.interior_shape()
    phi = O.ghosted(m, rng.uniform(0, 1, shp))
    cl = O.ghosted(m, rng.uniform(0.05, 0.5, shp))
    cs = O.ghosted(m, rng.uniform(0.02, 0.3, shp))
    Tf = O.ghosted(m, rng.uniform(1400, 1500, shp)) if field else None
    faces = m.face_shapes()
    out = [[np.zeros(faces[d]) if d < dim else np.zeros((1, 1, 1)) for d in range(3)]
           for _ in range(4)]
    orc.orc_conc_diffusion_mobility(C.byref(m), C.byref(mb), O.ptr(phi),
                                    O.ptr(Tf) if field else None, O.ptr(cl), O.ptr(cs),
                                    *[O.ptr(a) for grp in out for a in grp])
    g = m.ng
    gz = g if dim == 3 else 0
    if field:
        T = Tf
    else:
        i = np.arange(-g, m.n[0] + g)
        T = np.broadcast_to(m.T0 + m.gradT * ((i % m.n[0]) + 0.5) * m.dx[0], phi.shape)
    for d in range(dim):
        e = [0, 0, 0]
        e[2 - d] = 1  # arrays are (z, y, x)
        n = [faces[d][a] for a in range(3)]

        def hi(a):
            return a[gz:gz + n[0], g:g + n[1], g:g + n[2]]

        def lo(a):
            return a[gz - e[0]:gz - e[0] + n[0], g - e[1]:g - e[1] + n[1],
                     g - e[2]:g - e[2] + n[2]]

        Tm = 0.5 * (hi(T) + lo(T))
        DL = _diffusion(orc, m, mob, "L", 0.5 * (hi(cl) + lo(cl)), Tm)
        DS = _diffusion(orc, m, mob, "S", 0.5 * (hi(cs) + lo(cs)), Tm)
        pm = 0.5 * (hi(phi) + lo(phi))
        h = pm ** 3 * (10 - 15 * pm + 6 * pm ** 2)
        assert O.rel_l2(out[0][d], (1 - h) * DL) <= 1e-13
        assert O.rel_l2(out[1][d], h * DS) <= 1e-13
        assert O.rel_l2(out[2][d], DL) <= 1e-13
        assert O.rel_l2(out[3][d], DS) <= 1e-13
        # magnitudes: liquid ~1e3 um^2/s, fcc ~1 um^2/s (1400-1700 K here)
        assert 500 < DL.min() and DL.max() < 3000
        assert 0 < DS.min() and DS.max() < 50


def test_mobility_struct_defaults():
    """q<n>AB absent -> (0, 1); qA/qB with two values -> a2 = a3 = 0; the
    database reader keeps the block's species and phases apart."""
    mob = _db()["mobility"]
    mb = calphad_db.mobility_struct(mob)
    assert list(mb.q[0][1][1]) == [-306500.0, 0.0449132, 0.0, 0.0]  # Au in Ni, fcc
    assert list(mb.q[1][0][0]) == [-35921.87, 3.6471e-8, 0.0, 0.0]  # Ni, liquid, qA
    assert list(mb.qq[1][1][1]) == [-42800.0, 1.0]
    assert list(mb.qq[0][0][3]) == [0.0, 1.0]
    assert list(mb.qq[0][1][0]) == [232300.0, 7.6881435e-08]


def test_apply_database_fills_the_model():
    """apply_database copies the MobilityParameters block into the model
    and leaves the choice of diffusivities to conc_diffusion; the oracle's
    right-hand side then takes the atomic-mobility diffusivities exactly
    when conc_diffusion says so (orc_conc_diffusion_model)."""
    m = _model(3, False)
    ref = calphad_db.mobility_struct(_db()["mobility"])
    assert bytes(m.mobility) == bytes(ref)
    assert m.conc_diffusion == abi.DIFF_ARRHENIUS
    orc = O.lib()
    rng = np.random.default_rng(7)
    phi = O.ghosted(m, rng.uniform(0, 1, m.interior_shape()))
    cl = O.ghosted(m, rng.uniform(0.05, 0.3, m.interior_shape()))
    cs = O.ghosted(m, rng.uniform(0.05, 0.3, m.interior_shape()))
    fs = m.face_shapes()
    out = {}
    for kind in (abi.DIFF_ARRHENIUS, abi.DIFF_MOBILITY):
        m.conc_diffusion = kind
        dl = [np.zeros(s) for s in fs]
        ds = [np.zeros(s) for s in fs]
        orc.orc_conc_diffusion_model(C.byref(m), O.ptr(phi), None, O.ptr(cl), O.ptr(cs),
                                     *[O.ptr(a) for a in dl], *[O.ptr(a) for a in ds])
        out[kind] = (dl, ds)
    dl = [np.zeros(s) for s in fs]
    ds = [np.zeros(s) for s in fs]
    orc.orc_conc_diffusion_mobility(C.byref(m), C.byref(m.mobility), O.ptr(phi), None,
                                    O.ptr(cl), O.ptr(cs), *[O.ptr(a) for a in dl],
                                    *[O.ptr(a) for a in ds], *([None] * 6))
    for a, b in zip(out[abi.DIFF_MOBILITY][0] + out[abi.DIFF_MOBILITY][1], dl + ds):
        assert np.array_equal(a, b)
    dl = [np.zeros(s) for s in fs]
    ds = [np.zeros(s) for s in fs]
    orc.orc_conc_diffusion(C.byref(m), O.ptr(phi), None, *[O.ptr(a) for a in dl],
                           *[O.ptr(a) for a in ds])
    for a, b in zip(out[abi.DIFF_ARRHENIUS][0] + out[abi.DIFF_ARRHENIUS][1], dl + ds):
        assert np.array_equal(a, b)
