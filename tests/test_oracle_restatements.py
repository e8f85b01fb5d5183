"""Second, independent restatements (numpy, written from the reference's
Fortran loops) of stencil kernels that no reference known-answer test
covers, checked against the oracle's C++ on random fields (CPU):
gradient_flux (3d/quatrhs.m4:12-66), compute_flux_isotropic
(2d/quatrhs.m4:106-151), the 2D and 3D anisotropic_gradient_flux
(2d/quatrhs.m4:154-256, 3d/quatrhs.m4:149-349), concentration_pfmdiffusion_of_temperature
(3d/concentrationdiffusion.m4:310-428), add_flux (3d/flux.m4:15-100) and
the quaternion face coefficients (quatgrad_side, 3d/quatgrad.m4:213-335,
with compute_face_coef3d, 3d/quatfacops.m4:14-155, for the three gradient
floor types of fortran/quat.f:1497-1537), computerhspbg
(3d/quatrhs.m4:357-515), one colour of the red-black FAC smoother and
the FAC residual (3d/ellipticfacops.m4:16-177, 448-511), the phase block's
C coefficient (PhaseFACOps.cc:101-183), the "kks" composition flux
(KKSCompositionRHSStrategy.cc:98-441), the quaternion mobility
(3d/mobility.m4:13-95), the quaternion right-hand side
(3d/quatfacops.m4:227-311, 596-657) and the CALPHAD driving force
(CALPHADFreeEnergyStrategyBinary.cc:521-670).
The GPU leaf kernels are checked against the oracle to 1e-12, so these
close the chain to the reference's formulas."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from ampe_gb300 import abi, configs


def _model2d(flux, n=(14, 11)):
    m = configs.dilute2d(n[0])
    m.n[1] = n[1]
    m.dx[0], m.dx[1] = 0.7, 1.3
    m.epsilon_phi = 1.7
    m.flux_type = flux
    return m


def _oracle_flux(orc, m, ph, q=None):
    fs = [np.zeros(s) for s in m.face_shapes()]
    orc.orc_phase_flux(C.byref(m), O.ptr(ph), None if q is None else O.ptr(q),
                       *[O.ptr(f) for f in fs])
    return fs


def test_gradient_flux_3d(orc):
    m = configs.calphad3d(9, seed=3, T_run=1500.0)
    m.n[1], m.n[2] = 7, 6
    m.dx[0], m.dx[1], m.dx[2] = 0.5, 0.8, 1.1
    m.epsilon_phi = 0.9
    rng = np.random.default_rng(4)
    ph = O.ghosted(m, rng.uniform(0, 1, m.interior_shape()))
    f0, f1, f2 = _oracle_flux(orc, m, ph)
    e2 = m.epsilon_phi ** 2
    P = ph  # [k + 1, j + 1, i + 1]
    r0 = (P[1:-1, 1:-1, 1:] - P[1:-1, 1:-1, :-1]) * (e2 / m.dx[0])
    r1 = (P[1:-1, 1:, 1:-1] - P[1:-1, :-1, 1:-1]) * (e2 / m.dx[1])
    r2 = (P[1:, 1:-1, 1:-1] - P[:-1, 1:-1, 1:-1]) * (e2 / m.dx[2])
    for a, b in ((f0, r0), (f1, r1), (f2, r2)):
        assert a.shape == b.shape
        assert O.rel_l2(a, b) <= 1e-14


def test_isotropic_flux_2d(orc):
    m = _model2d(abi.FLUX_ISOTROPIC)
    rng = np.random.default_rng(5)
    ph = O.ghosted(m, rng.uniform(0, 1, m.interior_shape()))
    f0, f1, _ = _oracle_flux(orc, m, ph)
    e2 = m.epsilon_phi ** 2
    P = ph[0]  # [j + 1, i + 1]
    nx, ny = m.n[0], m.n[1]
    ax = (1.0 / 12.0) * e2 / m.dx[0]
    ay = (1.0 / 12.0) * e2 / m.dx[1]
    r0 = np.empty((ny, nx + 1))
    for j in range(ny):
        for i in range(nx + 1):
            p = lambda a, b: P[b + 1, a + 1]  # noqa: E731
            r0[j, i] = ax * ((p(i, j - 1) - p(i - 1, j - 1)) + (p(i, j) - p(i - 1, j)) * 10.0
                             + (p(i, j + 1) - p(i - 1, j + 1)))
    r1 = np.empty((ny + 1, nx))
    for j in range(ny + 1):
        for i in range(nx):
            p = lambda a, b: P[b + 1, a + 1]  # noqa: E731
            r1[j, i] = ay * ((p(i - 1, j) - p(i - 1, j - 1)) + (p(i, j) - p(i, j - 1)) * 10.0
                             + (p(i + 1, j) - p(i + 1, j - 1)))
    assert O.rel_l2(f0[0], r0) <= 1e-14
    assert O.rel_l2(f1[0], r1) <= 1e-14


@pytest.mark.parametrize("qlen", [2, 4])
def test_anisotropic_flux_2d(orc, qlen):
    m = _model2d(abi.FLUX_ANISOTROPIC)
    m.aniso_eps, m.aniso_k, m.qlen = 0.05, 4, qlen
    rng = np.random.default_rng(6)
    ph = O.ghosted(m, rng.uniform(0, 1, m.interior_shape()))
    g = rng.standard_normal((qlen,) + m.interior_shape())
    g /= np.linalg.norm(g, axis=0, keepdims=True)
    q = np.ascontiguousarray(np.stack([O.ghosted(m, x) for x in g]))
    f0, f1, _ = _oracle_flux(orc, m, ph, q)
    eps, nu, kn = m.epsilon_phi, m.aniso_eps, m.aniso_k
    dxi, dyi = 1.0 / m.dx[0], 1.0 / m.dx[1]
    P = ph[0]
    Q1 = q[0, 0]
    nx, ny = m.n[0], m.n[1]

    def p(a, b):
        return P[b + 1, a + 1]

    def angle(qa, qb):
        qq = min(1.0, max(-1.0, 0.5 * (qa + qb)))
        return 2.0 * np.arccos(qq) if qlen == 4 else np.arccos(qq)

    def eps_of(dpx, dpy, ph_o):
        theta = np.arctan(dpy / dpx) if abs(dpx) > 1e-12 else 0.5 * np.pi
        et = eps * (1.0 + nu * np.cos(kn * (theta - ph_o)))
        de = -kn * eps * nu * np.sin(kn * (theta - ph_o))
        return et, de

    r0 = np.empty((ny, nx + 1))
    for j in range(ny):
        for i in range(nx + 1):
            dpx = (p(i, j) - p(i - 1, j)) * dxi
            dpy = 0.25 * (p(i - 1, j + 1) - p(i - 1, j - 1) + p(i, j + 1) - p(i, j - 1)) * dyi
            et, de = eps_of(dpx, dpy, angle(Q1[j + 1, i], Q1[j + 1, i + 1]))
            r0[j, i] = et * et * dpx - et * de * dpy
    r1 = np.empty((ny + 1, nx))
    for j in range(ny + 1):
        for i in range(nx):
            dpx = 0.25 * (p(i + 1, j - 1) - p(i - 1, j - 1) + p(i + 1, j) - p(i - 1, j)) * dxi
            dpy = (p(i, j) - p(i, j - 1)) * dyi
            et, de = eps_of(dpx, dpy, angle(Q1[j, i + 1], Q1[j + 1, i + 1]))
            r1[j, i] = et * et * dpy + et * de * dpx
    assert O.rel_l2(f0[0], r0) <= 1e-12
    assert O.rel_l2(f1[0], r1) <= 1e-12


def _interp(phi, t):
    if t == b"l":
        return phi
    return phi ** 3 * (10.0 - 15.0 * phi + 6.0 * phi ** 2)  # 'p' (pbg)


@pytest.mark.parametrize("interp", [b"l", b"p"])
def test_diffusion_of_temperature_and_add_flux_3d(orc, interp):
    """concentration_pfmdiffusion_of_temperature
    (3d/concentrationdiffusion.m4:310-428, arithmetic average) and add_flux
    (3d/flux.m4:15-100) with a stored temperature field."""
    m = configs.calphad3d(8, seed=3, T_run=1500.0)
    m.n[1], m.n[2] = 7, 6
    m.dx[0], m.dx[1], m.dx[2] = 0.6, 0.9, 1.2
    m.temp_mode = abi.TEMP_FIELD
    m.D_liquid, m.D_solid = 3.0, 0.02
    m.Q_liquid, m.Q_solid = 2.0e4, 5.0e4
    m.diff_interp, m.avg_type = interp, b"a"
    rng = np.random.default_rng(7)
    phi = O.ghosted(m, rng.uniform(0, 1, m.interior_shape()))
    temp = O.ghosted(m, rng.uniform(1400, 1600, m.interior_shape()))
    u = O.ghosted(m, rng.uniform(0.1, 0.6, m.interior_shape()))
    shapes = m.face_shapes()
    dl = [np.zeros(s) for s in shapes]
    ds = [np.zeros(s) for s in shapes]
    orc.orc_conc_diffusion(C.byref(m), O.ptr(phi), O.ptr(temp), *[O.ptr(a) for a in dl],
                           *[O.ptr(a) for a in ds])
    fl = [np.zeros(s) for s in shapes]
    orc.orc_add_flux(C.byref(m), O.ptr(u), *[O.ptr(a) for a in dl], *[O.ptr(a) for a in fl])
    R = 8.314472  # KKSdiluteBinary.cc:45, the gas constant the kernels use
    sl = [np.s_[1:-1, 1:-1, 1:], np.s_[1:-1, 1:, 1:-1], np.s_[1:, 1:-1, 1:-1]]
    sm = [np.s_[1:-1, 1:-1, :-1], np.s_[1:-1, :-1, 1:-1], np.s_[:-1, 1:-1, 1:-1]]
    for d in range(3):
        vphi = 0.5 * (phi[sm[d]] + phi[sl[d]])
        h = _interp(vphi, interp)
        invT = 2.0 / (temp[sm[d]] + temp[sl[d]])
        rl = (1.0 - h) * (m.D_liquid * np.exp(-(m.Q_liquid / R) * invT))
        rs = h * (m.D_solid * np.exp(-(m.Q_solid / R) * invT))
        assert O.rel_l2(dl[d], rl) <= 1e-14
        assert O.rel_l2(ds[d], rs) <= 1e-14
        rf = (1.0 / m.dx[d]) * (rl * (u[sl[d]] - u[sm[d]]))
        assert O.rel_l2(fl[d], rf) <= 1e-14


def _grad_normi(g2, floor_type, floor):
    """eval_grad_normi (fortran/quat.f:1497-1537)."""
    fl2, mx = floor * floor, 1.0 / floor
    if floor_type == b"m":
        return np.where(g2 > fl2, g2 ** -0.5, mx)
    if floor_type == b"s":
        return (g2 + fl2) ** -0.5
    gng2 = g2 * mx * mx
    with np.errstate(divide="ignore", invalid="ignore"):
        big = np.tanh(mx * np.sqrt(g2)) / np.sqrt(g2)
    return np.where(gng2 > 0.01, big, mx * (1.0 - gng2 * (5.0 - 2.0 * gng2) / 15.0))


@pytest.mark.parametrize("floor_type", [b"m", b"s", b"t"])
def test_quat_face_coef_3d(orc, floor_type):
    """quatdiffs + quatgrad_side (3d/quatgrad.m4:213-335) and
    compute_face_coef3d (3d/quatfacops.m4:14-155) at constant T."""
    m = configs.polycrystal3d(9, seed=3, T=1500.0)
    m.n[1], m.n[2] = 8, 7
    m.dx[0], m.dx[1], m.dx[2] = 0.8, 1.0, 1.3
    m.quat_floor_type = floor_type
    rng = np.random.default_rng(8)
    shp = m.interior_shape()
    g = np.round(rng.standard_normal((4,) + shp)) + 0.05 * rng.standard_normal((4,) + shp)
    g /= np.linalg.norm(g, axis=0, keepdims=True)
    q = np.stack([O.ghosted(m, x) for x in g])  # (4, z, y, x) ghosted
    phi = O.ghosted(m, rng.uniform(0, 1, shp))
    fo = [np.zeros(s) for s in m.face_shapes()]
    orc.orc_quat_face_coef(C.byref(m), O.ptr(phi), None, O.ptr(np.ascontiguousarray(q)),
                           *[O.ptr(f) for f in fo])
    nx, ny, nz = m.n[0], m.n[1], m.n[2]
    dxi, dyi, dzi = 1.0 / m.dx[0], 1.0 / m.dx[1], 1.0 / m.dx[2]

    def Q(c, i, j, k):  # q of component c at cell (i, j, k), ghosts at -1 / n
        return q[c, k + 1, j + 1, i + 1]

    def dxq(c, i, j, k):
        return Q(c, i, j, k) - Q(c, i - 1, j, k)

    def dyq(c, i, j, k):
        return Q(c, i, j, k) - Q(c, i, j - 1, k)

    def dzq(c, i, j, k):
        return Q(c, i, j, k) - Q(c, i, j, k - 1)

    def coef(pa, pb, g2):
        pm = 0.5 * (pa + pb)  # arithmetic average
        p1 = _interp(pm, m.orient_interp1)
        p2 = _interp(pm, m.orient_interp2)
        diff = m.misorientation_factor * m.T0 * p1
        return -_grad_normi(np.array(g2), floor_type, m.quat_grad_floor) * diff \
            - m.epsilon_q ** 2 * p2

    P = phi
    rx = np.empty((nz, ny, nx + 1))
    for k in range(nz):
        for j in range(ny):
            for i in range(nx + 1):
                g2 = 0.0
                for c in range(4):
                    g2 += (dxi * dxq(c, i, j, k)) ** 2
                for c in range(4):
                    g2 += (0.25 * dyi * (dyq(c, i - 1, j + 1, k) + dyq(c, i - 1, j, k)
                                         + dyq(c, i, j + 1, k) + dyq(c, i, j, k))) ** 2
                for c in range(4):
                    g2 += (0.25 * dzi * (dzq(c, i - 1, j, k + 1) + dzq(c, i - 1, j, k)
                                         + dzq(c, i, j, k + 1) + dzq(c, i, j, k))) ** 2
                rx[k, j, i] = coef(P[k + 1, j + 1, i], P[k + 1, j + 1, i + 1], g2)
    rz = np.empty((nz + 1, ny, nx))
    for k in range(nz + 1):
        for j in range(ny):
            for i in range(nx):
                g2 = 0.0
                for c in range(4):
                    g2 += (0.25 * dxi * (dxq(c, i + 1, j, k - 1) + dxq(c, i, j, k - 1)
                                         + dxq(c, i + 1, j, k) + dxq(c, i, j, k))) ** 2
                for c in range(4):
                    g2 += (0.25 * dyi * (dyq(c, i, j + 1, k - 1) + dyq(c, i, j, k - 1)
                                         + dyq(c, i, j + 1, k) + dyq(c, i, j, k))) ** 2
                for c in range(4):
                    g2 += (dzi * dzq(c, i, j, k)) ** 2
                rz[k, j, i] = coef(P[k, j + 1, i + 1], P[k + 1, j + 1, i + 1], g2)
    assert O.rel_l2(fo[0], rx) <= 1e-13
    assert O.rel_l2(fo[2], rz) <= 1e-13


def _dinterp(phi, t):
    if t == b"l":
        return np.ones_like(phi)
    return 30.0 * phi ** 2 * (1.0 - phi) ** 2  # 'p' (pbg)


@pytest.mark.parametrize("orient", [0, 1])
def test_computerhspbg_3d(orc, orient):
    """computerhspbg (3d/quatrhs.m4:357-515), double well 'd'
    (g' = 32 phi (1 - phi)(1 - 2 phi), functions.f:275-302), constant T."""
    m = configs.calphad3d(8, seed=3, T_run=1500.0)
    m.n[1], m.n[2] = 7, 6
    m.dx[0], m.dx[1], m.dx[2] = 0.6, 0.9, 1.2
    m.temp_mode = abi.TEMP_CONSTANT
    m.T0 = 1450.0
    m.with_orient = orient
    m.misorientation_factor, m.epsilon_q = 0.3, 0.4
    m.phase_well_scale = 0.7
    rng = np.random.default_rng(9)
    fs = [rng.standard_normal(s) for s in m.face_shapes()]
    phi = O.ghosted(m, rng.uniform(0, 1, m.interior_shape()))
    ogm = rng.uniform(0, 2, size=m.interior_shape())
    out = np.zeros(m.interior_shape())
    orc.orc_computerhspbg(C.byref(m), *[O.ptr(f) for f in fs], None, O.ptr(phi), O.ptr(ogm),
                          O.ptr(out))
    f0, f1, f2 = fs
    p = phi[1:-1, 1:-1, 1:-1]
    r = ((f0[:, :, 1:] - f0[:, :, :-1]) * (1.0 / m.dx[0])
         + (f1[:, 1:, :] - f1[:, :-1, :]) * (1.0 / m.dx[1])
         + (f2[1:, :, :] - f2[:-1, :, :]) * (1.0 / m.dx[2]))
    r = r - m.phase_well_scale * (32.0 * p * (1.0 - p) * (1.0 - 2.0 * p))
    if orient:
        p1 = _dinterp(p, m.orient_interp1)
        p2 = _dinterp(p, m.orient_interp2)
        r = r - m.misorientation_factor * m.T0 * p1 * ogm \
            - p2 * (0.5 * m.epsilon_q ** 2) * ogm * ogm
    assert O.rel_l2(out, r) <= 1e-13


@pytest.mark.parametrize("offset", [0, 1])
def test_rbgs_colour_3d(orc, offset):
    """efo_compfluxvardc3d + efo_rbgswithfluxmaxvardcvarsf3d
    (3d/ellipticfacops.m4:16-177): one colour of the red-black update with
    face D, cell C and cell M arrays."""
    m = configs.calphad3d(8, seed=3, T_run=1500.0)
    m.n[1], m.n[2] = 6, 6
    m.dx[0], m.dx[1], m.dx[2] = 0.6, 0.9, 1.2
    rng = np.random.default_rng(10)
    D = [rng.uniform(-2.0, -0.5, s) for s in m.face_shapes()]
    Cc = O.ghosted(m, rng.uniform(1.0, 2.0, m.interior_shape()))
    Mc = O.ghosted(m, rng.uniform(0.5, 1.5, m.interior_shape()))
    f = O.ghosted(m, rng.uniform(-1, 1, m.interior_shape()))
    u = O.ghosted(m, rng.uniform(-1, 1, m.interior_shape()))
    uo = u.copy()
    mr = orc.orc_efo_rbgs(C.byref(m), *[O.ptr(a) for a in D], 0.0, O.ptr(Cc), 0.0, O.ptr(Mc), 0.0,
                          O.ptr(f), O.ptr(uo), offset)
    dxi = [1.0 / m.dx[d] for d in range(3)]
    fx = dxi[0] * D[0] * (u[1:-1, 1:-1, 1:] - u[1:-1, 1:-1, :-1])
    fy = dxi[1] * D[1] * (u[1:-1, 1:, 1:-1] - u[1:-1, :-1, 1:-1])
    fz = dxi[2] * D[2] * (u[1:, 1:-1, 1:-1] - u[:-1, 1:-1, 1:-1])
    Mi, Ci, fi, ui = (a[1:-1, 1:-1, 1:-1] for a in (Mc, Cc, f, u))
    res = fi - Mi * (dxi[0] * (fx[:, :, 1:] - fx[:, :, :-1]) + dxi[1] * (fy[:, 1:, :] - fy[:, :-1, :])
                     + dxi[2] * (fz[1:, :, :] - fz[:-1, :, :])) - Ci * ui
    dudr = 1.0 / (Mi * (dxi[0] ** 2 * (D[0][:, :, 1:] + D[0][:, :, :-1])
                        + dxi[1] ** 2 * (D[1][:, 1:, :] + D[1][:, :-1, :])
                        + dxi[2] ** 2 * (D[2][1:, :, :] + D[2][:-1, :, :])) - Ci)
    k, j, i = np.indices(m.interior_shape())
    colour = (i + j + k) % 2 == offset
    expect = np.where(colour, ui - res * dudr, ui)
    assert O.rel_l2(uo[1:-1, 1:-1, 1:-1], expect) <= 1e-14
    assert abs(mr - np.abs(res[colour]).max()) <= 1e-12 * max(1.0, mr)


def test_kks_form_flux_3d(orc):
    """The "kks" composition flux: concentration_pfmdiffusion
    (3d/concentrationdiffusion.m4:14-128), the coupling coefficient of
    KKSCompositionRHSStrategy::setDiffCoeffForPhaseOnPatch (:280-310) and
    concentrationflux (3d/concentrationrhs.m4:14-104); coefficients from the
    lagged (phi, cL, cS), differences of the current (phi, c)."""
    m = configs.calphad3d(8, seed=3, T_run=1500.0)
    m.n[1], m.n[2] = 7, 6
    m.dx[0], m.dx[1], m.dx[2] = 0.6, 0.9, 1.2
    m.conc_form = abi.CONC_KKS
    m.temp_mode = abi.TEMP_FIELD
    m.D_liquid, m.D_solid, m.Q_liquid, m.Q_solid = 3.0, 0.02, 2.0e4, 5.0e4
    m.energy_interp, m.avg_type = b"p", b"a"
    rng = np.random.default_rng(11)
    shp = m.interior_shape()
    phid, cld, csd = (O.ghosted(m, rng.uniform(lo, hi, shp))
                      for lo, hi in ((0, 1), (0.2, 0.5), (0.05, 0.3)))
    phi, conc = O.ghosted(m, rng.uniform(0, 1, shp)), O.ghosted(m, rng.uniform(0.1, 0.5, shp))
    temp = O.ghosted(m, rng.uniform(1400, 1600, shp))
    fo = [np.zeros(s) for s in m.face_shapes()]
    orc.orc_conc_flux_kks(C.byref(m), O.ptr(phid), O.ptr(cld), O.ptr(csd), O.ptr(temp),
                          O.ptr(phi), O.ptr(conc), *[O.ptr(f) for f in fo])
    R = 8.314472
    sl = [np.s_[1:-1, 1:-1, 1:], np.s_[1:-1, 1:, 1:-1], np.s_[1:, 1:-1, 1:-1]]
    sm = [np.s_[1:-1, 1:-1, :-1], np.s_[1:-1, :-1, 1:-1], np.s_[:-1, 1:-1, 1:-1]]
    for d in range(3):
        vphi = 0.5 * (phid[sm[d]] + phid[sl[d]])
        h = _interp(vphi, b"p")
        invT = 2.0 / (temp[sm[d]] + temp[sl[d]])
        d0 = (1.0 - h) * (m.D_liquid * np.exp(-(m.Q_liquid / R) * invT)) \
            + h * (m.D_solid * np.exp(-(m.Q_solid / R) * invT))
        cl = 0.5 * (cld[sl[d]] + cld[sm[d]])
        cs = 0.5 * (csd[sl[d]] + csd[sm[d]])
        dphi = d0 * _dinterp(vphi, b"p") * (cl - cs)
        r = (1.0 / m.dx[d]) * (d0 * (conc[sl[d]] - conc[sm[d]]) + dphi * (phi[sl[d]] - phi[sm[d]]))
        assert O.rel_l2(fo[d], r) <= 1e-13


def test_quat_mobility_and_rhs_3d(orc):
    """quatmobility, type 'p' (3d/mobility.m4:13-95), then compute_flux3d +
    add_quat_op3d (3d/quatfacops.m4:227-311, 596-657): q' = -M_q div(fc grad q)
    per component."""
    m = configs.polycrystal3d(8, seed=3, T=1500.0)
    m.n[1], m.n[2] = 7, 6
    m.dx[0], m.dx[1], m.dx[2] = 0.8, 1.0, 1.3
    rng = np.random.default_rng(12)
    shp = m.interior_shape()
    phi = O.ghosted(m, rng.uniform(-0.1, 1.1, shp))
    mq = np.zeros_like(phi)
    orc.orc_quat_mobility(C.byref(m), O.ptr(phi), O.ptr(mq))
    pc = np.clip(phi[1:-1, 1:-1, 1:-1], 0.0, 1.0)
    mq_r = m.min_quat_mobility + (m.quat_mobility - m.min_quat_mobility) * (
        1.0 - pc ** 3 * (10.0 - 15.0 * pc + 6.0 * pc * pc))
    assert O.rel_l2(mq[1:-1, 1:-1, 1:-1], mq_r) <= 1e-15
    g = rng.standard_normal((4,) + shp)
    g /= np.linalg.norm(g, axis=0, keepdims=True)
    q = np.ascontiguousarray(np.stack([O.ghosted(m, x) for x in g]))
    fc = [rng.uniform(-2, -0.1, s) for s in m.face_shapes()]
    out = np.empty(4 * m.cells())
    orc.orc_quat_rhs(C.byref(m), *[O.ptr(f) for f in fc], O.ptr(mq), O.ptr(q), O.ptr(out))
    out = out.reshape((4,) + shp)
    hi = [1.0 / m.dx[d] for d in range(3)]
    for c in range(4):
        Q = q[c]
        fx = fc[0] * hi[0] * (Q[1:-1, 1:-1, 1:] - Q[1:-1, 1:-1, :-1])
        fy = fc[1] * hi[1] * (Q[1:-1, 1:, 1:-1] - Q[1:-1, :-1, 1:-1])
        fz = fc[2] * hi[2] * (Q[1:, 1:-1, 1:-1] - Q[:-1, 1:-1, 1:-1])
        div = ((fx[:, :, 1:] - fx[:, :, :-1]) * hi[0] + (fy[:, 1:, :] - fy[:, :-1, :]) * hi[1]
               + (fz[1:, :, :] - fz[:-1, :, :]) * hi[2])
        assert O.rel_l2(out[c], -mq_r * div) <= 1e-13


def test_calphad_driving_force_3d(orc):
    """CALPHADFreeEnergyStrategyBinary::addDrivingForce
    (CALPHADFreeEnergyStrategyBinary.cc:521-670): rhs += h'(phi)
    [(f_L(cL) - f_A(cA)) - mu_A(cA) (cL - cA)], energies per volume; the
    free energy and its derivative are the oracle's (pinned on the
    reference's CALPHAD known-answer tests)."""
    import json
    import os

    from ampe_gb300.calphad_db import apply_database

    m = configs.calphad3d(6, seed=3, T_run=1500.0)
    m.n[1], m.n[2] = 5, 4
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                           "calphad_AuNi.json")) as f:
        apply_database(m, json.load(f))
    m.temp_mode = abi.TEMP_CONSTANT
    m.T0 = 1420.0
    m.inv_molar_volume[0], m.inv_molar_volume[1] = 0.11, 0.13
    rng = np.random.default_rng(13)
    shp = m.interior_shape()
    phi = O.ghosted(m, rng.uniform(0, 1, shp))
    cl = O.ghosted(m, rng.uniform(0.2, 0.4, shp))
    cs = O.ghosted(m, rng.uniform(0.05, 0.2, shp))
    rhs = rng.standard_normal(shp)
    r0 = rhs.copy()
    orc.orc_add_driving_force(C.byref(m), None, O.ptr(phi), O.ptr(cl), O.ptr(cs), O.ptr(rhs))
    fe = np.vectorize(lambda c, p: orc.orc_free_energy(C.byref(m), m.T0, c, p))
    mu = np.vectorize(lambda c: orc.orc_dfdc(C.byref(m), m.T0, c, 1))
    p, a, b = (x[1:-1, 1:-1, 1:-1] for x in (phi, cl, cs))
    fl = fe(a, 0) * m.inv_molar_volume[0]
    fa = fe(b, 1) * m.inv_molar_volume[1]
    dF = (fl - fa) - mu(b) * m.inv_molar_volume[1] * (a - b)
    expect = r0 + _dinterp(p, m.energy_interp) * dF
    assert O.rel_l2(rhs, expect) <= 1e-13


def _qmul(a, b):
    """quatmult4 (fortran/quat.f:867-894)."""
    return np.array([a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3],
                     a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2],
                     a[0] * b[2] + a[2] * b[0] + a[3] * b[1] - a[1] * b[3],
                     a[0] * b[3] + a[3] * b[0] + a[1] * b[2] - a[2] * b[1]])


def _dgamma(q, n):
    """compute_dgamma (3d/quatrhs.m4:149-178)."""
    qp = np.array([q[0], -q[1], -q[2], -q[3]])
    npr = _qmul(q, _qmul(n, qp))
    n4 = npr[1] ** 4 + npr[2] ** 4 + npr[3] ** 4
    dg = np.array([0.0, npr[1] * (npr[1] ** 2 - n4), npr[2] * (npr[2] ** 2 - n4),
                   npr[3] * (npr[3] ** 2 - n4)])
    return _qmul(qp, _qmul(dg, q)), n4


def test_anisotropic_flux_3d(orc):
    """anisotropic_gradient_flux 3D (3d/quatrhs.m4:180-349): cubic
    anisotropy through the quaternion rotation of the interface normal."""
    m = configs.calphad3d(7, seed=3, T_run=1500.0)
    m.n[1], m.n[2] = 6, 5
    m.dx[0], m.dx[1], m.dx[2] = 0.8, 1.0, 1.2
    m.flux_type = abi.FLUX_ANISOTROPIC
    m.aniso_eps, m.qlen, m.epsilon_phi = 0.05, 4, 1.3
    rng = np.random.default_rng(14)
    shp = m.interior_shape()
    ph = O.ghosted(m, rng.uniform(0, 1, shp))
    g = rng.standard_normal((4,) + shp)
    g /= np.linalg.norm(g, axis=0, keepdims=True)
    q = np.ascontiguousarray(np.stack([O.ghosted(m, x) for x in g]))
    fo = _oracle_flux(orc, m, ph, q)
    eps, e4 = m.epsilon_phi, m.aniso_eps
    factor = 4.0 * e4 / (1.0 - 3.0 * e4)
    dxi, dyi, dzi = (1.0 / m.dx[d] for d in range(3))
    nx, ny, nz = m.n[0], m.n[1], m.n[2]

    def P(i, j, k):
        return ph[k + 1, j + 1, i + 1]

    def flux(dpx, dpy, dpz, qa, qb, comp):
        g2 = dpx * dpx + dpy * dpy + dpz * dpz
        if abs(g2) > 1e-12:
            nn = np.array([0.0, dpx, dpy, dpz]) / np.sqrt(g2)
            dg, n4 = _dgamma(0.5 * (qa + qb), nn)
        else:
            dg, n4 = np.array([0.0, 0.0, 0.0, 1.0]), 0.0
        gam = eps * (1.0 - 3.0 * e4) * (1.0 + factor * n4)
        dp = (dpx, dpy, dpz)[comp - 1]
        return gam * gam * dp + 16.0 * eps * gam * e4 * np.sqrt(g2) * dg[comp]

    rx = np.empty((nz, ny, nx + 1))
    for k in range(nz):
        for j in range(ny):
            for i in range(nx + 1):
                dpx = (P(i, j, k) - P(i - 1, j, k)) * dxi
                dpy = 0.25 * (P(i - 1, j + 1, k) - P(i - 1, j - 1, k) + P(i, j + 1, k)
                              - P(i, j - 1, k)) * dyi
                dpz = 0.25 * (P(i - 1, j, k + 1) - P(i - 1, j, k - 1) + P(i, j, k + 1)
                              - P(i, j, k - 1)) * dzi
                rx[k, j, i] = flux(dpx, dpy, dpz, q[:, k + 1, j + 1, i], q[:, k + 1, j + 1, i + 1], 1)
    rz = np.empty((nz + 1, ny, nx))
    for k in range(nz + 1):
        for j in range(ny):
            for i in range(nx):
                dpx = 0.25 * (P(i + 1, j, k - 1) - P(i - 1, j, k - 1) + P(i + 1, j, k)
                              - P(i - 1, j, k)) * dxi
                dpy = 0.25 * (P(i, j + 1, k - 1) - P(i, j - 1, k - 1) + P(i, j + 1, k)
                              - P(i, j - 1, k)) * dyi
                dpz = (P(i, j, k) - P(i, j, k - 1)) * dzi
                rz[k, j, i] = flux(dpx, dpy, dpz, q[:, k, j + 1, i + 1], q[:, k + 1, j + 1, i + 1], 3)
    assert O.rel_l2(fo[0], rx) <= 1e-12
    assert O.rel_l2(fo[2], rz) <= 1e-12


def test_fac_residual_and_phase_c_3d(orc):
    """efo_compresvarsca3d (3d/ellipticfacops.m4:448-511) and
    PhaseFACOps::setCOnPatchPrivate (PhaseFACOps.cc:101-183): C = 1 + gamma M
    w g''(phi), double well 'd' (g'' = 32 (1 - 6 phi + 6 phi^2),
    functions.f:304-330)."""
    m = configs.calphad3d(7, seed=3, T_run=1500.0)
    m.n[1], m.n[2] = 6, 5
    m.dx[0], m.dx[1], m.dx[2] = 0.7, 1.0, 1.3
    m.phase_mobility, m.phase_well_scale = 1.7, 0.4
    rng = np.random.default_rng(15)
    shp = m.interior_shape()
    phi = O.ghosted(m, rng.uniform(0, 1, shp))
    cc = np.zeros_like(phi)
    orc.orc_phase_fac_set_c(C.byref(m), O.ptr(phi), 0.3, O.ptr(cc))
    p = phi[1:-1, 1:-1, 1:-1]
    c_r = 1.0 + (0.3 * m.phase_mobility) * m.phase_well_scale * (32.0 * (1.0 - 6.0 * p + 6.0 * p * p))
    assert O.rel_l2(cc[1:-1, 1:-1, 1:-1], c_r) <= 1e-15
    D = [rng.uniform(-2.0, -0.5, s) for s in m.face_shapes()]
    Mc = O.ghosted(m, rng.uniform(0.5, 1.5, shp))
    f = O.ghosted(m, rng.uniform(-1, 1, shp))
    u = O.ghosted(m, rng.uniform(-1, 1, shp))
    res = np.zeros_like(u)
    orc.orc_efo_residual(C.byref(m), *[O.ptr(a) for a in D], 0.0, O.ptr(cc), 0.0, O.ptr(Mc), 0.0,
                         O.ptr(f), O.ptr(u), O.ptr(res))
    dxi = [1.0 / m.dx[d] for d in range(3)]
    fx = dxi[0] * D[0] * (u[1:-1, 1:-1, 1:] - u[1:-1, 1:-1, :-1])
    fy = dxi[1] * D[1] * (u[1:-1, 1:, 1:-1] - u[1:-1, :-1, 1:-1])
    fz = dxi[2] * D[2] * (u[1:, 1:-1, 1:-1] - u[:-1, 1:-1, 1:-1])
    Mi, fi, ui = (a[1:-1, 1:-1, 1:-1] for a in (Mc, f, u))
    r = fi - Mi * (dxi[0] * (fx[:, :, 1:] - fx[:, :, :-1]) + dxi[1] * (fy[:, 1:, :] - fy[:, :-1, :])
                   + dxi[2] * (fz[1:, :, :] - fz[:-1, :, :])) - c_r * ui
    assert O.rel_l2(res[1:-1, 1:-1, 1:-1], r) <= 1e-14
