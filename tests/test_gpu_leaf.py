"""GPU parity of every leaf kernel of the C-ABI against the CPU oracle on
the same seeded inputs (FP64: relative L2 <= 1e-12; differences are FMA
contraction only)."""
import ctypes as C
import json
import os

import numpy as np
import pytest

import oracle as O
from ampe_gb300 import abi, configs
from ampe_gb300.calphad_db import mobility_struct

pytestmark = pytest.mark.gpu
TOL = 1e-12


_KEEP = []


@pytest.fixture(autouse=True)
def _keep_alive():
    """Device copies handed to the C-ABI as raw pointers must outlive the
    call: a temporary tensor's memory would be recycled by the allocator."""
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


def rnd_ghosted(m, rng, lo=0.0, hi=1.0):
    return O.ghosted(m, rng.uniform(lo, hi, size=m.interior_shape()))


def models():
    out = []
    m = configs.dilute2d(24)
    m.n[1] = 20
    out.append(("dilute2d_iso", m))
    m = configs.dilute2d(24)
    m.flux_type = abi.FLUX_SIMPLE
    out.append(("dilute2d_simple", m))
    m = configs.dilute2d(16)
    m.flux_type = abi.FLUX_ANISOTROPIC
    m.aniso_eps = 0.02
    m.aniso_k = 4
    m.qlen = 2
    out.append(("dilute2d_aniso", m))
    m = configs.calphad3d(12, seed=3, T_run=1500.0)
    m.n[1], m.n[2] = 10, 8
    out.append(("calphad3d_simple", m))
    m = configs.calphad3d(10, seed=4, T_run=1400.0)
    m.flux_type = abi.FLUX_ANISOTROPIC
    m.aniso_eps = 0.05
    m.qlen = 4
    out.append(("calphad3d_aniso", m))
    # composition-dependent diffusivities from the AuNi atomic mobilities
    m = configs.calphad3d(10, seed=3, T_run=1450.0)
    m.n[1], m.n[2] = 8, 6
    m.conc_diffusion = abi.DIFF_MOBILITY
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                           "calphad_AuNi.json")) as f:
        m.mobility = mobility_struct(json.load(f)["mobility"])
    out.append(("calphad3d_mobility", m))
    return out


def quat_field(m, rng):
    g = rng.standard_normal((m.qlen,) + m.interior_shape())
    g /= np.linalg.norm(g, axis=0, keepdims=True)
    return np.ascontiguousarray(np.stack([O.ghosted(m, q) for q in g]))


@pytest.mark.parametrize("name,m", models())
def test_fill_and_phase_flux(cuda, orc, name, m):
    rng = np.random.default_rng(1)
    phi_i = rng.uniform(0, 1, size=m.interior_shape())
    g = np.zeros(m.ghost_shape())
    gg = m.ng
    gz = gg if m.dim == 3 else 0
    g[gz:g.shape[0] - gz, gg:-gg, gg:-gg] = phi_i
    d = dev(g)
    assert cuda.lib.ampe_fill_ghosts(C.byref(m), P(d), None) == 0
    ref = O.ghosted(m, phi_i)
    assert np.array_equal(host(d), ref)
    q = quat_field(m, rng)
    fs_o = [np.zeros(s) for s in m.face_shapes()]
    orc.orc_phase_flux(C.byref(m), O.ptr(ref), O.ptr(q), *[O.ptr(f) for f in fs_o])
    fs_d = [dev(np.zeros(s)) for s in m.face_shapes()]
    rc = cuda.lib.ampe_phase_flux(C.byref(m), P(d), P(dev(q)), *[P(f) for f in fs_d], None)
    assert rc == 0
    for k in range(m.dim):
        assert O.rel_l2(host(fs_d[k]), fs_o[k]) <= TOL


@pytest.mark.parametrize("name,m", models()[:4])
@pytest.mark.parametrize("orient", [0, 1])
def test_computerhspbg(cuda, orc, name, m, orient):
    rng = np.random.default_rng(2)
    m.with_orient = orient
    m.misorientation_factor = 0.3
    m.epsilon_q = 0.4
    fs = [rng.standard_normal(s) for s in m.face_shapes()]
    phi = rnd_ghosted(m, rng)
    ogm = rng.uniform(0, 2, size=m.interior_shape())
    out_o = np.zeros(m.interior_shape())
    orc.orc_computerhspbg(C.byref(m), *[O.ptr(f) for f in fs], None, O.ptr(phi), O.ptr(ogm), O.ptr(out_o))
    out_d = dev(np.zeros(m.interior_shape()))
    assert cuda.lib.ampe_computerhspbg(C.byref(m), *[P(dev(f)) for f in fs], None, P(dev(phi)),
                                       P(dev(ogm)), P(out_d), None) == 0
    assert O.rel_l2(host(out_d), out_o) <= TOL


@pytest.mark.parametrize("name,m", models()[:4])
def test_driving_force_and_phase_concentrations(cuda, orc, name, m):
    rng = np.random.default_rng(3)
    phi = rnd_ghosted(m, rng)
    if m.thermo == abi.THERMO_DILUTE:
        conc = rnd_ghosted(m, rng, 0.01, 0.12)
    else:
        conc = rnd_ghosted(m, rng, 0.3, 0.5)
    clr = np.ascontiguousarray(conc * rng.uniform(0.9, 1.1, size=conc.shape))
    csr = np.ascontiguousarray(conc * rng.uniform(0.9, 1.1, size=conc.shape))
    cl_o, cs_o = np.zeros_like(conc), np.zeros_like(conc)
    nf = C.c_long(0)
    orc.orc_phase_concentrations(C.byref(m), None, O.ptr(phi), O.ptr(conc), O.ptr(clr), O.ptr(csr),
                                 O.ptr(cl_o), O.ptr(cs_o), C.byref(nf))
    assert nf.value == 0
    cl_d, cs_d = dev(np.zeros_like(conc)), dev(np.zeros_like(conc))
    import torch

    cnt = torch.zeros(2, dtype=torch.int64, device="cuda")
    rc = cuda.lib.ampe_phase_concentrations(C.byref(m), None, P(dev(phi)), P(dev(conc)), P(dev(clr)),
                                            P(dev(csr)), P(cl_d), P(cs_d), P(cnt), None)
    assert rc == 0
    assert O.rel_l2(host(cl_d), cl_o) <= TOL and O.rel_l2(host(cs_d), cs_o) <= TOL
    assert int(cnt[1]) == 0 and int(cnt[0]) > 0
    rhs_o = rng.standard_normal(m.interior_shape())
    rhs_d = dev(rhs_o.copy())
    orc.orc_add_driving_force(C.byref(m), None, O.ptr(phi), O.ptr(cl_o), O.ptr(cs_o), O.ptr(rhs_o))
    assert cuda.lib.ampe_add_driving_force(C.byref(m), None, P(dev(phi)), P(dev(cl_o)), P(dev(cs_o)),
                                           P(rhs_d), None) == 0
    assert O.rel_l2(host(rhs_d), rhs_o) <= TOL


def test_phase_concentrations_auni_temperature_field(cuda, orc):
    import json
    import os

    from ampe_gb300.calphad_db import apply_database

    m = configs.calphad3d(8, seed=1)
    with open(os.path.join(os.path.dirname(__file__), "golden", "calphad_AuNi.json")) as f:
        apply_database(m, json.load(f))
    m.temp_mode = abi.TEMP_FIELD
    rng = np.random.default_rng(9)
    T = rnd_ghosted(m, rng, 1350.0, 1500.0)
    phi = rnd_ghosted(m, rng)
    conc = rnd_ghosted(m, rng, 0.1, 0.3)
    ref = np.full_like(conc, 0.2)
    cl_o, cs_o = np.zeros_like(conc), np.zeros_like(conc)
    nf = C.c_long(0)
    orc.orc_phase_concentrations(C.byref(m), O.ptr(T), O.ptr(phi), O.ptr(conc), O.ptr(ref), O.ptr(ref),
                                 O.ptr(cl_o), O.ptr(cs_o), C.byref(nf))
    assert nf.value == 0
    cl_d, cs_d = dev(np.zeros_like(conc)), dev(np.zeros_like(conc))
    rc = cuda.lib.ampe_phase_concentrations(C.byref(m), P(dev(T)), P(dev(phi)), P(dev(conc)), P(dev(ref)),
                                            P(dev(ref)), P(cl_d), P(cs_d), None, None)
    assert rc == 0
    assert O.rel_l2(host(cl_d), cl_o) <= TOL and O.rel_l2(host(cs_d), cs_o) <= TOL


@pytest.mark.parametrize("name,m", models()[:4])
def test_composition_kernels(cuda, orc, name, m):
    rng = np.random.default_rng(4)
    m.Q_liquid = 3000.0
    m.Q_solid = 5000.0
    m.avg_type = b"h"
    phi = rnd_ghosted(m, rng, 0.0, 1.0)
    u = rnd_ghosted(m, rng)
    shapes = m.face_shapes()
    dl_o = [np.zeros(s) for s in shapes]
    ds_o = [np.zeros(s) for s in shapes]
    orc.orc_conc_diffusion(C.byref(m), O.ptr(phi), None, *[O.ptr(a) for a in dl_o], *[O.ptr(a) for a in ds_o])
    dl_d = [dev(np.zeros(s)) for s in shapes]
    ds_d = [dev(np.zeros(s)) for s in shapes]
    assert cuda.lib.ampe_conc_diffusion(C.byref(m), P(dev(phi)), None, *[P(a) for a in dl_d],
                                        *[P(a) for a in ds_d], None) == 0
    for k in range(m.dim):
        assert O.rel_l2(host(dl_d[k]), dl_o[k]) <= TOL
        assert O.rel_l2(host(ds_d[k]), ds_o[k]) <= TOL
    fl_o = [rng.standard_normal(s) for s in shapes]
    fl_d = [dev(a.copy()) for a in fl_o]
    orc.orc_add_flux(C.byref(m), O.ptr(u), *[O.ptr(a) for a in dl_o], *[O.ptr(a) for a in fl_o])
    assert cuda.lib.ampe_add_flux(C.byref(m), P(dev(u)), *[P(dev(a)) for a in dl_o], *[P(a) for a in fl_d],
                                  None) == 0
    for k in range(m.dim):
        assert O.rel_l2(host(fl_d[k]), fl_o[k]) <= TOL
    r_o = np.zeros(m.interior_shape())
    orc.orc_computerhsconcentration(C.byref(m), *[O.ptr(a) for a in fl_o], O.ptr(r_o))
    r_d = dev(np.zeros(m.interior_shape()))
    assert cuda.lib.ampe_computerhsconcentration(C.byref(m), *[P(dev(a)) for a in fl_o], P(r_d), None) == 0
    assert O.rel_l2(host(r_d), r_o) <= TOL


@pytest.mark.parametrize("name,m", models())
def test_fused_rhs(cuda, orc, name, m):
    rng = np.random.default_rng(5)
    phi = rnd_ghosted(m, rng)
    lo, hi = (0.01, 0.12) if m.thermo == abi.THERMO_DILUTE else (0.3, 0.5)
    cl = rnd_ghosted(m, rng, lo, hi)
    cs = rnd_ghosted(m, rng, lo, hi)
    q = quat_field(m, rng)
    fp_o = np.zeros(m.interior_shape())
    fc_o = np.zeros(m.interior_shape())
    orc.orc_rhs_phase_conc(C.byref(m), O.ptr(phi), O.ptr(q), None, O.ptr(cl), O.ptr(cs), O.ptr(phi),
                           O.ptr(fp_o), O.ptr(fc_o))
    fp_d = dev(np.zeros(m.interior_shape()))
    fc_d = dev(np.zeros(m.interior_shape()))
    rc = cuda.lib.ampe_rhs_phase_conc(C.byref(m), P(dev(phi)), P(dev(q)), None, P(dev(cl)), P(dev(cs)),
                                      P(fp_d), P(fc_d), None)
    assert rc == 0
    assert O.rel_l2(host(fp_d), fp_o) <= 1e-11
    assert O.rel_l2(host(fc_d), fc_o) <= TOL


@pytest.mark.parametrize("name,m", models()[:4])
@pytest.mark.parametrize("vard", [False, True])
def test_rbgs_and_residual(cuda, orc, name, m, vard):
    import torch

    rng = np.random.default_rng(6)
    shapes = m.face_shapes()
    D = [np.ascontiguousarray(-rng.uniform(0.5, 1.5, s)) for s in shapes] if vard else [None] * 3
    Cc = rnd_ghosted(m, rng, 1.0, 2.0)
    Mc = rnd_ghosted(m, rng, 0.5, 1.5)
    f = rnd_ghosted(m, rng, -1, 1)
    u = rnd_ghosted(m, rng, -1, 1)
    u_o = u.copy()
    u_d = dev(u)
    mx = torch.zeros(1, dtype=torch.float64, device="cuda")
    for off in (0, 1):
        mr = orc.orc_efo_rbgs(C.byref(m), *[O.ptr(a) for a in D], -0.7, O.ptr(Cc), 0.0, O.ptr(Mc), 0.0,
                              O.ptr(f), O.ptr(u_o), off)
        orc.orc_fill_ghosts(C.byref(m), O.ptr(u_o))
        mx.zero_()
        Dd = [None if a is None else dev(a) for a in D]
        assert cuda.lib.ampe_efo_rbgs(C.byref(m), *[P(a) for a in Dd], -0.7, P(dev(Cc)), 0.0, P(dev(Mc)),
                                      0.0, P(dev(f)), P(u_d), off, P(mx), None) == 0
        assert cuda.lib.ampe_fill_ghosts(C.byref(m), P(u_d), None) == 0
        assert abs(float(mx[0]) - mr) <= 1e-12 * max(1.0, mr)
    assert O.rel_l2(host(u_d), u_o) <= TOL
    r_o = np.zeros(m.ghost_shape())
    orc.orc_efo_residual(C.byref(m), *[O.ptr(a) for a in D], -0.7, O.ptr(Cc), 0.0, O.ptr(Mc), 0.0,
                         O.ptr(f), O.ptr(u_o), O.ptr(r_o))
    r_d = dev(np.zeros(m.ghost_shape()))
    Dd = [None if a is None else dev(a) for a in D]
    assert cuda.lib.ampe_efo_residual(C.byref(m), *[P(a) for a in Dd], -0.7, P(dev(Cc)), 0.0, P(dev(Mc)),
                                      0.0, P(dev(f)), P(dev(u_o)), P(r_d), None) == 0
    gg = m.ng
    gz = gg if m.dim == 3 else 0
    sl = (slice(gz, r_o.shape[0] - gz), slice(gg, -gg), slice(gg, -gg))
    assert O.rel_l2(host(r_d)[sl], r_o[sl]) <= TOL


@pytest.mark.parametrize("name,m", models()[:4])
def test_residual_rms(cuda, orc, name, m):
    import torch

    rng = np.random.default_rng(8)
    D = [np.ascontiguousarray(-rng.uniform(0.5, 1.5, s)) for s in m.face_shapes()]
    Cc = rnd_ghosted(m, rng, 1.0, 2.0)
    f = rnd_ghosted(m, rng, -1, 1)
    u = rnd_ghosted(m, rng, -1, 1)
    r_o = np.zeros(m.ghost_shape())
    orc.orc_efo_residual(C.byref(m), *[O.ptr(a) for a in D], 0.0, O.ptr(Cc), 0.0, None, 1.3,
                         O.ptr(f), O.ptr(u), O.ptr(r_o))
    rms_o = orc.orc_rms_interior(C.byref(m), O.ptr(r_o))
    nsc = cuda.lib.ampe_efo_residual_rms_scratch_doubles(C.byref(m))
    assert nsc >= np.prod(m.ghost_shape())
    scratch = torch.empty(nsc, dtype=torch.float64, device="cuda")
    rms = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert cuda.lib.ampe_efo_residual_rms(C.byref(m), *[P(dev(a)) for a in D], 0.0, P(dev(Cc)), 0.0, None,
                                          1.3, P(dev(f)), P(dev(u)), P(scratch), P(rms), None) == 0
    assert abs(float(rms[0]) - rms_o) <= 1e-12 * rms_o


def test_phase_set_c(cuda, orc):
    m = configs.calphad3d(8)
    rng = np.random.default_rng(7)
    phi = rnd_ghosted(m, rng)
    c_o = np.zeros(m.ghost_shape())
    orc.orc_phase_fac_set_c(C.byref(m), O.ptr(phi), 0.3, O.ptr(c_o))
    c_d = dev(np.zeros(m.ghost_shape()))
    assert cuda.lib.ampe_phase_fac_set_c(C.byref(m), P(dev(phi)), 0.3, P(c_d), None) == 0
    assert O.rel_l2(host(c_d), c_o) <= TOL


def sweep_models():
    out = []
    m = configs.dilute2d(64)
    m.n[1] = 40
    out.append(("2d_64x40", m))
    m = configs.calphad3d(12, seed=3, T_run=1500.0)
    m.n[1], m.n[2] = 10, 8
    out.append(("3d_12x10x8", m))
    m = configs.calphad3d(40, seed=3, T_run=1500.0)
    m.n[1], m.n[2] = 18, 22
    out.append(("3d_40x18x22", m))
    m = configs.calphad3d(64, seed=3, T_run=1500.0)
    out.append(("3d_64", m))
    return out


@pytest.mark.parametrize("name,m", sweep_models())
@pytest.mark.parametrize("vard", [False, True])
@pytest.mark.parametrize("zero", [False, True])
def test_rbgs_sweep_one_launch(cuda, orc, name, m, vard, zero):
    """The one-launch red+black sweep equals two colour calls plus a ghost
    fill (and the oracle), interior and ghosts, from u or from u = 0."""
    rng = np.random.default_rng(16)
    D = [np.ascontiguousarray(-rng.uniform(0.5, 1.5, s)) for s in m.face_shapes()] if vard \
        else [None] * 3
    Cc = rnd_ghosted(m, rng, 1.0, 2.0)
    Mc = rnd_ghosted(m, rng, 0.5, 1.5)
    f = rnd_ghosted(m, rng, -1, 1)
    u = np.zeros(m.ghost_shape()) if zero else rnd_ghosted(m, rng, -1, 1)
    Dd = [None if a is None else dev(a) for a in D]
    args = [P(a) for a in Dd] + [-0.7, P(dev(Cc)), 0.0, P(dev(Mc)), 0.0, P(dev(f))]
    u_two = dev(u)
    for off in (0, 1):
        assert cuda.lib.ampe_efo_rbgs(C.byref(m), *args, P(u_two), off, None, None) == 0
        assert cuda.lib.ampe_fill_ghosts(C.byref(m), P(u_two), None) == 0
    u_out = dev(np.full(m.ghost_shape(), 7.0))
    u_in = None if zero else dev(u)
    assert cuda.lib.ampe_efo_rbgs_sweep(C.byref(m), *args, P(u_in), P(u_out), None) == 0
    a, b = host(u_out), host(u_two)
    assert np.array_equal(a, b), np.abs(a - b).max()
    u_o = u.copy()
    for off in (0, 1):
        orc.orc_efo_rbgs(C.byref(m), *[O.ptr(x) for x in D], -0.7, O.ptr(Cc), 0.0, O.ptr(Mc), 0.0,
                         O.ptr(f), O.ptr(u_o), off)
        orc.orc_fill_ghosts(C.byref(m), O.ptr(u_o))
    assert O.rel_l2(a, u_o) <= TOL


def test_rbgs_sweep_rejects_odd(cuda):
    m = configs.calphad3d(12, seed=3, T_run=1500.0)
    m.n[2] = 9
    x = dev(np.zeros(m.ghost_shape()))
    y = dev(np.zeros(m.ghost_shape()))
    assert cuda.lib.ampe_efo_rbgs_sweep(C.byref(m), None, None, None, -1.0, None, 1.0, None, 1.0,
                                        P(x), P(x), P(y), None) == abi.AMPE_ERR_INVALID
