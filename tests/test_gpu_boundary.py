"""The drop-in boundary with SAMRAI's per-array ghost widths and the
caller's stream.

The reference hands each Fortran kernel a ghost width per array (e.g.
GRADIENT_FLUX(..., phase, phaseng, flux0, flux1, flux2, fluxng),
QuatFort.h:50-61; a call site is PhaseFluxStrategySimple.cc:54-65, and the
EBS diffusion side variables carry one ghost, QuatModel.cc:1268-1277).
Here cell fields have ghost width 2 and side fields ghost width 1
(ampe_model_t.ng_side); the leaf kernels must read and write the interior
faces of those arrays, leave their ghost faces alone, and match the oracle
run on ghost-free side arrays (FP64, relative L2 <= 1e-12).  The stepper
run on a caller's stream (ampe_stepper_set_stream) gives the same steps as
on its own stream."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from ampe_gb300 import abi, configs, initial
from ampe_gb300.stepper import ImplicitStepper

pytestmark = pytest.mark.gpu
TOL = 1e-12
SENTINEL = 7.0
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


def models():
    out = []
    m = configs.dilute2d(24)
    m.n[1] = 20
    out.append(("dilute2d_iso", m))
    m = configs.calphad3d(12, seed=3, T_run=1500.0)
    m.n[1], m.n[2] = 10, 8
    out.append(("calphad3d_simple", m))
    for _, mm in out:
        mm.ng = 2
    return out


def sided(m):
    """The same model with side arrays of ghost width 1."""
    s = abi.Model.from_buffer_copy(m)
    s.ng_side = 1
    return s


def embed(ms, plain, d):
    """Ghost-free side array of normal d -> ghost width ms.ng_side, the
    ghost faces set to SENTINEL."""
    g = ms.ng_side
    gz = g if ms.dim == 3 else 0
    out = np.full(ms.face_shapes()[d], SENTINEL)
    out[gz:out.shape[0] - gz, g:out.shape[1] - g, g:out.shape[2] - g] = plain
    return out


def interior(ms, a, d):
    g = ms.ng_side
    gz = g if ms.dim == 3 else 0
    return a[gz:a.shape[0] - gz, g:a.shape[1] - g, g:a.shape[2] - g]


def ghost_faces_untouched(ms, a, d):
    b = a.copy()
    g = ms.ng_side
    gz = g if ms.dim == 3 else 0
    b[gz:b.shape[0] - gz, g:b.shape[1] - g, g:b.shape[2] - g] = SENTINEL
    return np.all(b == SENTINEL)


@pytest.mark.parametrize("name,m", models())
def test_side_ghosts_phase(cuda, orc, name, m):
    ms = sided(m)
    rng = np.random.default_rng(1)
    phi = O.ghosted(m, rng.uniform(0, 1, size=m.interior_shape()))
    fo = [np.zeros(s) for s in m.face_shapes()]
    orc.orc_phase_flux(C.byref(m), O.ptr(phi), None, *[O.ptr(f) for f in fo])
    fd = [dev(np.full(s, SENTINEL)) for s in ms.face_shapes()]
    assert cuda.lib.ampe_phase_flux(C.byref(ms), P(dev(phi)), None, *[P(f) for f in fd],
                                    None) == 0
    for d in range(m.dim):
        a = host(fd[d])
        assert O.rel_l2(interior(ms, a, d), fo[d]) <= TOL
        assert ghost_faces_untouched(ms, a, d)
    # the divergence reads the interior faces of ghosted side arrays
    out_o = np.zeros(m.interior_shape())
    orc.orc_computerhspbg(C.byref(m), *[O.ptr(f) for f in fo], None, O.ptr(phi), None,
                          O.ptr(out_o))
    out_d = dev(np.zeros(m.interior_shape()))
    fe = [dev(embed(ms, fo[d], d)) if d < m.dim else dev(np.zeros((1, 1, 1)))
          for d in range(3)]
    assert cuda.lib.ampe_computerhspbg(C.byref(ms), *[P(f) for f in fe], None, P(dev(phi)),
                                       None, P(out_d), None) == 0
    assert O.rel_l2(host(out_d), out_o) <= TOL


@pytest.mark.parametrize("name,m", models())
def test_side_ghosts_composition(cuda, orc, name, m):
    ms = sided(m)
    rng = np.random.default_rng(4)
    phi = O.ghosted(m, rng.uniform(0, 1, size=m.interior_shape()))
    u = O.ghosted(m, rng.uniform(0, 1, size=m.interior_shape()))
    shapes, sshapes = m.face_shapes(), ms.face_shapes()
    dl_o = [np.zeros(s) for s in shapes]
    ds_o = [np.zeros(s) for s in shapes]
    orc.orc_conc_diffusion(C.byref(m), O.ptr(phi), None, *[O.ptr(a) for a in dl_o],
                           *[O.ptr(a) for a in ds_o])
    dl_d = [dev(np.full(s, SENTINEL)) for s in sshapes]
    ds_d = [dev(np.full(s, SENTINEL)) for s in sshapes]
    assert cuda.lib.ampe_conc_diffusion(C.byref(ms), P(dev(phi)), None, *[P(a) for a in dl_d],
                                        *[P(a) for a in ds_d], None) == 0
    for d in range(m.dim):
        assert O.rel_l2(interior(ms, host(dl_d[d]), d), dl_o[d]) <= TOL
        assert O.rel_l2(interior(ms, host(ds_d[d]), d), ds_o[d]) <= TOL
        assert ghost_faces_untouched(ms, host(dl_d[d]), d)
    fl_o = [rng.standard_normal(s) for s in shapes]
    fl_d = [dev(embed(ms, fl_o[d], d)) if d < m.dim else dev(np.zeros((1, 1, 1)))
            for d in range(3)]
    orc.orc_add_flux(C.byref(m), O.ptr(u), *[O.ptr(a) for a in dl_o], *[O.ptr(a) for a in fl_o])
    assert cuda.lib.ampe_add_flux(C.byref(ms), P(dev(u)), *[P(a) for a in dl_d],
                                  *[P(a) for a in fl_d], None) == 0
    for d in range(m.dim):
        assert O.rel_l2(interior(ms, host(fl_d[d]), d), fl_o[d]) <= TOL
    r_o = np.zeros(m.interior_shape())
    orc.orc_computerhsconcentration(C.byref(m), *[O.ptr(a) for a in fl_o], O.ptr(r_o))
    r_d = dev(np.zeros(m.interior_shape()))
    assert cuda.lib.ampe_computerhsconcentration(C.byref(ms), *[P(a) for a in fl_d], P(r_d),
                                                 None) == 0
    assert O.rel_l2(host(r_d), r_o) <= TOL
    # the FAC colour update with face coefficients in ghosted side arrays
    D = [np.ascontiguousarray(-rng.uniform(0.5, 1.5, s)) for s in shapes]
    f = O.ghosted(m, rng.uniform(-1, 1, size=m.interior_shape()))
    u_o = O.ghosted(m, rng.uniform(-1, 1, size=m.interior_shape()))
    u_d = dev(u_o)
    Dd = [dev(embed(ms, D[d], d)) if d < m.dim else dev(np.zeros((1, 1, 1))) for d in range(3)]
    for off in (0, 1):
        orc.orc_efo_rbgs(C.byref(m), *[O.ptr(x) for x in D], 0.0, None, -1.0, None, 1.0,
                         O.ptr(f), O.ptr(u_o), off)
        orc.orc_fill_ghosts(C.byref(m), O.ptr(u_o))
        assert cuda.lib.ampe_efo_rbgs(C.byref(ms), *[P(x) for x in Dd], 0.0, None, -1.0, None,
                                      1.0, P(dev(f)), P(u_d), off, None, None) == 0
        assert cuda.lib.ampe_fill_ghosts(C.byref(ms), P(u_d), None) == 0
    assert O.rel_l2(host(u_d), u_o) <= TOL


def test_caller_stream(cuda):
    import torch

    m = configs.calphad3d(16, seed=3, T_run=1500.0)
    phi, c = initial.calphad3d_state(16, seed=2, nseeds=2, radius=4.5)
    p = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6)
    a = ImplicitStepper(m, p)
    a.set_state(phi, c)
    a.advance(3)
    b = ImplicitStepper(m, p)
    st = torch.cuda.Stream()
    assert cuda.lib.ampe_stepper_set_stream(b._h, C.c_void_p(st.cuda_stream)) == 0
    assert cuda.lib.ampe_stepper_stream(b._h) == st.cuda_stream
    b.set_state(phi, c)
    b.advance(3)
    for x, y in zip(a.get_state(), b.get_state()):
        assert np.array_equal(x, y)
    assert cuda.lib.ampe_stepper_set_stream(b._h, None) == 0
    assert cuda.lib.ampe_stepper_stream(b._h) != st.cuda_stream
    b.advance(1)
