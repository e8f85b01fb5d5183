"""The z-marching single-pass red-black sweep (sweep_z.cu) against two
colour passes of the reference's update (efo_rbgswithfluxmaxvardcvarsf3d,
3d/ellipticfacops.m4:153-172, colour order of
EllipticFACOps::smoothErrorByRedBlack) on a 128^3 level, for the operator
shapes of the phase (cell C), composition (face D) and quaternion (face D,
cell M) blocks, from u and from u = 0, two sweeps in a row (the second
reads the first's output).  Bar: relative max difference <= 1e-14 over the
ghost box (interior and periodic images), FP64."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from ampe_gb300 import configs

pytestmark = pytest.mark.gpu
N = 128


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def _P(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _ghosted(m, rng, lo, hi):
    return O.ghosted(m, rng.uniform(lo, hi, size=m.interior_shape()))


@pytest.mark.parametrize("shape", ["phase", "conc", "quat"])
@pytest.mark.parametrize("zero", [False, True])
def test_sweep_z_equals_two_colours(cuda, shape, zero):
    import torch

    m = configs.calphad3d(N, seed=3, T_run=1500.0)
    rng = np.random.default_rng(41)
    D = [None] * 3
    Cc = Mc = None
    if shape == "phase":
        Cc = _dev(_ghosted(m, rng, 1.0, 2.0))
    else:
        D = [_dev(-rng.uniform(0.5, 1.5, s)) for s in m.face_shapes()]
        if shape == "quat":
            Mc = _dev(_ghosted(m, rng, 0.5, 1.5))
    f = _dev(_ghosted(m, rng, -1, 1))
    args = [_P(x) for x in D] + [-0.7, _P(Cc), 1.3, _P(Mc), 0.9, _P(f)]
    u0 = np.zeros(m.ghost_shape()) if zero else _ghosted(m, rng, -1, 1)
    L = cuda.lib
    two = _dev(u0)
    a = None if zero else _dev(u0)
    b = _dev(np.full(m.ghost_shape(), 7.0))
    for sweep in range(2):
        for off in (0, 1):
            assert L.ampe_efo_rbgs(C.byref(m), *args, _P(two), off, None, None) == 0
            assert L.ampe_fill_ghosts(C.byref(m), _P(two), None) == 0
        assert L.ampe_efo_rbgs_sweep(C.byref(m), *args, _P(a), _P(b), None) == 0
        torch.cuda.synchronize()
        x, y = b.cpu().numpy(), two.cpu().numpy()
        err = np.abs(x - y).max() / np.abs(y).max()
        print("%s zero=%s sweep %d: max rel difference %.3e (exact: %s)"
              % (shape, zero, sweep, err, np.array_equal(x, y)))
        assert err <= 1e-14
        if a is None:
            a = _dev(np.zeros(m.ghost_shape()))
        a, b = b, a
