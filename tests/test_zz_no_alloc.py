"""The allocation-free residual norm against the scratch-taking one.

ampe_efo_residual_rms_noalloc serves callers that cannot allocate device
memory (a host framework that owns every GPU byte through its own pool, or a
loop that must not call cudaMalloc/cudaFree because they synchronise the
device).  It must return exactly what ampe_efo_residual_rms returns with
caller-provided scratch, on consecutive calls that reuse its one internal
buffer, and refuse levels whose working set exceeds that buffer.  This file
is collected last so a failure here comes after every other GPU test ran."""
import ctypes as C

import numpy as np
import pytest

from ampe_gb300 import abi, configs

pytestmark = pytest.mark.gpu


def _fields(m, rng):
    import torch

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()

    def ghost(lo, hi):
        g = m.ng
        gz = g if m.dim == 3 else 0
        a = rng.uniform(lo, hi, size=m.interior_shape())
        return dev(np.pad(a, ((gz, gz), (g, g), (g, g)), mode="wrap"))

    D = [dev(-rng.uniform(0.5, 1.5, s)) for s in m.face_shapes()]
    return D, ghost(1.0, 2.0), ghost(-1, 1), ghost(-1, 1)


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("dim", [2, 3])
def test_noalloc_matches_scratch_version_twice(cuda, dim):
    import torch

    L = cuda.lib
    m = configs.dilute2d(48) if dim == 2 else configs.calphad3d(24)
    rng = np.random.default_rng(21)
    scratch = torch.empty(L.ampe_efo_residual_rms_scratch_doubles(C.byref(m)),
                          dtype=torch.float64, device="cuda")
    for call in range(2):  # two calls in a row reuse the internal buffer
        D, Cc, f, u = _fields(m, rng)
        a = torch.zeros(1, dtype=torch.float64, device="cuda")
        b = torch.zeros(1, dtype=torch.float64, device="cuda")
        args = [*[_p(x) for x in D], 0.0, _p(Cc), 0.0, None, 1.7, _p(f), _p(u)]
        assert L.ampe_efo_residual_rms(C.byref(m), *args, _p(scratch), _p(a), None) == 0
        assert L.ampe_efo_residual_rms_noalloc(C.byref(m), *args, _p(b), None) == 0
        torch.cuda.synchronize()
        ra, rb = float(a[0]), float(b[0])
        assert ra > 0.0
        assert abs(ra - rb) <= 1e-13 * ra, (call, ra, rb)


def test_noalloc_size_limit_edge(cuda):
    """78^3 (an 80^3 ghost box plus the reduction partials fits in 2^19
    doubles) matches the scratch version; 79^3 (an 81^3 ghost box does not
    fit) is refused."""
    import torch

    L = cuda.lib
    m = configs.calphad3d(78)
    assert L.ampe_efo_residual_rms_scratch_doubles(C.byref(m)) <= 1 << 19
    rng = np.random.default_rng(5)
    D, Cc, f, u = _fields(m, rng)
    scratch = torch.empty(L.ampe_efo_residual_rms_scratch_doubles(C.byref(m)),
                          dtype=torch.float64, device="cuda")
    a = torch.zeros(1, dtype=torch.float64, device="cuda")
    b = torch.zeros(1, dtype=torch.float64, device="cuda")
    args = [*[_p(x) for x in D], 0.0, _p(Cc), 0.0, None, 1.7, _p(f), _p(u)]
    assert L.ampe_efo_residual_rms(C.byref(m), *args, _p(scratch), _p(a), None) == 0
    assert L.ampe_efo_residual_rms_noalloc(C.byref(m), *args, _p(b), None) == 0
    torch.cuda.synchronize()
    assert float(a[0]) > 0.0 and abs(float(a[0]) - float(b[0])) <= 1e-13 * float(a[0])
    m79 = configs.calphad3d(79)
    assert L.ampe_efo_residual_rms_scratch_doubles(C.byref(m79)) > 1 << 19
    f79 = torch.zeros(int(np.prod(m79.ghost_shape())), dtype=torch.float64, device="cuda")
    x = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = L.ampe_efo_residual_rms_noalloc(C.byref(m79), None, None, None, -1.0, None, 1.0, None,
                                         1.0, _p(f79), _p(f79), _p(x), None)
    assert rc == abi.AMPE_ERR_TOO_LARGE


def test_noalloc_refuses_levels_beyond_its_buffer(cuda):
    import torch

    L = cuda.lib
    m = configs.calphad3d(96)  # 98^3 ghost box > 2^19 doubles
    # full-size inputs, so that the call is well defined even if it ran
    f = torch.zeros(int(np.prod(m.ghost_shape())), dtype=torch.float64, device="cuda")
    u = torch.zeros_like(f)
    x = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = L.ampe_efo_residual_rms_noalloc(C.byref(m), None, None, None, -1.0, None, 1.0, None,
                                         1.0, _p(f), _p(u), _p(x), None)
    assert rc == abi.AMPE_ERR_TOO_LARGE
