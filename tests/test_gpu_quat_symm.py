"""Symmetry-aware orientation kernels (ampe_quat_symm_rotation,
ampe_quat_fundamental, ampe_quat_diffs_symm, ampe_quat_grad_side_symm;
reference QuatModel.cc:4978-5105, 3d/quatrotation.m4, 3d/quatdiffs.m4:
131-219, 3d/quatgrad.m4:376-679) against the oracle on a 3D level whose
cells carry random symmetry relabellings of a smooth field plus noise, side
arrays with one ghost.  Bars: rotation indices equal, differences,
gradients and fundamental-region quaternions bit-identical (both sides
evaluate the same operations without fused multiply-add); the second
rotation pass, which starts from the first one's indices, equal too."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from ampe_gb300 import configs

pytestmark = pytest.mark.gpu


def _qmul(a, b):
    w = a[..., 0] * b[..., 0] - a[..., 1] * b[..., 1] - a[..., 2] * b[..., 2] - a[..., 3] * b[..., 3]
    x = a[..., 0] * b[..., 1] + a[..., 1] * b[..., 0] + a[..., 2] * b[..., 3] - a[..., 3] * b[..., 2]
    y = a[..., 0] * b[..., 2] + a[..., 2] * b[..., 0] + a[..., 3] * b[..., 1] - a[..., 1] * b[..., 3]
    z = a[..., 0] * b[..., 3] + a[..., 3] * b[..., 0] + a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1]
    return np.stack([w, x, y, z], -1)


def _field(m, orc, seed):
    qr = np.zeros((48, 4))
    conj = np.zeros(48, dtype=np.int32)
    orc.orc_quat_symm_table(O.ptr(qr), conj.ctypes.data)
    g = m.ng
    n2, n1, n0 = m.n[2], m.n[1], m.n[0]
    z, y, x = np.meshgrid(np.arange(-g, n2 + g), np.arange(-g, n1 + g), np.arange(-g, n0 + g),
                          indexing="ij")
    ang = 0.3 * (np.sin(2 * np.pi * x / n0) + np.cos(4 * np.pi * y / n1) +
                 np.sin(2 * np.pi * z / n2))
    axis = np.array([1.0, -2.0, 0.5]) / np.sqrt(5.25)
    s = np.stack([np.cos(ang / 2)] + [np.sin(ang / 2) * a for a in axis], -1)
    rng = np.random.default_rng(seed)
    lab = rng.integers(48, size=(n2, n1, n0))[z % n2, y % n1, x % n0]
    noise = 0.05 * rng.standard_normal((n2, n1, n0, 4))[z % n2, y % n1, x % n0]
    q = _qmul(s, qr[lab]) + noise
    return np.ascontiguousarray(np.moveaxis(q, -1, 0))


def test_quat_symm_kernels(cuda, orc):
    import torch

    m = configs.calphad3d(24, seed=1, T_run=1500.0)
    m.n[1], m.n[2] = 20, 16
    m.dx[2] = 1.2
    m.ng_side = 1
    q = _field(m, orc, 6)
    fs = m.face_shapes()
    L = cuda.lib

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()

    def P(t):
        return C.c_void_p(t.data_ptr())

    rot_o = [np.zeros(s, dtype=np.int32) for s in fs]
    rot_d = [dev(r) for r in rot_o]
    qd = dev(q)
    for rnd in range(2):
        orc.orc_quat_symm_rotation(C.byref(m), O.ptr(q), *[r.ctypes.data for r in rot_o])
        assert L.ampe_quat_symm_rotation(C.byref(m), P(qd), *[P(r) for r in rot_d], None) == 0
        torch.cuda.synchronize()
        for a, b in zip(rot_o, rot_d):
            assert np.array_equal(a, b.cpu().numpy()), "rotation indices, pass %d" % rnd
        if rnd == 0:
            # a nearby field: the second pass searches from these indices
            q = q + 0.02 * np.random.default_rng(2).standard_normal(q.shape)
            qd = dev(q)
    used = np.unique(np.concatenate([r.ravel() for r in rot_o]))
    assert len(used) > 20  # the relabelling does exercise the table
    diff_o = [np.zeros((4,) + s) for s in fs]
    diff_d = [dev(d) for d in diff_o]
    orc.orc_quat_diffs_symm(C.byref(m), O.ptr(q), *[r.ctypes.data for r in rot_o],
                            *[O.ptr(d) for d in diff_o])
    assert L.ampe_quat_diffs_symm(C.byref(m), P(qd), *[P(r) for r in rot_d],
                                  *[P(d) for d in diff_d], None) == 0
    torch.cuda.synchronize()
    for a, b in zip(diff_o, diff_d):
        assert np.array_equal(a, b.cpu().numpy())
    grad_o = [np.zeros((4,) + fs[d]) for d in range(3) for _ in range(3)]
    grad_d = [dev(x) for x in grad_o]
    orc.orc_quat_grad_side_symm(C.byref(m), *[O.ptr(d) for d in diff_o],
                                *[r.ctypes.data for r in rot_o], *[O.ptr(x) for x in grad_o])
    assert L.ampe_quat_grad_side_symm(C.byref(m), *[P(d) for d in diff_d],
                                      *[P(r) for r in rot_d], *[P(x) for x in grad_d],
                                      None) == 0
    torch.cuda.synchronize()
    for a, b in zip(grad_o, grad_d):
        assert np.array_equal(a, b.cpu().numpy())
    assert np.isfinite(np.concatenate([x.ravel() for x in grad_o])).all()
    qf = q.copy()
    orc.orc_quat_fundamental(C.byref(m), O.ptr(qf))
    assert L.ampe_quat_fundamental(C.byref(m), P(qd), None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(qd.cpu().numpy(), qf)
    # refused: side arrays without the ghost layer the loops need
    m.ng_side = 0
    assert L.ampe_quat_symm_rotation(C.byref(m), P(qd), *[P(r) for r in rot_d], None) < 0
