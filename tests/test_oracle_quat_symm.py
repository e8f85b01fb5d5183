"""Symmetry-aware orientation in the oracle (quat.f quatfindsymm4 /
quatsymmrotate4 / setqr, 3d/quatrotation.m4, 3d/quatdiffs.m4:131-219,
3d/quatgrad.m4:376-679) and the library's rotation table, on the CPU:

* the library's 48 rotations, built by rule, equal the oracle's restatement
  of setqr's listing (and its conjugate table), and form a group closed
  under products with the conjugate as inverse;
* the search returns the rotation that maps q2 onto q1 when q2 is q1 taken
  through a symmetry element, from any starting index;
* fundamental-region mapping picks the rotation closest to the identity
  (first one within the stop threshold in the listing order);
* with every rotation index 1 the symmetric differences and side gradients
  are the plain QUATDIFFS / QUATGRAD_SIDE formulas;
* relabelling each cell's orientation by a random symmetry element leaves
  the magnitudes of the symmetric differences those of the smooth field."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from ampe_gb300 import abi, configs

THR = (2 * np.sin(np.pi / 16)) ** 2


def _table(orc):
    qr = np.zeros((48, 4))
    conj = np.zeros(48, dtype=np.int32)
    orc.orc_quat_symm_table(O.ptr(qr), conj.ctypes.data)
    return qr, conj


def qmul(a, b):
    w = a[..., 0] * b[..., 0] - a[..., 1] * b[..., 1] - a[..., 2] * b[..., 2] - a[..., 3] * b[..., 3]
    x = a[..., 0] * b[..., 1] + a[..., 1] * b[..., 0] + a[..., 2] * b[..., 3] - a[..., 3] * b[..., 2]
    y = a[..., 0] * b[..., 2] + a[..., 2] * b[..., 0] + a[..., 3] * b[..., 1] - a[..., 1] * b[..., 3]
    z = a[..., 0] * b[..., 3] + a[..., 3] * b[..., 0] + a[..., 1] * b[..., 2] - a[..., 2] * b[..., 1]
    return np.stack([w, x, y, z], -1)


def conjq(a):
    return a * np.array([1, -1, -1, -1])


def test_table_matches_library_and_is_a_group(orc):
    from ampe_gb300 import _native

    qr, conj = _table(orc)
    lq = np.zeros((48, 4))
    lc = np.zeros(48, dtype=np.int32)
    assert _native.lib.ampe_quat_symm_table(lq.ctypes.data, lc.ctypes.data) == 0
    assert np.array_equal(lq, qr) and np.array_equal(lc, conj)
    assert np.allclose(np.linalg.norm(qr, axis=1), 1.0, atol=1e-15)
    for a in range(48):
        assert np.allclose(qr[conj[a] - 1], conjq(qr[a]))
        for b in range(48):
            p = qmul(qr[a], qr[b])
            assert np.min(np.abs(qr - p).max(axis=1)) < 1e-15  # closed


@pytest.mark.parametrize("start", [1, 0, 7, -12, 99])
def test_find_symm_recovers_the_rotation(orc, start):
    qr, _ = _table(orc)
    rng = np.random.default_rng(3)
    for t in range(60):
        q1 = rng.standard_normal(4)
        q1 /= np.linalg.norm(q1)
        r = int(rng.integers(48))
        q2 = qmul(q1, conjq(qr[r]))  # q2 qr[r] = q1
        out = np.zeros(4)
        iq = orc.orc_quat_find_symm(O.ptr(q1), O.ptr(q2), start, O.ptr(out))
        assert iq == r + 1
        assert np.allclose(out, q1, atol=1e-14)


def test_fundamental(orc):
    qr, _ = _table(orc)
    m = configs.calphad3d(4, seed=1, T_run=1500.0)
    m.n[1], m.n[2] = 3, 2
    rng = np.random.default_rng(5)
    q = rng.standard_normal((4,) + m.ghost_shape())
    q0 = q.copy()
    orc.orc_quat_fundamental(C.byref(m), O.ptr(q))
    g = m.ng
    sl = (slice(None), slice(g, -g), slice(g, -g), slice(g, -g))
    a = np.moveaxis(q0[sl], 0, -1).reshape(-1, 4)
    b = np.moveaxis(q[sl], 0, -1).reshape(-1, 4)
    ident = np.array([1.0, 0, 0, 0])
    for x, y in zip(a, b):
        cand = qmul(x[None], qr)  # all 48 images
        d = np.sum((cand / np.linalg.norm(cand, axis=1)[:, None] - ident) ** 2, axis=1)
        k = np.flatnonzero(np.all(np.abs(cand - y) < 1e-15, axis=1))
        assert len(k) == 1
        k = k[0]
        # the first in listing order within the threshold, else the minimum
        within = np.flatnonzero(d <= THR)
        assert k == (within[0] if len(within) else np.argmin(d))
    # ghosts untouched
    mask = np.ones(q.shape, bool)
    mask[sl] = False
    assert np.array_equal(q[mask], q0[mask])


def _model(ng_side=1):
    m = configs.calphad3d(6, seed=1, T_run=1500.0)
    m.n[1], m.n[2] = 5, 4
    m.dx[1], m.dx[2] = 0.8, 1.3
    m.ng_side = ng_side
    return m


def _sides(m, dtype=np.float64, depth=4):
    return [np.zeros((depth,) + s, dtype=dtype) if depth > 1 else np.zeros(s, dtype=dtype)
            for s in m.face_shapes()]


def test_identity_rotations_give_plain_formulas(orc):
    m = _model()
    rng = np.random.default_rng(8)
    q = np.stack([O.ghosted(m, rng.standard_normal(m.interior_shape())) for _ in range(4)])
    rot = [np.ones(s, dtype=np.int32) for s in m.face_shapes()]
    diff = _sides(m)
    orc.orc_quat_diffs_symm(C.byref(m), O.ptr(q), *[r.ctypes.data for r in rot],
                            *[O.ptr(x) for x in diff])
    g, s = m.ng, m.ng_side
    n0, n1, n2 = m.n
    # plain differences on every face the loops cover
    for d in range(3):
        e = [0, 0, 0]
        e[2 - d] = 1
        ext = [n2 + 2 - e[0], n1 + 2 - e[1], n0 + 2 - e[2]]  # faces incl. 1 transverse ghost
        lo = [g - 1 + e[0], g - 1 + e[1], g - 1 + e[2]]
        hi = q[:, lo[0]:lo[0] + ext[0], lo[1]:lo[1] + ext[1], lo[2]:lo[2] + ext[2]]
        lw = q[:, lo[0] - e[0]:lo[0] - e[0] + ext[0], lo[1] - e[1]:lo[1] - e[1] + ext[1],
               lo[2] - e[2]:lo[2] - e[2] + ext[2]]
        f0 = [s - 1 + e[0], s - 1 + e[1], s - 1 + e[2]]
        got = diff[d][:, f0[0]:f0[0] + ext[0], f0[1]:f0[1] + ext[1], f0[2]:f0[2] + ext[2]]
        assert np.array_equal(got, hi - lw)
    fs = m.face_shapes()
    grads = [[np.zeros((4,) + fs[d]) for _ in range(3)] for d in range(3)]  # [side][comp]
    outs = [grads[d][c] for d in range(3) for c in range(3)]
    orc.orc_quat_grad_side_symm(C.byref(m), *[O.ptr(x) for x in diff],
                                *[r.ctypes.data for r in rot], *[O.ptr(x) for x in outs])
    # QUATGRAD_SIDE: normal diff/h; tangential 1/4 of the four e-differences
    h = [m.dx[0], m.dx[1], m.dx[2]]

    def D(e, i, j, k):
        return diff[e][:, k + s, j + s, i + s]

    for d in range(3):
        ld = [d == 0, d == 1, d == 2]
        for (k, j, i) in [(0, 0, 0), (n2 - 1, n1 - 1, n0 - 1), (1, 2, 3)]:
            i2, j2, k2 = i + ld[0], j + ld[1], k + ld[2]  # also the last normal face
            for (ii, jj, kk) in [(i, j, k), (i2 if d == 0 else i, j2 if d == 1 else j,
                                             k2 if d == 2 else k)]:
                got = grads[d][d][:, kk + s, jj + s, ii + s]
                assert np.allclose(got, D(d, ii, jj, kk) / h[d], rtol=1e-15)
                for e in range(3):
                    if e == d:
                        continue
                    ue = [e == 0, e == 1, e == 2]
                    ref = 0.25 / h[e] * (D(e, ii + ue[0], jj + ue[1], kk + ue[2]) +
                                         D(e, ii + ue[0] - ld[0], jj + ue[1] - ld[1],
                                           kk + ue[2] - ld[2]) +
                                         D(e, ii - ld[0], jj - ld[1], kk - ld[2]) +
                                         D(e, ii, jj, kk))
                    got = grads[d][e][:, kk + s, jj + s, ii + s]
                    assert np.allclose(got, ref, rtol=1e-14, atol=1e-15)


def test_relabelling_invariance(orc):
    """A smooth unit-quaternion field with each cell's q replaced by
    q qr[random]: after QUAT_SYMM_ROTATION the symmetric differences have
    the magnitudes of the smooth field's plain differences."""
    qr, _ = _table(orc)
    m = _model()
    g = m.ng
    z, y, x = np.meshgrid(*[np.arange(-g, n + g) for n in (m.n[2], m.n[1], m.n[0])],
                          indexing="ij")
    # smooth and periodic: small rotation angles about a fixed axis
    ang = 0.15 * (np.sin(2 * np.pi * x / m.n[0]) + np.cos(2 * np.pi * y / m.n[1]) +
                  np.sin(2 * np.pi * z / m.n[2]))
    axis = np.array([1.0, 2.0, 3.0]) / np.sqrt(14.0)
    s = np.stack([np.cos(ang / 2)] + [np.sin(ang / 2) * a for a in axis], -1)
    rng = np.random.default_rng(4)
    # the same label on periodic images, as a ghost fill would leave them
    lab_i = rng.integers(48, size=(m.n[2], m.n[1], m.n[0]))
    lab = lab_i[(z % m.n[2]), (y % m.n[1]), (x % m.n[0])]
    q = np.ascontiguousarray(np.moveaxis(qmul(s, qr[lab]), -1, 0))
    rot = [np.zeros(sh, dtype=np.int32) for sh in m.face_shapes()]
    orc.orc_quat_symm_rotation(C.byref(m), O.ptr(q), *[r.ctypes.data for r in rot])
    diff = _sides(m)
    orc.orc_quat_diffs_symm(C.byref(m), O.ptr(q), *[r.ctypes.data for r in rot],
                            *[O.ptr(v) for v in diff])
    sg = m.ng_side
    for d in range(3):
        e = [0, 0, 0]
        e[2 - d] = 1
        n = [m.n[2], m.n[1], m.n[0]]
        hi = s[g:g + n[0] + e[0], g:g + n[1] + e[1], g:g + n[2] + e[2]]
        lo = s[g - e[0]:g + n[0], g - e[1]:g + n[1], g - e[2]:g + n[2]]
        ref = np.linalg.norm(hi - lo, axis=-1)
        got = diff[d][:, sg:sg + n[0] + e[0], sg:sg + n[1] + e[1], sg:sg + n[2] + e[2]]
        assert np.allclose(np.linalg.norm(got, axis=0), ref, atol=1e-14)
        assert ref.max() > 0.01  # the field does vary
