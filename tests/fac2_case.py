"""A two-level composite problem for the FAC tests: a periodic coarse level
and one fine box refined by 2, random positive face coefficients D, cell M
and a negative cell C on both levels (so A = M div(D grad) + C is negative
definite), seeded."""
import numpy as np

from ampe_gb300 import abi, configs


def make(n=(16, 12, 10), lo=(4, 3, 2), nbox=(6, 4, 4), level_dx=1, seed=0, variable=True,
         c_scale=1.0):
    m = configs.calphad3d(n[0], seed=1, T_run=1500.0)
    m.n[0], m.n[1], m.n[2] = n
    m.ng = 1
    m.ng_side = 0
    m.dx[0], m.dx[1], m.dx[2] = 1.0, 0.9, 1.1
    p = abi.Fac2()
    p.coarse = m
    for d in range(3):
        p.lo[d] = lo[d]
        p.nbox[d] = nbox[d]
    p.ng_fine = 1
    p.level_dx = level_dx
    p.presweeps = p.postsweeps = 2
    p.coarse_sweeps = 12
    p.d_const, p.c_const, p.m_const = 1.0, -c_scale, 1.0
    mf = p.fine_model()
    rng = np.random.default_rng(seed)
    lev = {}
    for name, mm in (("c", m), ("f", mf)):
        d = {}
        if variable:
            d["D"] = [rng.uniform(0.5, 1.5, s) for s in mm.face_shapes()]
            if name == "c":  # periodic level: the last face is the first one
                d["D"][0][:, :, -1] = d["D"][0][:, :, 0]
                d["D"][1][:, -1, :] = d["D"][1][:, 0, :]
                d["D"][2][-1, :, :] = d["D"][2][0, :, :]
            d["C"] = -c_scale * rng.uniform(1.0, 2.0, mm.ghost_shape())
            d["M"] = rng.uniform(0.5, 1.5, mm.ghost_shape())
        else:
            d["D"], d["C"], d["M"] = [None] * 3, None, None
        d["f"] = rng.standard_normal(mm.ghost_shape())
        d["u"] = np.zeros(mm.ghost_shape())
        lev[name] = d
    return p, m, mf, lev


def level_struct(d, ptr):
    s = abi.Fac2Level()
    for k in range(3):
        s.D[k] = ptr(d["D"][k]) if d["D"][k] is not None else None
    s.C = ptr(d["C"]) if d["C"] is not None else None
    s.M = ptr(d["M"]) if d["M"] is not None else None
    return s


def under_box(p, m):
    """(z, y, x) interior mask of the coarse cells under the fine box."""
    mask = np.zeros(tuple(m.interior_shape()), bool)
    idx = [((p.lo[d] + np.arange(p.nbox[d])) % m.n[d]) for d in range(3)]
    mask[np.ix_(idx[2], idx[1], idx[0])] = True
    return mask
