"""Seeded synthetic initial conditions (numpy, interior arrays z,y,x).

The reference reads its initial conditions from NetCDF files written by
utils/*.py; here the same kinds of fields are generated in memory.
"""
import numpy as np


def tanh_seed(shape, centers, radii, width):
    """phi = 1/2 [1 - tanh((r - R)/W)] around each centre (max over seeds)."""
    grids = np.meshgrid(*[np.arange(s) + 0.5 for s in shape], indexing="ij")
    phi = np.zeros(shape)
    for c, R in zip(centers, radii):
        r2 = np.zeros(shape)
        for g, cc, s in zip(grids, c, shape):
            d = np.abs(g - cc)
            d = np.minimum(d, s - d)  # periodic distance
            r2 += d * d
        phi = np.maximum(phi, 0.5 * (1.0 - np.tanh((np.sqrt(r2) - R) / width)))
    return phi


def dilute2d_state(n=256, seed=0, radius=20.0, width=3.0, c0=0.02, noise=1e-3):
    rng = np.random.default_rng(seed)
    phi = tanh_seed((n, n), [(n / 2, n / 2)], [radius], width)
    c = c0 + rng.uniform(-noise, noise, size=(n, n))
    return phi.reshape(1, n, n), c.reshape(1, n, n)


def calphad3d_state(n=256, seed=0, nseeds=16, radius=None, width=3.0,
                    clo=0.3, chi=0.5):
    rng = np.random.default_rng(seed)
    if radius is None:
        radius = max(3.0, n / 24.0)
    centers = [tuple(rng.uniform(0, n, size=3)) for _ in range(nseeds)]
    phi = tanh_seed((n, n, n), centers, [radius] * nseeds, width)
    c = rng.uniform(clo, chi, size=(n, n, n))
    return phi, c


def random_unit_quaternions(rng, k):
    """k unit quaternions uniform on S^3 (normalised Gaussian 4-vectors)."""
    q = rng.standard_normal((k, 4))
    return q / np.linalg.norm(q, axis=1, keepdims=True)


def polycrystal_state(n=128, ngrains=8, seed=0, channel=6.0, width=1.5,
                      clo=0.3, chi=0.5):
    """Periodic Voronoi polycrystal: grain interiors solid (phi = 1), a liquid
    channel `channel` cells wide along the grain boundaries, each grain's
    orientation a random unit quaternion (the channel cells take their
    nearest grain's), c ~ U[clo, chi].  Returns phi, c, q (4, z, y, x).
    Built slab by slab along z so that 512^3 levels fit in host memory."""
    rng = np.random.default_rng(seed)
    seeds = rng.uniform(0, n, size=(ngrains, 3))
    quats = random_unit_quaternions(rng, ngrains)
    ax = np.arange(n) + 0.5
    phi = np.empty((n, n, n))
    q = np.empty((4, n, n, n))
    y, x = np.meshgrid(ax, ax, indexing="ij")
    dxy = []
    for s_ in seeds:  # periodic in-plane squared distances, per seed
        dx = np.abs(x - s_[0])
        dx = np.minimum(dx, n - dx)
        dy = np.abs(y - s_[1])
        dy = np.minimum(dy, n - dy)
        dxy.append(dx * dx + dy * dy)
    for k in range(n):
        z = ax[k]
        d1 = np.full((n, n), np.inf)
        d2 = np.full((n, n), np.inf)
        g1 = np.zeros((n, n), dtype=np.int64)
        for g, s_ in enumerate(seeds):
            dz = abs(z - s_[2])
            dz = min(dz, n - dz)
            dd = np.sqrt(dxy[g] + dz * dz)
            closer = dd < d1
            d2 = np.where(closer, d1, np.minimum(d2, dd))
            g1 = np.where(closer, g, g1)
            d1 = np.where(closer, dd, d1)
        dist_gb = 0.5 * (d2 - d1)  # distance to the nearest grain boundary
        phi[k] = 0.5 * (1.0 + np.tanh((dist_gb - 0.5 * channel) / width))
        q[:, k] = np.moveaxis(quats[g1], -1, 0)
    c = rng.uniform(clo, chi, size=(n, n, n))
    return phi, c, q


def dendrite2d_state(n=2048, nseeds=16, radius=8.0, seed=0, width=3.0, c0=0.02,
                     noise=1e-3):
    """2D seeds of the given radius at seeded random centres, each with a
    random orientation angle theta in [0, pi); every cell takes its nearest
    seed's angle.  Returns phi, c (1, n, n) and q (2, 1, n, n) =
    (cos theta, sin theta), the 2-component orientation read by the 2D
    anisotropic flux (phi_orient = acos q0)."""
    rng = np.random.default_rng(seed)
    centers = [tuple(rng.uniform(0, n, size=2)) for _ in range(nseeds)]
    angles = rng.uniform(0.0, np.pi, size=nseeds)
    phi = tanh_seed((n, n), centers, [radius] * nseeds, width)
    ax = np.arange(n) + 0.5
    yy, xx = np.meshgrid(ax, ax, indexing="ij")
    best = np.full((n, n), np.inf)
    theta = np.zeros((n, n))
    for (cy, cx), a in zip(centers, angles):
        dy = np.abs(yy - cy)
        dy = np.minimum(dy, n - dy)
        dx = np.abs(xx - cx)
        dx = np.minimum(dx, n - dx)
        d = dx * dx + dy * dy
        closer = d < best
        theta = np.where(closer, a, theta)
        best = np.where(closer, d, best)
    c = c0 + rng.uniform(-noise, noise, size=(n, n))
    q = np.stack([np.cos(theta), np.sin(theta)]).reshape(2, 1, n, n)
    return phi.reshape(1, n, n), c.reshape(1, n, n), np.ascontiguousarray(q)
