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
