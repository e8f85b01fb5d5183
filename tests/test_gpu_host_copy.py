"""ampe_stepper_load_y / ampe_stepper_get_state with host buffers: pinned
host memory (copied by a kernel through the device's mapping of it) and
pageable memory (cudaMemcpyAsync) give the same bytes, for level sizes
with an even and an odd cell count."""
import ctypes as C

import numpy as np
import pytest

from ampe_gb300 import configs, initial
from ampe_gb300.stepper import ImplicitStepper

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [16, 15])
def test_pinned_and_pageable_copies_agree(cuda, n):
    import torch

    m = configs.calphad3d(n, seed=3, T_run=1500.0)
    phi, c = initial.calphad3d_state(n, seed=2, nseeds=2, radius=4.0)
    p = configs.step_params(dt=0.1, precond=2, mg_levels=2, atol=1e-6)
    g = ImplicitStepper(m, p)
    g.set_state(phi, c)
    g.advance(1)
    N = m.cells()
    L = cuda.lib
    # device -> host
    a_phi, a_c = np.zeros(N), np.zeros(N)
    assert L.ampe_stepper_get_state(g._h, a_phi.ctypes.data, a_c.ctypes.data, None, None, 1) == 0
    b_phi = torch.zeros(N, dtype=torch.float64).pin_memory()
    b_c = torch.zeros(N, dtype=torch.float64).pin_memory()
    assert L.ampe_stepper_get_state(g._h, C.c_void_p(b_phi.data_ptr()), C.c_void_p(b_c.data_ptr()),
                                    None, None, 1) == 0
    assert np.array_equal(a_phi, b_phi.numpy()) and np.array_equal(a_c, b_c.numpy())
    assert np.abs(a_phi).max() > 0
    # host -> device: a changed state loaded from pinned memory reads back
    rng = np.random.default_rng(1)
    new_phi = np.clip(a_phi + 1e-3 * rng.standard_normal(N), 0, 1)
    b_phi.copy_(torch.from_numpy(new_phi))
    assert L.ampe_stepper_load_y(g._h, C.c_void_p(b_phi.data_ptr()), C.c_void_p(b_c.data_ptr()),
                                 1) == 0
    r_phi, r_c = np.zeros(N), np.zeros(N)
    assert L.ampe_stepper_get_state(g._h, r_phi.ctypes.data, r_c.ctypes.data, None, None, 1) == 0
    assert np.array_equal(r_phi, new_phi) and np.array_equal(r_c, a_c)
    # and from pageable memory
    assert L.ampe_stepper_load_y(g._h, a_phi.ctypes.data, a_c.ctypes.data, 1) == 0
    assert L.ampe_stepper_get_state(g._h, r_phi.ctypes.data, r_c.ctypes.data, None, None, 1) == 0
    assert np.array_equal(r_phi, a_phi)
    g.close()
