"""Surrogate MLP: gradients of the GPU training kernels against the numpy
oracle, tensor-core (tcgen05) inference against the CUDA-core reference
kernel and numpy, training on Newton-labelled samples, and the mixed stepper
with the surrogate initial guess against the FP64 oracle; the surrogate is
evaluated only while no converged warm start exists (a cold start)."""
import ctypes as C

import numpy as np
import pytest

import mlp_oracle as MO
import oracle as O
from ampe_gb300 import configs, initial
from ampe_gb300.stepper import ImplicitStepper

pytestmark = pytest.mark.gpu


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _mlp(cuda, m, batch=512, seed=7):
    h = C.c_void_p()
    assert cuda.lib.ampe_mlp_create(C.byref(m), batch, seed, C.byref(h)) == 0
    return h


def test_gradients_match_oracle(cuda):
    import torch

    L = cuda.lib
    m = configs.calphad3d(16, seed=3, T_run=1500.0)
    h = _mlp(cuda, m, batch=256)
    npar = L.ampe_mlp_nparams(h)
    rng = np.random.default_rng(3)
    params = (rng.standard_normal(npar) * 0.3).astype(np.float32)
    assert L.ampe_mlp_set(h, params.ctypes.data, 1) == 0
    B = 256
    x = np.zeros((B, 4), np.float32)
    x[:, :3] = rng.uniform(-1, 1, (B, 3))
    tgt = rng.standard_normal((B, 2)).astype(np.float32)
    xd = torch.from_numpy(x).cuda()
    td = torch.from_numpy(tgt).cuda()
    loss = C.c_float()
    assert L.ampe_mlp_grad(h, _p(xd), _p(td), B, C.byref(loss)) == 0
    g = np.empty(npar, np.float32)
    assert L.ampe_mlp_get(h, None, g.ctypes.data, 1) == 0
    # the tensor-core products round every operand to BF16: against the
    # oracle that rounds the same operands the gradient agrees to FP32
    # accumulation (and the odd BF16 rounding flip); against the unrounded
    # FP64 gradient to BF16 resolution
    lo, go = MO.loss_and_grad_bf16(params.astype(np.float64), x.astype(np.float64),
                                   tgt.astype(np.float64))
    lx, gx = MO.loss_and_grad(params.astype(np.float64), x.astype(np.float64),
                              tgt.astype(np.float64))
    e_bf = np.linalg.norm(g - go) / np.linalg.norm(go)
    e_ex = np.linalg.norm(g - gx) / np.linalg.norm(gx)
    print("tensor-core gradient: rel L2 %.2e vs the BF16-operand oracle, %.2e vs FP64" % (e_bf, e_ex))
    assert abs(loss.value - lo) <= 1e-5 * lo
    assert e_bf <= 2e-3
    assert e_ex <= 3e-2
    L.ampe_mlp_destroy(h)


def test_tensor_core_wait_timeout(cuda):
    """The bounded mbarrier waits of the tcgen05 kernels: with the issue
    skipped (nothing in flight) a wait of 64 polls runs out, the status
    reports it, tensor memory is freed, and the next calls succeed."""
    import torch

    L = cuda.lib
    m = configs.calphad3d(16, seed=3, T_run=1500.0)
    h = _mlp(cuda, m, batch=256)
    phi = O.ghosted(m, np.full(m.interior_shape(), 0.5))
    c = O.ghosted(m, np.full(m.interior_shape(), 0.4))
    pd, cd = torch.from_numpy(phi).cuda(), torch.from_numpy(c).cuda()
    N = m.cells()
    gl = torch.zeros(N, dtype=torch.float32, device="cuda")
    gs = torch.zeros(N, dtype=torch.float32, device="cuda")
    x = torch.zeros((256, 4), dtype=torch.float32, device="cuda")
    t = torch.zeros((256, 2), dtype=torch.float32, device="cuda")
    loss = C.c_float()
    ref = []
    for skip in (0, 1, 0):
        assert L.ampe_mlp_set_wait_limit(h, 64 if skip else 1 << 22, skip) == 0
        assert L.ampe_mlp_clear_status(h) == 0
        assert L.ampe_mlp_infer(h, C.byref(m), _p(pd), _p(cd), None, _p(gl), _p(gs), 1, None) == 0
        torch.cuda.synchronize()
        assert L.ampe_mlp_status(h) == (-3 if skip else 0)
        assert L.ampe_mlp_clear_status(h) == 0
        assert L.ampe_mlp_grad(h, _p(x), _p(t), 256, C.byref(loss)) == 0
        assert L.ampe_mlp_status(h) == (-3 if skip else 0)
        if not skip:
            ref.append(gl.cpu().numpy().copy())
    assert np.array_equal(ref[0], ref[1])
    L.ampe_mlp_destroy(h)


def test_tensor_core_inference_matches_reference(cuda):
    import torch

    L = cuda.lib
    m = configs.calphad3d(24, seed=3, T_run=1500.0)
    h = _mlp(cuda, m)
    npar = L.ampe_mlp_nparams(h)
    rng = np.random.default_rng(5)
    params = (rng.standard_normal(npar) * 0.25).astype(np.float32)
    assert L.ampe_mlp_set(h, params.ctypes.data, 1) == 0
    assert L.ampe_mlp_set_normalization(h, 1450.0, 1550.0) == 0
    phi = O.ghosted(m, rng.uniform(0, 1, m.interior_shape()))
    c = O.ghosted(m, rng.uniform(0.3, 0.5, m.interior_shape()))
    pd, cd = torch.from_numpy(phi).cuda(), torch.from_numpy(c).cuda()
    N = m.cells()
    out = {}
    for tc in (1, 0):
        gl = torch.zeros(N, dtype=torch.float32, device="cuda")
        gs = torch.zeros(N, dtype=torch.float32, device="cuda")
        assert L.ampe_mlp_infer(h, C.byref(m), _p(pd), _p(cd), None, _p(gl), _p(gs), tc, None) == 0
        torch.cuda.synchronize()
        out[tc] = (gl.cpu().numpy(), gs.cpu().numpy())
    assert L.ampe_mlp_status(h) == 0
    # numpy forward with BF16 activations, as the reference kernel computes
    gi = m.ng
    gz = gi
    phi_i = phi[gz:-gz, gi:-gi, gi:-gi].ravel()
    c_i = c[gz:-gz, gi:-gi, gi:-gi].ravel()
    x = np.zeros((N, 4))
    x[:, 0] = 2 * phi_i - 1
    x[:, 1] = 2 * c_i - 1
    i = np.tile(np.arange(m.n[0]), m.n[1] * m.n[2])
    T = m.T0 + m.gradT * (i + 0.5)
    x[:, 2] = (T - 1500.0) / 50.0
    _, acts = MO.forward(params, x, round_acts=True)
    y = acts[-1]
    ref = 1.0 / (1.0 + np.exp(-y))
    # identical math up to FP32 vs FP64 accumulation; an activation landing on
    # a BF16 rounding tie can flip by one BF16 ulp, hence the max bound
    for k in range(2):
        d = np.abs(out[0][k] - ref[:, k])
        assert d.max() < 2e-3 and d.mean() < 1e-5, (k, d.max(), d.mean())
    # tensor cores with bf16x2 tanh-based SiLU: a few 1e-3
    for k in range(2):
        d = np.abs(out[1][k] - out[0][k])
        assert d.max() < 3e-2 and d.mean() < 5e-3, (k, d.max(), d.mean())
    L.ampe_mlp_destroy(h)


def _trained(cuda, m, nsamp=1 << 17, steps=1500):
    L = cuda.lib
    h = _mlp(cuda, m, batch=4096, seed=11)
    fails = C.c_longlong()
    assert L.ampe_mlp_generate(h, nsamp, 99, 1450.0, 1550.0, 0.01, 0.99, C.byref(fails)) == 0
    assert fails.value == 0
    loss = C.c_float()
    assert L.ampe_mlp_train(h, steps, 4096, 3e-3, C.byref(loss)) == 0
    return h, loss.value


def test_training_and_surrogate_stepper(cuda):
    m = configs.calphad3d(16, seed=3, T_run=1500.0)
    h, loss = _trained(cuda, m)
    assert loss < 0.05, loss
    phi, c = initial.calphad3d_state(16, seed=2, nseeds=2, radius=4.5)
    nsteps = 6
    p64 = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6)
    o = O.OracleStepper(m, p64)
    o.set_state(phi, c)
    rc, so = o.advance(nsteps)
    assert rc == 0
    ps = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6, precision=1, surrogate=1)
    g = ImplicitStepper(m, ps)
    assert cuda.lib.ampe_stepper_attach_surrogate(g._h, h) == 0
    g.set_state(phi, c)
    sg = g.advance(nsteps)
    assert sg["kks_fail"] == 0
    errs = [O.rel_l2(a, b) for a, b in zip(g.get_state()[:2], o.get_state()[:2])]
    print("surrogate stepper rel L2:", errs, sg, "train loss", loss)
    assert max(errs) <= 2e-6
    # the network removes most Newton work from a cold start (guess = c)
    pm = configs.step_params(dt=0.1, precond=2, mg_levels=3, atol=1e-6, precision=1)
    cold = ImplicitStepper(m, pm)
    cold.set_state(phi, c)
    st_cold = cold.advance(1)
    warm = ImplicitStepper(m, ps)
    cuda.lib.ampe_stepper_attach_surrogate(warm._h, h)
    warm.set_state(phi, c)
    st_warm = warm.advance(1)
    print("first step KKS iterations: plain", st_cold["kks_iters"], "surrogate", st_warm["kks_iters"],
          "fallbacks", st_warm["kks_fallback"])
    assert st_warm["kks_iters"] < st_cold["kks_iters"]
    # once a step has converged, its phase concentrations are the warm start
    # and the network is no longer evaluated
    kt_mlp = 3
    assert cuda.lib.ampe_stepper_profile(warm._h, 1) == 0
    warm.advance(1)
    t, cnt = C.c_double(), C.c_longlong()
    assert cuda.lib.ampe_stepper_kernel_time(warm._h, kt_mlp, C.byref(t), C.byref(cnt)) == 0
    assert cnt.value == 0
    cuda.lib.ampe_mlp_destroy(h)
