"""numpy restatement of the surrogate MLP used to check the GPU kernels
(test infrastructure).  Parameters are the FP32 master vector
[W0 b0 W1 b1 W2 b2 W3 b3], W row-major [out][in]; the forward pass rounds
the weights to BF16 (round to nearest even), activations stay unrounded,
SiLU exact; loss = 1/2 mean over samples of the squared logit errors."""
import numpy as np

SIZES = [(64, 3), (64, 64), (64, 64), (2, 64)]


def bf16(x):
    x32 = np.ascontiguousarray(x, dtype=np.float32)
    u = x32.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32)


def unpack(params):
    out, off = [], 0
    for n, k in SIZES:
        W = params[off:off + n * k].reshape(n, k)
        off += n * k
        b = params[off:off + n]
        off += n
        out.append((W, b))
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, x, round_acts=False):
    layers = unpack(np.asarray(params, np.float64))
    a = np.asarray(x[:, :3], np.float64)
    if round_acts:
        a = bf16(a).astype(np.float64)
    zs, acts = [], [a]
    for li, (W, b) in enumerate(layers):
        z = a @ bf16(W).astype(np.float64).T + b
        zs.append(z)
        a = silu(z) if li < 3 else z
        if round_acts and li < 3:
            a = bf16(a).astype(np.float64)
        acts.append(a)
    return zs, acts


def loss_and_grad(params, x, target):
    zs, acts = forward(params, x)
    y = acts[-1]
    B = x.shape[0]
    d = y - target
    loss = 0.5 * np.sum(d * d) / B
    dz = d / B
    layers = unpack(np.asarray(params, np.float64))
    grads = []
    for li in range(3, -1, -1):
        W, b = layers[li]
        xin = acts[li]
        gW = dz.T @ xin
        gb = dz.sum(axis=0)
        grads.append((gW, gb))
        if li > 0:
            dz = (dz @ bf16(W).astype(np.float64)) * dsilu(zs[li - 1])
    grads.reverse()
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat


def fp16(x):
    return np.asarray(x, np.float64).astype(np.float16).astype(np.float64)


def loss_and_grad_bf16(params, x, target):
    """The gradient as the tensor-core training kernel forms it: operands of
    every product rounded to BF16 (inputs, activations, weights, and the
    back-propagated dZ of each layer), silu'(z) stored in FP16, products and
    sums accumulated exactly here (FP32 on the GPU); the bias gradients are
    the sums of the BF16 dZ."""
    zs, acts = forward(params, x, round_acts=True)
    y = acts[-1]
    B = x.shape[0]
    d = y - target
    loss = 0.5 * np.sum(d * d) / B
    dz = d / B
    layers = unpack(np.asarray(params, np.float64))
    grads = []
    for li in range(3, -1, -1):
        W, b = layers[li]
        dzb = bf16(dz).astype(np.float64)
        xin = acts[li]
        grads.append((dzb.T @ xin, dzb.sum(axis=0)))
        if li > 0:
            dz = (dzb @ bf16(W).astype(np.float64)) * fp16(dsilu(zs[li - 1]))
    grads.reverse()
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat
