"""CPU oracle of the learned-closure MLP (float64 NumPy).

TEST INFRASTRUCTURE ONLY: checks the GPU forward pass and gradients of
pylbm_gb300's MLP kernels (lbm_mlp_forward / lbm_mlp_gradients /
lbm_mlp_vjp_tc).

Network x(16) -> 64 SiLU -> 64 SiLU -> y(8); loss = mean over samples and the
first 6 outputs of (y - target)^2.  Parameters use the FP32 block layout of
include/lbm_gb300.h (W1[64][16] b1[64] W2[64][64] b2[64] W3[8][64] b3[8]).
With ``bf16=True`` the values are rounded to bfloat16 where the kernels
round them (weights, inputs, hidden activations, dL/dy, hidden gradients),
so only the accumulation order differs from the GPU.
"""
import numpy as np

IN, H, OUT, NUSED = 16, 64, 8, 6
SHAPES = [("W1", (H, IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (OUT, H)), ("b3", (OUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)


def bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    b = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = ((b >> 16) & 1) + 0x7FFF
    return ((b + r) & 0xFFFF0000).view(np.float32).astype(np.float64)


def unpack(p):
    out, i = {}, 0
    for name, shape in SHAPES:
        k = int(np.prod(shape))
        out[name] = np.asarray(p[i:i + k], dtype=np.float64).reshape(shape)
        i += k
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def init_params(seed=0, scale=1.0):
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in SHAPES:
        if name.startswith("W"):
            fan_in = shape[1]
            d[name] = rng.normal(0.0, scale / np.sqrt(fan_in), shape)
        else:
            d[name] = np.zeros(shape)
    return pack(d).astype(np.float32)


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, x, bf16_points=True):
    r = bf16 if bf16_points else (lambda v: np.asarray(v, dtype=np.float64))
    w = unpack(p)
    W1, W2, W3 = (r(w[k]) for k in ("W1", "W2", "W3"))
    x = r(x)
    z1 = x @ W1.T + w["b1"]
    h1 = r(_silu(z1))
    z2 = h1 @ W2.T + w["b2"]
    h2 = r(_silu(z2))
    y = h2 @ W3.T + w["b3"]
    return y, (x, z1, h1, z2, h2, W1, W2, W3)


def _backward(dy, cache, r):
    xr, z1, h1, z2, h2, W1, W2, W3 = cache
    dy = r(dy)
    dh2 = r((dy @ W3) * _silu_grad(z2))
    dh1 = r((dh2 @ W2) * _silu_grad(z1))
    g = {"W3": dy.T @ h2, "b3": dy.sum(0), "W2": dh2.T @ h1, "b2": dh2.sum(0), "W1": dh1.T @ xr,
         "b1": dh1.sum(0)}
    return pack(g)


def loss_and_grad(p, x, target, bf16_points=True):
    r = bf16 if bf16_points else (lambda v: np.asarray(v, dtype=np.float64))
    n = x.shape[0]
    y, cache = forward(p, x, bf16_points)
    diff = np.zeros_like(y)
    diff[:, :NUSED] = y[:, :NUSED] - target[:, :NUSED]
    loss = float((diff ** 2).sum() / (NUSED * n))
    return loss, _backward(2.0 * diff / (NUSED * n), cache, r)


def vjp(p, x, dy, bf16_points=True):
    """(sum of dy . y, gradient of that sum) over the first 6 outputs: the
    backward step of the MLP inside a larger differentiated computation, dy
    being the loss gradient with respect to the outputs."""
    r = bf16 if bf16_points else (lambda v: np.asarray(v, dtype=np.float64))
    y, cache = forward(p, x, bf16_points)
    d = np.zeros_like(y)
    d[:, :NUSED] = np.asarray(dy, dtype=np.float64)[:, :NUSED]
    return float((d * y).sum()), _backward(d, cache, r)


def finite_difference(p, x, target, idx, eps=1e-6):
    """Central difference of the exact (unrounded) loss along parameters ``idx``."""
    out = []
    for i in idx:
        pp = np.asarray(p, dtype=np.float64).copy()
        pp[i] += eps
        lp, _ = loss_and_grad(pp, x, target, bf16_points=False)
        pp[i] -= 2 * eps
        lm, _ = loss_and_grad(pp, x, target, bf16_points=False)
        out.append((lp - lm) / (2 * eps))
    return np.array(out)
