"""Learned-closure MLP kernels against the CPU oracle (oracle/mlp_oracle.py).

Forward outputs and gradients of the BF16/FP32 tensor-core kernels are
compared with a float64 NumPy evaluation that rounds to BF16 at the same
points, and with the exact float64 gradient.
"""
import ctypes

import numpy as np
import pytest

import mlp_oracle as mo
from pylbm_gb300 import runtime
from pylbm_gb300.closure import Mlp

pytestmark = pytest.mark.gpu


def _data(n, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, mo.IN))
    x[:, 9:] = 0.0
    t = rng.normal(size=(n, mo.OUT))
    return mo.bf16(x), t


def test_forward_matches_oracle():
    mlp = Mlp(seed=3)
    x, _ = _data(256)
    y = mlp.forward(x)
    ref, _ = mo.forward(mlp.params_host().astype(np.float64), x)
    assert np.abs(y - ref).max() <= 2e-3 * np.abs(ref).max()


@pytest.mark.parametrize("n", [128, 1000, 20000])
def test_tensor_memory_forward_matches_oracle_and_warp_forward(n):
    """lbm_mlp_forward_tc (tcgen05.mma, FP32 accumulators in tensor memory,
    partial last tile) against the oracle and the warp-level kernel."""
    mlp = Mlp(seed=3)
    x, _ = _data(n, seed=7)
    y_tc = mlp.forward_tc(x)
    ref, _ = mo.forward(mlp.params_host().astype(np.float64), x)
    scale = np.abs(ref).max()
    # the FP32 accumulation order inside a layer differs from the oracle's and
    # the warp kernel's: a hidden activation can round to the neighbouring
    # BF16 value (measured up to 2.2e-3 of the output scale at n = 1000)
    assert np.abs(y_tc - ref).max() <= 5e-3 * scale
    assert np.abs(y_tc - mlp.forward(x)).max() <= 5e-3 * scale
    count = ctypes.c_uint32()
    runtime.check(runtime.core().lbm_mlp_tc_timeouts(ctypes.byref(count)))
    assert count.value == 0


@pytest.mark.parametrize("kernel,n", [("warp", 16), ("warp", 4096), ("warp", 10000 - 10000 % 16),
                                      ("tc", 16), ("tc", 1000), ("tc", 4096), ("tc", 40000)])
def test_gradients_match_oracle(kernel, n):
    """warp: k_mlp_fwd_bwd + k_mlp_wgrad; tc: k_mlp_train_tc (tcgen05, one
    kernel, gradients accumulated in tensor memory; any n, partial last
    tile, several tiles per block at n = 40000)."""
    mlp = Mlp(seed=5)
    mlp.train_kernel = kernel
    x, t = _data(n, seed=n)
    loss, grad = mlp.gradients(x, t)
    p = mlp.params_host().astype(np.float64)
    ref_loss, ref = mo.loss_and_grad(p, x, t, bf16_points=True)
    _, exact = mo.loss_and_grad(p, x, t, bf16_points=False)
    assert abs(loss - ref_loss) <= 1e-4 * ref_loss
    rel = np.linalg.norm(grad - ref) / np.linalg.norm(ref)
    assert rel < 5e-3, rel
    rel_exact = np.linalg.norm(grad - exact) / np.linalg.norm(exact)
    assert rel_exact < 5e-2, rel_exact
    # per-block agreement (each weight matrix and bias)
    i = 0
    for name, shape in mo.SHAPES:
        k = int(np.prod(shape))
        blk = slice(i, i + k)
        if np.linalg.norm(ref[blk]) > 0:
            assert np.linalg.norm(grad[blk] - ref[blk]) / np.linalg.norm(ref[blk]) < 2e-2, name
        i += k
    if kernel == "tc":
        count = ctypes.c_uint32()
        runtime.check(runtime.core().lbm_mlp_tc_timeouts(ctypes.byref(count)))
        assert count.value == 0


def test_tensor_core_gradients_equal_warp_gradients():
    """The two training paths on the same batch: the same loss and gradients
    up to the FP32 accumulation order (a BF16 activation or gradient may round
    to its neighbour)."""
    x, t = _data(4096, seed=11)
    out = {}
    for kernel in ("warp", "tc"):
        mlp = Mlp(seed=9)
        mlp.train_kernel = kernel
        out[kernel] = mlp.gradients(x, t)
    (lw, gw), (lt, gt) = out["warp"], out["tc"]
    assert abs(lw - lt) <= 1e-5 * lw
    assert np.linalg.norm(gt - gw) / np.linalg.norm(gw) < 5e-3


@pytest.mark.parametrize("kernel", ["warp", "tc"])
def test_adam_training_reduces_loss(kernel):
    """Fit a smooth map with the GPU training step; the loss must drop."""
    rng = np.random.default_rng(7)
    n = 8192
    x = rng.normal(size=(n, mo.IN))
    x[:, 9:] = 0.0
    x = mo.bf16(x)
    t = np.zeros((n, mo.OUT))
    t[:, :6] = np.tanh(x[:, :6] * 0.7) + 0.3 * x[:, 1:7] * x[:, 2:8]
    mlp = Mlp(seed=11)
    mlp.train_kernel = kernel
    first = mlp.train_step(x, t, lr=3e-3)
    for _ in range(300):
        last = mlp.train_step(x, t, lr=3e-3)
    assert last < 0.2 * first, (first, last)


@pytest.mark.parametrize("n", [16, 1000, 40000])
def test_vector_jacobian_product_matches_oracle(n):
    """lbm_mlp_vjp_tc: the gradient of sum(dy . y) for a given output
    gradient dy (the backward step of the a-posteriori training), against
    the oracle with the same BF16 rounding points and the exact float64 one."""
    mlp = Mlp(seed=4)
    x, dy = _data(n, seed=n + 1)
    dot, grad = mlp.vjp(x, dy)
    p = mlp.params_host().astype(np.float64)
    ref_dot, ref = mo.vjp(p, x, dy, bf16_points=True)
    _, exact = mo.vjp(p, x, dy, bf16_points=False)
    y_ref, _ = mo.forward(p, x)
    assert abs(dot - ref_dot) <= 5e-3 * np.abs(dy[:, :6] * y_ref[:, :6]).sum()
    assert np.linalg.norm(grad - ref) / np.linalg.norm(ref) < 5e-3
    assert np.linalg.norm(grad - exact) / np.linalg.norm(exact) < 5e-2
    count = ctypes.c_uint32()
    runtime.check(runtime.core().lbm_mlp_tc_timeouts(ctypes.byref(count)))
    assert count.value == 0
