"""Learned collision closure: a per-node MLP that corrects the post-collision
non-conserved moments of a coarse simulation.

``Mlp`` owns the FP32 master parameters, their BF16 copies, the Adam moments
and the gradient buffer on the device, and drives the tensor-core kernels of
liblbm_gb300.so (lbm_mlp_forward / lbm_mlp_gradients / lbm_mlp_adam).  The
inputs are the node's pre-collision moments (normalised), the outputs the
corrections of the non-conserved moments (normalised); conserved moments are
never touched, so mass and momentum stay exactly conserved.
"""
import ctypes

import numpy as np

from . import runtime
from .simulation import to_storage

IN, H, OUT, NUSED = 16, 64, 8, 6


def sizes():
    npar, nw = ctypes.c_int32(), ctypes.c_int32()
    runtime.check(runtime.core().lbm_mlp_sizes(ctypes.byref(npar), ctypes.byref(nw)))
    return npar.value, nw.value


def init_params(seed=0):
    """He-style initialisation of the FP32 parameter block (biases zero)."""
    rng = np.random.default_rng(seed)
    parts = []
    for fan_out, fan_in in ((H, IN), (H, H), (OUT, H)):
        parts.append(rng.normal(0.0, np.sqrt(1.0 / fan_in), (fan_out, fan_in)).ravel())
        parts.append(np.zeros(fan_out))
    return np.concatenate(parts).astype(np.float32)


def _bf16_bits(x):
    x = np.asarray(x, dtype=np.float64)
    if x.ndim != 2 or x.shape[1] != IN:
        raise ValueError(f"inputs must be (n, {IN})")
    return to_storage(x, "bfloat16")


class Mlp:
    """Device-resident MLP parameters with training and inference entry points."""

    def __init__(self, seed=0, params=None, stream=None):
        self.nparam, self.nweights = sizes()
        self._core = runtime.core()
        self.stream = stream
        p = init_params(seed) if params is None else np.asarray(params, dtype=np.float32)
        if p.size != self.nparam:
            raise ValueError(f"expected {self.nparam} parameters")
        self.p = runtime.DeviceBuffer(4 * self.nparam)
        self.m = runtime.DeviceBuffer(4 * self.nparam)
        self.v = runtime.DeviceBuffer(4 * self.nparam)
        self.g = runtime.DeviceBuffer(4 * self.nparam)
        self.w = runtime.DeviceBuffer(2 * self.nweights)
        self.loss = runtime.DeviceBuffer(16)
        self.p.upload(p, stream=stream)
        for b in (self.m, self.v, self.g):
            b.zero(stream)
        self.step = 0
        self._scratch = None
        self.sync()

    def sync(self):
        runtime.check(self._core.lbm_mlp_sync_weights(self.p.handle, self.w.handle, self.stream))

    def params_host(self):
        out = np.empty(self.nparam, dtype=np.float32)
        self.p.download(out, stream=self.stream)
        return out

    def set_params(self, p):
        self.p.upload(np.asarray(p, dtype=np.float32), stream=self.stream)
        self.sync()

    def _scratch_for(self, n):
        size = ctypes.c_size_t()
        runtime.check(self._core.lbm_mlp_scratch_bytes(n, ctypes.byref(size)))
        if self._scratch is None or self._scratch.nbytes < size.value:
            self._scratch = runtime.DeviceBuffer(size.value)
        return self._scratch

    # ------------------------------------------------------------ host arrays
    def forward(self, x):
        """Outputs (n, 8) float64 for inputs (n, 16) (rounded to BF16)."""
        xb = _bf16_bits(x)
        n = xb.shape[0]
        pad = (-n) % 16
        if pad:
            xb = np.concatenate([xb, np.zeros((pad, IN), dtype=np.uint16)])
        dx = runtime.DeviceBuffer(xb.nbytes)
        dx.upload(xb, stream=self.stream)
        dy = runtime.DeviceBuffer(4 * OUT * xb.shape[0])
        runtime.check(self._core.lbm_mlp_forward(dx.handle, xb.shape[0], self.w.handle, self.p.handle, dy.handle,
                                                 self.stream))
        y = np.empty((xb.shape[0], OUT), dtype=np.float32)
        dy.download(y, stream=self.stream)
        return y[:n].astype(np.float64)

    def _device_data(self, x, t):
        xb = _bf16_bits(x)
        n = xb.shape[0]
        if n % 16:
            raise ValueError("the batch size must be a multiple of 16")
        dx = runtime.DeviceBuffer(xb.nbytes)
        dx.upload(xb, stream=self.stream)
        tt = np.zeros((n, OUT), dtype=np.float32)
        tt[:, :] = np.asarray(t, dtype=np.float32)[:, :OUT]
        dt = runtime.DeviceBuffer(tt.nbytes)
        dt.upload(tt, stream=self.stream)
        return dx, dt, n

    def gradients(self, x, t):
        """(loss, gradient float64) of the mean squared error on the 6 outputs."""
        dx, dt, n = self._device_data(x, t)
        self.g.zero(self.stream)
        loss = self.gradients_device(dx, dt, n)
        grad = np.empty(self.nparam, dtype=np.float32)
        self.g.download(grad, stream=self.stream)
        self.g.zero(self.stream)
        return loss, grad.astype(np.float64)

    def train_step(self, x, t, lr=1e-3):
        dx, dt, n = self._device_data(x, t)
        return self.train_step_device(dx, dt, n, lr)

    # ---------------------------------------------------------- device arrays
    def gradients_device(self, dx, dt, n, read_loss=True):
        scratch = self._scratch_for(n)
        runtime.check(self._core.lbm_mlp_gradients(dx.handle if hasattr(dx, "handle") else dx,
                                                   dt.handle if hasattr(dt, "handle") else dt, n, self.w.handle,
                                                   self.p.handle, self.g.handle, self.loss.handle, scratch.handle,
                                                   scratch.nbytes, self.stream))
        if not read_loss:
            return None
        out = np.empty(1, dtype=np.float32)
        self.loss.download(out, stream=self.stream)
        return float(out[0])

    def train_step_device(self, dx, dt, n, lr=1e-3, read_loss=True):
        loss = self.gradients_device(dx, dt, n, read_loss)
        self.step += 1
        runtime.check(self._core.lbm_mlp_adam(self.p.handle, self.m.handle, self.v.handle, self.g.handle, lr, 0.9,
                                              0.999, 1e-8, self.step, self.w.handle, self.stream))
        return loss
