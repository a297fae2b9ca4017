"""Learned collision closure: a per-node MLP that corrects the post-collision
non-conserved moments of a coarse simulation.

``Mlp`` owns the FP32 master parameters, their BF16 copies, the Adam moments
and the gradient buffer on the device, and drives the tensor-core kernels of
liblbm_gb300.so (lbm_mlp_forward(_tc) / lbm_mlp_gradients(_tc) /
lbm_mlp_vjp_tc / lbm_mlp_adam).  The inputs are the node's pre-collision
moments (normalised), the outputs the corrections of the non-conserved
moments (additive form) or the factors of their relaxation rates (rate
form); conserved moments are never touched, so mass and momentum stay
exactly conserved.  The first, one-step training of this module
(generate_training_data / train) is kept beside the a-posteriori training
of closure_train.py, which produced the shipped model.
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
        # "tc": k_mlp_train_tc (tcgen05, one kernel; 26.6 us per Adam step of
        # 2048 samples); "warp": k_mlp_fwd_bwd + k_mlp_wgrad (mma.sync, 279 us)
        self.train_kernel = "tc"
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

    def forward_tc(self, x):
        """The same outputs from the tcgen05 kernel (lbm_mlp_forward_tc: tiles of
        128 samples, accumulators in tensor memory), any number of rows."""
        xb = _bf16_bits(x)
        n = xb.shape[0]
        dx = runtime.DeviceBuffer(max(xb.nbytes, 32))
        dx.upload(xb, stream=self.stream)
        dy = runtime.DeviceBuffer(max(4 * OUT * n, 4))
        runtime.check(self._core.lbm_mlp_forward_tc(dx.handle, n, self.p.handle, dy.handle, self.stream))
        y = np.empty((n, OUT), dtype=np.float32)
        dy.download(y, stream=self.stream)
        dx.free()
        dy.free()
        return y.astype(np.float64)

    def forward_device(self, x, n, y, stream=None):
        """lbm_mlp_forward_tc on device pointers: x (n, 16) BF16 rows, y (n, 8)
        FP32; on ``stream`` (a raw CUDA stream handle) if given, else the Mlp's."""
        runtime.check(self._core.lbm_mlp_forward_tc(ctypes.c_void_p(x), n, self.p.handle, ctypes.c_void_p(y),
                                                    self.stream if stream is None else stream))

    def vjp_device(self, x, dy, n, stream=None):
        """Adds the gradient of sum(dy . y) over the 6 used outputs to the
        gradient buffer (lbm_mlp_vjp_tc; device pointers, dy (n, 8) FP32)."""
        runtime.check(self._core.lbm_mlp_vjp_tc(ctypes.c_void_p(x), ctypes.c_void_p(dy), n, self.p.handle,
                                                self.g.handle, self.loss.handle,
                                                self.stream if stream is None else stream))

    def vjp(self, x, dy):
        """(sum of dy . y, gradient float64) for host arrays x (n, 16), dy (n, 8)."""
        dx, ddy, n = self._device_data(x, dy)
        self.g.zero(self.stream)
        self.vjp_device(dx.ptr, ddy.ptr, n)
        grad = np.empty(self.nparam, dtype=np.float32)
        self.g.download(grad, stream=self.stream)
        self.g.zero(self.stream)
        dot = np.empty(1, dtype=np.float32)
        self.loss.download(dot, stream=self.stream)
        return float(dot[0]), grad.astype(np.float64)

    def grad_host(self):
        out = np.empty(self.nparam, dtype=np.float32)
        self.g.download(out, stream=self.stream)
        return out

    def set_grad(self, g):
        self.g.upload(np.asarray(g, dtype=np.float32), stream=self.stream)

    def adam_step(self, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        """Adam update from the accumulated gradient (which it zeroes)."""
        self.step += 1
        runtime.check(self._core.lbm_mlp_adam(self.p.handle, self.m.handle, self.v.handle, self.g.handle, lr, beta1,
                                              beta2, eps, self.step, self.w.handle, self.stream))

    def _device_data(self, x, t):
        xb = _bf16_bits(x)
        n = xb.shape[0]
        if n % 16 and self.train_kernel == "warp":
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
        xh = dx.handle if hasattr(dx, "handle") else dx
        th = dt.handle if hasattr(dt, "handle") else dt
        if self.train_kernel == "tc":
            # forward, backward and weight gradients of 128-sample tiles in one
            # tcgen05 kernel, nothing staged in global memory
            runtime.check(self._core.lbm_mlp_gradients_tc(xh, th, n, self.p.handle, self.g.handle, self.loss.handle,
                                                          self.stream))
        elif self.train_kernel == "warp":
            scratch = self._scratch_for(n)
            runtime.check(self._core.lbm_mlp_gradients(xh, th, n, self.w.handle, self.p.handle, self.g.handle,
                                                       self.loss.handle, scratch.handle, scratch.nbytes, self.stream))
        else:
            raise ValueError(f"train_kernel: {self.train_kernel!r} (tc or warp)")
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


# ---------------------------------------------------------------------------
# Closure model: MLP + normalisation, training data from restricted fine runs
# ---------------------------------------------------------------------------
class ClosureModel:
    """A trained closure: MLP parameters and the normalisation of its inputs
    (pre-collision moments) and outputs (non-conserved moment corrections).

    ``rate`` (16 floats lo[8], hi[8], or None): the rate form of the fused
    step, in which output j sets lam_j in [lo_j, hi_j] and the node relaxes
    moment j at s_j (1 + lam_j) instead of adding y_j sig_j + mu_j.
    """

    def __init__(self, params, norm, meta=None, seed=0, rate=None):
        self.mlp = Mlp(seed=seed, params=params)
        self.norm = np.ascontiguousarray(norm, dtype=np.float32)
        if self.norm.size != 48:
            raise ValueError("norm holds mu_in[16], isig_in[16], mu_out[8], sig_out[8]")
        self.rate = None
        if rate is not None:
            self.rate = np.ascontiguousarray(rate, dtype=np.float32)
            if self.rate.size != 16 or np.any(self.rate[:8] > self.rate[8:]) or np.any(self.rate[:8] < -1.0):
                raise ValueError("rate holds lo[8], hi[8] with -1 <= lo <= hi")
        self.meta = dict(meta or {})
        sm, _ = runtime.device_info()
        self.grid = 2 * sm  # fused closure step: persistent blocks, two per SM
        # guard of the fused step: corrections beyond 8x the relaxation's own
        # change plus 8 output standard deviations (or not finite) fall back
        # to the plain collision at that node
        self.guard = np.array([8.0, 8.0 * float(np.max(self.norm[40:48]))], dtype=np.float32)

    def norm_ptr(self):
        return self.norm.ctypes.data_as(ctypes.c_void_p)

    def guard_ptr(self):
        return self.guard.ctypes.data_as(ctypes.c_void_p)

    def rate_ptr(self):
        return None if self.rate is None else self.rate.ctypes.data_as(ctypes.c_void_p)

    def save(self, path):
        extra = {} if self.rate is None else {"rate": self.rate}
        np.savez(path, params=self.mlp.params_host(), norm=self.norm, guard=self.guard,
                 meta=np.array(repr(self.meta)), **extra)

    @classmethod
    def load(cls, path):
        d = np.load(path, allow_pickle=False)
        import ast
        model = cls(d["params"], d["norm"], ast.literal_eval(str(d["meta"])),
                    rate=d["rate"] if "rate" in d.files else None)
        if "guard" in d.files:
            model.guard = np.ascontiguousarray(d["guard"], dtype=np.float32)
        return model


def _restrict(sim, factor):
    """Restricted physical populations (nv, n0/f, n1/f) of a simulation, float64."""
    lat = sim._lat
    nc = [lat.n[d] // factor for d in range(sim.dim)]
    out = runtime.DeviceBuffer(8 * sim.scheme.nv * int(np.prod(nc)))
    runtime.check(runtime.core().lbm_restrict(sim._F.handle, ctypes.byref(lat), out.handle, factor, sim._stream))
    host = np.empty([sim.scheme.nv] + nc)
    out.download(host, stream=sim._stream)
    out.free()
    return host


def _pull(f, vel):
    """Periodic pull of populations (nv, n0, n1): g_k(x) = f_k(x - v_k)."""
    return np.array([np.roll(f[k], shift=tuple(int(c) for c in vel[k]), axis=(0, 1)) for k in range(f.shape[0])])


def closure_pairs(scheme, c_now, c_next, rates, rng, nodes):
    """Inputs (pre-collision moments) and targets (corrections) at random nodes.

    c_now, c_next: restricted fine populations at coarse steps n and n+1.
    The coarse step pulls c_now, relaxes, and should produce c_next at every
    node; the target of the non-conserved moments is the difference between
    M c_next and the plain relaxation.
    """
    nv, nc = scheme.nv, scheme.nconsm
    vel = scheme.stencil.get_all_velocities()
    pre = np.einsum("ij,j...->i...", scheme.M, _pull(c_now, vel))
    flat = pre.reshape(nv, -1)
    sel = rng.choice(flat.shape[1], size=min(nodes, flat.shape[1]), replace=False)
    m = flat[:, sel]
    meq = scheme.equilibrium_numpy(m[:nc])
    relaxed = m + rates[:, None] * (meq - m)
    target = (scheme.M @ c_next.reshape(nv, -1)[:, sel])
    return m.T.copy(), (target - relaxed)[nc:].T.copy()


def subfilter_pairs(scheme, c_now, fine_cons, factor, rng, nodes):
    """Inputs and sub-filter targets at random coarse nodes.

    The coarse step relaxes toward m_eq(R(c)), the equilibrium of the
    restricted conserved moments, while the restricted fine flow relaxes
    toward R(m_eq(c)); for the quadratic terms of the equilibrium the
    difference is the sub-filter flux R(q_i q_j) - R(q_i) R(q_j) that the
    coarse grid cannot represent.  The target correction of non-conserved
    moment k is s_k * (R(m_eq,k(c)) - m_eq,k(R(c))), evaluated for the
    pre-collision state of the next coarse step (``fine_cons``: the fine
    conserved moments at that time).  The inputs are that step's
    pre-collision moments M pull(c_now).
    """
    nv, nc = scheme.nv, scheme.nconsm
    vel = scheme.stencil.get_all_velocities()
    pre = np.einsum("ij,j...->i...", scheme.M, _pull(c_now, vel)).reshape(nv, -1)

    def restrict(a):
        n0, n1 = a.shape
        return a.reshape(n0 // factor, factor, n1 // factor, factor).mean(axis=(1, 3)).ravel()

    fine = np.array([np.asarray(c, dtype=np.float64).ravel() for c in fine_cons])
    n0, n1 = np.asarray(fine_cons[0]).shape
    meq_fine = scheme.equilibrium_numpy(fine)                      # (nv, fine nodes)
    r_meq = np.array([restrict(meq_fine[k].reshape(n0, n1)) for k in range(nv)])
    r_cons = np.array([restrict(np.asarray(c, dtype=np.float64)) for c in fine_cons])
    meq_r = scheme.equilibrium_numpy(r_cons)
    rates = scheme.rates_numpy()
    sel = rng.choice(pre.shape[1], size=min(nodes, pre.shape[1]), replace=False)
    target = (rates[:, None] * (r_meq - meq_r))[nc:, sel]
    return pre[:, sel].T.copy(), target.T.copy()


def study_dicos(seed, n, re=30000.0, u0=0.05):
    """Double shear layer at Reynolds number ``re`` (U0 L / nu) on n^2 nodes."""
    from . import workloads as W
    nu = u0 * n / re
    return W.shear_layer(n=n, nu=nu, u0=u0, seed=seed)


def generate_training_data(seeds, n_fine=1024, factor=4, re=30000.0, times=(300, 500, 700, 900, 1100, 1300, 1500),
                           nodes_per_pair=4096, fine_dtype="float64", rng_seed=0):
    """(inputs, targets) pairs from fine runs restricted ``factor`` times."""
    from .scheme import Scheme
    from .simulation import Simulation

    rng = np.random.default_rng(rng_seed)
    n_coarse = n_fine // factor
    coarse_scheme = Scheme(study_dicos(0, n_coarse, re))
    xs, ys = [], []
    for s in seeds:
        sim = Simulation(study_dicos(int(s), n_fine, re), dtype=fine_dtype, parity=False)
        step = 0
        for tc in times:
            sim.run(factor * tc - step)
            step = factor * tc
            now = _restrict(sim, factor)
            sim.run(factor)
            step += factor
            fine = (sim.m[0], sim.m[1], sim.m[2])
            x, y = subfilter_pairs(coarse_scheme, now, fine, factor, rng, nodes_per_pair)
            xs.append(x)
            ys.append(y)
        sim.free()
    return np.concatenate(xs), np.concatenate(ys)


def fit_normalisation(x, y):
    mu_in = np.zeros(16, np.float32)
    isig_in = np.zeros(16, np.float32)
    mu_out = np.zeros(8, np.float32)
    sig_out = np.zeros(8, np.float32)
    mu_in[:x.shape[1]] = x.mean(0)
    sd = x.std(0)
    isig_in[:x.shape[1]] = np.where(sd > 0, 1.0 / np.maximum(sd, 1e-30), 0.0)
    mu_out[:y.shape[1]] = y.mean(0)
    sig_out[:y.shape[1]] = np.maximum(y.std(0), 1e-30)
    return np.concatenate([mu_in, isig_in, mu_out, sig_out])


def train(x, y, steps=6000, batch=2048, lr=2e-3, seed=0, val_fraction=0.05, log=None, report_every=500,
          corrected=None):
    """Train the MLP with the GPU kernels (Adam, cosine learning-rate decay).

    ``corrected``: indices (into the non-conserved moments) whose corrections
    the closure applies; the others get a zero target and a zero output scale
    (the network keeps its 6 outputs, the step leaves those moments to the
    plain relaxation).  None corrects all of them.

    Each block of ``report_every`` steps draws its minibatches from the
    training samples, gathered on the host and uploaded once.  Returns
    (ClosureModel, history).
    """
    import math
    rng = np.random.default_rng(seed)
    y = np.array(y, dtype=np.float64)
    if corrected is not None:
        keep = np.zeros(y.shape[1], dtype=bool)
        keep[list(corrected)] = True
        y[:, ~keep] = 0.0
    norm = fit_normalisation(x, y)
    if corrected is not None:
        norm[40:40 + y.shape[1]][~keep] = 0.0  # zero output scale: no correction applied
    nin, nout = x.shape[1], y.shape[1]
    xn = np.zeros((x.shape[0], IN))
    xn[:, :nin] = (x - norm[:nin]) * norm[16:16 + nin]
    yn = np.zeros((y.shape[0], OUT))
    scale = np.where(norm[40:40 + nout] > 0, norm[40:40 + nout], 1.0)
    yn[:, :nout] = (y - norm[32:32 + nout]) / scale
    perm = rng.permutation(x.shape[0])
    nval = min(int(val_fraction * x.shape[0]), 65536) // 16 * 16
    val, tr = perm[:nval], perm[nval:]
    model = ClosureModel(init_params(seed), norm, {"nin": nin, "nout": nout})
    mlp = model.mlp
    xb_all = to_storage(xn, "bfloat16")
    yf_all = yn.astype(np.float32)
    history = []
    done = 0
    while done < steps:
        chunk = min(report_every, steps - done)
        idx = tr[rng.integers(0, tr.size, chunk * batch)]
        dxe = runtime.DeviceBuffer(chunk * batch * IN * 2)
        dxe.upload(xb_all[idx])
        dye = runtime.DeviceBuffer(chunk * batch * OUT * 4)
        dye.upload(yf_all[idx])
        losses = []
        for b in range(chunk):
            s = done + b
            lr_s = lr * 0.5 * (1.0 + math.cos(math.pi * s / steps))
            xo = ctypes.c_void_p(dxe.ptr + b * batch * IN * 2)
            yo = ctypes.c_void_p(dye.ptr + b * batch * OUT * 4)
            losses.append(mlp.train_step_device(xo, yo, batch, lr_s, read_loss=(b % 16 == 0)))
        dxe.free()
        dye.free()
        done += chunk
        vl = validation_loss(mlp, xn[val], yn[val]) if nval else float("nan")
        tl = float(np.mean([l for l in losses if l is not None]))
        history.append({"step": done, "train": tl, "val": vl})
        if log:
            log(f"step {done}: train {tl:.4e} val {vl:.4e}")
    return model, history


def validation_loss(mlp, xn, yn):
    y = mlp.forward(xn)
    return float(((y[:, :NUSED] - yn[:, :NUSED]) ** 2).mean())


def vorticity(q, rho=None):
    """z-vorticity of the velocity q/rho on a periodic grid (central differences, unit spacing)."""
    ux, uy = (q[0], q[1]) if rho is None else (q[0] / rho, q[1] / rho)
    dux_dy = (np.roll(ux, -1, 1) - np.roll(ux, 1, 1)) / 2
    duy_dx = (np.roll(uy, -1, 0) - np.roll(uy, 1, 0)) / 2
    return duy_dx - dux_dy


def restrict_moments(m, factor):
    nv, a, b = m.shape
    return m.reshape(nv, a // factor, factor, b // factor, factor).mean(axis=(2, 4))
