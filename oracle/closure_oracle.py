"""CPU oracle of the fused learned-closure step (float64 NumPy).

TEST INFRASTRUCTURE ONLY: checks the CUDA closure step kernels
(k_step_periodic_closure, k_step_periodic_closure_tc) and the PyTorch
restatement of the coarse step used for training
(pylbm_gb300/closure_train.py).  The pylbm_gb300 package never imports it.

One periodic MRT step with the closure, in the order the fused kernels use:
pull f_k(x - v_k) with periodic wrap (pylbm/algorithm/pull.py:11-59), m = M f,
the plain relaxation m + s (m_eq(conserved) - m) (pylbm/algorithm/base.py:
404-428), the network's outputs y = MLP(bf16((m - mu_in) * isig_in)) with
BF16 rounding at the kernels' points (mlp_oracle.forward), then the
corrections of the non-conserved moments -- additive: z = y * sig_out +
mu_out; rate form: lam (m_relaxed - m) with lam = lo + (hi - lo) *
sigmoid(z) -- judged by the guard (every correction finite and at most
ratio * (largest change the relaxation made) + floor, else the node keeps
the plain collision), and f = M^-1 m.  The conserved moments are never
corrected.
"""
import numpy as np

import mlp_oracle as mo


def pull(f, velocities):
    """Periodic pull of populations (nv, n0, n1[, n2]): g_k(x) = f_k(x - v_k)."""
    dims = tuple(range(f.ndim - 1))
    return np.array([np.roll(f[k], shift=tuple(int(c) for c in velocities[k]), axis=dims)
                     for k in range(f.shape[0])])


def closure_step(f, scheme, params, norm, rate=None, guard=None):
    """One closure step of absolute populations ``f`` (float64); returns
    (f_new, number of nodes that kept the plain collision)."""
    nv, nc = scheme.nv, scheme.nconsm
    nn = nv - nc
    g = pull(np.asarray(f, dtype=np.float64), scheme.stencil.get_all_velocities())
    m = np.einsum("ij,j...->i...", np.asarray(scheme.M, dtype=np.float64), g)
    rows = m.reshape(nv, -1).T.copy()  # (nodes, nv)
    norm = np.asarray(norm, dtype=np.float64)
    x = np.zeros((rows.shape[0], mo.IN))
    x[:, :nv] = (rows - norm[:nv]) * norm[16:16 + nv]
    y, _ = mo.forward(np.asarray(params, dtype=np.float64), x)
    s = scheme.rates_numpy()
    meq = scheme.equilibrium_numpy(rows[:, :nc].T).T
    relaxed = rows + s * (meq - rows)
    d = relaxed[:, nc:] - rows[:, nc:]
    z = y[:, :nn] * norm[40:40 + nn] + norm[32:32 + nn]
    if rate is None:
        corr = z
    else:
        rate = np.asarray(rate, dtype=np.float64)
        lo, hi = rate[:nn], rate[8:8 + nn]
        with np.errstate(over="ignore"):
            corr = (lo + (hi - lo) / (1.0 + np.exp(-z))) * d
    ok = np.ones(rows.shape[0], dtype=bool)
    if guard is not None and guard[0] > 0.0:
        limit = guard[0] * np.abs(d).max(axis=1) + guard[1]
        with np.errstate(invalid="ignore"):
            ok = np.all(np.isfinite(corr) & (np.abs(corr) <= limit[:, None]), axis=1)
    post = relaxed.copy()
    post[ok, nc:] += corr[ok]
    f_new = (np.asarray(scheme.invM, dtype=np.float64) @ post.T).reshape(f.shape)
    return f_new, int((~ok).sum())
