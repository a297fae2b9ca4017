"""The CPU oracle against the reference's own outputs (golden fixtures).

The fixtures were produced by running pylbm 0.11.0's Cython generator on the
same dictionaries (tests/golden/make_golden.py).  The bound here is the
oracle's, not the GPU's: the oracle evaluates M f and M^-1 m in full float64
where the reference's generated code rounds its constants to the printed
decimal digits, which leaves ~1e-12 after a few hundred steps.
"""
import numpy as np
import pytest

from conftest import golden, rel_err
from oracle import OracleSimulation, equilibrium_table
from pylbm_gb300 import workloads as W


def test_cavity_n32_against_reference():
    g = golden("cavity_n32.npz")
    o = OracleSimulation(W.cavity(n=32))
    o.initialize()
    assert rel_err(o.moments(), g["m0"]).max() < 1e-14
    o.run(50)
    assert rel_err(o.moments(), g["m50"]).max() < 1e-12
    o.run(250)
    assert rel_err(o.moments(), g["m300"]).max() < 2e-12


def test_cylinder_against_reference():
    g = golden("cylinder_small.npz")
    o = OracleSimulation(W.cylinder(nx=96, ny=32, radius=5, center=(24, 17), re=40.0))
    o.run(100)
    assert rel_err(o.moments(), g["m100"]).max() < 5e-12


def test_tgv3d_against_reference():
    g = golden("tgv3d_n16.npz")
    o = OracleSimulation(W.tgv3d(n=16))
    o.initialize()
    assert rel_err(o.moments(), g["m0"]).max() < 1e-12
    o.run(20)
    assert rel_err(o.moments(), g["m20"]).max() < 5e-12


def test_shear_layer_against_reference():
    g = golden("shear_n64.npz")
    o = OracleSimulation(W.shear_layer(n=64))
    o.initialize()
    assert rel_err(o.moments(), g["m0"]).max() < 1e-12
    o.run(200)
    assert rel_err(o.moments(), g["m200"]).max() < 5e-12


def test_cavity_full_size_sampled():
    """The 256^2 x 1000-step cavity of the reference, at every 4th node and the edges."""
    g = golden("cavity_n256_sampled.npz")
    o = OracleSimulation(W.cavity(n=256), nthreads=8)
    o.run(int(g["steps"]))
    m = o.moments()
    assert rel_err(m[:, ::4, ::4], g["sub"]).max() < 1e-11
    assert rel_err(m[:, :2], g["lo_x"]).max() < 1e-11
    assert rel_err(m[:, :, -2:], g["hi_y"]).max() < 1e-11


def test_equilibrium_table_monomials():
    from pylbm_gb300.scheme import Scheme
    sc = Scheme(W.cavity(n=8))
    rows, coefs, expos = equilibrium_table(sc)
    # m3 = -2 rho + 3 qx^2 + 3 qy^2
    sel = rows == 3
    terms = {tuple(e): c for e, c in zip(expos[sel], coefs[sel])}
    assert terms == {(1, 0, 0): -2.0, (0, 2, 0): 3.0, (0, 0, 2): 3.0}


def test_planted_error_is_detected():
    """A wrong relaxation rate in the oracle must break the parity check."""
    g = golden("cavity_n32.npz")
    d = W.cavity(n=32, omega=1.9)
    o = OracleSimulation(d)
    o.run(50)
    assert rel_err(o.moments(), g["m50"]).max() > 1e-6


def test_reference_kernel_baseline_computes_the_step():
    """The CPU baseline's reference kernel (pylbm's generated one_time_step) agrees with the oracle."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle"))
    import build_ref
    import ref_baseline
    mod = build_ref.load("tgv3d")
    if mod is None:
        pytest.skip("oracle/_ref not generated (needs the reference sources and Cython)")
    n = 12
    # one slab process: one untimed step and two timed ones
    _, _, f = ref_baseline.run_slabs(n=n, steps=2, procs=1, keep_state=True)
    o = OracleSimulation(W.tgv3d(n=n))
    o.run(3)
    got = np.moveaxis(f, -1, 0)
    assert np.abs(got - o.f[:, 1:-1, 1:-1, 1:-1]).max() < 1e-13


def test_mlp_oracle_gradient_matches_finite_differences():
    """The MLP oracle's backward pass (float64, no rounding) against central differences."""
    import mlp_oracle as mo
    rng = np.random.default_rng(0)
    p = mo.init_params(seed=1).astype(np.float64)
    x = rng.normal(size=(48, mo.IN))
    x[:, 9:] = 0.0
    t = rng.normal(size=(48, mo.OUT))
    _, g = mo.loss_and_grad(p, x, t, bf16_points=False)
    idx = np.concatenate([rng.choice(mo.NPARAM, 40, replace=False), [mo.NPARAM - 1, mo.NPARAM - 3]])
    fd = mo.finite_difference(p, x, t, idx)
    assert np.allclose(g[idx], fd, rtol=1e-5, atol=1e-9)
    # the two unused outputs carry no gradient
    assert g[-2] == 0.0 and g[-1] == 0.0


def test_mlp_oracle_bf16_rounding():
    import mlp_oracle as mo
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 3.14159265, -2.71828])
    r = mo.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125  # 1 + 2^-8 is a tie: to even
    assert abs(r[3] - 3.140625) < 1e-12
