"""The benchmark configurations at their full sizes.

* D3Q19 MRT Taylor-Green vortex, 256^3 nodes, 500 steps: the FP64 run
  against the reference's own run of the same dictionary (pylbm's Cython
  generator, tests/golden/tgv3d_n256_sampled.npz: every moment at every 16th
  node, the conserved moments on three grid lines, per-moment sums and sums
  of squares over all 16.8 M nodes, kinetic energy every 100 steps); then the
  FP32, FP16 and BF16 shifted-storage runs against that FP64 run.
* D2Q9 MRT flow past a disc, 2048x512, Re 200, 20 000 steps: the FP64 run
  against the reference's run (tests/golden/cylinder_2048x512_sampled.npz,
  including the cross-stream momentum at two wake probes every 20 steps),
  then the FP32 run against the FP64 run (velocity and vorticity).
* The 512-instance ensemble (D2Q9 double shear layers, sides 64..512,
  viscosity log-uniform in [5e-4, 5e-2], FP16 shifted storage), 2000 steps:
  every instance against its own FP64 run.

The parity bound of the FP64 runs is 1e-12 relative to each moment's
largest value; the reduced-precision bounds are stated beside each check.
"""
import numpy as np
import pytest
import sympy as sp

from conftest import golden, rel_err
from pylbm_gb300 import Simulation
from pylbm_gb300 import workloads as W

pytestmark = pytest.mark.gpu

PARITY = 1e-12


def _all_moments(sim):
    return np.array([sim.m[k] for k in range(sim.scheme.nv)])


def _sum_checks(m, g):
    """Per-moment sums and sums of squares over every node against the reference's."""
    flat = m.reshape(m.shape[0], -1)
    s1, s2 = flat.sum(axis=1), (flat * flat).sum(axis=1)
    scale = np.sqrt(flat.shape[1] * g["sumsq"])
    assert np.all(np.abs(s1 - g["sum"]) <= PARITY * np.maximum(scale, 1e-300)), np.abs(s1 - g["sum"]) / scale
    assert np.all(np.abs(s2 - g["sumsq"]) <= PARITY * np.maximum(g["sumsq"], 1e-300))


def _velocity(fields):
    rho = fields[0]
    return np.stack([q / rho for q in fields[1:]])


def _rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


# ---------------------------------------------------------------- TGV 256^3
@pytest.fixture(scope="module")
def tgv_fp64():
    g = golden("tgv3d_n256_sampled.npz")
    n, steps = int(g["n"]), int(g["steps"])
    sim = Simulation(W.tgv3d(n=n))  # float64, the reference generator's printed forms
    energy = []
    for s in range(0, steps + 1, 100):
        if s:
            sim.run(100)
        f = sim.fields()
        energy.append(0.5 * float(((f["qx"] ** 2 + f["qy"] ** 2 + f["qz"] ** 2) / f["rho"]).sum()))
    m = _all_moments(sim)
    sim.free()
    return g, m, np.array(energy)


def test_tgv256_fp64_500_steps_matches_reference_run(tgv_fp64):
    g, m, energy = tgv_fp64
    st, off = int(g["stride"]), int(g["offset"])
    sl = slice(off, None, st)
    sub_err = rel_err(m[:, sl, sl, sl], g["sub"])
    i, j, k = (int(x) for x in g["line"])
    cons = [0, 1, 2, 3]
    for got, want in ((m[cons][:, :, j, k], g["line_x"]), (m[cons][:, i, :, k], g["line_y"]),
                      (m[cons][:, i, j, :], g["line_z"])):
        assert rel_err(got, want).max() <= PARITY
    _sum_checks(m, g)
    e_ref = g["energy"][:, 1]
    assert np.all(np.abs(energy - e_ref) <= PARITY * e_ref), (energy, e_ref)
    print(f"TGV 256^3 x 500 FP64 vs reference: max rel err {sub_err.max():.3e}, "
          f"bit-identical samples: {np.array_equal(m[:, sl, sl, sl], g['sub'])}")
    assert sub_err.max() <= PARITY, sub_err


@pytest.mark.parametrize("dtype,bound", [("float32", 3e-5), ("float16", 3e-3), ("bfloat16", 3e-2)])
def test_tgv256_reduced_precision_against_fp64(tgv_fp64, dtype, bound):
    """Shifted storage, FP32 arithmetic: velocity and kinetic-energy density
    relative L2 error after 500 steps against the FP64 run (which equals the
    reference's run, test above)."""
    _, m, _ = tgv_fp64
    u_ref = _velocity(m[:4])
    ke_ref = 0.5 * m[0] * (u_ref ** 2).sum(axis=0)
    sim = Simulation(W.tgv3d(n=256), dtype=dtype)
    sim.run(500)
    f = sim.fields()
    sim.free()
    cons = np.stack([f["rho"], f["qx"], f["qy"], f["qz"]])
    u = _velocity(cons)
    e_u = _rel_l2(u, u_ref)
    e_ke = _rel_l2(0.5 * cons[0] * (u ** 2).sum(axis=0), ke_ref)
    print(f"TGV 256^3 x 500 {dtype}: velocity rel L2 {e_u:.3e}, kinetic energy rel L2 {e_ke:.3e}")
    assert e_u < bound and e_ke < 2 * bound


# ------------------------------------------------------- disc flow 2048x512
@pytest.fixture(scope="module")
def disc_fp64():
    g = golden("cylinder_2048x512_sampled.npz")
    steps, every = int(g["steps"]), int(g["probe_every"])
    nodes = [tuple(int(x) for x in p) for p in g["probe_nodes"]]
    sim = Simulation(W.cylinder())  # float64, the reference generator's printed forms
    probes = []
    for s in range(0, steps + 1, every):
        if s:
            sim.run(every)
        probes.append([float(sim.m[2, px, py]) for px, py in nodes])
    m = _all_moments(sim)
    sim.free()
    return g, m, np.array(probes)


def test_disc_flow_fp64_20000_steps_matches_reference_run(disc_fp64):
    g, m, probes = disc_fp64
    st = int(g["stride"])
    x0, y0 = (int(v) for v in g["patch_origin"])
    ph, pw = g["patch"].shape[1:]
    assert rel_err(m[:3, ::st, ::st], g["sub"]).max() <= PARITY
    patch_err = rel_err(m[:, x0:x0 + ph, y0:y0 + pw], g["patch"])
    _sum_checks(m, g)
    scale = np.abs(g["probes"]).max(axis=0)
    probe_err = (np.abs(probes - g["probes"]).max(axis=0) / scale).max()
    print(f"disc flow 2048x512 x 20000 FP64 vs reference: moments {patch_err.max():.3e}, "
          f"probe series {probe_err:.3e}, bit-identical: {np.array_equal(m[:3, ::st, ::st], g['sub'])}")
    assert patch_err.max() <= PARITY and probe_err <= PARITY


def _vorticity(u):
    return np.gradient(u[1], axis=0) - np.gradient(u[0], axis=1)


def test_disc_flow_fp32_20000_steps_against_fp64(disc_fp64):
    """FP32 shifted storage and arithmetic over the full 20 000 steps: velocity
    and vorticity relative L2 error against the FP64 run over the fluid."""
    _, m, _ = disc_fp64
    u_ref = _velocity(m[:3])
    sim = Simulation(W.cylinder(), dtype="float32")
    sim.run(20000)
    f = sim.fields()
    inner = tuple(slice(int(h), -int(h)) for h in sim.domain.halo)
    fluid = sim.domain.in_or_out[inner] == sim.domain.valin
    sim.free()
    u = _velocity(np.stack([f["rho"], f["qx"], f["qy"]]))
    mask = np.broadcast_to(fluid, u.shape)
    e_u = _rel_l2(np.where(mask, u, 0), np.where(mask, u_ref, 0))
    w, w_ref = _vorticity(np.where(mask, u, 0)), _vorticity(np.where(mask, u_ref, 0))
    e_w = _rel_l2(w, w_ref)
    print(f"disc flow 2048x512 x 20000 float32: velocity rel L2 {e_u:.3e}, vorticity rel L2 {e_w:.3e}")
    assert e_u < 1e-4 and e_w < 1e-3


# ------------------------------------------------------------- ensemble 512
def test_ensemble_512_every_instance_against_its_fp64_run():
    from pylbm_gb300.ensemble import shear_ensemble

    steps = 2000
    e16, sides, nus = shear_ensemble(count=512, seed=0, dtype="float16")
    e64, _, _ = shear_ensemble(count=512, seed=0, dtype="float64", tile=(64, 4, 0))
    e16.run(steps)
    e64.run(steps)
    e16.synchronize()
    e64.synchronize()
    errs = []
    for i in range(len(sides)):
        got = e16.moments(i, keys=range(3))
        ref = e64.moments(i, keys=range(3))
        err_rho = float(np.abs(got[0] - ref[0]).max() / np.abs(ref[0]).max())
        err_q = float(np.abs(got[1:] - ref[1:]).max() / np.abs(ref[1:]).max())
        errs.append((err_rho, err_q))
    errs = np.array(errs)
    worst = int(np.argmax(errs[:, 1]))
    print(f"ensemble 512 x {steps} float16 vs own float64 runs: max rho err {errs[:, 0].max():.3e}, "
          f"max q err {errs[:, 1].max():.3e} (instance {worst}, side {sides[worst]}, nu {nus[worst]:.2e}), "
          f"median q err {np.median(errs[:, 1]):.3e}")
    # the FP64 ensemble is each instance's own single run: three of them checked bit for bit
    omega = sp.Symbol("omega")
    for i in (0, worst, int(np.argmax(sides))):
        sim = Simulation(e64.dicos[i], dtype="float64", parity=False)
        sim.extra_parameters = {omega: e64.params[i]["omega"]}
        sim.run(steps)
        single = np.array([sim.m[k] for k in range(3)])
        assert np.array_equal(e64.moments(i, keys=range(3)), single), i
        sim.free()
    e16.free()
    e64.free()
    assert errs[:, 0].max() < 1e-2 and errs[:, 1].max() < 1e-1


def _strouhal(qy, every, diameter=64, u_in=0.05):
    """Shedding frequency from upward zero crossings of a wake probe signal."""
    x = qy - qy.mean()
    up = np.where((x[:-1] < 0) & (x[1:] >= 0))[0]
    period = every * float(np.mean(np.diff(up)))
    return diameter / (u_in * period), len(up)


def test_disc_flow_sheds_vortices_at_the_expected_strouhal_number():
    """The Re 200 disc flow (radius 32, centre one node above mid-channel),
    FP32 shifted storage: the wake's asymmetry grows from the start (the
    20 000 steps of the workload show it growing, not yet shedding) and the
    disc sheds from about 1e5 steps on; over steps 200 000 - 250 000 the
    cross-stream momentum behind the disc oscillates at St = f D / U in the
    range of a confined Re 200 disc."""
    every = 100
    sim = Simulation(W.cylinder(), dtype="float32")
    sim.run(200000)
    qy = []
    for _ in range(500):
        sim.run(every)
        qy.append(float(sim.m[2, 560, 257]))
    sim.free()
    qy = np.array(qy)
    assert np.ptp(qy) > 0.05  # a developed wake oscillation (u_in = 0.05)
    st, cycles = _strouhal(qy, every)
    print(f"disc flow Re 200 (float32) Strouhal number {st:.4f} over {cycles} cycles")
    assert cycles >= 6
    assert 0.18 < st < 0.23
