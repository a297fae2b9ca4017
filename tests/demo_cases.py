"""Scheme dictionaries of pylbm's demos whose results pylbm pins in tests/reference/*.h5.

TEST INFRASTRUCTURE.  Each function restates, as a pylbm dictionary, the
physics of one reference demo run by pylbm's own regression tests
(tests/test_demo_1d.py, test_demo_2d.py, test_demo_3d.py): same lattice,
moment basis, equilibrium, relaxation rates, initial state and boundary
conditions, at the space step and final time those tests use.  The golden
fields (converted from the reference's HDF5 files by
golden/make_demo_golden.py) are compared at pylbm's own tolerance
(tests/conftest.py:306-307: rel 1e-14, abs 1e-7).

``bc`` defaults to pylbm_gb300.boundary; passing the reference's ``pylbm.bc``
gives the dictionary pylbm itself accepts.
"""
import math

import numpy as np
import sympy as sp

X, Y, Z, LA = sp.symbols("X, Y, Z, lambda")
RHO, QX, QY = sp.symbols("rho, qx, qy")


def _bc(bc):
    if bc is None:
        from pylbm_gb300 import boundary as bc
    return bc


def run_to(sim, final_time):
    """Advance as the demos do: ``while sol.t < Tf: sol.one_time_step()``."""
    while sim.t < final_time:
        sim.one_time_step()
    return sim


def poiseuille(dx=1.0 / 64, bc=None, generator="cuda"):
    """Channel flow, D2Q9 MRT (demo/2D/Poiseuille.py:21-104).

    Box [0, 2] x [-0.5, 0.5]; inflow (label 2) by Bouzidi bounce-back with
    the parabolic profile and a linear pressure; outflow (label 1) NeumannX;
    walls (label 0) Bouzidi bounce-back.
    """
    bc = _bc(bc)
    la, width, height = 1.0, 2, 1
    max_velocity, rhoo, mu, zeta = 0.1, 1.0, 0.00185, 1.0e-2
    grad_pressure = -max_velocity * 8.0 / height**2 * 3.0 / (la**2 * rhoo) * mu
    c = 3.0 / (la * rhoo * dx)
    s1 = 1.0 / (0.5 + zeta * c)
    s2 = 1.0 / (0.5 + mu * c)
    inv = 1.0 / (LA**2 * rhoo)
    qx2, qy2, qxy = inv * QX**2, inv * QY**2, inv * QX * QY
    q2 = qx2 + qy2

    def bc_in(f, m, x, y, width, height, max_velocity, grad_pressure):
        m[RHO] = (x - 0.5 * width) * grad_pressure
        m[QX] = max_velocity * (1.0 - 4.0 * y**2 / height**2)

    return {
        "box": {"x": [0.0, width], "y": [-0.5 * height, 0.5 * height], "label": [2, 1, 0, 0]},
        "space_step": dx,
        "scheme_velocity": la,
        "schemes": [{
            "velocities": list(range(9)),
            "polynomials": [1, LA * X, LA * Y, 3 * (X**2 + Y**2) - 4,
                            0.5 * (9 * (X**2 + Y**2)**2 - 21 * (X**2 + Y**2) + 8),
                            3 * X * (X**2 + Y**2) - 5 * X, 3 * Y * (X**2 + Y**2) - 5 * Y,
                            X**2 - Y**2, X * Y],
            "relaxation_parameters": [0.0, 0.0, 0.0, s1, s1, s1, s1, s2, s2],
            "equilibrium": [RHO, QX, QY, -2 * RHO + 3 * q2, RHO - 3 * q2, -QX / LA, -QY / LA,
                            qx2 - qy2, qxy],
            "conserved_moments": [RHO, QX, QY],
        }],
        "parameters": {LA: la},
        "init": {RHO: 1.0, QX: 0.0, QY: 0.0},
        "boundary_conditions": {
            0: {"method": {0: bc.BouzidiBounceBack}},
            1: {"method": {0: bc.NeumannX}},
            2: {"method": {0: bc.BouzidiBounceBack},
                "value": (bc_in, (width, height, max_velocity, grad_pressure))},
        },
        "generator": generator,
    }


def poiseuille_vec(dx=1.0 / 64, bc=None, generator="cuda"):
    """Channel flow with three coupled D2Q4 (demo/2D/Poiseuille_vec.py:48-130).

    Box [0, 1] x [-0.25, 0.25]; p, ux, uy each carried by one D2Q4; Bouzidi
    bounce-back / anti-bounce-back walls, pressure given at both ends.
    """
    bc = _bc(bc)
    P, UX, UY = sp.symbols("p, ux, uy")
    width, height, la = 1.0, 0.5, 1.0
    max_velocity, mu, zeta, cte = 0.1, 0.00185, 1.0e-5, 3.0
    grad_pressure = -mu * max_velocity * 8.0 / height**2
    c = 3.0 / (la * dx)
    s1 = 1.0 / (0.5 + zeta * c)
    s2 = 1.0 / (0.5 + mu * c)
    vel = list(range(1, 5))
    polys = [1, LA * X, LA * Y, X**2 - Y**2]

    def bc_in(f, m, x, y, width, height, max_velocity, grad_pressure, cte):
        m[P] = (x - 0.5 * width) * grad_pressure * cte
        m[UX] = max_velocity * (1.0 - 4.0 * y**2 / height**2)

    def bc_out(f, m, x, y, width, grad_pressure, cte):
        m[P] = (x - 0.5 * width) * grad_pressure * cte

    return {
        "box": {"x": [0.0, width], "y": [-0.5 * height, 0.5 * height], "label": [2, 1, 0, 0]},
        "space_step": dx,
        "scheme_velocity": la,
        "schemes": [
            {"velocities": vel, "polynomials": polys, "relaxation_parameters": [0.0, s1, s1, 1.0],
             "equilibrium": [P, UX, UY, 0.0], "conserved_moments": P},
            {"velocities": vel, "polynomials": polys, "relaxation_parameters": [0.0, s2, s2, 1.0],
             "equilibrium": [UX, UX**2 + P / cte, UX * UY, 0.0], "conserved_moments": UX},
            {"velocities": vel, "polynomials": polys, "relaxation_parameters": [0.0, s2, s2, 1.0],
             "equilibrium": [UY, UX * UY, UY**2 + P / cte, 0.0], "conserved_moments": UY},
        ],
        "parameters": {LA: la},
        "init": {P: 0.0, UX: 0.0, UY: 0.0},
        "boundary_conditions": {
            0: {"method": {0: bc.BouzidiBounceBack, 1: bc.BouzidiAntiBounceBack, 2: bc.BouzidiAntiBounceBack}},
            1: {"method": {0: bc.BouzidiAntiBounceBack, 1: bc.NeumannX, 2: bc.NeumannX},
                "value": (bc_out, (width, grad_pressure, cte))},
            2: {"method": {0: bc.BouzidiAntiBounceBack, 1: bc.BouzidiAntiBounceBack, 2: bc.BouzidiAntiBounceBack},
                "value": (bc_in, (width, height, max_velocity, grad_pressure, cte))},
        },
        "generator": generator,
    }


def orszag_tang(dx=2.0 * np.pi / 64, bc=None, generator="cuda"):
    """Orszag-Tang vortex of 2D MHD, six coupled D2Q4 (demo/2D/Orszag_Tang_vortex.py:25-168).

    Periodic [0, 2 pi]^2, la = 10, all relaxation rates 1.95.
    """
    GA = sp.Symbol("GA")
    rho, qx, qy, E, Bx, By = sp.symbols("rho, qx, qy, E, Bx, By")
    gamma, la = 5.0 / 3.0, 10.0
    s0 = s1 = s2 = s3 = 1.95
    p = (GA - 1) * (E - (qx**2 + qy**2) / (2 * rho) - (Bx**2 + By**2) / 2)
    ps = p + (Bx**2 + By**2) / 2
    vB = (qx * Bx + qy * By) / rho
    vel, polys = list(range(1, 5)), [1, LA * X, LA * Y, X**2 - Y**2]

    def init_rho(x, y, gamma):
        return gamma**2 * np.ones(x.shape)

    def init_qx(x, y, gamma):
        return -(gamma**2) * np.sin(y)

    def init_qy(x, y, gamma):
        return gamma**2 * np.sin(x)

    def init_bx(x, y):
        return -np.sin(y)

    def init_by(x, y):
        return np.sin(2 * x)

    def init_e(x, y, gamma):
        kinetic = 0.5 * (init_qx(x, y, gamma)**2 + init_qy(x, y, gamma)**2) / init_rho(x, y, gamma)
        magnetic = 0.5 * (init_bx(x, y)**2 + init_by(x, y)**2)
        return kinetic + magnetic + gamma / (gamma - 1)

    def scheme(cons, rates, eq):
        return {"velocities": vel, "conserved_moments": cons, "polynomials": polys,
                "relaxation_parameters": rates, "equilibrium": eq}

    return {
        "box": {"x": [0.0, 2 * np.pi], "y": [0.0, 2 * np.pi], "label": -1},
        "space_step": dx,
        "scheme_velocity": la,
        "schemes": [
            scheme(rho, [0.0, s1, s1, s0], [rho, qx, qy, 0.0]),
            scheme(qx, [0.0, s2, s2, s0], [qx, qx**2 / rho + ps - Bx**2, qx * qy / rho - Bx * By, 0.0]),
            scheme(qy, [0.0, s2, s2, s0], [qy, qx * qy / rho - Bx * By, qy**2 / rho + ps - By**2, 0.0]),
            scheme(E, [0.0, s3, s3, s0], [E, (E + ps) * qx / rho - vB * Bx, (E + ps) * qy / rho - vB * By, 0.0]),
            scheme(Bx, [0.0, s3, s3, s0], [Bx, 0, (qy * Bx - qx * By) / rho, 0.0]),
            scheme(By, [0.0, s3, s3, s0], [By, (qx * By - qy * Bx) / rho, 0, 0.0]),
        ],
        "init": {rho: (init_rho, (gamma,)), qx: (init_qx, (gamma,)), qy: (init_qy, (gamma,)),
                 E: (init_e, (gamma,)), Bx: init_bx, By: init_by},
        "parameters": {LA: la, GA: gamma},
        "generator": generator,
    }


def advection_3d(dx=1.0 / 64, bc=None, generator="cuda"):
    """Advection on the 3D torus, D3Q6 (demo/3D/advection.py:30-91): c = (0.5, 0.2, 0.1), s = 1."""
    U = sp.Symbol("u")
    ux, uy, uz, s, la = 0.5, 0.2, 0.1, 1.0, 1.0

    def u0(x, y, z):
        return 0.5 * np.ones((x.size, y.size, z.size)) + 0.5 * (
            ((x - 0.5)**2 + (y - 0.5)**2 + (z - 0.5)**2) < 0.25**2)

    return {
        "box": {"x": [0.0, 1.0], "y": [0.0, 1.0], "z": [0.0, 1.0], "label": -1},
        "space_step": dx,
        "scheme_velocity": la,
        "schemes": [{
            "velocities": list(range(1, 7)),
            "conserved_moments": [U],
            "polynomials": [1, LA * X, LA * Y, LA * Z, X**2 - Y**2, X**2 - Z**2],
            "equilibrium": [U, ux * U, uy * U, uz * U, 0.0, 0.0],
            "relaxation_parameters": [0.0, s, s, s, s, s],
        }],
        "init": {U: u0},
        "parameters": {LA: la},
        "generator": generator,
    }


def reduce_field(a):
    """What a fixture keeps of a field: all of it up to 8192 nodes; beyond, in
    2D every 2nd node, the middle row and the sum, in 3D the middle z-plane,
    every 4th node and the sum (the reference's 64^3 files are 2 MB)."""
    a = np.asarray(a, dtype=np.float64)
    if a.size <= 8192:
        return {"": a}
    if a.ndim == 2:
        return {"__every2": np.ascontiguousarray(a[::2, ::2]), "__midrow": np.ascontiguousarray(a[a.shape[0] // 2]),
                "__sum": np.array(a.sum())}
    return {"__mid": np.ascontiguousarray(a[:, :, a.shape[2] // 2]),
            "__every4": np.ascontiguousarray(a[::4, ::4, ::4]), "__sum": np.array(a.sum())}


def poiseuille_3d(dx=1.0 / 64, bc=None, generator="cuda"):
    """Channel flow with four coupled D3Q6 (demo/3D/poiseuille.py:60-155).

    Box [0, 1] x [-0.25, 0.25] x [-2 dx, 2 dx], periodic in z; Bouzidi walls,
    pressure given at both ends (outflow NeumannX for the velocities).
    """
    bc = _bc(bc)
    P, UX, UY, UZ = sp.symbols("p,ux,uy,uz")
    width, height, la = 1.0, 0.5, 1.0
    max_velocity, mu, cte = 0.1, 1.0e-3, 10.0
    grad_pressure = -mu * max_velocity * 8.0 / height**2
    s = 1.0 / (0.5 + 1.0 / np.sqrt(12))
    rates = [0.0, s, s, s, s, s]
    vel = list(range(1, 7))
    polys = [1, LA * X, LA * Y, LA * Z, X**2 - Y**2, X**2 - Z**2]

    def bc_in(f, m, x, y, z):
        m[P] = (x - 0.5 * width) * grad_pressure * cte
        m[UX] = max_velocity * (1.0 - 4.0 * y**2 / height**2)

    def bc_out(f, m, x, y, z):
        m[P] = (x - 0.5 * width) * grad_pressure * cte

    def scheme(cons, eq):
        return {"velocities": vel, "conserved_moments": cons, "polynomials": polys,
                "relaxation_parameters": rates, "equilibrium": eq}

    walls = {0: bc.BouzidiBounceBack, 1: bc.BouzidiAntiBounceBack, 2: bc.BouzidiAntiBounceBack,
             3: bc.BouzidiAntiBounceBack}
    return {
        "box": {"x": [0.0, width], "y": [-0.5 * height, 0.5 * height], "z": [-2 * dx, 2 * dx],
                "label": [1, 2, 0, 0, -1, -1]},
        "space_step": dx,
        "scheme_velocity": la,
        "schemes": [
            scheme(P, [P, UX, UY, UZ, 0.0, 0.0]),
            scheme(UX, [UX, UX**2 + P / cte, UX * UY, UX * UZ, 0.0, 0.0]),
            scheme(UY, [UY, UY * UX, UY**2 + P / cte, UY * UZ, 0.0, 0.0]),
            scheme(UZ, [UZ, UZ * UX, UZ * UY, UZ**2 + P / cte, 0.0, 0.0]),
        ],
        "init": {P: 0.0, UX: 0.0, UY: 0.0, UZ: 0.0},
        "boundary_conditions": {
            0: {"method": walls},
            1: {"method": {0: bc.BouzidiAntiBounceBack, 1: bc.NeumannX, 2: bc.NeumannX, 3: bc.NeumannX},
                "value": bc_out},
            2: {"method": {0: bc.BouzidiAntiBounceBack, 1: bc.BouzidiAntiBounceBack, 2: bc.BouzidiAntiBounceBack,
                           3: bc.BouzidiAntiBounceBack},
                "value": bc_in},
        },
        "parameters": {LA: la},
        "generator": generator,
    }


def euler_1d(dx=1.0 / 64, bc=None, generator="cuda"):
    """Sod shock tube, three coupled D1Q2 (demo/1D/euler.py:45-118): la = 3, Neumann ends."""
    bc = _bc(bc)
    rho, q, E = sp.symbols("rho, q, E")
    la_c = sp.symbols("lambda", constants=True)
    gamma, xmin, xmax, la = 1.4, 0.0, 1.0, 3.0
    rho_l, rho_r, p_l, p_r, u_l, u_r = 1.0, 1.0 / 8.0, 1.0, 0.1, 0.0, 0.0
    q_l, q_r = rho_l * u_l, rho_r * u_r
    e_l = rho_l * u_l**2 + p_l / (gamma - 1.0)
    e_r = rho_r * u_r**2 + p_r / (gamma - 1.0)

    def riemann(x, xmin, xmax, left, right):
        xm = 0.5 * (xmin + xmax)
        u = np.empty(x.shape)
        u[x < xm] = left
        u[x == xm] = 0.5 * (left + right)
        u[x > xm] = right
        return u

    def scheme(cons, rate, flux):
        return {"velocities": [1, 2], "conserved_moments": cons, "polynomials": [1, la_c * X],
                "relaxation_parameters": [0, rate], "equilibrium": [cons, flux]}

    return {
        "box": {"x": [xmin, xmax], "label": 0},
        "space_step": dx,
        "scheme_velocity": la,
        "schemes": [
            scheme(rho, 1.9, q),
            scheme(q, 1.5, (gamma - 1.0) * E + 0.5 * (3.0 - gamma) * q**2 / rho),
            scheme(E, 1.4, gamma * E * q / rho - 0.5 * (gamma - 1.0) * q**3 / rho**2),
        ],
        "init": {rho: (riemann, (xmin, xmax, rho_l, rho_r)), q: (riemann, (xmin, xmax, q_l, q_r)),
                 E: (riemann, (xmin, xmax, e_l, e_r))},
        "boundary_conditions": {0: {"method": {0: bc.Neumann, 1: bc.Neumann, 2: bc.Neumann}}},
        "parameters": {la_c: la},
        "generator": generator,
    }


def lid_driven_cavity(dx=1.0 / 64, bc=None, generator="cuda"):
    """Lid-driven cavity, D2Q9 Geier scheme with relative velocity
    (demo/2D/lid_driven_cavity.py:57-229, scheme_name "Geier").

    Bouzidi bounce-back walls; the lid (label 1) moves at 0.05.
    """
    bc = _bc(bc)
    la_c = sp.symbols("lambda", constants=True)
    la, rho_o, driven_velocity, mu = 1.0, 1.0, 0.05, 5.0e-6
    zeta = 100 * mu
    ux, uy = QX / RHO, QY / RHO
    rhou2 = RHO * (ux**2 + uy**2)
    c = 3.0 / (la * rho_o * dx)
    s_1 = 1 / (0.5 + c * (zeta - 2 * mu / 3))
    s_2 = 1 / (0.5 + c * mu)

    def bc_up(f, m, x, y, rho_o, driven_velocity):
        m[RHO] = rho_o
        m[QX] = rho_o * driven_velocity
        m[QY] = 0.0

    return {
        "parameters": {la_c: la},
        "box": {"x": [0.0, 1.0], "y": [0.0, 1.0], "label": [0, 0, 0, 1]},
        "space_step": dx,
        "scheme_velocity": la_c,
        "schemes": [{
            "velocities": list(range(9)),
            "polynomials": [1, X, Y, X**2 + Y**2, X * Y**2, Y * X**2, X**2 * Y**2, X**2 - Y**2, X * Y],
            "relaxation_parameters": [0.0, 0.0, 0.0, s_1, s_1, s_1, s_1, s_2, s_2],
            "equilibrium": [RHO, QX, QY, rhou2 + 2 / 3 * RHO * la_c**2, QX * (la_c**2 / 3 + uy**2),
                            QY * (la_c**2 / 3 + ux**2), RHO * (la_c**2 / 3 + ux**2) * (la_c**2 / 3 + uy**2),
                            RHO * (ux**2 - uy**2), RHO * ux * uy],
            "conserved_moments": [RHO, QX, QY],
        }],
        "init": {RHO: rho_o, QX: 0.0, QY: 0.0},
        "boundary_conditions": {
            0: {"method": {0: bc.BouzidiBounceBack}},
            1: {"method": {0: bc.BouzidiBounceBack}, "value": (bc_up, (rho_o, driven_velocity))},
        },
        "generator": generator,
        "relative_velocity": [QX / RHO, QY / RHO],
    }


def _geier(la_c, dx, la, rho_o, mu, zeta):
    """D2Q9 Geier basis, equilibrium and rates (moments_choice "Geier" of the 2D Navier-Stokes demos)."""
    ux, uy = QX / RHO, QY / RHO
    rhou2 = RHO * (ux**2 + uy**2)
    c = 3.0 / (la * rho_o * dx)
    s_1 = 1 / (0.5 + c * (zeta - 2 * mu / 3))
    s_2 = 1 / (0.5 + c * mu)
    return {
        "velocities": list(range(9)),
        "polynomials": [1, X, Y, X**2 + Y**2, X * Y**2, Y * X**2, X**2 * Y**2, X**2 - Y**2, X * Y],
        "relaxation_parameters": [0.0, 0.0, 0.0, s_1, s_1, s_1, s_1, s_2, s_2],
        "equilibrium": [RHO, QX, QY, rhou2 + 2 / 3 * RHO * la_c**2, QX * (la_c**2 / 3 + uy**2),
                        QY * (la_c**2 / 3 + ux**2), RHO * (la_c**2 / 3 + ux**2) * (la_c**2 / 3 + uy**2),
                        RHO * (ux**2 - uy**2), RHO * ux * uy],
        "conserved_moments": [RHO, QX, QY],
    }


def kelvin_helmholtz(dx=1.0 / 64, bc=None, generator="cuda"):
    """Periodic double shear layer, D2Q9 Geier with relative velocity
    (demo/2D/Kelvin_Helmoltz.py:44-219): Mach 0.1 (la = sqrt(3)/0.1), k = 80, delta = 0.05."""
    la_c = sp.symbols("lambda", constants=True)
    la, rho_o, u_o, zeta, mu, k, delta = np.sqrt(3) / 0.1, 1.0, 0.5, 0.0366, 1.0e-6, 80, 0.05

    def qx_init(x, y, U, k):
        return np.zeros_like(x) + U * np.tanh(k * (y - 0.25)) * (y <= 0.5) + U * np.tanh(k * (0.75 - y)) * (y > 0.5)

    def qy_init(x, y, U, delta):
        return np.zeros_like(y) + U * delta * np.sin(2 * np.pi * (x + 0.25))

    return {
        "parameters": {la_c: la},
        "box": {"x": [0.0, 1.0], "y": [0.0, 1.0], "label": -1},
        "space_step": dx,
        "scheme_velocity": la_c,
        "schemes": [_geier(la_c, dx, la, rho_o, mu, zeta)],
        "init": {RHO: rho_o, QX: (qx_init, (u_o, k)), QY: (qy_init, (u_o, delta))},
        "relative_velocity": [QX / RHO, QY / RHO],
        "generator": generator,
    }


def karman_vortex_street(dx=1.0 / 64, bc=None, circle=None, generator="cuda"):
    """Flow past a disc, D2Q9 Geier with relative velocity (demo/2D/Karman_vortex_street.py:49-225).

    Box [0, 2] x [0, 1]; label 0 (inflow and channel walls) Bouzidi
    bounce-back with the inflow state, label 1 NeumannX, disc (label 2,
    radius 1/32 at (0.3, 0.5 + 2 dx)) Bouzidi bounce-back.
    """
    bc = _bc(bc)
    if circle is None:
        from pylbm_gb300.geometry import Circle as circle
    la_c = sp.symbols("lambda", constants=True)
    la, rho_o, u_o, mu, radius = 1.0, 1.0, 0.05, 5.0e-6, 1.0 / 32
    zeta = 10 * mu

    def bc_in(f, m, x, y, rho_o, u_o):
        m[RHO] = rho_o
        m[QX] = rho_o * u_o
        m[QY] = 0.0

    return {
        "box": {"x": [0.0, 2.0], "y": [0.0, 1.0], "label": [0, 1, 0, 0]},
        "elements": [circle([0.3, 0.5 + 2 * dx], radius, label=2)],
        "space_step": dx,
        "scheme_velocity": la,
        "schemes": [_geier(la_c, dx, la, rho_o, mu, zeta)],
        "parameters": {la_c: la},
        "init": {RHO: rho_o, QX: rho_o * u_o, QY: 0.0},
        "boundary_conditions": {
            0: {"method": {0: bc.BouzidiBounceBack}, "value": (bc_in, (rho_o, u_o))},
            1: {"method": {0: bc.NeumannX}},
            2: {"method": {0: bc.BouzidiBounceBack}},
        },
        "generator": generator,
        "relative_velocity": [QX / RHO, QY / RHO],
    }


def advection_2d(dx=1.0 / 64, bc=None, generator="cuda"):
    """Advection on the torus, D2Q4 with a constant relative velocity (demo/2D/advection.py:21-115).

    c = (0.2, 0.5), la = 2, rates given through the parameters sigma_0, sigma_1.
    """
    U = sp.Symbol("U")
    CX, CY, la_c = sp.symbols("c_0, c_1, lambda", constants=True)
    sigma0, sigma1 = sp.symbols("sigma_0, sigma_1", constants=True)
    xmin, xmax, ymin, ymax = 0.0, 1.0, 0.0, 1.0
    sq, sxy = 1 / (0.5 + sigma0), 1 / (0.5 + sigma1)

    def u_init(x, y, xmin, xmax, ymin, ymax):
        center = (0.75 * xmin + 0.25 * xmax, 0.50 * ymin + 0.50 * ymax)
        return 1 + 0.5 * ((x - center[0])**2 + (y - center[1])**2 < 0.1**2)

    return {
        "box": {"x": [xmin, xmax], "y": [ymin, ymax], "label": -1},
        "space_step": dx,
        "scheme_velocity": la_c,
        "schemes": [{
            "velocities": list(range(1, 5)),
            "conserved_moments": U,
            "polynomials": [1, X, Y, X**2 - Y**2],
            "relaxation_parameters": [0.0, sq, sq, sxy],
            "equilibrium": [U, CX * U, CY * U, 0],
        }],
        "init": {U: (u_init, (xmin, xmax, ymin, ymax))},
        "generator": generator,
        "parameters": {la_c: 2.0, CX: 0.2, CY: 0.5, sigma0: 1.0e-2, sigma1: 0.5},
        "relative_velocity": [CX, CY],
    }


def air_conditioning(dx=1.0 / 64, bc=None, parallelogram=None, generator="cuda"):
    """Buoyant flow with a cold inflow: D2Q9 MRT for (rho, q) with the buoyancy
    source term on qy, coupled to a D2Q5 for T (demo/2D/air_conditioning.py:36-158).

    Two solid blocks (parallelograms) at the bottom corners; label 0 walls
    and label 1 inflow by Bouzidi bounce-back (flow) / anti-bounce-back (T),
    label 2 NeumannX.
    """
    bc = _bc(bc)
    if parallelogram is None:
        from pylbm_gb300.geometry import Parallelogram as parallelogram
    rho, qx, qy, T = sp.symbols("rho, qx, qy, T")
    T0, Tin = 0.5, -0.5
    xmin, xmax, ymin, ymax = 0.0, 1.0, 0.0, 1.0
    Ra, Pr, alpha, la, rhoo, g, uo = 2000, 0.71, 0.005, 1.0, 1.0, 9.81, 0.025
    nu = np.sqrt(Pr * alpha * 9.81 * (T0 - Tin) * (ymax - ymin) / Ra)
    kappa = nu / Pr
    eta = nu
    snu = 1.0 / (0.5 + 3 * nu)
    seta = 1.0 / (0.5 + 3 * eta)
    sq = 8 * (2 - snu) / (8 - snu)
    se = seta
    sf = [0.0, 0.0, 0.0, seta, se, sq, sq, snu, snu]
    a = 0.5
    skappa = 1.0 / (0.5 + 10 * kappa / (4 + a))
    se = 1.0 / (0.5 + np.sqrt(3) / 3)
    snu = se
    sT = [0.0, skappa, skappa, se, snu]

    def init_T(x, y, T0):
        return T0

    def bc_wall(f, m, x, y, T0):
        m[qx] = 0.0
        m[qy] = 0.0
        m[T] = T0

    def bc_in(f, m, x, y, T0, Tin, ymax, rhoo, uo):
        m[qx] = rhoo * uo
        m[qy] = 0.0
        m[T] = T0 + (Tin - T0) * (ymax - y) * (y - 0.8) * 100

    return {
        "box": {"x": [xmin, xmax], "y": [ymin, ymax], "label": [1, 2, 0, 0]},
        "elements": [parallelogram([xmin, ymin], [0.1, 0], [0, 0.8], label=0),
                     parallelogram([xmax, ymin], [-0.1, 0], [0, 0.8], label=0)],
        "space_step": dx,
        "scheme_velocity": la,
        "schemes": [
            {"velocities": list(range(9)), "conserved_moments": [rho, qx, qy],
             "polynomials": [1, X, Y, 3 * (X**2 + Y**2) - 4,
                             sp.Rational(1, 2) * (9 * (X**2 + Y**2)**2 - 21 * (X**2 + Y**2) + 8),
                             3 * X * (X**2 + Y**2) - 5 * X, 3 * Y * (X**2 + Y**2) - 5 * Y, X**2 - Y**2, X * Y],
             "relaxation_parameters": sf,
             "equilibrium": [rho, qx, qy, -2 * rho + 3 * (qx**2 + qy**2), rho - 3 * (qx**2 + qy**2), -qx, -qy,
                             qx**2 - qy**2, qx * qy],
             "source_terms": {qy: alpha * g * T}},
            {"velocities": list(range(5)), "conserved_moments": T,
             "polynomials": [1, X, Y, 5 * (X**2 + Y**2) - 4, (X**2 - Y**2)],
             "equilibrium": [T, T * qx, T * qy, a * T, 0.0], "relaxation_parameters": sT},
        ],
        "init": {rho: 1.0, qx: 0.0, qy: 0.0, T: (init_T, (T0,))},
        "boundary_conditions": {
            0: {"method": {0: bc.BouzidiBounceBack, 1: bc.BouzidiAntiBounceBack}, "value": (bc_wall, (T0,))},
            1: {"method": {0: bc.BouzidiBounceBack, 1: bc.BouzidiAntiBounceBack},
                "value": (bc_in, (T0, Tin, ymax, rhoo, uo))},
            2: {"method": {0: bc.NeumannX, 1: bc.NeumannX}},
        },
        "generator": generator,
    }


def rayleigh_benard(dx=1.0 / 64, bc=None, generator="cuda"):
    """Rayleigh-Benard convection: D2Q9 MRT with buoyancy source on qy coupled
    to a D2Q5 for T (demo/2D/Rayleigh-Benard.py:87-206, time_bc=True).

    Periodic in x; bottom wall (label 0) with a bottom temperature that
    switches every 5 time units (time-dependent boundary value), top wall
    (label 1); Bouzidi bounce-back (flow) / anti-bounce-back (T).
    """
    bc = _bc(bc)
    la_c = sp.symbols("lambda")
    rho, qx, qy, T = sp.symbols("rho, qx, qy, T")
    Td, Tu = 0.5, -0.5
    xmin, xmax, ymin, ymax = 0.0, 2.0, 0.0, 1.0
    Ra, Pr, alpha, la, g = 2000, 0.71, 0.005, 1.0, 9.81
    nu = np.sqrt(Pr * alpha * 9.81 * (Td - Tu) * (ymax - ymin) / Ra)
    kappa = nu / Pr
    eta = nu
    snu = 1.0 / (0.5 + 3 * nu)
    seta = 1.0 / (0.5 + 3 * eta)
    sq = 8 * (2 - snu) / (8 - snu)
    se = seta
    sf = [0.0, 0.0, 0.0, seta, se, sq, sq, snu, snu]
    a = 0.5
    skappa = 1.0 / (0.5 + 10 * kappa / (4 + a))
    se = 1.0 / (0.5 + np.sqrt(3) / 3)
    snu = se
    sT = [0.0, skappa, skappa, se, snu]

    def init_T(x, y, Td, Tu, xmin, xmax, ymin, ymax):
        xmid, ymid = (xmax + xmin) / 2, (ymax + ymin) / 2
        return Td + (Tu - Td) / (ymax - ymin) * (y - ymin) + Td * (x < 1.1 * xmid) * (x > 0.9 * xmid) * (y < ymid)

    def bc_up(f, m, x, y, Tu):
        m[qx] = 0.0
        m[qy] = 0.0
        m[T] = Tu

    def bc_down_with_time(f, m, t, x, y, Td, Tu):
        m[qx] = 0.0
        m[qy] = 0.0
        if 0 <= t % 10.0 <= 5:
            m[T] = Td
        else:
            m[T] = Tu

    walls = {0: bc.BouzidiBounceBack, 1: bc.BouzidiAntiBounceBack}
    return {
        "box": {"x": [xmin, xmax], "y": [ymin, ymax], "label": [-1, -1, 0, 1]},
        "space_step": dx,
        "scheme_velocity": la,
        "schemes": [
            {"velocities": list(range(9)), "conserved_moments": [rho, qx, qy],
             "polynomials": [1, X, Y, 3 * (X**2 + Y**2) - 4, 0.5 * (9 * (X**2 + Y**2)**2 - 21 * (X**2 + Y**2) + 8),
                             3 * X * (X**2 + Y**2) - 5 * X, 3 * Y * (X**2 + Y**2) - 5 * Y, X**2 - Y**2, X * Y],
             "relaxation_parameters": sf,
             "equilibrium": [rho, qx, qy, -2 * rho + 3 * (qx**2 + qy**2), rho - 3 * (qx**2 + qy**2), -qx, -qy,
                             qx**2 - qy**2, qx * qy],
             "source_terms": {qy: alpha * g * T}},
            {"velocities": list(range(5)), "conserved_moments": T,
             "polynomials": [1, X, Y, 5 * (X**2 + Y**2) - 4, (X**2 - Y**2)],
             "equilibrium": [T, T * qx, T * qy, a * T, 0.0], "relaxation_parameters": sT},
        ],
        "init": {rho: 1.0, qx: 0.0, qy: 0.0, T: (init_T, (Td, Tu, xmin, xmax, ymin, ymax))},
        "boundary_conditions": {
            0: {"method": dict(walls), "value": (bc_down_with_time, (Td, Tu)), "time_bc": True},
            1: {"method": dict(walls), "value": (bc_up, (Tu,))},
        },
        "generator": generator,
    }


def _bump(x, xmin, xmax, reg):
    """Compactly supported bump of regularity ``reg`` centred at a quarter of
    the domain (u_init of demo/1D/advection.py and demo/1D/burgers.py)."""
    middle, width = 0.75 * xmin + 0.25 * xmax, 0.125 * (xmax - xmin)
    coeffs = [(-1)**k * math.comb(reg, k) / (2 * k + 1) for k in range(reg + 1)]
    cte = sum(coeffs)
    out = np.zeros(x.shape)
    left = (x > middle - width) & (x <= middle)
    right = (x < middle + width) & (x > middle)
    sl = (x[left] - (middle - width) - 0.5 * width) / (0.5 * width)
    sr = (x[right] - middle - 0.5 * width) / (0.5 * width)
    out[left] = sum(c * sl**(2 * k + 1) for k, c in enumerate(coeffs)) + cte
    out[right] = cte - sum(c * sr**(2 * k + 1) for k, c in enumerate(coeffs))
    return out / (2 * cte)


def advection_1d(dx=1.0 / 64, bc=None, generator="cuda"):
    """Periodic advection, D1Q2 with a symbolic rate (demo/1D/advection.py:81-112, the D1Q2 run)."""
    U, Xs = sp.symbols("u, X")
    C, la_c = sp.symbols("c, lambda", constants=True)
    sigma0 = sp.Symbol("sigma_0", constants=True)
    return {
        "box": {"x": [0.0, 1.0], "label": -1},
        "space_step": dx,
        "scheme_velocity": la_c,
        "schemes": [{"velocities": [1, 2], "conserved_moments": U, "polynomials": [1, Xs],
                     "relaxation_parameters": [0.0, 1 / (0.5 + sigma0)], "equilibrium": [U, C * U]}],
        "init": {U: (_bump, (0.0, 1.0, 0))},
        "generator": generator,
        "parameters": {la_c: 1.0, C: 0.25, sigma0: 1 / 2.0 - 0.5},
    }


def burgers_1d(dx=1.0 / 64, bc=None, generator="cuda"):
    """Burgers equation, D1Q2 with Neumann ends (demo/1D/burgers.py:82-113, the D1Q2 run)."""
    bc = _bc(bc)
    U, Xs = sp.symbols("u, X")
    la_c = sp.symbols("lambda", constants=True)
    sigma0 = sp.Symbol("sigma_0", constants=True)
    return {
        "box": {"x": [-1.0, 1.0], "label": 0},
        "space_step": dx,
        "scheme_velocity": la_c,
        "schemes": [{"velocities": [1, 2], "conserved_moments": U, "polynomials": [1, Xs],
                     "relaxation_parameters": [0.0, 1 / (0.5 + sigma0)], "equilibrium": [U, U**2 / 2]}],
        "init": {U: (_bump, (-1.0, 1.0, 1))},
        "boundary_conditions": {0: {"method": {0: bc.Neumann}}},
        "generator": generator,
        "parameters": {la_c: 1.0, sigma0: 1 / 1.8 - 0.5},
    }


def advection_reaction_1d(dx=1.0 / 64, bc=None, generator="cuda"):
    """Advection with a logistic reaction source mu u (1 - u), D1Q2
    (demo/1D/advection_reaction.py:50-105)."""
    Xs, U = sp.symbols("X, u")
    C, MU, la_c = sp.symbols("c, mu, lambda", constants=True)

    def u_init(x, xmin, xmax):
        middle, width = 0.5 * (xmin + xmax), 0.1 * (xmax - xmin)
        xc = xmin + x % (xmax - xmin)
        return 0.25 + 0.125 / width**10 * (xc - middle - width)**5 * (middle - xc - width)**5 * (
            abs(xc - middle) <= width)

    return {
        "box": {"x": [0.0, 1.0], "label": -1},
        "space_step": dx,
        "scheme_velocity": la_c,
        "schemes": [{"velocities": [1, 2], "conserved_moments": U, "polynomials": [1, Xs],
                     "relaxation_parameters": [0.0, 2.0], "equilibrium": [U, C * U],
                     "source_terms": {U: MU * U * (1 - U)}}],
        "init": {U: (u_init, (0.0, 1.0))},
        "generator": generator,
        "parameters": {la_c: 1.0, C: 0.25, MU: 1.0},
    }


def shallow_water(dx=1.0 / 64, bc=None, generator="cuda"):
    """Shallow water, three D2Q4 with relative velocity q/h (demo/2D/shallow_water.py:36-115).

    Periodic [-1, 1]^2, la = 4, g = 1, a raised disc of water.
    """
    H, QXs, QYs = sp.symbols("h, qx, qy")
    la_c, G = sp.symbols("lambda, g", constants=True)
    s_hx, s_hxy, s_qx, s_qxy = sp.symbols("sigma_0, sigma_1, sigma_2, sigma_3", constants=True)
    xmin, xmax, ymin, ymax = -1.0, 1.0, -1.0, 1.0
    rate_hx, rate_hxy = 1 / (0.5 + s_hx), 1 / (0.5 + s_hxy)
    rate_qx, rate_qxy = 1 / (0.5 + s_qx), 1 / (0.5 + s_qxy)
    vel, polys = list(range(1, 5)), [1, X, Y, X**2 - Y**2]

    def h_init(x, y, xmin, xmax, ymin, ymax):
        center = (0.5 * xmin + 0.5 * xmax, 0.5 * ymin + 0.5 * ymax)
        return 1 + 0.5 * ((x - center[0])**2 + (y - center[1])**2 < 0.1**2)

    return {
        "parameters": {la_c: 4, G: 1.0, s_hx: 1.0e-3, s_hxy: 0.5, s_qx: 1.0e-1, s_qxy: 0.5},
        "box": {"x": [xmin, xmax], "y": [ymin, ymax], "label": -1},
        "space_step": dx,
        "scheme_velocity": la_c,
        "schemes": [
            {"velocities": vel, "conserved_moments": H, "polynomials": polys,
             "relaxation_parameters": [0.0, rate_hx, rate_hx, rate_hxy], "equilibrium": [H, QXs, QYs, 0.0]},
            {"velocities": vel, "conserved_moments": QXs, "polynomials": polys,
             "relaxation_parameters": [0.0, rate_qx, rate_qx, rate_qxy],
             "equilibrium": [QXs, QXs**2 / H + G * H**2 / 2, QXs * QYs / H, 0.0]},
            {"velocities": vel, "conserved_moments": QYs, "polynomials": polys,
             "relaxation_parameters": [0.0, rate_qx, rate_qx, rate_qxy],
             "equilibrium": [QYs, QXs * QYs / H, QYs**2 / H + G * H**2 / 2, 0.0]},
        ],
        "init": {H: (h_init, (xmin, xmax, ymin, ymax)), QXs: 0.0, QYs: 0.0},
        "relative_velocity": [QXs / H, QYs / H],
        "generator": generator,
    }


# name: (dictionary builder, final time, golden file, {golden field: conserved moment name})
CASES = {
    "poiseuille": (poiseuille, 0.5, "test2D_poiseuille", {"rho": "rho", "qx": "qx", "qy": "qy"}),
    "poiseuille_vec": (poiseuille_vec, 0.5, "test2D_poiseuille_vec", {"p": "p", "ux": "ux", "uy": "uy"}),
    "orszag_tang": (orszag_tang, 0.5, "test2D_orszag_Tang_vortex",
                    {k: k for k in ("rho", "qx", "qy", "E", "Bx", "By")}),
    "advection_3d": (advection_3d, 0.5, "test3D_advection", {"u": "u"}),
    "lid_driven_cavity": (lid_driven_cavity, 0.5, "test2D_lid_driven_cavity", {"rho": "rho", "qx": "qx", "qy": "qy"}),
    "kelvin_helmholtz": (kelvin_helmholtz, 0.5, "test2D_kelvin_Helmoltz", {"rho": "rho", "qx": "qx", "qy": "qy"}),
    "karman_vortex_street": (karman_vortex_street, 0.5, "test2D_karman_vortex_street",
                             {"rho": "rho", "qx": "qx", "qy": "qy"}),
    "advection_2d": (advection_2d, 0.5, "test2D_advection", {"U": "U"}),
    "air_conditioning": (air_conditioning, 0.5, "test2D_air_conditioning",
                         {"rho": "rho", "qx": "qx", "qy": "qy", "T": "T"}),
    "rayleigh_benard": (rayleigh_benard, 0.5, "test2D_rayleigh_benard",
                        {"rho": "rho", "qx": "qx", "qy": "qy", "T": "T"}),
    "advection_1d": (advection_1d, 0.5, "test1D_advection", {"u": "u"}),
    "burgers_1d": (burgers_1d, 0.5, "test1D_burgers", {"u": "u"}),
    "advection_reaction_1d": (advection_reaction_1d, 0.5, "test1D_advection_reaction", {"u": "u"}),
    "shallow_water": (shallow_water, 0.5, "test2D_shallow_water", {"h": "h", "qx": "qx", "qy": "qy"}),
    "euler_1d": (euler_1d, 0.5, "test1D_euler", {"rho": "rho", "q": "q", "E": "E"}),
    "poiseuille_3d": (poiseuille_3d, 0.5, "test3D_poseuille", {"p": "p", "ux": "ux", "uy": "uy", "uz": "uz"}),
}


def advection_init_f(dx=1.0 / 64, bc=None, generator="cuda"):
    """2D advection initialised by its distributions (demo/2D/advection_init_f.py:25-105)."""
    d = advection_2d(dx=dx, bc=bc, generator=generator)
    cx, cy, la = 0.2, 0.5, 2.0
    xmin, xmax, ymin, ymax = 0.0, 1.0, 0.0, 1.0

    def u_init(x, y, xmin, xmax, ymin, ymax):
        center = (0.75 * xmin + 0.25 * xmax, 0.50 * ymin + 0.50 * ymax)
        return 1 + (1.5 - 1) * ((x - center[0])**2 + (y - center[1])**2 < 0.1**2)

    def f_init(x, y, k, cx, cy, xmin, xmax, ymin, ymax):
        coeff = 0.25 + 0.5 * (cx, cy, -cx, -cy)[k]
        return coeff * u_init(x, y, xmin, xmax, ymin, ymax)

    d["inittype"] = "distributions"
    d["init"] = {k: (f_init, (k, cx / la, cy / la, xmin, xmax, ymin, ymax)) for k in range(4)}
    return d


CASES["advection_init_f"] = (advection_init_f, 0.5, "test2D_advection_init_f", {"U": "U"})


# ---------------------------------------------------------------------------
# 1D Riemann problems (demo/1D/riemann_problems/*.py): D1Q2 per conserved
# quantity, symbolic rates 1/(1/2 + sigma), Neumann ends, piecewise-constant
# initial state (riemann_pb of exact_solvers/riemann_solvers.py:21-48).

def _riemann(x, xmid, left, right):
    out = np.empty(x.shape)
    out[x < xmid] = left
    out[x >= xmid] = right
    return out


def _riemann_system(xmin, xmax, la, fields, rates, flux, states, params, dx, bc, generator):
    """fields: conserved symbols; rates: sigma symbol -> s; flux: equilibrium
    of the first-order moment of each field; states: (left, right) per field."""
    bc = _bc(bc)
    Xs = sp.Symbol("X")
    la_c = sp.symbols("lambda", constants=True)
    xmid = 0.5 * (xmin + xmax)
    schemes = [{"velocities": [1, 2], "conserved_moments": f, "polynomials": [1, Xs],
                "relaxation_parameters": [0, 1 / (0.5 + sig)], "equilibrium": [f, fl]}
               for f, sig, fl in zip(fields, rates, flux)]
    prm = {la_c: la}
    prm.update({sig: 1 / s - 0.5 for sig, s in rates.items()})
    prm.update(params)
    return {
        "box": {"x": [xmin, xmax], "label": 0},
        "space_step": dx,
        "scheme_velocity": la_c,
        "schemes": schemes,
        "init": {f: (_riemann, (xmid, l, r)) for f, (l, r) in zip(fields, states)},
        "boundary_conditions": {0: {"method": {i: bc.Neumann for i in range(len(fields))}}},
        "generator": generator,
        "parameters": prm,
    }


def riemann_advection(dx=1.0 / 64, bc=None, generator="cuda"):
    """demo/1D/riemann_problems/advection.py:24-82: u_t + c u_x = 0, c = 1/4, s = 1.9."""
    U = sp.Symbol("u")
    C, SIG = sp.symbols("c, sigma", constants=True)
    return _riemann_system(0.0, 1.0, 1.0, [U], {SIG: 1.9}, [C * U], [(1.0, 0.0)], {C: 0.25}, dx, bc, generator) | {
        "init": {U: (_riemann, (0.25, 1.0, 0.0))}}


def riemann_burgers(dx=1.0 / 64, bc=None, generator="cuda"):
    """demo/1D/riemann_problems/burgers.py:28-81: rarefaction 0 | 0.3 on [-1, 1], s = 1.8."""
    U = sp.Symbol("u")
    SIG = sp.Symbol("sigma", constants=True)
    return _riemann_system(-1.0, 1.0, 1.0, [U], {SIG: 1.8}, [U**2 / 2], [(0.0, 0.3)], {}, dx, bc, generator)


def riemann_euler(dx=1.0 / 64, bc=None, generator="cuda"):
    """demo/1D/riemann_problems/euler.py:38-121: Sod tube, gamma = 1.4, la = 3."""
    RHOs, Q, E = sp.symbols("rho, q, E")
    GAMMA = sp.Symbol("gamma", constants=True)
    s1, s2, s3 = sp.symbols("sigma_1, sigma_2, sigma_3", constants=True)
    gamma = 1.4
    flux = [Q, (GAMMA - 1) * E + (3 - GAMMA) / 2 * Q**2 / RHOs,
            GAMMA * E * Q / RHOs - (GAMMA - 1) / 2 * Q**3 / RHOs**2]
    states = [(1, 1 / 8), (0, 0), (1 / (gamma - 1.0), 0.1 / (gamma - 1.0))]
    return _riemann_system(0.0, 1.0, 3.0, [RHOs, Q, E], {s1: 1.9, s2: 1.5, s3: 1.4}, flux, states,
                           {GAMMA: gamma}, dx, bc, generator)


def riemann_euler_isothermal(dx=1.0 / 64, bc=None, generator="cuda"):
    """demo/1D/riemann_problems/euler_isothermal.py:40-109: c0 = la / sqrt(3), rho 2/3 | 4/3."""
    RHOs, Q = sp.symbols("rho, q")
    CO = sp.Symbol("c_0", constants=True)
    s1, s2 = sp.symbols("sigma_1, sigma_2", constants=True)
    return _riemann_system(-1, 1, 1.0, [RHOs, Q], {s1: 2.0, s2: 1.85}, [Q, Q**2 / RHOs + CO**2 * RHOs],
                           [(1 - 1 / 3, 1 + 1 / 3), (0, 0)], {CO: 1.0 / np.sqrt(3)}, dx, bc, generator)


def riemann_p_system(dx=1.0 / 64, bc=None, generator="cuda"):
    """demo/1D/riemann_problems/p_system.py:28-95: p(u) = u^-gamma, gamma = 2/3, la = 2."""
    U1, U2 = sp.symbols("u_1, u_2")
    GAMMA = sp.Symbol("gamma", constants=True)
    s1, s2 = sp.symbols("sigma_1, sigma_2", constants=True)
    return _riemann_system(0.0, 1.0, 2.0, [U1, U2], {s1: 1.9, s2: 1.9}, [-U2, U1**(-GAMMA)],
                           [(1.50, 0.50), (1.25, 1.50)], {GAMMA: 2.0 / 3.0}, dx, bc, generator)


def riemann_shallow_water(dx=1.0 / 64, bc=None, generator="cuda"):
    """demo/1D/riemann_problems/shallow_water.py:27-92: dam break h 2 | 1, q 0.1 | 0, g = 1, la = 2."""
    H, Q = sp.symbols("h, q")
    G = sp.Symbol("g", constants=True)
    s1, s2 = sp.symbols("sigma_1, sigma_2", constants=True)
    return _riemann_system(-1, 1.0, 2.0, [H, Q], {s1: 1.5, s2: 1.5}, [Q, Q**2 / H + 0.5 * G * H**2],
                           [(2, 1), (0.1, 0.0)], {G: 1}, dx, bc, generator)


CASES.update({
    "riemann_advection": (riemann_advection, 0.5, "test1D_riemann_advection", {"u": "u"}),
    "riemann_burgers": (riemann_burgers, 0.5, "test1D_riemann_burgers", {"u": "u"}),
    "riemann_euler": (riemann_euler, 0.5, "test1D_riemann_euler", {"rho": "rho", "q": "q", "E": "E"}),
    "riemann_euler_isothermal": (riemann_euler_isothermal, 0.5, "test1D_riemann_euler_isothermal",
                                 {"rho": "rho", "q": "q"}),
    "riemann_p_system": (riemann_p_system, 0.5, "test1D_riemann_p_system", {"u_1": "u_1", "u_2": "u_2"}),
    "riemann_shallow_water": (riemann_shallow_water, 0.5, "test1D_riemann_shallow_water", {"h": "h", "q": "q"}),
})


def bend(dx=1.0 / 64, bc=None, parallelogram=None, generator="cuda"):
    """Flow around a bend, D2Q9 Geier with relative velocity (demo/2D/bend.py:58-240).

    A solid block fills [0, 0.75]^2 (label 0, Bouzidi bounce-back); parabolic
    inflow through the left strip (label 2), outflow through the bottom
    strip (label 1, NeumannY).
    """
    bc = _bc(bc)
    if parallelogram is None:
        from pylbm_gb300.geometry import Parallelogram as parallelogram
    la_c = sp.symbols("lambda", constants=True)
    xmin, xmax, ymin, ymax = 0.0, 1.0, 0.0, 1.0
    radius, la, rho_o, u_o, mu = 0.25, 1.0, 1.0, 0.05, 2.5e-6
    zeta = 100 * mu
    xc, yc = xmax - radius, ymax - radius

    def bc_in(f, m, x, y, rho_o, u_o, ymin, ymax, radius):
        y_bound = ymax - radius
        m[RHO] = rho_o
        m[QX] = rho_o * u_o * 4 * (ymax - y) * (y - y_bound) / (ymax - y_bound)**2
        m[QY] = 0.0

    return {
        "box": {"x": [xmin, xmax], "y": [ymin, ymax], "label": [2, 0, 1, 0]},
        "elements": [parallelogram((xmin, ymin), (xc, ymin), (xmin, yc), label=0)],
        "space_step": dx,
        "scheme_velocity": la,
        "schemes": [_geier(la_c, dx, la, rho_o, mu, zeta)],
        "parameters": {la_c: la},
        "init": {RHO: rho_o, QX: rho_o * u_o, QY: 0.0},
        "boundary_conditions": {
            0: {"method": {0: bc.BouzidiBounceBack}},
            1: {"method": {0: bc.NeumannY}},
            2: {"method": {0: bc.BouzidiBounceBack}, "value": (bc_in, (rho_o, u_o, ymin, ymax, radius))},
        },
        "generator": generator,
        "relative_velocity": [QX / RHO, QY / RHO],
    }


CASES["bend"] = (bend, 0.5, "test2D_coude", {"rho": "rho", "qx": "qx", "qy": "qy"})


# ---------------------------------------------------------------------------
# Stencils reaching two nodes (vmax = 2, two ghost layers).  pylbm has no
# golden file for them; their fixtures are the reference's own run of the
# same dictionary (golden file None).

def d1q5_advection(dx=1.0 / 64, bc=None, generator="cuda"):
    """D1Q5 (velocities 0, +-1, +-2) advection, Neumann ends, Riemann initial state."""
    bc = _bc(bc)
    U, Xs = sp.symbols("u, X")
    la_c, C = sp.symbols("lambda, c", constants=True)
    return {
        "box": {"x": [0.0, 1.0], "label": 0},
        "space_step": dx,
        "scheme_velocity": la_c,
        "schemes": [{"velocities": list(range(5)), "conserved_moments": U,
                     "polynomials": [1, Xs, Xs**2 / 2, Xs**3 / 6, Xs**4 / 24],
                     "relaxation_parameters": [0.0, 1.5, 1.4, 1.3, 1.2],
                     "equilibrium": [U, C * U, C**2 * U / 2, C**3 * U / 6, C**4 * U / 24]}],
        "init": {U: (_riemann, (0.3, 1.0, 0.2))},
        "boundary_conditions": {0: {"method": {0: bc.Neumann}}},
        "generator": generator,
        "parameters": {la_c: 2.0, C: 0.25},
    }


def d2q13_advection(dx=1.0 / 32, bc=None, generator="cuda"):
    """D2Q13 (D2Q9 plus (+-2, 0), (0, +-2)) advection on the torus."""
    U = sp.Symbol("u")
    la_c, CX, CY = sp.symbols("lambda, c_x, c_y", constants=True)
    polys = [1, X, Y, X**2, Y**2, X * Y, X**2 * Y, X * Y**2, X**2 * Y**2, X**3, Y**3, X**4, Y**4]
    eq = [sp.sympify(p).subs({X: CX, Y: CY}) * U for p in polys]

    def u0(x, y):
        return 1.0 + 0.5 * ((x - 0.3)**2 + (y - 0.6)**2 < 0.15**2)

    return {
        "box": {"x": [0.0, 1.0], "y": [0.0, 1.0], "label": -1},
        "space_step": dx,
        "scheme_velocity": la_c,
        "schemes": [{"velocities": list(range(13)), "conserved_moments": U, "polynomials": polys,
                     "relaxation_parameters": [0.0] + [1.2] * 12, "equilibrium": eq}],
        "init": {U: u0},
        "generator": generator,
        "parameters": {la_c: 2.0, CX: 0.3, CY: -0.2},
    }


CASES.update({
    "d1q5_advection": (d1q5_advection, 0.5, None, {"u": "u"}),
    "d2q13_advection": (d2q13_advection, 0.25, None, {"u": "u"}),
})


def karman_3d(dx=1.0 / 32, bc=None, sphere=None, generator="cuda"):
    """Flow past a sphere, D3Q15 MRT (demo/3D/Karman.py:29-125), Re 2000.

    Box [0, 2] x [0, 1]^2 periodic in y and z; inflow (label 1) Bouzidi
    bounce-back with qx = 0.01, outflow (label 2) NeumannX, sphere of radius
    1/8 at (0.3, 0.5, 0.5) (label 0) Bouzidi bounce-back.  pylbm has no golden
    file for it; the fixture is the reference run (space step 1/32).
    """
    bc = _bc(bc)
    if sphere is None:
        from pylbm_gb300.geometry import Sphere as sphere
    mass, qx, qy, qz = sp.symbols("mass, qx, qy, qz")
    la_c = sp.Symbol("lambda")
    nu = 5.0 / 2000
    s1, s2, s4 = 1.6, 1.2, 1.6
    s9 = 1.0 / (3 * nu + 0.5)
    s11, s14 = s9, 1.2
    r = X**2 + Y**2 + Z**2

    def bc_up(f, m, x, y, z):
        m[qx] = 0.01

    return {
        "box": {"x": [0.0, 2.0], "y": [0.0, 1.0], "z": [0.0, 1.0], "label": [1, 2, -1, -1, -1, -1]},
        "elements": [sphere((0.3, 0.5, 0.5), 0.125, 0)],
        "space_step": dx,
        "scheme_velocity": 1.0,
        "schemes": [{
            "velocities": list(range(7)) + list(range(19, 27)),
            "conserved_moments": [mass, qx, qy, qz],
            "polynomials": [1, r - 2, 0.5 * (15 * r**2 - 55 * r + 32), X, 0.5 * (5 * r - 13) * X, Y,
                            0.5 * (5 * r - 13) * Y, Z, 0.5 * (5 * r - 13) * Z, 3 * X**2 - r, Y**2 - Z**2,
                            X * Y, Y * Z, Z * X, X * Y * Z],
            "relaxation_parameters": [0, s1, s2, 0, s4, 0, s4, 0, s4, s9, s9, s11, s11, s11, s14],
            "equilibrium": [mass, -mass + qx**2 + qy**2 + qz**2, -mass, qx, -7.0 / 3 * qx, qy, -7.0 / 3 * qy, qz,
                            -7.0 / 3 * qz, 1.0 / 3 * (2 * qx**2 - (qy**2 + qz**2)), qy**2 - qz**2, qx * qy,
                            qy * qz, qz * qx, 0],
        }],
        "init": {mass: 1.0, qx: 0.0, qy: 0.0, qz: 0.0},
        "boundary_conditions": {
            0: {"method": {0: bc.BouzidiBounceBack}},
            1: {"method": {0: bc.BouzidiBounceBack}, "value": bc_up},
            2: {"method": {0: bc.NeumannX}},
        },
        "parameters": {la_c: 1.0},
        "generator": generator,
    }


CASES["karman_3d"] = (karman_3d, 0.25, None, {"mass": "mass", "qx": "qx", "qy": "qy", "qz": "qz"})


def lid_cavity_3d(dx=1.0 / 32, bc=None, generator="cuda"):
    """3D lid-driven cavity, D3Q15 MRT at Re 200 (demo/3D/lid_cavity.py:33-124): the lid
    (label 1, top z face) moves diagonally; Bouzidi bounce-back everywhere.
    The fixture is the reference run (space step 1/32)."""
    d = karman_3d(dx=dx, bc=bc, generator=generator)
    mass, qx, qy, qz = sp.symbols("mass, qx, qy, qz")
    nu = 5.0 / 200
    s9 = 1.0 / (3 * nu + 0.5)
    rates = list(d["schemes"][0]["relaxation_parameters"])
    rates[9:14] = [s9] * 5
    d["schemes"][0]["relaxation_parameters"] = rates
    bc = _bc(bc)

    def bc_up(f, m, x, y, z):
        m[qx] = -math.sqrt(2) / 20.0
        m[qy] = -math.sqrt(2) / 20.0

    d["box"] = {"x": [0.0, 1.0], "y": [0.0, 1.0], "z": [0.0, 1.0], "label": [0, 0, 0, 0, 0, 1]}
    del d["elements"]
    d["boundary_conditions"] = {0: {"method": {0: bc.BouzidiBounceBack}},
                                1: {"method": {0: bc.BouzidiBounceBack}, "value": bc_up}}
    return d


CASES["lid_cavity_3d"] = (lid_cavity_3d, 0.25, None, {"mass": "mass", "qx": "qx", "qy": "qy", "qz": "qz"})
