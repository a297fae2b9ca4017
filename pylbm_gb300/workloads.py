"""Scheme dictionaries of the benchmark workloads.

Each function returns a pylbm scheme dictionary (the format of
pylbm/simulation.py:33 and of the demos in pylbm's demo/ folder).  ``bc`` and
``elements`` default to this package's classes; passing the reference's
``pylbm.bc`` module and ``pylbm.Circle`` yields the same dictionary for
pylbm itself, which is how the golden fixtures are produced.

* ``cavity``       D2Q9 d'Humieres MRT lid-driven cavity (moment basis and
                   equilibrium of demo/2D/lid_driven_cavity.py, dHumiere
                   branch), bounce-back walls, lid by bounce-back with a
                   prescribed velocity.
* ``tgv3d``        D3Q19 MRT (d'Humieres et al. 2002 basis) periodic
                   Taylor-Green vortex with its pressure perturbation.
* ``cylinder``     D2Q9 MRT flow past a disc: anti-bounce-back inflow,
                   Neumann-x outflow, periodic in y, bounce-back obstacle.
* ``shear_layer``  D2Q9 MRT periodic double shear layer (profile of
                   demo/2D/Kelvin_Helmoltz.py).
"""
import numpy as np
import sympy as sp

X, Y, Z = sp.symbols("X, Y, Z")
RHO, QX, QY, QZ = sp.symbols("rho, qx, qy, qz")
LA = sp.symbols("lambda", constants=True)


def _bc(bc):
    if bc is None:
        from . import boundary as bc
    return bc


def d2q9_dhumieres(rates):
    """Polynomials and equilibrium of the D2Q9 d'Humieres basis (rho0 = 1)."""
    polys = [1, X, Y, 3 * (X**2 + Y**2) - 4 * LA**2,
             sp.Rational(1, 2) * (9 * (X**2 + Y**2)**2 - 21 * (X**2 + Y**2) * LA**2 + 8 * LA**4),
             3 * X * (X**2 + Y**2) - 5 * X * LA**2, 3 * Y * (X**2 + Y**2) - 5 * Y * LA**2,
             X**2 - Y**2, X * Y]
    q2 = QX**2 + QY**2
    eq = [RHO, QX, QY, -2 * RHO * LA**2 + 3 * q2, RHO * LA**2 - 3 * q2, -QX * LA**2, -QY * LA**2,
          QX**2 - QY**2, QX * QY]
    return {"velocities": list(range(9)), "polynomials": polys, "relaxation_parameters": list(rates),
            "equilibrium": eq, "conserved_moments": [RHO, QX, QY]}


def omega_from_nu(nu):
    """Shear relaxation rate for a lattice viscosity nu (la = dx/dt = 1)."""
    return 1.0 / (0.5 + 3.0 * nu)


def cavity(n=256, nu=1e-3, lid=0.05, bc=None, generator="cuda", omega=None):
    bc = _bc(bc)
    w = omega_from_nu(nu) if omega is None else omega
    rho_o = 1.0

    def bc_up(f, m, x, y, rho, u):
        m[RHO] = rho
        m[QX] = rho * u
        m[QY] = 0.0

    return {
        "parameters": {LA: 1.0},
        "box": {"x": [0.0, 1.0], "y": [0.0, 1.0], "label": [0, 0, 0, 1]},
        "space_step": 1.0 / n,
        "scheme_velocity": LA,
        "schemes": [d2q9_dhumieres([0.0, 0.0, 0.0, 1.5, 1.5, 1.2, 1.2, w, w])],
        "init": {RHO: rho_o, QX: 0.0, QY: 0.0},
        "boundary_conditions": {
            0: {"method": {0: bc.BounceBack}},
            1: {"method": {0: bc.BounceBack}, "value": (bc_up, (rho_o, lid))},
        },
        "generator": generator,
    }


def d3q19_dhumieres(s_nu, s_e=1.2, s_eps=1.4, s_q=1.5, s_pi=1.6, s_m=1.8):
    """D3Q19 MRT basis of d'Humieres et al. (2002), incompressible equilibria (rho0 = 1)."""
    c2 = X**2 + Y**2 + Z**2
    polys = [1,
             19 * c2 - 30 * LA**2,
             sp.Rational(1, 2) * (21 * c2**2 - 53 * c2 * LA**2 + 24 * LA**4),
             X, (5 * c2 - 9 * LA**2) * X,
             Y, (5 * c2 - 9 * LA**2) * Y,
             Z, (5 * c2 - 9 * LA**2) * Z,
             3 * X**2 - c2, (3 * c2 - 5 * LA**2) * (3 * X**2 - c2),
             Y**2 - Z**2, (3 * c2 - 5 * LA**2) * (Y**2 - Z**2),
             X * Y, Y * Z, X * Z,
             (Y**2 - Z**2) * X, (Z**2 - X**2) * Y, (X**2 - Y**2) * Z]
    j2 = QX**2 + QY**2 + QZ**2
    pxx = 2 * QX**2 - QY**2 - QZ**2
    pww = QY**2 - QZ**2
    eq = [RHO,
          -11 * RHO * LA**2 + 19 * j2,
          3 * RHO * LA**4 - sp.Rational(11, 2) * j2 * LA**2,
          QX, -sp.Rational(2, 3) * QX * LA**2,
          QY, -sp.Rational(2, 3) * QY * LA**2,
          QZ, -sp.Rational(2, 3) * QZ * LA**2,
          pxx, -sp.Rational(1, 2) * pxx * LA**2,
          pww, -sp.Rational(1, 2) * pww * LA**2,
          QX * QY, QY * QZ, QX * QZ,
          0, 0, 0]
    rates = [0.0, s_e, s_eps, 0.0, s_q, 0.0, s_q, 0.0, s_q, s_nu, s_pi, s_nu, s_pi, s_nu, s_nu, s_nu,
             s_m, s_m, s_m]
    return {"velocities": list(range(19)), "polynomials": polys, "relaxation_parameters": rates,
            "equilibrium": eq, "conserved_moments": [RHO, QX, QY, QZ]}


def cavity3d(n=128, nu=1e-3, lid=0.05, bc=None, generator="cuda"):
    """Lid-driven cube, D3Q19 MRT: bounce-back on every wall, the top wall
    (z = 1) moving at ``lid`` along x (the 3D analogue of ``cavity``)."""
    bc = _bc(bc)
    w = omega_from_nu(nu)
    rho_o = 1.0

    def bc_up(f, m, x, y, z, rho, u):
        m[RHO] = rho
        m[QX] = rho * u
        m[QY] = 0.0
        m[QZ] = 0.0

    return {
        "parameters": {LA: 1.0},
        "box": {"x": [0.0, 1.0], "y": [0.0, 1.0], "z": [0.0, 1.0], "label": [0, 0, 0, 0, 0, 1]},
        "space_step": 1.0 / n,
        "scheme_velocity": LA,
        "schemes": [d3q19_dhumieres(w)],
        "init": {RHO: rho_o, QX: 0.0, QY: 0.0, QZ: 0.0},
        "boundary_conditions": {
            0: {"method": {0: bc.BounceBack}},
            1: {"method": {0: bc.BounceBack}, "value": (bc_up, (rho_o, lid))},
        },
        "generator": generator,
    }


def tgv3d(n=256, nu=2e-3, u0=0.04, generator="cuda"):
    """Periodic Taylor-Green vortex on [0, 2pi)^3 with n^3 nodes (lattice units, la = 1)."""
    w = omega_from_nu(nu)
    L = 2 * np.pi
    dx = L / n
    cs2 = 1.0 / 3.0

    def rho_init(x, y, z):
        p = u0**2 / 16.0 * (np.cos(2 * x) + np.cos(2 * y)) * (np.cos(2 * z) + 2.0)
        return 1.0 + p / cs2

    def qx_init(x, y, z):
        return u0 * np.sin(x) * np.cos(y) * np.cos(z)

    def qy_init(x, y, z):
        return -u0 * np.cos(x) * np.sin(y) * np.cos(z)

    def qz_init(x, y, z):
        return np.zeros_like(x * y * z)

    return {
        "parameters": {LA: 1.0},
        "box": {"x": [0.0, L], "y": [0.0, L], "z": [0.0, L], "label": -1},
        "space_step": dx,
        "scheme_velocity": LA,
        "schemes": [d3q19_dhumieres(w)],
        "init": {RHO: rho_init, QX: qx_init, QY: qy_init, QZ: qz_init},
        "generator": generator,
    }


def cylinder(nx=2048, ny=512, radius=32, center=(400, 257), u_in=0.05, re=200.0, bc=None, circle=None,
             generator="cuda"):
    """Flow past a disc of ``radius`` nodes; Re from the diameter."""
    bc = _bc(bc)
    if circle is None:
        from .geometry import Circle as circle
    dx = 1.0 / ny
    nu = u_in * 2 * radius / re
    w = omega_from_nu(nu)

    def bc_in(f, m, x, y, rho, u):
        m[RHO] = rho
        m[QX] = rho * u
        m[QY] = 0.0

    return {
        "parameters": {LA: 1.0},
        "box": {"x": [0.0, nx * dx], "y": [0.0, 1.0], "label": [1, 2, -1, -1]},
        "elements": [circle((center[0] * dx, center[1] * dx), radius * dx, label=0)],
        "space_step": dx,
        "scheme_velocity": LA,
        "schemes": [d2q9_dhumieres([0.0, 0.0, 0.0, 1.5, 1.5, 1.2, 1.2, w, w])],
        "init": {RHO: 1.0, QX: u_in, QY: 0.0},
        "boundary_conditions": {
            0: {"method": {0: bc.BounceBack}},
            1: {"method": {0: bc.AntiBounceBack}, "value": (bc_in, (1.0, u_in))},
            2: {"method": {0: bc.NeumannX}},
        },
        "generator": generator,
    }


def shear_layer(n=256, nu=1e-3, u0=0.05, width=1.0 / 80.0, delta=0.05, omega=None, generator="cuda", seed=None):
    """Periodic double shear layer on the unit square (n^2 nodes).

    ``omega`` may be a sympy symbol: it then becomes a run-time parameter
    (``sim.extra_parameters``).  ``seed`` adds a random low-mode perturbation
    (used for ensembles of distinct instances).
    """
    w = omega_from_nu(nu) if omega is None else omega
    k = 1.0 / width
    rng = np.random.default_rng(seed) if seed is not None else None
    phases = rng.uniform(0, 2 * np.pi, 3) if rng is not None else None
    amps = rng.uniform(0.5, 1.5, 3) if rng is not None else None

    def qx_init(x, y):
        return np.zeros_like(x) + u0 * np.tanh(k * (y - 0.25)) * (y <= 0.5) + u0 * np.tanh(k * (0.75 - y)) * (y > 0.5)

    def qy_init(x, y):
        base = u0 * delta * np.sin(2 * np.pi * (x + 0.25))
        if phases is not None:
            for i in range(3):
                base = base + 0.3 * u0 * delta * amps[i] * np.sin(2 * np.pi * (i + 2) * x + phases[i])
        return np.zeros_like(y) + base

    return {
        "parameters": {LA: 1.0},
        "box": {"x": [0.0, 1.0], "y": [0.0, 1.0], "label": -1},
        "space_step": 1.0 / n,
        "scheme_velocity": LA,
        "schemes": [d2q9_dhumieres([0.0, 0.0, 0.0, 1.5, 1.5, 1.2, 1.2, w, w])],
        "init": {RHO: 1.0, QX: qx_init, QY: qy_init},
        "generator": generator,
    }


def geier_d2q9(dx, la=1.0, rho_o=1.0, mu=5.0e-6, zeta=5.0e-5):
    """D2Q9 Geier basis with relative velocity q/rho: central moments (pylbm's
    2D Navier-Stokes demos, moments_choice "Geier"); rates from the bulk and
    shear viscosities."""
    ux, uy = QX / RHO, QY / RHO
    rhou2 = RHO * (ux**2 + uy**2)
    c = 3.0 / (la * rho_o * dx)
    s_1 = 1 / (0.5 + c * (zeta - 2 * mu / 3))
    s_2 = 1 / (0.5 + c * mu)
    return {
        "velocities": list(range(9)),
        "polynomials": [1, X, Y, X**2 + Y**2, X * Y**2, Y * X**2, X**2 * Y**2, X**2 - Y**2, X * Y],
        "relaxation_parameters": [0.0, 0.0, 0.0, s_1, s_1, s_1, s_1, s_2, s_2],
        "equilibrium": [RHO, QX, QY, rhou2 + 2 / 3 * RHO * LA**2, QX * (LA**2 / 3 + uy**2),
                        QY * (LA**2 / 3 + ux**2), RHO * (LA**2 / 3 + ux**2) * (LA**2 / 3 + uy**2),
                        RHO * (ux**2 - uy**2), RHO * ux * uy],
        "conserved_moments": [RHO, QX, QY],
    }


def karman(dx=1.0 / 64, u_o=0.05, mu=5.0e-6, bc=None, circle=None, generator="cuda"):
    """Flow past a disc in a channel, D2Q9 Geier with relative velocity and
    Bouzidi walls (the physics of pylbm's demo/2D/Karman_vortex_street.py at
    any resolution): box [0, 2] x [0, 1], disc of radius 1/32 at
    (0.3, 0.5 + 2 dx), inflow state on label 0, NeumannX outflow."""
    bc = _bc(bc)
    if circle is None:
        from .geometry import Circle as circle
    rho_o, la = 1.0, 1.0

    def bc_in(f, m, x, y, rho_o, u_o):
        m[RHO] = rho_o
        m[QX] = rho_o * u_o
        m[QY] = 0.0

    return {
        "box": {"x": [0.0, 2.0], "y": [0.0, 1.0], "label": [0, 1, 0, 0]},
        "elements": [circle([0.3, 0.5 + 2 * dx], 1.0 / 32, label=2)],
        "space_step": dx,
        "scheme_velocity": la,
        "schemes": [geier_d2q9(dx, la, rho_o, mu, 10 * mu)],
        "parameters": {LA: la},
        "init": {RHO: rho_o, QX: rho_o * u_o, QY: 0.0},
        "boundary_conditions": {
            0: {"method": {0: bc.BouzidiBounceBack}, "value": (bc_in, (rho_o, u_o))},
            1: {"method": {0: bc.NeumannX}},
            2: {"method": {0: bc.BouzidiBounceBack}},
        },
        "generator": generator,
        "relative_velocity": [QX / RHO, QY / RHO],
    }
