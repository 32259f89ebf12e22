"""Workload definitions shared by the tests and the fixture generator.

Initial data are evaluated at cell midpoints origin + dx*(i + 1/2)
(alsfvm/src/grid/Grid.cpp:148-165) with Python's math module, which calls the
C library, so the values equal what the library's C++ initial-data code
computes. Arrays are interior-only primitive variables (rho, u..., p) or (u),
one block per variable, x fastest.
"""
import math

import numpy as np

NVAR = {"euler1": 3, "euler2": 4, "euler3": 5, "burgers": 1}
RECONSTRUCTIONS = ["none", "weno2", "eno2", "eno3", "eno4"]
# the limiter reconstructions (MC.hpp, MM.hpp) and the fluxes beyond HLL /
# HLL3 / Godunov (numerical_flux_list.hpp): their fixtures live in
# golden/flux_extra.npz
LIMITER_RECONSTRUCTIONS = ["mc", "mm"]
EULER_RECONSTRUCTIONS = ["wenof2"]  # WENOF2.hpp: primitive-variable WENO2, Euler only
EXTRA_FLUXES = {"euler1": ["central"], "euler2": ["central"], "euler3": ["central"],
                "burgers": ["central", "rusanov", "roe"]}
BASE_FLUXES = {"euler1": ["hll", "hll3"], "euler2": ["hll", "hll3"], "euler3": ["hll", "hll3"],
               "burgers": ["godunov"]}
_GHOSTS = {"none": 1, "weno2": 2, "eno2": 2, "eno3": 3, "eno4": 4, "mc": 2, "mm": 2, "wenof2": 2}


def ghost_cells(recon):
    return _GHOSTS[recon]


def dimension(n):
    return 3 if n[2] > 1 else (2 if n[1] > 1 else 1)


def padded_shape(n, g):
    dim = dimension(n)
    return [n[d] + 2 * g if d < dim else n[d] for d in range(3)]


def smooth_random_state(eq, t, rng):
    """A positive conserved state on a padded grid of shape t: smooth waves in
    every direction plus 1% noise, so high-order reconstructions stay physical."""
    z, y, x = np.meshgrid(np.arange(t[2]), np.arange(t[1]), np.arange(t[0]), indexing="ij")
    x, y, z = x.ravel(), y.ravel(), z.ravel()
    tot = x.size
    nv = NVAR[eq]
    U = np.zeros((nv, tot))
    wave = np.sin(0.41 * x + 0.2) + np.cos(0.33 * y + 0.5) + np.sin(0.29 * z + 1.1)
    if eq == "burgers":
        U[0] = 0.3 * wave + rng.uniform(-0.01, 0.01, tot)
        return U
    nsd = nv - 2
    rho = 1.5 + 0.15 * wave + rng.uniform(0, 0.01, tot)
    u = 0.2 * np.sin(0.37 * x[None, :] + 0.7 * np.arange(nsd)[:, None]) + rng.uniform(-0.01, 0.01, (nsd, tot))
    p = 1.5 + 0.15 * np.cos(0.23 * x + 0.31 * y + 0.17 * z) + rng.uniform(0, 0.01, tot)
    U[0] = rho
    U[1:1 + nsd] = rho * u
    U[-1] = p / 0.4 + 0.5 * rho * (u * u).sum(0)
    return U


def midpoints(n, lower, upper):
    return [[lower[d] + (upper[d] - lower[d]) / n[d] * i + (upper[d] - lower[d]) / n[d] / 2.0
             for i in range(n[d])] for d in range(3)]


def sod_prim(n, lower=-5.0, upper=5.0):
    """Sod shock tube: (rho, u, p) = (1, 0, 1) for x < 0, (0.125, 0, 0.1) otherwise."""
    xs = midpoints((n, 1, 1), (lower, 0, 0), (upper, 1, 1))[0]
    prim = np.zeros((3, n))
    for i, x in enumerate(xs):
        left = x < 0
        prim[0, i] = 1.0 if left else 0.125
        prim[2, i] = 1.0 if left else 0.1
    return prim


def kh_perturbation(x, a, b):
    """d(x) = 0.01 * sum_j a_j cos(b_j + 2 pi j x), j = 1..10."""
    s = 0.0
    for j in range(10):
        s += a[j] * math.cos(b[j] + 2 * math.pi * (j + 1) * x)
    return 0.01 * s


def kh_parameters(X):
    """Maps 40 uniform draws to (a1, b1, a2, b2): a_j normalised to sum 1, b_j
    scaled to [0, 2 pi]. X[0:10] -> a1, X[10:20] -> b1, X[20:30] -> a2,
    X[30:40] -> b2."""
    X = list(X)
    a1 = X[0:10]
    s1 = sum(a1)
    a1 = [v / s1 for v in a1]
    b1 = [2 * math.pi * v for v in X[10:20]]
    a2 = X[20:30]
    s2 = sum(a2)
    a2 = [v / s2 for v in a2]
    b2 = [2 * math.pi * v for v in X[30:40]]
    return a1, b1, a2, b2


def kh_prim(n, X):
    """Kelvin-Helmholtz on [0,1]^2: rho=2, u=-0.5 inside 0.25+d1(x) < y < 0.75+d2(x),
    rho=1, u=0.5 outside; v=0, p=2.5. The interface heights come from math.cos
    per column; the inside test is a comparison of doubles, done for all rows
    at once (numpy's addition and comparison are the IEEE operations)."""
    a1, b1, a2, b2 = kh_parameters(X)
    xs, ys, _ = midpoints((n, n, 1), (0, 0, 0), (1, 1, 0))
    lo = 0.25 + np.array([kh_perturbation(x, a1, b1) for x in xs])
    hi = 0.75 + np.array([kh_perturbation(x, a2, b2) for x in xs])
    y = np.array(ys)[:, None]
    inside = ((lo[None, :] < y) & (y < hi[None, :])).ravel()
    prim = np.zeros((4, n * n))
    prim[0] = np.where(inside, 2.0, 1.0)
    prim[1] = np.where(inside, -0.5, 0.5)
    prim[3] = 2.5
    return prim


def tg_prim(n):
    """Taylor-Green on [0, 2 pi]^3: rho=1, u=sin x cos y cos z, v=-cos x sin y cos z,
    w=0, p=100+((cos 2x + cos 2y)(cos 2z + 2) - 2)/16."""
    L = 2 * math.pi
    xs, ys, zs = midpoints((n, n, n), (0, 0, 0), (L, L, L))
    prim = np.zeros((5, n * n * n))
    for kz, z in enumerate(zs):
        for j, y in enumerate(ys):
            for i, x in enumerate(xs):
                k = (kz * n + j) * n + i
                prim[0, k] = 1.0
                prim[1, k] = math.sin(x) * math.cos(y) * math.cos(z)
                prim[2, k] = -math.cos(x) * math.sin(y) * math.cos(z)
                prim[4, k] = 100 + ((math.cos(2 * x) + math.cos(2 * y)) * (math.cos(2 * z) + 2) - 2) / 16
    return prim


def burgers_prim(n, phase):
    """u0 = sin(2 pi x) + 0.5 * phase on [0,1], phase a U[-1,1] draw."""
    xs = midpoints((n, 1, 1), (0, 0, 0), (1, 1, 1))[0]
    return np.array([[math.sin(2 * math.pi * x) + 0.5 * phase for x in xs]])


_KH_X = [((k * 7919) % 1000) / 1000.0 + 0.0005 for k in range(40)]

GOLDEN_RUNS = {
    "sod256": dict(equation="euler1", flux="hll3", recon="weno2", integrator="rungekutta3",
                   boundary="neumann", n=(256, 1, 1), lower=(-5, 0, 0), upper=(5, 1, 1), gamma=1.4,
                   cfl=0.475, end_time=1.3, number_of_saves=1, max_steps=0,
                   prim=lambda: sod_prim(256)),
    "sod128_hll_eno3_rk2": dict(equation="euler1", flux="hll", recon="eno3", integrator="rungekutta2",
                                boundary="neumann", n=(128, 1, 1), lower=(-5, 0, 0), upper=(5, 1, 1),
                                gamma=1.4, cfl=0.475, end_time=1.3, number_of_saves=1, max_steps=0,
                                prim=lambda: sod_prim(128)),
    "kh32": dict(equation="euler2", flux="hll3", recon="weno2", integrator="rungekutta3",
                 boundary="periodic", n=(32, 32, 1), lower=(0, 0, 0), upper=(1, 1, 0), gamma=1.4,
                 cfl=0.4, end_time=2.0, number_of_saves=0, max_steps=20,
                 prim=lambda: kh_prim(32, _KH_X)),
    "kh24_eno2_fe": dict(equation="euler2", flux="hll", recon="eno2", integrator="forwardeuler",
                         boundary="periodic", n=(24, 24, 1), lower=(0, 0, 0), upper=(1, 1, 0),
                         gamma=1.4, cfl=0.4, end_time=2.0, number_of_saves=0, max_steps=10,
                         prim=lambda: kh_prim(24, _KH_X)),
    "tg8": dict(equation="euler3", flux="hll3", recon="weno2", integrator="rungekutta3",
                boundary="periodic", n=(8, 8, 8), lower=(0, 0, 0), upper=(2 * math.pi,) * 3, gamma=1.4,
                cfl=0.4, end_time=100.0, number_of_saves=0, max_steps=5, prim=lambda: tg_prim(8)),
    "burgers128": dict(equation="burgers", flux="godunov", recon="weno2", integrator="rungekutta2",
                       boundary="periodic", n=(128, 1, 1), lower=(0, 0, 0), upper=(1, 1, 1), gamma=1.4,
                       cfl=0.475, end_time=0.5, number_of_saves=1, max_steps=0,
                       prim=lambda: burgers_prim(128, 0.3)),
    "burgers96_eno4_rk3": dict(equation="burgers", flux="godunov", recon="eno4", integrator="rungekutta3",
                               boundary="periodic", n=(96, 1, 1), lower=(0, 0, 0), upper=(1, 1, 1),
                               gamma=1.4, cfl=0.475, end_time=0.5, number_of_saves=1, max_steps=0,
                               prim=lambda: burgers_prim(96, -0.4)),
}


# Functional fixtures (tests/golden/functional.npz, made by make_golden.py)
# name: (functional, equation, boundary, n, ghosts, lower, upper, params, weight)
FUNCTIONAL_CASES = {
    "identity_euler2": ("identity", "euler2", "periodic", (9, 7, 1), 2, (0, 0, 0), (1, 1, 0), {}, 0.7),
    "identity_burgers1d": ("identity", "burgers", "neumann", (20, 1, 1), 3, (0, 0, 0), (1, 1, 1), {}, 1.0),
    "identity_euler3": ("identity", "euler3", "periodic", (5, 4, 3), 2, (0, 0, 0), (1, 1, 1), {}, 1.3),
    "moment2_euler2": ("moment", "euler2", "periodic", (8, 6, 1), 2, (0, 0, 0), (1, 1, 0), {"degree": 2}, 0.5),
    "moment3_burgers1d": ("moment", "burgers", "periodic", (17, 1, 1), 2, (0, 0, 0), (1, 1, 1), {"degree": 3}, 1.0),
    "moment1_euler3": ("moment", "euler3", "neumann", (4, 5, 3), 1, (0, 0, 0), (1, 1, 1), {"degree": 1}, 2.0),
    "legendre3_euler2": ("legendre_pointwise", "euler2", "periodic", (7, 6, 1), 2, (0, 0, 0), (1, 1, 0),
                         {"degree": 3, "min_value": 0.0, "max_value": 10.0}, 1.0),
    "legendre5_euler2_rhoE": ("legendre_pointwise", "euler2", "neumann", (6, 8, 1), 2, (0, 0, 0), (1, 1, 0),
                              {"degree": 5, "min_value": -2.0, "max_value": 8.0, "variables": "rho E"}, 0.25),
    "legendre0_burgers2d": ("legendre_pointwise", "burgers", "periodic", (5, 6, 1), 2, (0, 0, 0), (1, 1, 0),
                            {"degree": 0, "min_value": -1.0, "max_value": 1.0}, 1.0),
    "log_entropy_euler2": ("log_entropy", "euler2", "periodic", (8, 7, 1), 2, (0, 0, 0), (2, 1, 0),
                           {"gamma": 1.4}, 0.9),
    "log_entropy_euler1": ("log_entropy", "euler1", "neumann", (16, 1, 1), 2, (-5, 0, 0), (5, 1, 1),
                           {"gamma": 5.0 / 3.0}, 1.0),
    "log_entropy_euler3": ("log_entropy", "euler3", "periodic", (5, 4, 3), 2, (0, 0, 0), (1, 1, 1),
                           {"gamma": 1.4}, 1.0),
    "bv1_euler2": ("bv", "euler2", "periodic", (8, 7, 1), 2, (0, 0, 0), (1, 1, 0), {"degree": 1}, 1.0),
    "bv2_burgers1d": ("bv", "burgers", "periodic", (19, 1, 1), 2, (0, 0, 0), (1, 1, 1), {"degree": 2}, 0.5),
    "bv1_euler1": ("bv", "euler1", "neumann", (12, 1, 1), 3, (0, 0, 0), (1, 1, 1), {"degree": 1}, 1.0),
    "structure_cube_euler2": ("structure_cube", "euler2", "periodic", (8, 6, 1), 2, (0, 0, 0), (1, 1, 0),
                              {"p": 2.0, "number_of_h": 4}, 0.3),
}

# name: (equation, n, ghosts, direction, p)
BV_DIRECTION_CASES = {
    "euler2_x_p1": ("euler2", (8, 7, 1), 2, 0, 1),
    "euler2_y_p1": ("euler2", (8, 7, 1), 2, 1, 1),
    "euler3_z_p2": ("euler3", (5, 4, 3), 2, 2, 2),
    "burgers1d_x_p3": ("burgers", (15, 1, 1), 2, 0, 3),
}

# Axis structure functions (StructureBasic; tests/golden/structure_basic.npz)
# name: (equation, boundary, n, ghosts, number_of_h, p, direction)
STRUCTURE_BASIC_CASES = {
    "euler2_periodic_x_p2": ("euler2", "periodic", (12, 10, 1), 2, 5, 2.0, 0),
    "euler2_neumann_y_p1_5": ("euler2", "neumann", (9, 11, 1), 2, 6, 1.5, 1),
    "burgers1d_periodic_p3": ("burgers", "periodic", (20, 1, 1), 3, 7, 3.0, 0),
    "euler3_periodic_z_p2": ("euler3", "periodic", (5, 4, 6), 2, 4, 2.0, 2),
}
