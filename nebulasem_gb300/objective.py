"""The rising-bubble sensitivity problem: objective, its state gradient, and
the map from the initial potential-temperature perturbation to the state.

J = 1/2 sum over nodes inside x in [x0, x1], z in [z0, z1] of theta'^2 at the
final time, theta' = rho theta / rho - T0.  The control is the initial
theta' field; with p' = 0 initially (euler.cpp:136-149)
    rho = P0 / (R (theta' + T0)) (p_ref / P0)^(1/gamma),   rho theta = rho (theta' + T0),
so d rho / d theta' = -rho / (theta' + T0) and d(rho theta) / d theta' = 0.
"""
import numpy as np


def box_mask(xyz, box=(800.0, 1200.0, 1200.0, 1600.0)):
    x0, x1, z0, z1 = box
    x, z = xyz[:, 0], xyz[:, 2]
    return (x >= x0) & (x <= x1) & (z >= z0) & (z <= z1)


def objective(u, mask, T0=300.0):
    th = u[4] / u[0] - T0
    return 0.5 * float(np.sum(th[mask] ** 2))


def objective_grad(u, mask, T0=300.0):
    """dJ/du for the five conserved variables."""
    rho, rt = u[0], u[4]
    th = rt / rho - T0
    g = [np.zeros_like(rho) for _ in range(5)]
    g[4][mask] = th[mask] / rho[mask]
    g[0][mask] = -th[mask] * rt[mask] / rho[mask] ** 2
    return g


def state_from_theta(theta_p, p_ref, P0=1e5, T0=300.0, cp=1004.5, cv=717.5):
    R = cp - cv
    gam = cp / cv
    rho = (P0 / (R * (theta_p + T0))) * np.power(p_ref / P0, 1 / gam)
    z = np.zeros_like(rho)
    return [rho, z, z.copy(), z.copy(), rho * (theta_p + T0)]


def theta_grad(lam0, u0, theta_p, T0=300.0):
    """dJ/dtheta' from dJ/du0 (chain rule of state_from_theta)."""
    return lam0[0] * (-u0[0] / (theta_p + T0))
