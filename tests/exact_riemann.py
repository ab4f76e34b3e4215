"""Exact solution of the ideal-gas Riemann problem (Toro, "Riemann Solvers
and Numerical Methods for Fluid Dynamics", ch. 4), used as an independent
check of the Sod configuration."""
import math

import numpy as np


def _f(p, rho, pk, a, g):
    if p > pk:
        A = 2.0 / ((g + 1.0) * rho)
        B = (g - 1.0) / (g + 1.0) * pk
        return (p - pk) * math.sqrt(A / (p + B))
    return 2.0 * a / (g - 1.0) * ((p / pk) ** ((g - 1.0) / (2.0 * g)) - 1.0)


def star_state(rl, ul, pl, rr, ur, pr, g=1.4):
    al, ar = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    lo, hi = 1e-12, 10.0 * max(pl, pr)
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if _f(mid, rl, pl, al, g) + _f(mid, rr, pr, ar, g) + ur - ul > 0.0:
            hi = mid
        else:
            lo = mid
    p = 0.5 * (lo + hi)
    u = 0.5 * (ul + ur) + 0.5 * (_f(p, rr, pr, ar, g) - _f(p, rl, pl, al, g))
    return p, u


def sample(x, t, x0, rl, ul, pl, rr, ur, pr, g=1.4):
    """Density, velocity, pressure at positions x and time t (left rarefaction /
    right shock branch, as in Sod's problem)."""
    p, u = star_state(rl, ul, pl, rr, ur, pr, g)
    al = math.sqrt(g * pl / rl)
    rho = np.empty_like(x)
    vel = np.empty_like(x)
    pre = np.empty_like(x)
    s = (x - x0) / t
    rls = rl * (p / pl) ** (1.0 / g)
    als = al * (p / pl) ** ((g - 1.0) / (2.0 * g))
    shl, stl = ul - al, u - als
    rrs = rr * ((p / pr + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * p / pr + 1.0))
    ar = math.sqrt(g * pr / rr)
    sr = ur + ar * math.sqrt((g + 1) / (2 * g) * p / pr + (g - 1) / (2 * g))
    for i, si in enumerate(s):
        if si < shl:
            rho[i], vel[i], pre[i] = rl, ul, pl
        elif si < stl:
            c = 2.0 / (g + 1) + (g - 1) / ((g + 1) * al) * (ul - si)
            rho[i] = rl * c ** (2.0 / (g - 1))
            vel[i] = 2.0 / (g + 1) * (al + (g - 1) / 2 * ul + si)
            pre[i] = pl * c ** (2 * g / (g - 1))
        elif si < u:
            rho[i], vel[i], pre[i] = rls, u, p
        elif si < sr:
            rho[i], vel[i], pre[i] = rrs, u, p
        else:
            rho[i], vel[i], pre[i] = rr, ur, pr
    return rho, vel, pre
