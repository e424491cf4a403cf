"""Exact solution of the 1D Euler Riemann problem for an ideal gas (Toro 2009, chapter 4):
Newton iteration for the star pressure, then sampling of the self-similar solution."""
from __future__ import annotations

import math

import numpy as np


def _f(p, dk, pk, ck, g):
    if p > pk:  # shock
        A = 2.0 / ((g + 1.0) * dk)
        B = (g - 1.0) / (g + 1.0) * pk
        q = math.sqrt(A / (p + B))
        return (p - pk) * q, q * (1.0 - 0.5 * (p - pk) / (B + p))
    pr = p / pk  # rarefaction
    return 2.0 * ck / (g - 1.0) * (pr ** ((g - 1.0) / (2.0 * g)) - 1.0), 1.0 / (dk * ck) * pr ** (-(g + 1.0) / (2.0 * g))


def star_state(dl, ul, pl, dr, ur, pr, g):
    cl, cr = math.sqrt(g * pl / dl), math.sqrt(g * pr / dr)
    p = max(1e-8, 0.5 * (pl + pr))
    for _ in range(100):
        fl, dfl = _f(p, dl, pl, cl, g)
        fr, dfr = _f(p, dr, pr, cr, g)
        dp = (fl + fr + ur - ul) / (dfl + dfr)
        p_new = max(1e-12, p - dp)
        if abs(p_new - p) < 1e-14 * (p_new + p):
            p = p_new
            break
        p = p_new
    fl, _ = _f(p, dl, pl, cl, g)
    fr, _ = _f(p, dr, pr, cr, g)
    return p, 0.5 * (ul + ur) + 0.5 * (fr - fl)


def sod_exact(x, t, gamma=1.4, left=(1.0, 0.0, 1.0), right=(0.125, 0.0, 0.1), x0=0.5):
    """Return (rho, u, p) at positions x and time t."""
    g = gamma
    dl, ul, pl = left
    dr, ur, pr = right
    ps, us = star_state(dl, ul, pl, dr, ur, pr, g)
    cl, cr = math.sqrt(g * pl / dl), math.sqrt(g * pr / dr)
    rho = np.empty_like(x)
    u = np.empty_like(x)
    p = np.empty_like(x)
    for i, xi in enumerate(x):
        s = (xi - x0) / t
        if s <= us:  # left of contact
            if ps > pl:  # left shock
                sl = ul - cl * math.sqrt((g + 1) / (2 * g) * ps / pl + (g - 1) / (2 * g))
                if s <= sl:
                    rho[i], u[i], p[i] = dl, ul, pl
                else:
                    rho[i] = dl * ((ps / pl + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pl + 1))
                    u[i], p[i] = us, ps
            else:  # left rarefaction
                shl = ul - cl
                cls = cl * (ps / pl) ** ((g - 1) / (2 * g))
                stl = us - cls
                if s <= shl:
                    rho[i], u[i], p[i] = dl, ul, pl
                elif s >= stl:
                    rho[i] = dl * (ps / pl) ** (1 / g)
                    u[i], p[i] = us, ps
                else:
                    c = 2 / (g + 1) * (cl + (g - 1) / 2 * (ul - s))
                    u[i] = 2 / (g + 1) * (cl + (g - 1) / 2 * ul + s)
                    rho[i] = dl * (c / cl) ** (2 / (g - 1))
                    p[i] = pl * (c / cl) ** (2 * g / (g - 1))
        else:  # right of contact
            if ps > pr:  # right shock
                sr = ur + cr * math.sqrt((g + 1) / (2 * g) * ps / pr + (g - 1) / (2 * g))
                if s >= sr:
                    rho[i], u[i], p[i] = dr, ur, pr
                else:
                    rho[i] = dr * ((ps / pr + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pr + 1))
                    u[i], p[i] = us, ps
            else:  # right rarefaction
                shr = ur + cr
                crs = cr * (ps / pr) ** ((g - 1) / (2 * g))
                str_ = us + crs
                if s >= shr:
                    rho[i], u[i], p[i] = dr, ur, pr
                elif s <= str_:
                    rho[i] = dr * (ps / pr) ** (1 / g)
                    u[i], p[i] = us, ps
                else:
                    c = 2 / (g + 1) * (cr - (g - 1) / 2 * (ur - s))
                    u[i] = 2 / (g + 1) * (-cr + (g - 1) / 2 * ur + s)
                    rho[i] = dr * (c / cr) ** (2 / (g - 1))
                    p[i] = pr * (c / cr) ** (2 * g / (g - 1))
    return rho, u, p
