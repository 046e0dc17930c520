"""Exact solution of the 1-D Riemann problem for an ideal gas.

The classical exact solver (pressure function with Newton iteration for the
star pressure, then sampling of the self-similar solution), as published in
E. F. Toro, "Riemann Solvers and Numerical Methods for Fluid Dynamics",
chapter 4.  Used as a known answer for the Sod shock tube.
"""
import math

import numpy as np


def _f(p, rho, pk, ck, g):
    if p > pk:  # shock
        A = 2.0 / ((g + 1.0) * rho)
        B = (g - 1.0) / (g + 1.0) * pk
        q = math.sqrt(A / (p + B))
        return (p - pk) * q, q * (1.0 - 0.5 * (p - pk) / (B + p))
    # rarefaction
    r = (p / pk) ** ((g - 1.0) / (2.0 * g))
    return 2.0 * ck / (g - 1.0) * (r - 1.0), 1.0 / (rho * ck) * (p / pk) ** (-(g + 1.0) / (2.0 * g))


def star_state(rl, ul, pl, rr, ur, pr, g):
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    p = max(1e-10, 0.5 * (pl + pr))
    for _ in range(100):
        fl, dl = _f(p, rl, pl, cl, g)
        fr, dr = _f(p, rr, pr, cr, g)
        dp = (fl + fr + ur - ul) / (dl + dr)
        p_new = max(1e-12, p - dp)
        if abs(p_new - p) < 1e-14 * p:
            p = p_new
            break
        p = p_new
    fl, _ = _f(p, rl, pl, cl, g)
    fr, _ = _f(p, rr, pr, cr, g)
    u = 0.5 * (ul + ur) + 0.5 * (fr - fl)
    return p, u


def sample(x, t, x0, left, right, g):
    """Density, velocity and pressure at positions x and time t."""
    rl, ul, pl = left
    rr, ur, pr = right
    ps, us = star_state(rl, ul, pl, rr, ur, pr, g)
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    out = np.zeros((3, len(x)))
    for i, xi in enumerate(x):
        s = (xi - x0) / t
        if s <= us:  # left of contact
            if ps > pl:
                sl = ul - cl * math.sqrt((g + 1) / (2 * g) * ps / pl + (g - 1) / (2 * g))
                if s <= sl:
                    w = (rl, ul, pl)
                else:
                    r = rl * ((ps / pl + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pl + 1))
                    w = (r, us, ps)
            else:
                shl = ul - cl
                cml = cl * (ps / pl) ** ((g - 1) / (2 * g))
                stl = us - cml
                if s <= shl:
                    w = (rl, ul, pl)
                elif s > stl:
                    w = (rl * (ps / pl) ** (1 / g), us, ps)
                else:
                    u = 2 / (g + 1) * (cl + (g - 1) / 2 * ul + s)
                    c = 2 / (g + 1) * (cl + (g - 1) / 2 * (ul - s))
                    r = rl * (c / cl) ** (2 / (g - 1))
                    w = (r, u, pl * (c / cl) ** (2 * g / (g - 1)))
        else:
            if ps > pr:
                sr = ur + cr * math.sqrt((g + 1) / (2 * g) * ps / pr + (g - 1) / (2 * g))
                if s >= sr:
                    w = (rr, ur, pr)
                else:
                    r = rr * ((ps / pr + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pr + 1))
                    w = (r, us, ps)
            else:
                shr = ur + cr
                cmr = cr * (ps / pr) ** ((g - 1) / (2 * g))
                str_ = us + cmr
                if s >= shr:
                    w = (rr, ur, pr)
                elif s <= str_:
                    w = (rr * (ps / pr) ** (1 / g), us, ps)
                else:
                    u = 2 / (g + 1) * (-cr + (g - 1) / 2 * ur + s)
                    c = 2 / (g + 1) * (cr - (g - 1) / 2 * (ur - s))
                    r = rr * (c / cr) ** (2 / (g - 1))
                    w = (r, u, pr * (c / cr) ** (2 * g / (g - 1)))
        out[:, i] = w
    return out
