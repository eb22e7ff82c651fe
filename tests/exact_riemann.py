"""Exact solution of the 1D Riemann problem for an ideal gas (Toro, "Riemann Solvers and
Numerical Methods for Fluid Dynamics", ch. 4: pressure function + Newton iteration, then
self-similar sampling).  Test helper for the Sod configuration at an arbitrary final time.
"""
import numpy as np


def _f(p, rho, pk, ck, g):
    if p > pk:   # shock
        A = 2.0 / ((g + 1.0) * rho)
        B = (g - 1.0) / (g + 1.0) * pk
        f = (p - pk) * np.sqrt(A / (p + B))
        df = np.sqrt(A / (B + p)) * (1.0 - (p - pk) / (2.0 * (B + p)))
    else:        # rarefaction
        f = 2.0 * ck / (g - 1.0) * ((p / pk) ** ((g - 1.0) / (2.0 * g)) - 1.0)
        df = 1.0 / (rho * ck) * (p / pk) ** (-(g + 1.0) / (2.0 * g))
    return f, df


def star_state(rl, ul, pl, rr, ur, pr, g):
    cl, cr = np.sqrt(g * pl / rl), np.sqrt(g * pr / rr)
    p = max(1e-8, 0.5 * (pl + pr))
    for _ in range(100):
        fl, dfl = _f(p, rl, pl, cl, g)
        fr, dfr = _f(p, rr, pr, cr, g)
        pn = p - (fl + fr + ur - ul) / (dfl + dfr)
        pn = max(pn, 1e-12)
        if abs(pn - p) / (0.5 * (pn + p)) < 1e-14:
            p = pn
            break
        p = pn
    fl, _ = _f(p, rl, pl, cl, g)
    fr, _ = _f(p, rr, pr, cr, g)
    u = 0.5 * (ul + ur) + 0.5 * (fr - fl)
    return p, u


def sample(x, t, x0, rl, ul, pl, rr, ur, pr, g):
    """rho, u, p at positions x (array) and time t for an interface at x0."""
    ps, us = star_state(rl, ul, pl, rr, ur, pr, g)
    cl, cr = np.sqrt(g * pl / rl), np.sqrt(g * pr / rr)
    out = np.zeros((3, len(x)))
    for i, xi in enumerate(x):
        s = (xi - x0) / t
        if s <= us:   # left of contact
            if ps > pl:   # left shock
                sl = ul - cl * np.sqrt((g + 1) / (2 * g) * ps / pl + (g - 1) / (2 * g))
                if s <= sl:
                    r, u, p = rl, ul, pl
                else:
                    r = rl * ((ps / pl + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pl + 1))
                    u, p = us, ps
            else:         # left rarefaction
                shl = ul - cl
                csl = cl * (ps / pl) ** ((g - 1) / (2 * g))
                stl = us - csl
                if s <= shl:
                    r, u, p = rl, ul, pl
                elif s >= stl:
                    r, u, p = rl * (ps / pl) ** (1 / g), us, ps
                else:
                    u = 2 / (g + 1) * (cl + (g - 1) / 2 * ul + s)
                    c = 2 / (g + 1) * (cl + (g - 1) / 2 * (ul - s))
                    r = rl * (c / cl) ** (2 / (g - 1))
                    p = pl * (c / cl) ** (2 * g / (g - 1))
        else:         # right of contact
            if ps > pr:   # right shock
                sr = ur + cr * np.sqrt((g + 1) / (2 * g) * ps / pr + (g - 1) / (2 * g))
                if s >= sr:
                    r, u, p = rr, ur, pr
                else:
                    r = rr * ((ps / pr + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pr + 1))
                    u, p = us, ps
            else:
                shr = ur + cr
                csr = cr * (ps / pr) ** ((g - 1) / (2 * g))
                str_ = us + csr
                if s >= shr:
                    r, u, p = rr, ur, pr
                elif s <= str_:
                    r, u, p = rr * (ps / pr) ** (1 / g), us, ps
                else:
                    u = 2 / (g + 1) * (-cr + (g - 1) / 2 * ur + s)
                    c = 2 / (g + 1) * (cr - (g - 1) / 2 * (ur - s))
                    r = rr * (c / cr) ** (2 / (g - 1))
                    p = pr * (c / cr) ** (2 * g / (g - 1))
        out[:, i] = (r, u, p)
    return out
