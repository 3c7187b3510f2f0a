"""Exact solution of the 1D Euler Riemann problem (test infrastructure).

Restates the exact solver of Toro, "Riemann Solvers and Numerical Methods
for Fluid Dynamics", 3rd ed., ch. 4: pressure function f_K (4.6-4.7), Newton
iteration for the star pressure (4.44), star velocity (4.9), and sampling of
the self-similar solution at x/t (4.4-4.5 shock/rarefaction structure).  Used
as the secondary check of the Sod-tube runs.
"""
import math

import numpy as np


def _fk(p, rho, pk, ak, g):
    if p > pk:  # shock
        A = 2.0 / ((g + 1.0) * rho)
        B = (g - 1.0) / (g + 1.0) * pk
        q = math.sqrt(A / (p + B))
        return (p - pk) * q, q * (1.0 - 0.5 * (p - pk) / (B + p))
    # rarefaction
    f = 2.0 * ak / (g - 1.0) * ((p / pk) ** ((g - 1.0) / (2.0 * g)) - 1.0)
    df = (p / pk) ** (-(g + 1.0) / (2.0 * g)) / (rho * ak)
    return f, df


def star_state(WL, WR, g=1.4):
    rl, ul, pl = WL
    rr, ur, pr = WR
    al, ar = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    p = max(1e-12, 0.5 * (pl + pr) - 0.125 * (ur - ul) * (rl + rr) * (al + ar))
    for _ in range(100):
        fl, dfl = _fk(p, rl, pl, al, g)
        fr, dfr = _fk(p, rr, pr, ar, g)
        dp = (fl + fr + ur - ul) / (dfl + dfr)
        pn = max(1e-14, p - dp)
        if abs(pn - p) < 1e-15 * (pn + p):
            p = pn
            break
        p = pn
    fl, _ = _fk(p, rl, pl, al, g)
    fr, _ = _fk(p, rr, pr, ar, g)
    return p, 0.5 * (ul + ur) + 0.5 * (fr - fl)


def sample(WL, WR, xi, g=1.4):
    """(rho, u, p) at the similarity coordinates xi = (x - x0) / t."""
    rl, ul, pl = WL
    rr, ur, pr = WR
    al, ar = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    ps, us = star_state(WL, WR, g)
    out = np.empty((len(xi), 3))
    for n, s in enumerate(np.asarray(xi, dtype=float)):
        if s <= us:  # left of the contact
            if ps > pl:
                sl = ul - al * math.sqrt((g + 1) / (2 * g) * ps / pl + (g - 1) / (2 * g))
                if s <= sl:
                    out[n] = (rl, ul, pl)
                else:
                    r = rl * ((ps / pl + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pl + 1))
                    out[n] = (r, us, ps)
            else:
                shl = ul - al
                asl = al * (ps / pl) ** ((g - 1) / (2 * g))
                stl = us - asl
                if s <= shl:
                    out[n] = (rl, ul, pl)
                elif s >= stl:
                    out[n] = (rl * (ps / pl) ** (1 / g), us, ps)
                else:
                    c = 2 / (g + 1) + (g - 1) / ((g + 1) * al) * (ul - s)
                    out[n] = (rl * c ** (2 / (g - 1)), 2 / (g + 1) * (al + (g - 1) / 2 * ul + s),
                              pl * c ** (2 * g / (g - 1)))
        else:  # right of the contact
            if ps > pr:
                sr = ur + ar * math.sqrt((g + 1) / (2 * g) * ps / pr + (g - 1) / (2 * g))
                if s >= sr:
                    out[n] = (rr, ur, pr)
                else:
                    r = rr * ((ps / pr + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pr + 1))
                    out[n] = (r, us, ps)
            else:
                shr = ur + ar
                asr = ar * (ps / pr) ** ((g - 1) / (2 * g))
                str_ = us + asr
                if s >= shr:
                    out[n] = (rr, ur, pr)
                elif s <= str_:
                    out[n] = (rr * (ps / pr) ** (1 / g), us, ps)
                else:
                    c = 2 / (g + 1) - (g - 1) / ((g + 1) * ar) * (ur - s)
                    out[n] = (rr * c ** (2 / (g - 1)), 2 / (g + 1) * (-ar + (g - 1) / 2 * ur + s),
                              pr * c ** (2 * g / (g - 1)))
    return out
