"""Exact solution of the hydrodynamic shock tube -- TEST INFRASTRUCTURE ONLY.

A restatement of the reference's analytic overlay for its shock-tube model,
cans1d/md_shktb/hdmlw/shktb_analytic.pro (the same file ships with every
md_shktb scheme): the Riemann problem of an ideal gas at rest, high state 4
on the left (x < x0), low state 1 on the right, solved for the pressure
ratio across the shock p2/p1 from "Sawada's Note" eq. (8.274)
(shktb_analytic.pro:8-17), then the post-shock state, the contact, the
state behind the rarefaction and the fan itself (shktb_analytic.pro:40-113).

It is the known answer the tests hold the mLW step to with B = 0, where the
ideal-MHD step is the hydrodynamic one: the L1 error of the computed profile
against it, and its decrease under grid refinement.  Only tests/ and
bench.py's parity legs use it.
"""
from __future__ import annotations

import math

import numpy as np


def _f(x: float, gm: float, ro4: float, pr4: float, ro1: float, pr1: float) -> float:
    """shktb_analytic.pro:1-20: Sawada's eq. (8.274) as a function of
    x = p2/p1, zero at the solution."""
    cs1 = math.sqrt(gm * pr1 / ro1)
    cs4 = math.sqrt(gm * pr4 / ro4)
    cs14 = cs1 / cs4
    power = 2.0 * gm / (gm - 1.0)
    base = 1.0 - (gm - 1.0) / 2.0 * cs14 * (x - 1.0) * math.sqrt(
        2.0 / gm / ((gm + 1.0) * x + (gm - 1.0)))
    return base ** power - pr1 / pr4 * x


def pressure_ratio(gm: float, ro4: float, pr4: float, ro1: float, pr1: float) -> float:
    """p2/p1, the root of eq. (8.274) between 1 (no shock) and the ratio at
    which the rarefaction empties the left state.  The reference finds it
    with IDL's newton() from 2 to 1e-8 (shktb_analytic.pro:23-24,45); here
    bisection runs to the last bit, since the root is the reference value
    of the whole solution."""
    def g(x):
        b = 1.0 - (gm - 1.0) / 2.0 * (math.sqrt(gm * pr1 / ro1) / math.sqrt(gm * pr4 / ro4)) \
            * (x - 1.0) * math.sqrt(2.0 / gm / ((gm + 1.0) * x + (gm - 1.0)))
        if b <= 0.0:  # past the vacuum limit: the left state is exhausted
            return -pr1 / pr4 * x
        return _f(x, gm, ro4, pr4, ro1, pr1)

    lo, hi = 1.0, 2.0
    if g(lo) <= 0.0:
        raise ValueError("no shock: the left pressure does not exceed the right")
    while g(hi) > 0.0:
        lo, hi = hi, 2.0 * hi
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if mid <= lo or mid >= hi:
            break
        if g(mid) > 0.0:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def solution(x: np.ndarray, t: float, x0: float, gm: float, ro1: float, pr1: float,
             ro4: float = 1.0, pr4: float = 1.0):
    """shktb_analytic.pro:26-137: (ro, pr, vx) of the exact solution at the
    positions x and time t > 0, the interface at x0 at t = 0.  Returns the
    arrays and a dict of the wave positions and plateau states."""
    u1 = u4 = 0.0
    cs1 = math.sqrt(gm * pr1 / ro1)
    cs4 = math.sqrt(gm * pr4 / ro4)
    pr21 = pressure_ratio(gm, ro4, pr4, ro1, pr1)
    # shock (shktb_analytic.pro:48-50)
    us = cs1 * math.sqrt(((gm - 1.0) + (gm + 1.0) * pr21) / (2.0 * gm))
    xs = x0 + us * t
    # behind the shock (:55-58)
    u2 = cs1 * (pr21 - 1.0) * math.sqrt((2.0 / gm) / ((gm + 1.0) * pr21 + (gm - 1.0)))
    ro2 = ro1 * us / (us - u2)
    pr2 = pr21 * pr1
    # contact (:64-65)
    uc = u2
    xc = x0 + uc * t
    # behind the expansion fan (:71-74): isentropic from the left state
    u3, pr3 = u2, pr2
    ro3 = ro4 * (pr3 / pr4) ** (1.0 / gm)
    cs3 = math.sqrt(gm * pr3 / ro3)
    # the fan (:80-99); the reference writes rofan = (csfan^2/gm)^(1/(gm-1)),
    # the isentrope through (ro4, pr4) = (1, 1); the general form is used here
    xhead = x0 + (u4 - cs4) * t
    xtail = x0 + (u3 - cs3) * t
    x = np.asarray(x, dtype=np.float64)
    ro = np.empty_like(x)
    pr = np.empty_like(x)
    vx = np.empty_like(x)
    fan = (x > xhead) & (x < xtail)
    phi = (x[fan] - x0) / t
    csfan = (gm - 1.0) / (gm + 1.0) * (2.0 * cs4 / (gm - 1.0) - phi)
    rofan = ro4 * (csfan / cs4) ** (2.0 / (gm - 1.0))
    ro[fan] = rofan
    pr[fan] = pr4 * (rofan / ro4) ** gm
    vx[fan] = csfan + phi
    # plateaus, in the reference's order of assignment (:103-134)
    for sel, (r, p, u) in (((x <= xhead), (ro4, pr4, u4)),
                           ((x >= xtail) & (x <= xc), (ro3, pr3, u3)),
                           ((x >= xc) & (x <= xs), (ro2, pr2, u2)),
                           ((x >= xs), (ro1, pr1, u1))):
        ro[sel], pr[sel], vx[sel] = r, p, u
    waves = {"pr21": pr21, "x_shock": xs, "x_contact": xc, "x_fan_head": xhead,
             "x_fan_tail": xtail, "ro2": ro2, "pr2": pr2, "u2": u2, "ro3": ro3}
    return ro, pr, vx, waves


def l1_errors(x: np.ndarray, dx: np.ndarray, ro, pr, vx, t: float, x0: float, gm: float,
              ro1: float, pr1: float, ro4: float = 1.0, pr4: float = 1.0) -> dict:
    """Cell-weighted L1 distance sum |q - q_exact(x_i)| dx_i of each profile
    from the exact solution at the cell centres."""
    er, ep, ev, _ = solution(x, t, x0, gm, ro1, pr1, ro4, pr4)
    return {"ro": float(np.sum(np.abs(ro - er) * dx)), "pr": float(np.sum(np.abs(pr - ep) * dx)),
            "vx": float(np.sum(np.abs(vx - ev) * dx))}


def observed_order(ns, errs) -> float:
    """Least-squares slope of -log(err) against log(n)."""
    a = np.log(np.asarray(ns, dtype=np.float64))
    b = -np.log(np.asarray(errs, dtype=np.float64))
    return float(np.polyfit(a, b, 1)[0])
