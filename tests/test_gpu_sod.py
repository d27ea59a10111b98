"""The device mLW loops against the reference's known answer: the exact
hydrodynamic shock-tube solution of cans1d/md_shktb/hdmlw/
shktb_analytic.pro (oracle/shktb_analytic.py), run to its tend = 0.14154
with B = 0 in 1-D (mlw_m), 2-D (mlw_m3, an x-aligned tube) and 3-D (mlw_m).
The fast policy is held to the exact answer (L1 distance and its order under
refinement up to 2048 cells) and to the oracle's own distance; the exact
policy equals the oracle bit for bit over the whole run."""
import numpy as np
import pytest

import oracle
from oracle import shktb_analytic as an
from utrip_gb300 import capi, drivers, setups

pytestmark = pytest.mark.gpu

NS = (256, 512, 1024, 2048)
# the oracle's L1 at 2048 cells (rho 7.4e-4 / 8.1e-4, p 3.0e-4 / 3.1e-4,
# vx 7.1e-4 / 6.7e-4 in 1-D / 2-D and 3-D), with 20-30 % room; its orders
# over 256..2048 are 0.70-0.74 (rho), 0.94-0.99 (p) and 0.87-0.99 (vx)
L1_2048 = {"ro": 1.0e-3, "pr": 3.8e-4, "vx": 8.5e-4}
MIN_ORDER = {"ro": 0.65, "pr": 0.85, "vx": 0.8}
RUN = {1: "run_1d", 2: "run_2d", 3: "run_3d"}


def l1(s, st, t):
    x, dx, ro, pr, vx = setups.sod_interior_profile(s, st)
    sd = s["sod"]
    return an.l1_errors(x, dx, ro, pr, vx, t, sd["x0"], sd["gm"], sd["ro1"], sd["pr1"])


@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_device_converges_to_exact_shock_tube(gpu, oracle_lib, ndim):
    errs = []
    for n in NS:
        s = setups.sod_shock_tube(n, ndim)
        got = setups.copy_state(s)
        t, ns, merr, nexec = drivers.run_resident(s, got, 10 ** 6, exact=False)
        assert merr == 0 and t >= s["tend"] and nexec == ns
        e = l1(s, got, t)
        errs.append(e)
        if n <= 1024:  # the oracle's own distance, same set-up and loop
            ref = setups.copy_state(s)
            t_ref, ns_ref, _, _ = getattr(oracle, RUN[ndim])(s, ref, 10 ** 6)
            assert ns == ns_ref and t == pytest.approx(t_ref, rel=1e-12)
            er = l1(s, ref, t_ref)
            for k in e:
                assert e[k] == pytest.approx(er[k], rel=1e-6), (n, k, e[k], er[k])
    for k in ("ro", "pr", "vx"):
        e = [d[k] for d in errs]
        assert e[-1] <= L1_2048[k], (k, e)
        assert an.observed_order(NS, e) >= MIN_ORDER[k], (k, e)


@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_exact_policy_equals_oracle_to_tend(gpu, oracle_lib, ndim):
    s = setups.sod_shock_tube(256, ndim)
    ref = setups.copy_state(s)
    t_ref, ns_ref, _, _ = getattr(oracle, RUN[ndim])(s, ref, 10 ** 6)
    got = setups.copy_state(s)
    t, ns, merr, _ = drivers.run_resident(s, got, 10 ** 6, exact=True)
    assert (t, ns, merr) == (t_ref, ns_ref, 0)
    for k, a, b in zip(s["names"], got, ref):
        assert np.array_equal(a, b), k


# ---- the Riemann-solver steps on the same known answer -------------------------
# Roe-MUSCL (1-D roe_m, 2-D roe_m3, 3-D roe_m) and HLLD (the engine along x)
# with B = 0 and three ghost layers (setups.sod_shock_tube_riemann).  The
# oracle's L1 at 2048 cells is 5.9-6.0e-4 (rho), 3.1-3.2e-4 (p) and
# 7.3-7.8e-4 (vx), held here with 25 % room; its orders over 256..2048 are
# 0.82-0.84, 0.98-0.99 and 0.96-0.99.
RIEMANN_L1_2048 = {"ro": 7.5e-4, "pr": 4.0e-4, "vx": 9.7e-4}
RIEMANN_MIN_ORDER = {"ro": 0.75, "pr": 0.9, "vx": 0.9}
RIEMANN_RUN = {"roe_m_1d": "run_1d", "roe_m3": "run_2d", "roe_m_3d": "run_3d",
               "hlld_3d": "run_3d"}


def run_device(s, st, exact=False, df64=False):
    """The package loop to tend on the device: the 1-D Roe step through the
    drop-in calls on registered arrays (it has no run handle), the others
    through the run handle."""
    if s["solver"] == "roe_m_1d":
        assert not df64
        capi.set_exact(exact)
        try:
            t, ns, merr, _ = drivers.run_literal(s, st, 10 ** 6, resident=True)
        finally:
            capi.set_exact(False)
        return t, ns, merr
    t, ns, merr, nexec = drivers.run_resident(s, st, 10 ** 6, exact=exact, df64=df64)
    assert nexec == ns
    return t, ns, merr


@pytest.mark.parametrize("solver", ["roe_m_1d", "roe_m3", "roe_m_3d", "hlld_3d"])
def test_device_riemann_solvers_converge_to_exact_shock_tube(gpu, oracle_lib, solver):
    errs = []
    for n in NS:
        s = setups.sod_shock_tube_riemann(n, solver)
        got = setups.copy_state(s)
        t, ns, merr = run_device(s, got)
        assert merr == 0 and t >= s["tend"]
        e = l1(s, got, t)
        errs.append(e)
        if n <= 512:  # the oracle's own distance, same set-up and loop
            ref = setups.copy_state(s)
            t_ref, ns_ref, _, _ = getattr(oracle, RIEMANN_RUN[solver])(s, ref, 10 ** 6)
            assert ns == ns_ref and t == pytest.approx(t_ref, rel=1e-12)
            er = l1(s, ref, t_ref)
            for k in e:
                assert e[k] == pytest.approx(er[k], rel=1e-6), (n, k, e[k], er[k])
    for k in ("ro", "pr", "vx"):
        e = [d[k] for d in errs]
        assert e[-1] <= RIEMANN_L1_2048[k], (k, e)
        assert an.observed_order(NS, e) >= RIEMANN_MIN_ORDER[k], (k, e)


@pytest.mark.parametrize("solver", ["roe_m_1d", "roe_m3", "roe_m_3d", "hlld_3d"])
def test_riemann_exact_policy_equals_oracle_to_tend(gpu, oracle_lib, solver):
    s = setups.sod_shock_tube_riemann(256, solver)
    ref = setups.copy_state(s)
    t_ref, ns_ref, _, _ = getattr(oracle, RIEMANN_RUN[solver])(s, ref, 10 ** 6)
    got = setups.copy_state(s)
    t, ns, merr = run_device(s, got, exact=True)
    assert (t, ns, merr) == (t_ref, ns_ref, 0)
    for k, a, b in zip(s["names"], got, ref):
        assert np.array_equal(a, b), k


@pytest.mark.parametrize("solver", ["roe_m3", "roe_m_3d", "hlld_3d"])
def test_double_float_riemann_steps_on_the_exact_shock_tube(gpu, solver):
    """The double-float face fluxes reach the same distance from the exact
    answer as the FP64 fast policy (within 1e-6 of it) at 1024 cells."""
    s = setups.sod_shock_tube_riemann(1024, solver)
    res = {}
    for df in (False, True):
        st = setups.copy_state(s)
        t, ns, merr = run_device(s, st, df64=df)
        assert merr == 0 and t >= s["tend"]
        res[df] = (ns, l1(s, st, t))
    assert res[True][0] == res[False][0]
    for k in ("ro", "pr", "vx"):
        assert res[True][1][k] == pytest.approx(res[False][1][k], rel=1e-6), k


@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_double_float_mlw_steps_on_the_exact_shock_tube(gpu, ndim):
    """The double-float mLW loops (1-D mlw_m, 2-D mlw_m3, 3-D mlw_m) take the
    FP64 fast policy's steps and reach its distance from the exact answer
    (within 1e-6 of it) at 1024 cells."""
    s = setups.sod_shock_tube(1024, ndim)
    res = {}
    for df in (False, True):
        st = setups.copy_state(s)
        t, ns, merr, nexec = drivers.run_resident(s, st, 10 ** 6, df64=df)
        assert merr == 0 and t >= s["tend"] and nexec == ns
        res[df] = (ns, l1(s, st, t))
    assert res[True][0] == res[False][0]
    for k in ("ro", "pr", "vx"):
        assert res[True][1][k] == pytest.approx(res[False][1][k], rel=1e-6), k
