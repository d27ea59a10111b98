"""The double-float policy of the 1-D loop (cans_run_set_df64 on MLW_M_1D and
MLW_M_BG_1D runs: the step's arithmetic as pairs of floats on the FP32 pipes,
the state in FP64) against the oracle's reference arithmetic.  Shock tubes
and a periodic state stay within 1e-10 (relative L-inf per variable) to the
end of their runs.  The spicule model stays within the fast policy's own
bounds (1e-10; vx 1e-4, the quantity its corona amplifies): the static B_x
terms of mlw_m_bg's energy and x-momentum, B_x^2/8pi many orders above the
corona's gas pressure, are carried in FP64 and never meet the 48-bit
significand.  A group of double-float runs ends where the runs end alone."""
import numpy as np
import pytest

import oracle
from utrip_gb300 import capi, drivers, setups

pytestmark = pytest.mark.gpu
TOL = 1e-10


def rel_linf(a, b):
    scale = float(np.max(np.abs(b))) or 1.0
    return float(np.max(np.abs(a - b))) / scale


def loop_df64(s, nstop, tend=None):
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, nstop, tend=tend, df64=True,
                                              chunk=100000)
    return got, (t, ns, merr, nexec)


@pytest.mark.parametrize("nstop", [100, 10 ** 6])
def test_shock_tube(gpu, oracle_lib, nstop):
    """1024 cells, 100 steps and the whole run to t = 0.1 (996 steps)."""
    s = setups.shock_tube_1d(1024)
    ref = setups.copy_state(s)
    t_ref, ns_ref, _, _ = oracle.run_1d(s, ref, nstop)
    got, (t, ns, merr, nexec) = loop_df64(s, nstop)
    assert merr == 0 and ns == ns_ref and t == pytest.approx(t_ref, rel=1e-12)
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) <= TOL, (k, rel_linf(a, b))


def test_periodic_state(gpu, oracle_lib):
    s = setups.random_state_1d(301, seed=5)
    ref = setups.copy_state(s)
    oracle.run_1d(s, ref, 40)
    got, (t, ns, merr, nexec) = loop_df64(s, 40)
    assert ns == 40
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) <= TOL, (k, rel_linf(a, b))


def spicule_loop(s, nstop):
    run = drivers.make_run(s, exact=False, df64=True)
    try:
        run.push(setups.copy_state(s))
        run.start(tend=s["tend"], nstop=nstop, safety=s["safety"], dtmin=s["dtmin"])
        run.advance(nstop)
        return run.pull(), run.query()
    finally:
        run.close()


@pytest.mark.parametrize("nsteps", [100, 1000])
def test_spicule_loop(gpu, oracle_lib, nsteps):
    """The spicule model (torque and floor on) at the fast policy's bounds."""
    s = setups.spicule_1d(1024, seed=1)
    ref = setups.copy_state(s)
    oracle.run_spicule_c(s, ref, nsteps)
    got, st = spicule_loop(s, nsteps)
    assert st.ns == nsteps and st.merr == 0
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) < (1e-4 if k == "vx" else TOL), (k, rel_linf(a, b))


def test_spicule_loop_every_source_term(gpu, oracle_lib):
    """A varying distance from the axis (every rotation term of mlw_m_bg non-zero)
    and a perturbed state with flows and twist, 200 steps."""
    s = setups.spicule_1d(1024)
    rng = np.random.default_rng(9)
    xs = (s["x"] - s["x"][0]) / (s["x"][-1] - s["x"][0])
    s["rr"] = 1.0 + 0.2 * np.sin(2 * np.pi * xs + 0.3)
    s["rrm"] = 1.0 + 0.2 * np.sin(2 * np.pi * (xs + 0.5 / xs.size) + 0.3)
    s["drr"], s["drrm"] = setups.scrdy(s["rr"], s["rrm"], s["dx"], s["dxm"])
    ro, pr, vx, vy, by = s["state"]
    n = xs.size
    s["state"] = [ro * (1 + 0.05 * rng.standard_normal(n)), pr * (1 + 0.05 * rng.standard_normal(n)),
                  0.05 * rng.standard_normal(n), 0.05 * rng.standard_normal(n),
                  0.1 * rng.standard_normal(n)]
    ref = setups.copy_state(s)
    oracle.run_spicule_c(s, ref, 200)
    got, st = spicule_loop(s, 200)
    assert st.ns == 200 and st.merr == 0
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) < (1e-4 if k == "vx" else 1e-9), (k, rel_linf(a, b))


def test_mhd_wind_loop(gpu, oracle_lib):
    """cans1d/md_mhdwind on its stretched grid: the cross-section (0.7 to
    1.1e4), B_x and the radius vary, and the gas pressure falls to 6e-6 of
    B_x^2/8pi, so every static field term of the double-float mlw_m_bg is in
    play.  200 iterations: 1e-10, vx 1e-6 (the fast policy ends 1.9e-8 from
    the oracle in vx there; over longer runs this wind amplifies any
    rounding, and only the exact policy stays on the oracle's trajectory)."""
    s = setups.mhd_wind_1d(1024)
    ref = setups.copy_state(s)
    t_ref, ns_ref, _, _ = oracle.run_1d(s, ref, 200)
    got, (t, ns, merr, nexec) = loop_df64(s, 200)
    assert merr == 0 and ns == ns_ref and t == pytest.approx(t_ref, rel=1e-10)
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) < (1e-6 if k == "vx" else TOL), (k, rel_linf(a, b))


def test_group_equals_runs_alone(gpu):
    """Spicule runs at beta 0.3, 1 and 3 advanced as one double-float group
    end where each ends alone, to the fast policy's group bounds: the
    torque's FP64 multiply-adds may fuse differently in the group kernel,
    and the corona amplifies that in vx."""
    sets = [setups.spicule_1d(1024, beta=b, seed=k) for k, b in enumerate((0.3, 1.0, 3.0))]

    def started(s):
        run = drivers.make_run(s, df64=True)
        run.push(setups.copy_state(s))
        run.start(tend=s["tend"], nstop=10 ** 6, safety=s["safety"], dtmin=s["dtmin"])
        return run

    alone = []
    for s in sets:
        r = started(s)
        try:
            r.advance(300)
            alone.append((r.pull(), r.query().ns))
        finally:
            r.close()
    runs = [started(s) for s in sets]
    try:
        capi.Run.advance_group(runs, 300)
        for s, r, (a, ns) in zip(sets, runs, alone):
            assert r.query().ns == ns
            for k, x, y in zip(s["names"], r.pull(), a):
                assert rel_linf(x, y) <= (1e-4 if k == "vx" else 1e-10), (k, rel_linf(x, y))
    finally:
        for r in runs:
            r.close()


def test_group_refuses_mixed_policies(gpu):
    s = setups.spicule_1d(256)
    runs = [drivers.make_run(s, df64=df) for df in (False, True)]
    try:
        for r in runs:
            r.push(setups.copy_state(s))
            r.start(tend=s["tend"], nstop=10, safety=s["safety"], dtmin=s["dtmin"])
        with pytest.raises(capi.CansError) as e:
            capi.Run.advance_group(runs, 5)
        assert e.value.code == capi.CANS_ERR_ARG
    finally:
        for r in runs:
            r.close()


def test_exact_policy_refuses_double_float(gpu):
    s = setups.shock_tube_1d(256)
    run = drivers.make_run(s, exact=True)
    try:
        with pytest.raises(capi.CansError) as e:
            run.set_df64(True)
        assert e.value.code == capi.CANS_ERR_ARG
    finally:
        run.close()
