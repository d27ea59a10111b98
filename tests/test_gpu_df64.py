"""The double-float policy of the 2-D mlw_m3 and 3-D mlw_m steps
(cans_run_set_df64): the step's arithmetic in pairs of floats on the FP32
pipes, the conserved density and field accumulated in FP64.  It is held to the fast policy's bar
against the oracle -- relative L-infinity <= 1e-10 per variable after 100
steps -- on the benchmark vortex, the shear layer and a ragged random state,
and it must converge to the exact shock-tube solution like the oracle."""
import numpy as np
import pytest

import oracle
from oracle import shktb_analytic as an
from utrip_gb300 import capi, drivers, setups

pytestmark = pytest.mark.gpu
TOL = 1e-10


def rel_linf(a, b):
    scale = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) / scale if scale else float(np.max(np.abs(a - b)))


@pytest.mark.parametrize("tile", [0, 4])
@pytest.mark.parametrize("make,steps", [
    (lambda: setups.orszag_tang(64), 100),
    (lambda: setups.shear_layer(128, beta=0.5, seed=2), 100),
    (lambda: setups.random_state(53, 41, seed=7), 20),
])
def test_df64_loop_against_oracle(gpu, oracle_lib, make, steps, tile):
    s = make()
    ref = setups.copy_state(s)
    t_ref, ns_ref, _, _ = oracle.run_2d(s, ref, steps)
    got = setups.copy_state(s)
    run = drivers.make_run(s, df64=True, tile=tile)
    try:
        t, ns, merr, nexec = drivers.run_resident(s, got, steps, run=run)
    finally:
        run.close()
    assert merr == 0 and ns == ns_ref and nexec == ns
    assert t == pytest.approx(t_ref, rel=1e-12)
    for k, a, b in zip(s["names"], got, ref):
        assert np.isfinite(a).all(), k
        assert rel_linf(a, b) <= TOL, (k, rel_linf(a, b))


def test_df64_one_step_close_to_oracle(gpu, oracle_lib):
    """One step of a ragged random state (every variable non-zero): within a
    few 2^-48 of the reference arithmetic."""
    s = setups.random_state(45, 38, seed=11)
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_2d(s, ref, 0.4)
    oracle.step_2d(s, ref, dt)
    run = drivers.make_run(s, df64=True)
    try:
        run.push(s["state"])
        run.step(dt, apply_bc=False)
        got = run.pull()
    finally:
        run.close()
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) <= 2e-13, (k, rel_linf(a, b))


@pytest.mark.parametrize("n", [96, 130])
def test_df64_tiles_agree_bitwise(gpu, n):
    """Every tile shape, the y-marching ones included (segments and chunks
    ragged at 130), gives the same bits."""
    s = setups.orszag_tang(n)
    outs = []
    for tile in range(7):
        run = drivers.make_run(s, df64=True)
        try:
            run.set_tile(tile)
            st = setups.copy_state(s)
            drivers.run_resident(s, st, 30, run=run)
            outs.append(st)
        finally:
            run.close()
    for o in outs[1:]:
        for a, b in zip(o, outs[0]):
            assert np.array_equal(a, b)


def test_df64_shock_tube_converges_like_the_oracle(gpu, oracle_lib):
    for n in (256, 1024):
        s = setups.sod_shock_tube(n, 2)
        got = setups.copy_state(s)
        t, ns, merr, _ = drivers.run_resident(s, got, 10 ** 6, df64=True)
        ref = setups.copy_state(s)
        t_ref, ns_ref, _, _ = oracle.run_2d(s, ref, 10 ** 6)
        assert merr == 0 and ns == ns_ref
        sd = s["sod"]
        e = an.l1_errors(*setups.sod_interior_profile(s, got), t, sd["x0"], sd["gm"],
                         sd["ro1"], sd["pr1"])
        er = an.l1_errors(*setups.sod_interior_profile(s, ref), t_ref, sd["x0"], sd["gm"],
                          sd["ro1"], sd["pr1"])
        for k in e:
            assert e[k] == pytest.approx(er[k], rel=1e-6), (n, k)


def test_df64_refused_where_it_does_not_apply(gpu):
    for s, exact in ((setups.orszag_tang(32, solver="mlw_m"), False),
                     (setups.orszag_tang(32), True),
                     (setups.random_state_1d(40, seed=1), True),
                     (setups.random_state_3d(12, 12, 12, seed=1), True)):
        run = drivers.make_run(s, exact=exact)
        try:
            with pytest.raises(capi.CansError):
                run.set_df64(True)
        finally:
            run.close()


# ---- the 3-D mlw_m step ------------------------------------------------------

@pytest.mark.parametrize("tile", [0, 1])
@pytest.mark.parametrize("make,steps", [
    (lambda: setups.turbulence_3d(24, rms=0.05), 100),
    (lambda: setups.random_state_3d(21, 18, 23, seed=4), 20),
])
def test_df64_3d_loop_against_oracle(gpu, oracle_lib, make, steps, tile):
    s = make()
    ref = setups.copy_state(s)
    t_ref, ns_ref, _, _ = oracle.run_3d(s, ref, steps)
    got = setups.copy_state(s)
    run = drivers.make_run(s, df64=True, tile=tile)
    try:
        t, ns, merr, nexec = drivers.run_resident(s, got, steps, run=run)
    finally:
        run.close()
    assert merr == 0 and ns == ns_ref and nexec == ns
    assert t == pytest.approx(t_ref, rel=1e-12)
    for k, a, b in zip(s["names"], got, ref):
        assert np.isfinite(a).all(), k
        assert rel_linf(a, b) <= TOL, (k, rel_linf(a, b))


def test_df64_3d_tiles_agree_bitwise(gpu):
    s = setups.turbulence_3d(40, rms=0.05)
    outs = []
    for tile in range(2):
        run = drivers.make_run(s, df64=True)
        try:
            run.set_tile(tile)
            st = setups.copy_state(s)
            drivers.run_resident(s, st, 12, run=run)
            outs.append(st)
        finally:
            run.close()
    for a, b in zip(outs[1], outs[0]):
        assert np.array_equal(a, b)


def test_df64_3d_shock_tube_converges_like_the_oracle(gpu, oracle_lib):
    s = setups.sod_shock_tube(512, 3)
    got = setups.copy_state(s)
    t, ns, merr, _ = drivers.run_resident(s, got, 10 ** 6, df64=True)
    ref = setups.copy_state(s)
    t_ref, ns_ref, _, _ = oracle.run_3d(s, ref, 10 ** 6)
    assert merr == 0 and ns == ns_ref
    sd = s["sod"]
    e = an.l1_errors(*setups.sod_interior_profile(s, got), t, sd["x0"], sd["gm"], sd["ro1"],
                     sd["pr1"])
    er = an.l1_errors(*setups.sod_interior_profile(s, ref), t_ref, sd["x0"], sd["gm"],
                      sd["ro1"], sd["pr1"])
    for k in e:
        assert e[k] == pytest.approx(er[k], rel=1e-6), k


# ---- the Roe-MUSCL steps: the face flux in double-float ----------------------

@pytest.mark.parametrize("make,steps,run_oracle", [
    (lambda: setups.turbulence_3d(24, solver="roe_m_3d", rms=0.05, b0=(0.8, 0.48, 0.36)), 100,
     "run_3d"),
    (lambda: setups.shear_layer(128, beta=1.0, solver="roe_m3"), 100, "run_2d"),
])
def test_df64_roe_against_oracle(gpu, oracle_lib, make, steps, run_oracle):
    """With an oblique mean field (away from the c_f = c_a degeneracy, whose
    conditioning tests/test_oracle.py measures) the double-float Roe flux
    holds the fast policy's bar."""
    s = make()
    ref = setups.copy_state(s)
    t_ref, ns_ref, _, _ = getattr(oracle, run_oracle)(s, ref, steps)
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, steps, df64=True)
    assert merr == 0 and ns == ns_ref and nexec == ns
    for k, a, b in zip(s["names"], got, ref):
        assert np.isfinite(a).all(), k
        assert rel_linf(a, b) <= TOL, (k, rel_linf(a, b))


def test_df64_hlld_against_oracle(gpu, oracle_lib):
    """The HLLD face flux in double-float, on the oblique-field box of the
    fast policy's own test (safety 0.2: the CANS-unit cfl_m over three
    active axes), held to the same bar."""
    s = setups.turbulence_3d(24, solver="hlld_3d", rms=0.05, b0=(0.8, 0.48, 0.36))
    s["safety"] = 0.2
    ref = setups.copy_state(s)
    t_ref, ns_ref, _, _ = oracle.run_3d(s, ref, 100)
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, 100, df64=True)
    assert merr == 0 and ns == ns_ref and nexec == ns
    for k, a, b in zip(s["names"], got, ref):
        assert np.isfinite(a).all(), k
        assert rel_linf(a, b) <= TOL, (k, rel_linf(a, b))


def test_df64_hlld_brio_wu_like_the_oracle(gpu, oracle_lib):
    """Across the Brio-Wu shock tube's shocks, compound wave and rarefactions
    (every branch of the flux) the double-float flux stays within 1e-10 of
    the oracle to t = 0.1."""
    s = setups.shock_tube_hlld_1d(256)
    ref = setups.copy_state(s)
    t_ref, ns_ref, _, _ = oracle.run_3d(s, ref, 10 ** 6)
    got = setups.copy_state(s)
    t, ns, merr, _ = drivers.run_resident(s, got, 10 ** 6, df64=True)
    assert merr == 0 and ns == ns_ref
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) <= TOL, (k, rel_linf(a, b))


@pytest.mark.parametrize("solver", ["roe_m_3d", "hlld_3d"])
def test_df64_riemann_degenerate_faces_take_fp64(gpu, oracle_lib, solver):
    """On the x-aligned box every x face sits at the c_f = c_a degeneracy,
    where the reference algorithm amplifies rounding and the double-float flux
    alone ended 3e-5 from the oracle (HLLD, 256^3, 20 steps).  With the
    ill-conditioned faces evaluated in FP64 the double-float step stays within
    a small factor of the FP64 fast policy there."""
    s = setups.turbulence_3d(40, solver=solver)
    if solver == "hlld_3d":
        s["safety"] = 0.2
    ref = setups.copy_state(s)
    oracle.run_3d(s, ref, 20)
    err = {}
    for pol in ("fast", "df64"):
        got = setups.copy_state(s)
        t, ns, merr, _ = drivers.run_resident(s, got, 20, df64=pol == "df64")
        assert merr == 0 and ns == 20
        err[pol] = max(rel_linf(a, b) for a, b in zip(got, ref))
    assert err["df64"] <= max(10 * err["fast"], 1e-11), err
