"""GPU parity of the 3-D Roe-MUSCL path (cans3d/hdroe/roe_m.f, roeflux_m.f,
tvdminmod.f; loop of cans3d/md_mhdshktb/hdroe/main.f) against the CPU oracle,
through the C ABI.  Exact policy: bit-identical.  Fast policy: relative
L-infinity <= 1e-10 per variable after the stated steps."""
import numpy as np
import pytest

import oracle
from utrip_gb300 import capi, drivers, setups

pytestmark = pytest.mark.gpu
TOL_FAST = 1e-10


def rel_linf(a, b):
    scale = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) / scale if scale else float(np.max(np.abs(a - b)))


def assert_same(names, got, ref, what=""):
    for k, a, b in zip(names, got, ref):
        assert np.isfinite(b).all(), f"{what} {k}: oracle produced non-finite values"
        if not np.array_equal(a, b):
            d = np.argwhere(a != b)
            raise AssertionError(f"{what} {k}: {len(d)} cells differ, first {d[:3].tolist()}, "
                                 f"rel {rel_linf(a, b):.3e}")


@pytest.fixture(autouse=True)
def _exact_reset(gpu):
    gpu.set_exact(False)
    yield
    gpu.set_exact(False)


@pytest.mark.parametrize("shape", [(14, 12, 13), (21, 9, 30), (40, 17, 8)])
def test_one_step_exact_bitwise(gpu, oracle_lib, shape):
    s = setups.random_state_3d(*shape, seed=sum(shape), solver="roe_m_3d")
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_3d(s, ref, 0.4)
    oracle.step_3d(s, ref, dt)
    got = setups.copy_state(s)
    gpu.set_exact(True)
    drivers._step(s, got, dt)
    assert_same(s["names"], got, ref, "roe3d")


def test_minimum_extent(gpu, oracle_lib):
    # 5 cells along x: one updated cell layer (index 3); a margin-1 grid
    # supplies the arrays, roe_m itself takes any extents >= 5
    s = setups.random_state_3d(5, 6, 7, seed=3)
    s["solver"] = "roe_m_3d"
    ref = setups.copy_state(s)
    oracle.step_3d(s, ref, 1e-3)
    got = setups.copy_state(s)
    gpu.set_exact(True)
    drivers._step(s, got, 1e-3)
    assert_same(s["names"], got, ref, "roe3d 5x6x7")
    with pytest.raises(capi.CansError):
        capi.roe_m_3d(*[np.zeros((4, 6, 7), order="F") for _ in range(8)], 1e-3, 2.0,
                      np.ones(4), np.ones(6), np.ones(7))


def test_shock_tube_loop_exact(gpu, oracle_lib):
    """The oblique shock tube of md_mhdshktb/hdroe to tend = 0.1, bdfre on
    every face, margin 3: resident loop bit-identical to the oracle loop."""
    s = setups.shock_tube_3d(16)
    ref = setups.copy_state(s)
    t_ref, ns_ref, merr_ref, _ = oracle.run_3d(s, ref, 100000)
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, 100000, exact=True)
    assert (t, ns, merr) == (t_ref, ns_ref, merr_ref)
    assert nexec == ns and t >= 0.1
    assert_same(s["names"], got, ref, "shock tube")


def test_resident_loop_mixed_boundaries_exact(gpu, oracle_lib):
    s = setups.random_state_3d(22, 19, 26, seed=5, solver="roe_m_3d")
    ref = setups.copy_state(s)
    t_ref, ns_ref, merr_ref, _ = oracle.run_3d(s, ref, 12)
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, 12, exact=True)
    assert (t, ns, merr, nexec) == (t_ref, ns_ref, merr_ref, 12)
    assert_same(s["names"], got, ref, "roe loop")


def test_literal_loop_resident_and_not(gpu, oracle_lib):
    s = setups.random_state_3d(15, 14, 16, seed=7, solver="roe_m_3d")
    ref = setups.copy_state(s)
    oracle.run_3d(s, ref, 4)
    gpu.set_exact(True)
    for resident in (False, True):
        got = setups.copy_state(s)
        drivers.run_literal(s, got, 4, resident=resident)
        assert_same(s["names"], got, ref, f"literal resident={resident}")


def test_fast_policy_tolerance_100_steps(gpu, oracle_lib):
    """Fast policy against the oracle on the 3-D beta = 1 turbulence set-up
    (24^3) after 100 steps of the resident loop."""
    s = setups.turbulence_3d(24, solver="roe_m_3d", rms=0.05)
    ex = setups.copy_state(s)
    oracle.run_3d(s, ex, 100)
    fa = setups.copy_state(s)
    drivers.run_resident(s, fa, 100, exact=False)
    for k, a, b in zip(s["names"], fa, ex):
        assert np.isfinite(a).all()
        if k in ("by", "bz") and float(np.max(np.abs(b))) < 1e-6:
            assert float(np.max(np.abs(a - b))) <= 1e-12, k
            continue
        assert rel_linf(a, b) <= TOL_FAST, (k, rel_linf(a, b))


def test_pause_resume_and_graph_off(gpu, oracle_lib):
    s = setups.shock_tube_3d(12)
    ref = setups.copy_state(s)
    oracle.run_3d(s, ref, 9)
    run = drivers.make_run(s, exact=True)
    try:
        run.set_graph(False)
        got = setups.copy_state(s)
        run.push(got)
        run.start(t0=0.0, tend=1.0, nstop=9, safety=0.4, dtmin=1e-10)
        run.advance(12)
        st = run.query()
        assert st.done and st.ns == 9
        run.pull(got)
        assert_same(s["names"], got, ref, "graph off")
    finally:
        run.close()
