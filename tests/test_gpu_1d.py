"""GPU parity of the 1-D mLW path (cans1d/hdmlw/mlw_m.f, cfl_m.f, bd*) and of
the whole 1-D loop run as one thread-block-cluster kernel, against the CPU
oracle through the C ABI."""
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
        if not np.array_equal(a, b):
            d = np.argwhere(a != b)
            raise AssertionError(f"{what} {k}: {len(d)} cells differ, first {d[:3].ravel()}, "
                                 f"rel {rel_linf(a, b):.3e}")


@pytest.fixture(autouse=True)
def _exact_reset(gpu):
    gpu.set_exact(False)
    yield
    gpu.set_exact(False)


@pytest.mark.parametrize("ix", [35, 130, 1026, 4099])
def test_one_step_exact_bitwise(gpu, oracle_lib, ix):
    s = setups.random_state_1d(ix, seed=ix)
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_m_1d(0.4, 1e-10, s["gm"], s["bx"], *ref, s["dx"])
    oracle.mlw_m_1d(*ref, s["bx"], s["bxm"], dt, s["qav"], s["gm"], s["dx"], s["dxm"])
    got = setups.copy_state(s)
    gpu.set_exact(True)
    drivers._step(s, got, dt)
    assert_same(s["names"], got, ref, "step1d")


def test_cfl_exact(gpu, oracle_lib):
    s = setups.shock_tube_1d(1024)
    gpu.set_exact(True)
    a = oracle.cfl_m_1d(0.4, 1e-10, s["gm"], s["bx"], *s["state"], s["dx"])
    b = drivers._cfl(s, s["state"], 0.4)
    assert a == b


def test_every_boundary_kind_bitwise(gpu, oracle_lib):
    rng = np.random.default_rng(3)
    q = rng.standard_normal(13)
    dxm = np.linspace(0.1, 0.2, 13)
    for kind in range(8):
        for mbnd in (0, 1):
            for margin in (1, 2):
                a, b = q.copy(), q.copy()
                oracle.bd_1d(kind, mbnd, margin, a, q0=0.25, dxm=dxm)
                capi.bd_1d(kind, mbnd, margin, b, q0=0.25, dxm=dxm)
                assert np.array_equal(a, b), (kind, mbnd, margin)


def test_shock_tube_to_tend_exact(gpu, oracle_lib):
    s = setups.shock_tube_1d(1024)
    ref = setups.copy_state(s)
    t_ref, ns_ref, merr_ref, _ = oracle.run_1d(s, ref, 10 ** 6)
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, 10 ** 6, exact=True, chunk=100000)
    assert (t, ns, merr, nexec) == (t_ref, ns_ref, merr_ref, ns_ref)
    assert t >= 0.1 and ns > 100
    assert_same(s["names"], got, ref, "shock tube")


def test_shock_tube_fast_100_steps_within_tolerance(gpu, oracle_lib):
    s = setups.shock_tube_1d(1024)
    ref = setups.copy_state(s)
    oracle.run_1d(s, ref, 100)
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, 100, exact=False)
    assert ns == 100
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) <= TOL_FAST, (k, rel_linf(a, b))


def test_periodic_loop_exact(gpu, oracle_lib):
    s = setups.random_state_1d(301, seed=5)
    ref = setups.copy_state(s)
    r = oracle.run_1d(s, ref, 40)
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, 40, exact=True)
    assert (t, ns, merr) == (r[0], r[1], r[2])
    assert_same(s["names"], got, ref, "periodic 1d")


def test_literal_loop_matches_oracle(gpu, oracle_lib):
    s = setups.shock_tube_1d(256)
    ref = setups.copy_state(s)
    oracle.run_1d(s, ref, 20)
    for resident in (False, True):
        got = setups.copy_state(s)
        gpu.set_exact(True)
        drivers.run_literal(s, got, 20, resident=resident)
        assert_same(s["names"], got, ref, f"literal1d resident={resident}")


def test_pause_at_output_times(gpu):
    s = setups.shock_tube_1d(1024)
    run = drivers.make_run(s, exact=False)
    try:
        run.push(setups.copy_state(s))
        run.start(tend=0.1, nstop=10 ** 6, safety=0.4, dtmin=1e-10, dtout=0.01,
                  pause_on_output=True)
        run.advance(100000)
        st = run.query()
        assert st.pause == 1 and not st.done and st.t >= 0.01
        run.resume()
        run.advance(100000)
        assert run.query().t >= 0.02
    finally:
        run.close()
