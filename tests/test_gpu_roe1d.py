"""GPU parity of the 1-D Roe-MUSCL step (cans1d/hdroe/roe_m.f with the
two-component roeflux_m.f and tvdminmod.f) through the C ABI, against the
CPU oracle: one step on ragged grids and the md_mhdshktb/hdroe Brio-Wu run
to t = 0.1 (cfl_m, roe_m and bnd drop-ins).  Exact policy: bit-identical;
fast policy: relative L-infinity <= 1e-10 after 100 steps."""
import numpy as np
import pytest

import oracle
from utrip_gb300 import capi, drivers, setups

pytestmark = pytest.mark.gpu


def rel_linf(a, b):
    scale = float(np.max(np.abs(b)))
    return float(np.max(np.abs(a - b))) / scale if scale else float(np.max(np.abs(a - b)))


def assert_same(names, got, ref, what=""):
    for k, a, b in zip(names, got, ref):
        assert np.isfinite(b).all(), f"{what} {k}: oracle produced non-finite values"
        if not np.array_equal(a.view(np.int64), b.view(np.int64)):
            d = np.nonzero(a.view(np.int64) != b.view(np.int64))[0]
            raise AssertionError(f"{what} {k}: {d.size} cells differ, first {d[:4]}, "
                                 f"rel {rel_linf(a, b):.3e}")


@pytest.fixture(autouse=True)
def _exact_reset(gpu):
    gpu.set_exact(False)
    yield
    gpu.set_exact(False)


@pytest.mark.parametrize("ix", [5, 37, 130, 1030, 4099])
def test_one_step_exact_bitwise(gpu, oracle_lib, ix):
    s = setups.random_state_1d(ix, seed=ix)
    s["solver"] = "roe_m_1d"
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_m_1d(0.5, 1e-10, s["gm"], s["bx"], *ref, s["dx"])
    oracle.roe_m_1d(*ref, s["bx"], s["bxm"], dt, s["gm"], s["dx"])
    got = setups.copy_state(s)
    gpu.set_exact(True)
    drivers._step(s, got, dt)
    assert_same(s["names"], got, ref, "roe1d")


def test_rejects_short_grids(gpu):
    with pytest.raises(capi.CansError):
        capi.roe_m_1d(*[np.ones(4) for _ in range(7)], 1e-3, 2.0, np.ones(4))


@pytest.mark.parametrize("resident", [False, True])
def test_brio_wu_run_to_tend_exact(gpu, oracle_lib, resident):
    s = setups.shock_tube_1d(1024, solver="roe_m_1d")
    ref = setups.copy_state(s)
    t_ref, ns_ref, merr_ref, dts_ref = oracle.run_1d(s, ref, 10 ** 6)
    got = setups.copy_state(s)
    gpu.set_exact(True)
    t, ns, merr, dts = drivers.run_literal(s, got, 10 ** 6, resident=resident)
    assert (t, ns, merr) == (t_ref, ns_ref, merr_ref) and dts == dts_ref
    assert t >= 0.1 and ns > 100
    assert_same(s["names"], got, ref, "Brio-Wu")


def test_fast_policy_100_steps_within_tolerance(gpu, oracle_lib):
    s = setups.shock_tube_1d(1024, solver="roe_m_1d")
    ref = setups.copy_state(s)
    oracle.run_1d(s, ref, 100)
    got = setups.copy_state(s)
    drivers.run_literal(s, got, 100, resident=True)
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) < 1e-10, (k, rel_linf(a, b))
