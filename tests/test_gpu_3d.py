"""GPU parity of the 3-D mLW path (cans3d/hdmlw/mlw_m.f, cfl_m.f, bd*) against
the CPU oracle, through the C ABI.  Exact policy: bit-identical.  Fast
policy: relative L-infinity <= 1e-10 per variable after the stated steps."""
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
            raise AssertionError(f"{what} {k}: {len(d)} cells differ, first {d[:3].tolist()}, "
                                 f"rel {rel_linf(a, b):.3e}")


@pytest.fixture(autouse=True)
def _exact_reset(gpu):
    gpu.set_exact(False)
    yield
    gpu.set_exact(False)


@pytest.mark.parametrize("shape", [(20, 18, 16), (35, 21, 70), (19, 37, 9)])
def test_one_step_exact_bitwise(gpu, oracle_lib, shape):
    s = setups.random_state_3d(*shape, seed=sum(shape))
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_3d(s, ref, 0.4)
    oracle.step_3d(s, ref, dt)
    got = setups.copy_state(s)
    gpu.set_exact(True)
    drivers._step(s, got, dt)
    assert_same(s["names"], got, ref, "step3d")


def test_cfl_exact(gpu, oracle_lib):
    s = setups.random_state_3d(23, 19, 17, seed=8)
    gpu.set_exact(True)
    assert drivers._cfl(s, s["state"], 0.4) == oracle.cfl_3d(s, s["state"], 0.4)


def test_every_boundary_kind_bitwise(gpu, oracle_lib):
    rng = np.random.default_rng(5)
    q = np.asfortranarray(rng.standard_normal((9, 8, 7)))
    dm = {0: np.linspace(0.1, 0.2, 9), 1: np.linspace(0.1, 0.3, 8), 2: np.linspace(0.2, 0.3, 7)}
    for kind in range(8):
        for axis in (0, 1, 2):
            for mbnd in (0, 1):
                a = q.copy(order="F")
                b = q.copy(order="F")
                oracle.bd_3d(kind, axis, mbnd, 2, a, q0=0.5, dxm=dm[axis])
                capi.bd_3d(kind, axis, mbnd, 2, b, q0=0.5, dxm=dm[axis])
                assert np.array_equal(a, b), (kind, axis, mbnd)


def test_resident_loop_exact_20_steps(gpu, oracle_lib):
    s = setups.random_state_3d(28, 24, 70, seed=1)
    ref = setups.copy_state(s)
    t_ref, ns_ref, merr_ref, _ = oracle.run_3d(s, ref, 20)
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, 20, exact=True)
    assert (t, ns, merr, nexec) == (t_ref, ns_ref, merr_ref, 20)
    assert_same(s["names"], got, ref, "loop3d")


def test_literal_loop_matches_oracle(gpu, oracle_lib):
    s = setups.random_state_3d(18, 16, 14, seed=6)
    ref = setups.copy_state(s)
    oracle.run_3d(s, ref, 5)
    for resident in (False, True):
        got = setups.copy_state(s)
        gpu.set_exact(True)
        drivers.run_literal(s, got, 5, resident=resident)
        assert_same(s["names"], got, ref, f"literal3d resident={resident}")


def test_turbulence_fast_within_tolerance(gpu, oracle_lib):
    s = setups.turbulence_3d(32)
    ref = setups.copy_state(s)
    oracle.run_3d(s, ref, 100)
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, 100, exact=False)
    assert ns == 100 and nexec == 100
    for k, a, b in zip(s["names"], got, ref):
        if k in ("by", "bz") and np.max(np.abs(b)) < 1e-12:
            continue
        assert rel_linf(a, b) <= TOL_FAST, (k, rel_linf(a, b))


def test_all_tiles_agree_bitwise(gpu, oracle_lib):
    s = setups.random_state_3d(37, 30, 75, seed=12)
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_3d(s, ref, 0.4)
    oracle.step_3d(s, ref, dt)
    for tile in range(3):
        run = drivers.make_run(s, exact=True, tile=tile)
        try:
            run.push(setups.copy_state(s))
            run.step(dt, apply_bc=False)
            got = run.pull()
        finally:
            run.close()
        assert_same(s["names"], got, ref, f"tile {tile}")


def test_full_size_256_fast_vs_exact_and_mass(gpu):
    s = setups.turbulence_3d(256)
    a = setups.copy_state(s)
    b = setups.copy_state(s)
    ta = drivers.run_resident(s, a, 20, exact=True)
    tb = drivers.run_resident(s, b, 20, exact=False)
    assert ta[1] == tb[1] == 20
    for k, x, y in zip(s["names"], b, a):
        if k in ("by", "bz", "vx", "vy", "vz"):
            scale = max(float(np.max(np.abs(y))), 1e-2)
            assert float(np.max(np.abs(x - y))) <= TOL_FAST * scale, k
        else:
            assert rel_linf(x, y) <= TOL_FAST, (k, rel_linf(x, y))
    m0 = s["state"][0][1:-1, 1:-1, 1:-1].sum()
    assert abs(a[0][1:-1, 1:-1, 1:-1].sum() - m0) <= 1e-12 * m0
