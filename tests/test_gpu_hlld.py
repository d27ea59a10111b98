"""GPU parity of the HLLD path (cansxx-nosupport: engine.f, hlld_mh.f,
hlld_flux.f90, inp_const.f, inp_tvdminmod.f, adddfdx.f; loop of
md_mhdshktb/hdhlld-x/main.f) against the CPU oracle, through the C ABI.
Exact policy: bit-identical.  Fast policy: relative L-infinity <= 1e-10
per variable after the stated steps."""
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
    s = setups.random_state_3d(*shape, seed=sum(shape) + 1, solver="hlld_3d")
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_3d(s, ref, 0.4)
    oracle.step_3d(s, ref, dt)
    got = setups.copy_state(s)
    gpu.set_exact(True)
    drivers._step(s, got, dt)
    assert_same(s["names"], got, ref, "hlld3d")


@pytest.mark.parametrize("mfdim", [(1, 0, 0), (0, 1, 0), (1, 0, 1), (0, 1, 1)])
def test_partial_axis_masks_exact(gpu, oracle_lib, mfdim):
    s = setups.random_state_3d(12, 13, 11, seed=17, solver="hlld_3d")
    s["mfdim"] = mfdim
    ref = setups.copy_state(s)
    oracle.step_3d(s, ref, 4e-3)
    got = setups.copy_state(s)
    gpu.set_exact(True)
    drivers._step(s, got, 4e-3)
    assert_same(s["names"], got, ref, f"hlld mfdim={mfdim}")


def test_brio_wu_loop_exact(gpu, oracle_lib):
    """md_mhdshktb/hdhlld-x: 1024 cells (+3 ghosts each side), x only, to
    t = 0.1; resident loop bit-identical to the oracle loop."""
    s = setups.shock_tube_hlld_1d(1024)
    ref = setups.copy_state(s)
    t_ref, ns_ref, merr_ref, _ = oracle.run_3d(s, ref, 100000)
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, 100000, exact=True)
    assert (t, ns, merr) == (t_ref, ns_ref, merr_ref)
    assert nexec == ns and t >= 0.1
    assert_same(s["names"], got, ref, "brio-wu")


def test_literal_loop_resident_and_not(gpu, oracle_lib):
    s = setups.random_state_3d(15, 14, 16, seed=7, solver="hlld_3d")
    ref = setups.copy_state(s)
    oracle.run_3d(s, ref, 4)
    gpu.set_exact(True)
    for resident in (False, True):
        got = setups.copy_state(s)
        drivers.run_literal(s, got, 4, resident=resident)
        assert_same(s["names"], got, ref, f"literal resident={resident}")


def test_resident_loop_mixed_boundaries_exact(gpu, oracle_lib):
    s = setups.random_state_3d(22, 19, 26, seed=5, solver="hlld_3d")
    ref = setups.copy_state(s)
    t_ref, ns_ref, merr_ref, _ = oracle.run_3d(s, ref, 12)
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, 12, exact=True)
    assert (t, ns, merr, nexec) == (t_ref, ns_ref, merr_ref, 12)
    assert_same(s["names"], got, ref, "hlld loop")


def test_fast_policy_tolerance_100_steps(gpu, oracle_lib):
    # Two properties of the reference set the terms of this comparison:
    # (1) its driver pairs the CANS-unit cfl_m (ca^2 = B^2/4 pi rho) with the
    # Heaviside-unit HLLD state, which underestimates the Alfven speed; with
    # three active axes safety 0.4 is beyond the stability limit, so the run
    # here uses 0.2; (2) with the field along an axis the faces of that axis
    # sit at the cf = ca degeneracy, where hlld_flux's zfloor = 1e-10 guard
    # leaves a relative sensitivity near eps/1e-10 to rounding; an oblique
    # mean field (|b0| = 1, beta = 1) keeps every face away from it.
    s = setups.turbulence_3d(24, solver="hlld_3d", rms=0.05, b0=(0.8, 0.48, 0.36))
    s["safety"] = 0.2
    ex = setups.copy_state(s)
    oracle.run_3d(s, ex, 100)
    fa = setups.copy_state(s)
    drivers.run_resident(s, fa, 100, exact=False)
    for k, a, b in zip(s["names"], fa, ex):
        assert np.isfinite(a).all()
        assert rel_linf(a, b) <= TOL_FAST, (k, rel_linf(a, b))


def test_argument_checks(gpu):
    z = [np.zeros((3, 6, 7), order="F") for _ in range(8)]
    one = np.ones(8)
    with pytest.raises(capi.CansError):  # an active axis shorter than 4 cells
        capi.hlld_engine_3d(*z, 2.0, 1.0, 1e-3, one[:3], one[:3], one[:6], one[:6], one[:7],
                            one[:7], (1, 1, 1))
