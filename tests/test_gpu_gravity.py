"""GPU parity of the 2-D steps with gravity, mlw_m_g (cans2d/hdmlw/mlw_m_g.f)
and mlw_m3_g (mlw_m3_g.f), through the C ABI against the CPU oracle: one step
with seeded non-uniform gravity on ragged grids, and the md_mhdgwave model
loop (cfl_m, mlw_m_g, bnd) on the device.  Exact policy: bit-identical; fast
policy: relative L-infinity <= 1e-10 after 100 steps."""
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
        if not np.array_equal(a, b):
            d = np.argwhere(a != b)
            raise AssertionError(f"{what} {k}: {len(d)} cells differ, first {d[:3].tolist()}, "
                                 f"rel {rel_linf(a, b):.3e}")


@pytest.fixture(autouse=True)
def _exact_reset(gpu):
    gpu.set_exact(False)
    yield
    gpu.set_exact(False)


@pytest.mark.parametrize("solver", ["mlw_m", "mlw_m3"])
@pytest.mark.parametrize("shape", [(19, 16), (45, 23), (70, 41)])
def test_one_step_exact_bitwise(gpu, oracle_lib, solver, shape):
    s = setups.random_gravity(setups.random_state(*shape, seed=sum(shape), solver=solver),
                              seed=shape[0])
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_2d(s, ref, 0.4)
    oracle.step_2d(s, ref, dt)
    got = setups.copy_state(s)
    gpu.set_exact(True)
    drivers._step(s, got, dt)
    assert_same(s["names"], got, ref, f"{solver}_g")


def test_rejects_missing_fields(gpu):
    s = setups.random_state(12, 12, seed=1, solver="mlw_m")
    z = np.zeros((12, 12), order="F")
    with pytest.raises(capi.CansError):
        capi.mlw_m_g(*s["state"], 1e-3, 3.0, 5 / 3, z, z, None, z, s["dx"], s["dxm"],
                     s["dy"], s["dym"])


@pytest.mark.parametrize("solver", ["mlw_m", "mlw_m3"])
def test_gravity_wave_loop_exact_bitwise(gpu, oracle_lib, solver):
    """md_mhdgwave: stratified atmosphere, pressure pulse, 100 iterations of
    cfl_m -> mlw_m_g -> bnd (free/constant-gradient y faces) on the device."""
    s = setups.mhd_gravity_wave(64, solver=solver)
    ref = setups.copy_state(s)
    t, ns, merr, _ = oracle.run_2d(s, ref, 100)
    for tile in range(2):
        got = setups.copy_state(s)
        run = drivers.make_run(s, exact=True, tile=tile)
        try:
            out = drivers.run_resident(s, got, 100, run=run)
        finally:
            run.close()
        assert out == (t, ns, merr, ns)
        assert_same(s["names"], got, ref, f"gravity wave tile {tile}")


def test_gravity_wave_literal_loop_equals_oracle(gpu, oracle_lib):
    s = setups.mhd_gravity_wave(48)
    ref = setups.copy_state(s)
    oracle.run_2d(s, ref, 20)
    got = setups.copy_state(s)
    gpu.set_exact(True)
    drivers.run_literal(s, got, 20, resident=True)
    assert_same(s["names"], got, ref, "literal gravity wave")


def test_fast_policy_100_steps_within_tolerance(gpu, oracle_lib):
    s = setups.mhd_gravity_wave(128)
    ref = setups.copy_state(s)
    oracle.run_2d(s, ref, 100)
    got = setups.copy_state(s)
    drivers.run_resident(s, got, 100, exact=False)
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) < 1e-10, (k, rel_linf(a, b))


def test_emerging_flux_2d_loop_exact_bitwise(gpu, oracle_lib):
    """cans2d/md_efr: the Parker-unstable flux sheet at 64 x 128 (the
    reference's size), 100 iterations of cfl_m -> mlw_m_g -> bnd with the
    held y faces."""
    s = setups.emerging_flux_2d(64, 128)
    ref = setups.copy_state(s)
    t, ns, merr, _ = oracle.run_2d(s, ref, 100)
    got = setups.copy_state(s)
    out = drivers.run_resident(s, got, 100, exact=True)
    assert out == (t, ns, merr, ns)
    assert_same(s["names"], got, ref, "emerging flux 2-D")


def test_parker_instability_loop_exact_bitwise(gpu, oracle_lib):
    """cans2d/md_parkerinst at the reference's 64 x 128: 100 iterations of
    cfl_m -> mlw_m_g -> bnd -> chkdav (ro, pr; floor 1e-9) on the device."""
    s = setups.parker_instability(64, 128)
    ref = setups.copy_state(s)
    t, ns, merr, _ = oracle.run_2d(s, ref, 100)
    got = setups.copy_state(s)
    out = drivers.run_resident(s, got, 100, exact=True)
    assert out == (t, ns, merr, ns)
    assert_same(s["names"], got, ref, "Parker instability")


def oracle_loop_with_events(s, state, nstop):
    """oracle.run_2d with the chkdav events counted."""
    events, ns, t = 0, 0, 0.0
    while True:
        ns += 1
        dt, _ = oracle.cfl_2d(s, state, s["safety"])
        t += dt
        oracle.step_2d(s, state, dt)
        oracle.apply_bc_program(state, s["bc"], s["margin"], s)
        events += oracle.chkdav_state(s, state)
        if not (ns < nstop and t < s["tend"]):
            return t, ns, events


def test_chkdav_floor_events_exact(gpu, oracle_lib):
    """A floor above the coronal density of the Parker set-up makes chkdav
    act in every iteration: the resident loop floors ro and pr and zeroes
    vx, vy where the oracle does, and counts the same events."""
    s = dict(setups.parker_instability(48, 96), floor=0.012)
    ref = setups.copy_state(s)
    t, ns, events = oracle_loop_with_events(s, ref, 40)
    assert events > 0
    got = setups.copy_state(s)
    run = drivers.make_run(s, exact=True)
    try:
        run.push(got)
        run.start(tend=s["tend"], nstop=40, safety=s["safety"], dtmin=s["dtmin"])
        run.advance(41)
        st = run.query()
        run.pull(got)
    finally:
        run.close()
    assert (st.t, st.ns, st.merr) == (t, ns, 0)
    assert st.n_floor == events
    assert_same(s["names"], got, ref, "chkdav loop")


@pytest.mark.parametrize("resident", [False, True])
def test_chkdav_drop_in_2d_3d(gpu, oracle_lib, resident):
    rng = np.random.default_rng(3)
    for shape in ((23, 17), (9, 11, 13)):
        da = np.asfortranarray(rng.random(shape))
        vel = [np.asfortranarray(rng.standard_normal(shape)) for _ in shape]
        ref = [da.copy(order="F")] + [v.copy(order="F") for v in vel]
        n_ref = oracle.chkdav_nd(ref[0], ref[1:], 0.3)
        got = [da] + vel
        if resident:
            capi.register(got)
        try:
            fn = capi.chkdav_3d if len(shape) == 3 else capi.chkdav_2d
            n = fn(*got, 0.3)
        finally:
            if resident:
                capi.pull(got[0])
                capi.release(got[0])
        assert n == n_ref > 0
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
