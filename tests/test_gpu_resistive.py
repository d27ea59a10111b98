"""GPU parity of the resistive 2-D steps, mlw_m_e (cans2d/hdmlw/mlw_m_e.f),
mlw_m3_e (mlw_m3_e.f) and with gravity mlw_m_ge / mlw_m3_ge (mlw_m_ge.f,
mlw_m3_ge.f), and of their time step cfl_m_e / cfl_m3_e, through the C ABI
against the CPU oracle: one step with seeded resistivity on ragged grids, the
frozen fixtures, and the md_recon model loop (cfl_m_e, mlw_m_e, bnd) on the
device.  Exact policy: bit-identical; fast policy: relative L-infinity
<= 1e-10 after 100 steps."""
from pathlib import Path

import numpy as np
import pytest

import oracle
from utrip_gb300 import capi, drivers, setups

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


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


def resistive_case(solver, shape, grav, scale=0.02):
    s = setups.random_resistivity(
        setups.random_state(*shape, seed=sum(shape), solver=solver, margin=2),
        seed=shape[0], scale=scale)
    if grav:
        s = setups.random_gravity(s, seed=shape[1])
    return s


@pytest.mark.parametrize("solver", ["mlw_m", "mlw_m3"])
@pytest.mark.parametrize("grav", [False, True])
@pytest.mark.parametrize("shape", [(19, 16), (45, 23), (70, 41)])
def test_one_step_exact_bitwise(gpu, oracle_lib, solver, grav, shape):
    s = resistive_case(solver, shape, grav)
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_2d(s, ref, 0.4)
    oracle.step_2d(s, ref, dt)
    got = setups.copy_state(s)
    gpu.set_exact(True)
    drivers._step(s, got, dt)
    assert_same(s["names"], got, ref, f"{solver}_{'ge' if grav else 'e'}")


@pytest.mark.parametrize("solver", ["mlw_m", "mlw_m3"])
def test_one_step_fast_close(gpu, oracle_lib, solver):
    s = resistive_case(solver, (66, 50), True)
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_2d(s, ref, 0.4)
    oracle.step_2d(s, ref, dt)
    got = setups.copy_state(s)
    drivers._step(s, got, dt)
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) < 1e-12, (k, rel_linf(a, b))


@pytest.mark.parametrize("solver", ["mlw_m", "mlw_m3"])
@pytest.mark.parametrize("scale", [0.02, 0.5])
def test_cfl_e_exact(gpu, oracle_lib, solver, scale):
    """cfl_m_e / cfl_m3_e; with scale 0.5 the diffusion limit binds."""
    s = resistive_case(solver, (37, 29), False, scale=scale)
    want = oracle.cfl_2d(s, s["state"], 0.4)
    gpu.set_exact(True)
    assert drivers._cfl(s, s["state"], 0.4) == want
    gpu.set_exact(False)
    dt, merr = drivers._cfl(s, s["state"], 0.4)
    assert merr == want[1] and abs(dt - want[0]) <= 1e-14 * want[0]


def test_frozen_fixtures_exact(gpu):
    gpu.set_exact(True)
    for name, solver, grav in (("mlw_m_e_2d_18x17", "mlw_m", False),
                               ("mlw_m3_ge_2d_17x19", "mlw_m3", True)):
        z = np.load(GOLD / f"{name}.npz")
        names = setups.VARS[solver]
        st = [np.asfortranarray(z["in_" + k]) for k in names]
        src = {k[4:]: np.asfortranarray(z[k]) for k in z.files if k.startswith("src_")}
        s = dict(solver=solver, gravity=grav, qav=3.0, gm=5.0 / 3.0, dtmin=1e-10, **src,
                 **{k: z["grid_" + k] for k in ("dx", "dxm", "dy", "dym")})
        dt, _ = drivers._cfl(s, st, 0.4)
        assert dt == float(z["dt"]), name
        drivers._step(s, st, dt)
        for k, a in zip(names, st):
            assert np.array_equal(a, z["out_" + k]), (name, k)


def test_rejects_missing_fields(gpu):
    s = setups.random_state(12, 12, seed=1, solver="mlw_m", margin=2)
    z = np.zeros((12, 12), order="F")
    with pytest.raises(capi.CansError):
        capi.mlw_m_e(*s["state"], 1e-3, 3.0, 5 / 3, z, None, s["dx"], s["dxm"], s["dy"],
                     s["dym"])
    bad = dict(s, et=z)  # et without etm
    bad["etm"] = None
    with pytest.raises(capi.CansError):
        drivers.make_run(bad)


def test_batch_refuses_variant_setups(gpu):
    """The batch runs the plain step: a set-up with resistivity or gravity is
    refused instead of being run without its source terms."""
    s = setups.random_resistivity(setups.random_state(20, 20, seed=3, solver="mlw_m"), 4)
    with pytest.raises(capi.CansError):
        capi.Batch([s, s])
    g = setups.random_gravity(setups.random_state(20, 20, seed=3, solver="mlw_m"), 4)
    with pytest.raises(capi.CansError):
        capi.Batch([g])


def test_reconnection_loop_exact_bitwise(gpu, oracle_lib):
    """md_recon: Harris sheet with localised resistivity, 100 iterations of
    cfl_m_e -> mlw_m_e -> bnd on the device."""
    s = setups.magnetic_reconnection(64)
    ref = setups.copy_state(s)
    t, ns, merr, _ = oracle.run_2d(s, ref, 100)
    got = setups.copy_state(s)
    out = drivers.run_resident(s, got, 100, exact=True)
    assert out == (t, ns, merr, ns)
    assert_same(s["names"], got, ref, "reconnection")


def test_reconnection_literal_loop_equals_oracle(gpu, oracle_lib):
    s = setups.magnetic_reconnection(32)
    ref = setups.copy_state(s)
    oracle.run_2d(s, ref, 20)
    got = setups.copy_state(s)
    gpu.set_exact(True)
    drivers.run_literal(s, got, 20, resident=True)
    assert_same(s["names"], got, ref, "literal reconnection")


@pytest.mark.parametrize("solver", ["mlw_m", "mlw_m3"])
def test_diffusion_limited_loop_exact(gpu, oracle_lib, solver):
    """A loop whose time step is set by the diffusion limit: the run handle
    folds the constant min over cells of dtdif into each step's CFL."""
    s = resistive_case(solver, (40, 36), True, scale=0.5)
    ref = setups.copy_state(s)
    t, ns, merr, dts = oracle.run_2d(s, ref, 30)
    dtdif = 0.4 * 0.5 * np.minimum(s["dx"][:, None], s["dy"][None, :]) ** 2 / s["et"]
    assert dts[0] == float(np.min(dtdif))  # the diffusion limit binds
    got = setups.copy_state(s)
    out = drivers.run_resident(s, got, 30, exact=True)
    assert out == (t, ns, merr, ns)
    assert_same(s["names"], got, ref, "diffusion-limited")


def test_fast_policy_100_steps_within_tolerance(gpu, oracle_lib):
    s = setups.magnetic_reconnection(128)
    ref = setups.copy_state(s)
    oracle.run_2d(s, ref, 100)
    got = setups.copy_state(s)
    drivers.run_resident(s, got, 100, exact=False)
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) < 1e-10, (k, rel_linf(a, b))
