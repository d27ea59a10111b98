"""GPU parity of the 3-D resistive step, mlw_m_e (cans3d/hdmlw/mlw_m_e.f),
and its time step cfl_m_e (cans3d/common/cfl_m_e.f), through the C ABI
against the CPU oracle: one step with seeded resistivity on ragged grids, the
frozen fixture, and the md_recon 3-D model loop (cfl_m_e, mlw_m_e, bnd) on the
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


@pytest.mark.parametrize("shape", [(12, 13, 11), (37, 21, 19), (20, 4, 70)])
def test_one_step_exact_bitwise(gpu, oracle_lib, shape):
    s = setups.random_resistivity(setups.random_state_3d(*shape, seed=sum(shape)),
                                  seed=shape[0])
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_3d(s, ref, 0.4)
    oracle.step_3d(s, ref, dt)
    got = setups.copy_state(s)
    gpu.set_exact(True)
    gdt, merr = drivers._cfl(s, got, 0.4)
    assert (gdt, merr) == (dt, 0)
    drivers._step(s, got, dt)
    assert_same(s["names"], got, ref, "mlw_m_e 3-D")


def test_cfl_diffusion_limit_exact(gpu, oracle_lib):
    s = setups.random_state_3d(14, 12, 10, seed=8)
    s = dict(s, et=np.full(s["state"][0].shape, 40.0, order="F"),
             etm=np.zeros(s["state"][0].shape, order="F"))
    gpu.set_exact(True)
    assert drivers._cfl(s, s["state"], 0.4) == oracle.cfl_3d(s, s["state"], 0.4)


def test_one_step_fast_close(gpu, oracle_lib):
    s = setups.random_resistivity(setups.random_state_3d(40, 36, 33, seed=5), seed=6)
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_3d(s, ref, 0.4)
    oracle.step_3d(s, ref, dt)
    got = setups.copy_state(s)
    drivers._step(s, got, dt)
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) < 1e-12, (k, rel_linf(a, b))


def test_frozen_fixture_exact(gpu):
    z = np.load(GOLD / "mlw_m_e_3d_12x13x11.npz")
    names = setups.VARS["mlw_m_3d"]
    st = [np.asfortranarray(z["in_" + k]) for k in names]
    s = dict(solver="mlw_m_3d", qav=3.0, gm=5.0 / 3.0,
             et=np.asfortranarray(z["src_et"]), etm=np.asfortranarray(z["src_etm"]),
             **{k: z["grid_" + k] for k in ("dx", "dxm", "dy", "dym", "dz", "dzm")})
    gpu.set_exact(True)
    drivers._step(s, st, float(z["dt"]))
    for k, a in zip(names, st):
        assert np.array_equal(a, z["out_" + k]), k


def test_rejects_missing_fields(gpu):
    s = setups.random_resistivity(setups.random_state_3d(12, 12, 12, seed=1), seed=2)
    with pytest.raises(capi.CansError):
        capi.mlw_m_e_3d(*s["state"], 1e-3, 3.0, 5 / 3, s["et"], None, s["dx"], s["dxm"],
                        s["dy"], s["dym"], s["dz"], s["dzm"])
    bad = dict(s, etm=None)
    with pytest.raises(capi.CansError):
        drivers.make_run(bad)
    both = setups.random_gravity(s, seed=3)  # no 3-D step has gravity and resistivity
    with pytest.raises(capi.CansError):
        drivers.make_run(both)


@pytest.mark.parametrize("tile", [0, 1, 2])
def test_reconnection_loop_exact_bitwise(gpu, oracle_lib, tile):
    """md_recon 3-D at 48 x 48 x 4 (the reference's thin z axis): 40
    iterations of cfl_m_e -> mlw_m_e -> bnd on the device."""
    s = setups.magnetic_reconnection_3d(48, 4)
    ref = setups.copy_state(s)
    t, ns, merr, _ = oracle.run_3d(s, ref, 40)
    got = setups.copy_state(s)
    run = drivers.make_run(s, exact=True, tile=tile)
    try:
        out = drivers.run_resident(s, got, 40, run=run)
    finally:
        run.close()
    assert out == (t, ns, merr, ns)
    assert_same(s["names"], got, ref, f"reconnection 3-D tile {tile}")


def test_reconnection_reference_size_loop_exact_bitwise(gpu, oracle_lib):
    """md_recon 3-D at the reference's 128 x 128 x 4 (main.f:6): 60
    iterations of cfl_m_e -> mlw_m_e -> bnd on the device, autotuned tile."""
    s = setups.magnetic_reconnection_3d(128, 4)
    ref = setups.copy_state(s)
    t, ns, merr, _ = oracle.run_3d(s, ref, 60)
    got = setups.copy_state(s)
    run = drivers.make_run(s, exact=True)
    try:
        run.push(got)
        run.autotune(1)
        out = drivers.run_resident(s, got, 60, run=run)
    finally:
        run.close()
    assert out == (t, ns, merr, ns)
    assert_same(s["names"], got, ref, "reconnection 3-D 128x128x4")


def test_reconnection_literal_loop_equals_oracle(gpu, oracle_lib):
    s = setups.magnetic_reconnection_3d(24, 6)
    ref = setups.copy_state(s)
    oracle.run_3d(s, ref, 10)
    got = setups.copy_state(s)
    gpu.set_exact(True)
    drivers.run_literal(s, got, 10, resident=True)
    assert_same(s["names"], got, ref, "literal reconnection 3-D")


def test_fast_policy_100_steps_within_tolerance(gpu, oracle_lib):
    """vz and bz of this model stay ~1e-7 of the other components (they grow
    only from the zero current of the outer layer), so velocity and field
    are compared as vectors: the error of each component relative to the
    largest component of its vector."""
    s = setups.magnetic_reconnection_3d(64, 8)
    ref = setups.copy_state(s)
    oracle.run_3d(s, ref, 100)
    got = setups.copy_state(s)
    drivers.run_resident(s, got, 100, exact=False)
    names = s["names"]
    vec = {"v": [names.index(k) for k in ("vx", "vy", "vz")],
           "b": [names.index(k) for k in ("bx", "by", "bz")]}
    for v, (k, a, b) in enumerate(zip(names, got, ref)):
        group = vec.get(k[0]) if k[0] in "vb" else None
        scale = (max(float(np.max(np.abs(ref[q]))) for q in group) if group
                 else float(np.max(np.abs(b))))
        err = float(np.max(np.abs(a - b))) / scale
        assert err < 1e-10, (k, err)
