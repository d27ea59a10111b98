"""GPU parity of the spicule path: mlw_m_bg (cans1d/hdmlw/mlw_m_bg.f), chkdav
(cans1d/common/chkdav.f), the torque source (trqalfven.f) and the spicule
loop (cans1d/md_spicule/hdmlw/main.f) run as the 1-D cluster kernel, against
the CPU oracle through the C ABI, and the whole reference run (100000 steps)
against the reference's own output."""
from pathlib import Path

import numpy as np
import pytest

import oracle
from utrip_gb300 import capi, dac, drivers, setups

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden" / "spicule_reference.npz"


def bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def assert_bitwise(names, got, ref, what=""):
    for k, a, b in zip(names, got, ref):
        if not np.array_equal(bits(a), bits(b)):
            d = np.nonzero(bits(a) != bits(b))[0]
            scale = float(np.max(np.abs(b))) or 1.0
            raise AssertionError(f"{what} {k}: {d.size} cells differ, first {d[:4]}, "
                                 f"rel {float(np.max(np.abs(a - b))) / scale:.3e}")


def rel_linf(a, b):
    scale = float(np.max(np.abs(b))) or 1.0
    return float(np.max(np.abs(a - b))) / scale


@pytest.fixture(autouse=True)
def _exact_reset(gpu):
    gpu.set_exact(False)
    yield
    gpu.set_exact(False)


def bg_random(nx, seed):
    """The spicule set-up on nx cells with every term of mlw_m_bg switched
    on: a varying distance from the axis rr (so drr, drrm and the rotation
    terms are non-zero) and a perturbed state with flows and twist."""
    s = setups.spicule_1d(nx)
    rng = np.random.default_rng(seed)
    x = s["x"]
    xs = (x - x[0]) / (x[-1] - x[0])
    s["rr"] = 1.0 + 0.2 * np.sin(2 * np.pi * xs + 0.3)
    s["rrm"] = 1.0 + 0.2 * np.sin(2 * np.pi * (xs + 0.5 / nx) + 0.3)
    s["drr"], s["drrm"] = setups.scrdy(s["rr"], s["rrm"], s["dx"], s["dxm"])
    ro, pr, vx, vy, by = s["state"]
    n = x.size
    s["state"] = [ro * (1 + 0.05 * rng.standard_normal(n)), pr * (1 + 0.05 * rng.standard_normal(n)),
                  0.05 * rng.standard_normal(n), 0.05 * rng.standard_normal(n),
                  0.1 * rng.standard_normal(n)]
    return s


@pytest.mark.parametrize("nx", [33, 128, 1024, 4097])
def test_mlw_m_bg_one_step_exact_bitwise(gpu, oracle_lib, nx):
    s = bg_random(nx, seed=nx)
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_m_1d(0.8, 1e-10, s["gm"], s["bx"], *ref, s["dx"])
    oracle.step_bg(s, ref, dt)
    got = setups.copy_state(s)
    gpu.set_exact(True)
    drivers._step(s, got, dt)
    assert_bitwise(s["names"], got, ref, "mlw_m_bg")


def test_mlw_m_bg_one_step_fast_within_tolerance(gpu, oracle_lib):
    s = bg_random(1024, seed=5)
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_m_1d(0.8, 1e-10, s["gm"], s["bx"], *ref, s["dx"])
    oracle.step_bg(s, ref, dt)
    got = setups.copy_state(s)
    drivers._step(s, got, dt)
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) < 1e-12, k


def test_chkdav_dropin_bitwise(gpu, oracle_lib):
    rng = np.random.default_rng(2)
    da = rng.uniform(-1.0, 1.0, 5000)
    vx = rng.standard_normal(5000)
    a_da, a_vx, b_da, b_vx = da.copy(), vx.copy(), da.copy(), vx.copy()
    n_ref = oracle.chkdav(a_da, a_vx, 0.25)
    n = capi.chkdav(b_da, b_vx, 0.25)
    assert n == n_ref and n > 1000
    assert np.array_equal(bits(a_da), bits(b_da)) and np.array_equal(bits(a_vx), bits(b_vx))


def _loop_gpu(s, nstop, exact, floor=True, torque=True, chunk=100000):
    got = setups.copy_state(s)
    run = drivers.make_run(s, exact=exact, floor=floor, torque=torque)
    try:
        run.push(got)
        run.start(t0=0.0, tend=s["tend"], nstop=nstop, safety=s["safety"], dtmin=s["dtmin"])
        while True:
            st = run.query()
            if st.done:
                break
            run.advance(min(chunk, nstop))
        run.pull(got)
        return got, st
    finally:
        run.close()


@pytest.mark.parametrize("nx", [128, 1024])
def test_spicule_loop_exact_bitwise(gpu, oracle_lib, nx):
    """cfl_m -> mlw_m_bg -> torque -> bnd -> chkdav, 3000 iterations."""
    s = setups.spicule_1d(nx, seed=7)
    ref = setups.copy_state(s)
    t, ns, merr, nev = oracle.run_spicule_c(s, ref, 3000)
    got, st = _loop_gpu(s, 3000, exact=True)
    assert (st.t, st.ns, st.merr, st.n_floor) == (t, ns, merr, nev)
    assert_bitwise(s["names"], got, ref, "spicule loop")


def test_spicule_loop_with_floor_events_bitwise(gpu, oracle_lib):
    """A floor above the coronal density: chkdav raises cells and stops
    their flow every step; the event count and the state match."""
    s = setups.spicule_1d(512, seed=3)
    s["floor"] = float(np.quantile(s["state"][0], 0.5))
    ref = setups.copy_state(s)
    t, ns, merr, nev = oracle.run_spicule_c(s, ref, 400)
    got, st = _loop_gpu(s, 400, exact=True)
    assert nev > 1000
    assert (st.t, st.ns, st.merr, st.n_floor) == (t, ns, merr, nev)
    assert_bitwise(s["names"], got, ref, "floor loop")


@pytest.mark.parametrize("nsteps", [100, 1000])
def test_spicule_loop_fast_within_tolerance(gpu, oracle_lib, nsteps):
    """Fast policy against the oracle.  ro, pr, vy and by stay within 1e-10
    (relative L-inf).  vx gets 1e-4: in the corona of this model the uniform
    field's B^2/8pi is 1e6 times the gas pressure, so the last-bit rounding
    of the total energy in any step reappears 1e6 times larger in p and
    drives vx; injecting just that rounding into the oracle's own loop moves
    vx by ~1e-5 (test_oracle.py::test_spicule_corona_amplifies_energy_rounding).
    The exact policy equals the oracle bit for bit (the tests above)."""
    s = setups.spicule_1d(1024, seed=1)
    ref = setups.copy_state(s)
    oracle.run_spicule_c(s, ref, nsteps)
    got, st = _loop_gpu(s, nsteps, exact=False)
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) < (1e-4 if k == "vx" else 1e-10), k


def test_reference_spicule_run_exact_and_against_the_reference_output(gpu, oracle_lib):
    """The reference run (1024 cells, nstop = 100000, torque 30, floor 1e-9):
    the exact GPU loop equals the oracle bit for bit after 100000 steps, and
    both agree with the output the reference ships for that run: the time
    reached to 1e-7, the density and pressure profiles to 1e-3 and vx to
    5e-2 (relative L2).  vy and by are driven by the random torque, whose
    stream differs from the reference's, so only their amplitude is
    compared."""
    s = setups.spicule_1d()
    ref = setups.copy_state(s)
    t, ns, merr, nev = oracle.run_spicule_c(s, ref, 100000)
    got, st = _loop_gpu(s, 100000, exact=True)
    assert (st.t, st.ns, st.merr, st.n_floor) == (t, ns, merr, nev)
    assert_bitwise(s["names"], got, ref, "reference run")
    gold = dict(np.load(GOLD))
    t_ref = float(gold["t_records"][1])
    assert abs(st.t - t_ref) / t_ref < 1e-7
    for k, name in enumerate(s["names"]):
        r = gold[f"{name}_records"][1]
        d = np.linalg.norm(got[k] - r) / np.linalg.norm(r)
        if name in ("ro", "pr"):
            assert d < 1e-3, (name, d)
        elif name == "vx":
            assert d < 5e-2, (name, d)
        else:
            rms, rms_ref = np.sqrt(np.mean(got[k] ** 2)), np.sqrt(np.mean(r ** 2))
            assert 0.3 < rms / rms_ref < 3.0, (name, rms, rms_ref)


def test_run_spicule_files_and_restart(gpu, oracle_lib, tmp_path):
    """The model package on the device writes the reference's file set;
    a restart (mcont=1) from the last record continues the run exactly."""
    a = drivers.run_spicule(tmp_path / "a", nstop=300, dtout=1e-4, torque=False)
    files = sorted(p.name for p in (tmp_path / "a").iterdir())
    want = sorted([f"{k}.dac" for k in ("x", "bx", "bxm", "sc", "scm", "gx", "gxm", "rr", "rrm",
                                        "t", "ro", "pr", "vx", "vy", "by")] +
                  ["params.txt", "out.txt"])
    assert files == want
    tt = dac.dacopnr(tmp_path / "a" / "t.dac", 0).records
    assert a["records"] == tt.size and tt.size >= 3 and np.all(np.diff(tt) > 0)
    for k, name in enumerate(["ro", "pr", "vx", "vy", "by"]):
        f = dac.dacopnr(tmp_path / "a" / f"{name}.dac", 1)
        assert f.nx == tt.size
        assert np.array_equal(bits(f.last()), bits(a["state"][k]))
    assert (tmp_path / "a" / "out.txt").read_text().endswith("   ### normal stop ###\n")
    # the same 300 steps as 180 + a restart for 120
    b = drivers.run_spicule(tmp_path / "b", nstop=180, dtout=1e-4, torque=False)
    c = drivers.run_spicule(tmp_path / "c", nstop=120, dtout=1e-4, torque=False, mcont=1,
                            in_dir=tmp_path / "b")
    assert b["ns"] == 180 and c["ns"] == 120 and c["t"] == a["t"]
    assert_bitwise(["ro", "pr", "vx", "vy", "by"], c["state"], a["state"], "restart")
    t0 = dac.dacopnr(tmp_path / "c" / "t.dac", 0).records[0]
    assert t0 == dac.dacopnr(tmp_path / "b" / "t.dac", 0).records[-1]


def test_mhd_wind_loop_exact_bitwise(gpu, oracle_lib):
    """cans1d/md_mhdwind: the rotating magnetised wind on the stretched grid
    (1024 cells, held base values, free outer face), 2000 iterations of
    cfl_m -> mlw_m_bg -> bnd in one cluster launch, against the oracle."""
    s = setups.mhd_wind_1d(1024)
    ref = setups.copy_state(s)
    t, ns, merr, _ = oracle.run_1d(s, ref, 2000)
    got = setups.copy_state(s)
    out = drivers.run_resident(s, got, 2000, exact=True)
    assert out == (t, ns, merr, ns)
    for k, a, b in zip(s["names"], got, ref):
        assert np.array_equal(a, b), k
