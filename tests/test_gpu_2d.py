"""GPU parity of the 2-D mLW path against the CPU oracle, through the C ABI.

Exact policy: bit-identical to the oracle (same operations, same order, no
FMA contraction), after one step and after 100 steps of the full loop.
Fast policy: relative L-infinity error per variable <= 1e-10 after 100 steps
(the tolerance the target states), relative to max|reference| of that
variable.
"""
import numpy as np
import pytest

import oracle
from utrip_gb300 import capi, drivers, setups

pytestmark = pytest.mark.gpu
TOL_FAST = 1e-10


def rel_linf(a, b):
    scale = float(np.max(np.abs(b)))
    if scale == 0.0:
        return float(np.max(np.abs(a - b)))
    return float(np.max(np.abs(a - b))) / scale


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


@pytest.mark.parametrize("solver", ["mlw_m3", "mlw_m"])
@pytest.mark.parametrize("shape", [(18, 14), (37, 29), (130, 70), (67, 131)])
def test_one_step_exact_bitwise(gpu, oracle_lib, solver, shape):
    s = setups.random_state(*shape, seed=shape[0], solver=solver)
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_2d(s, ref, 0.4)
    oracle.step_2d(s, ref, dt)
    got = setups.copy_state(s)
    gpu.set_exact(True)
    drivers._step(s, got, dt)
    assert_same(s["names"], got, ref, "step")


@pytest.mark.parametrize("solver", ["mlw_m3", "mlw_m"])
def test_cfl_exact(gpu, oracle_lib, solver):
    s = setups.random_state(45, 33, seed=9, solver=solver)
    gpu.set_exact(True)
    ref = oracle.cfl_2d(s, s["state"], 0.4)
    got = drivers._cfl(s, s["state"], 0.4)
    assert got == ref
    _, merr = drivers._cfl(dict(s, dtmin=1.0), s["state"], 0.4)
    assert merr == 9001


def test_every_boundary_kind_bitwise(gpu, oracle_lib):
    rng = np.random.default_rng(21)
    q = np.asfortranarray(rng.standard_normal((11, 9)))
    dxm = np.linspace(0.1, 0.2, 11)
    dym = np.linspace(0.1, 0.3, 9)
    for kind in range(8):
        for axis in (0, 1):
            for mbnd in (0, 1):
                for margin in (1, 2):
                    a = q.copy(order="F")
                    b = q.copy(order="F")
                    oracle.bd(kind, axis, mbnd, margin, a, q0=0.75, dxm=dxm if axis == 0 else dym)
                    capi.bd(kind, axis, mbnd, margin, b, q0=0.75, dxm=dxm if axis == 0 else dym)
                    assert np.array_equal(a, b), (kind, axis, mbnd, margin)


@pytest.mark.parametrize("case", ["ot64", "shear48x40", "random70x50"])
def test_resident_loop_exact_100_steps(gpu, oracle_lib, case):
    if case == "ot64":
        s = setups.orszag_tang(64)
    elif case == "shear48x40":
        s = setups.shear_layer(48, beta=0.5, ny=40)
    else:
        s = setups.random_state(70, 50, seed=2)
    ref = setups.copy_state(s)
    t_ref, ns_ref, merr_ref, dts = oracle.run_2d(s, ref, 100)
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, 100, exact=True)
    # Orszag-Tang reaches tend = pi/2 before 100 steps, in both
    assert (ns, merr, nexec) == (ns_ref, merr_ref, ns_ref)
    assert t == t_ref
    assert_same(s["names"], got, ref, case)


@pytest.mark.parametrize("solver", ["mlw_m3", "mlw_m"])
def test_resident_loop_fast_100_steps_within_tolerance(gpu, oracle_lib, solver):
    s = setups.orszag_tang(96, solver=solver)
    ref = setups.copy_state(s)
    oracle.run_2d(s, ref, 100)
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, 100, exact=False)
    assert ns == 100 and nexec == 100
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) <= TOL_FAST, (k, rel_linf(a, b))


def test_literal_drop_in_loop_matches_oracle(gpu, oracle_lib):
    s = setups.shear_layer(40, beta=2.0, ny=36)
    ref = setups.copy_state(s)
    oracle.run_2d(s, ref, 12)
    for resident in (False, True):
        got = setups.copy_state(s)
        gpu.set_exact(True)
        t, ns, merr, dts = drivers.run_literal(s, got, 12, resident=resident)
        assert ns == 12
        assert_same(s["names"], got, ref, f"literal resident={resident}")


N_TILES_2D = 6  # 32x16, 32x8, 16x16, 64x8, 32x9 (one row per thread), 32x10
# tiles 6 and 7 are the y-marching kernel of the fast mlw_m3 step, its
# segments balanced per SM or by waves (the exact policy takes the 32x9 tile
# in their place)
MARCH_TILES = (6, 7)


@pytest.mark.parametrize("solver", ["mlw_m3", "mlw_m"])
def test_all_tiles_agree_bitwise(gpu, oracle_lib, solver):
    s = setups.random_state(150, 77, seed=4, solver=solver)
    ref = setups.copy_state(s)
    dt, _ = oracle.cfl_2d(s, ref, 0.4)
    oracle.step_2d(s, ref, dt)
    for tile in range(N_TILES_2D):
        run = drivers.make_run(s, exact=True, tile=tile)
        try:
            run.push(setups.copy_state(s))
            run.step(dt, apply_bc=False)
            got = run.pull()
        finally:
            run.close()
        assert_same(s["names"], got, ref, f"tile {tile}")


def test_loop_stops_on_dtmin_like_reference(gpu, oracle_lib):
    s = dict(setups.orszag_tang(32), dtmin=0.05)
    ref = setups.copy_state(s)
    r = oracle.run_2d(s, ref, 50)
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, 50, exact=True)
    assert (t, ns, merr) == (r[0], r[1], r[2]) and merr == 9001 and nexec == 0


def test_tend_stops_loop_like_reference(gpu, oracle_lib):
    s = setups.orszag_tang(40)
    ref = setups.copy_state(s)
    t_ref, ns_ref, _, _ = oracle.run_2d(s, ref, 10 ** 6, tend=0.05)
    got = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, got, 10 ** 6, tend=0.05, exact=True)
    assert t == t_ref and ns == ns_ref and nexec == ns_ref
    assert_same(s["names"], got, ref, "tend")


def test_pause_on_output_time(gpu):
    s = setups.orszag_tang(32)
    run = drivers.make_run(s, exact=False)
    try:
        run.push(setups.copy_state(s))
        run.start(tend=1.0, nstop=10 ** 6, safety=0.4, dtmin=1e-10, dtout=0.1,
                  pause_on_output=True)
        run.advance(500)
        st = run.query()
        assert st.pause == 1 and not st.done
        assert int((st.t - st.dt) / 0.1) < int(st.t / 0.1)
        n1 = st.nexec
        run.resume()
        run.advance(500)
        st2 = run.query()
        assert st2.nexec > n1
    finally:
        run.close()


def test_launch_counter_counts_graph_kernels(gpu):
    s = setups.orszag_tang(32)
    c0 = capi.launch_count()
    got = setups.copy_state(s)
    drivers.run_resident(s, got, 64, exact=False, chunk=32)
    # 2 kernels per iteration (the step, then the boundary program with the
    # frame CFL and the loop bookkeeping) plus start-up
    assert capi.launch_count() - c0 >= 2 * 64


def test_full_size_512_fast_vs_exact_and_conservation(gpu):
    s = setups.orszag_tang(512)
    a = setups.copy_state(s)
    b = setups.copy_state(s)
    ta = drivers.run_resident(s, a, 100, exact=True)
    tb = drivers.run_resident(s, b, 100, exact=False)
    assert ta[1] == tb[1] == 100
    for k, x, y in zip(s["names"], b, a):
        assert rel_linf(x, y) <= TOL_FAST, (k, rel_linf(x, y))
    # periodic box: total mass is conserved to rounding
    m0 = s["state"][0][1:-1, 1:-1].sum()
    assert abs(a[0][1:-1, 1:-1].sum() - m0) <= 1e-12 * m0


def test_oblique_shock_tube_to_tend_exact_bitwise(gpu, oracle_lib):
    """cans2d/md_mhd3shktb at the reference's 64 x 64: the whole run to
    t = 0.1 (cfl_m3 -> mlw_m3 -> free boundaries) on the device."""
    s = setups.oblique_shock_tube_2d(64)
    ref = setups.copy_state(s)
    t, ns, merr, _ = oracle.run_2d(s, ref, 10 ** 6)
    got = setups.copy_state(s)
    out = drivers.run_resident(s, got, 10 ** 6, exact=True)
    assert out == (t, ns, merr, ns) and t >= 0.1
    for k, a, b in zip(s["names"], got, ref):
        assert np.array_equal(a, b), k


@pytest.mark.parametrize("tile", MARCH_TILES)
@pytest.mark.parametrize("make,steps", [
    (lambda: setups.orszag_tang(64), 100),
    (lambda: setups.shear_layer(130, beta=0.5, seed=2), 100),
    (lambda: setups.random_state(53, 41, seed=7), 20),
])
def test_fast_marching_tile_against_oracle(gpu, oracle_lib, make, steps, tile):
    """The y-marching tile of the fast policy (32-column strips taking their
    rows in chunks, the symmetric momentum flux formed once) holds the fast
    policy's 1e-10 against the oracle, ragged strips and segments included."""
    s = make()
    ref = setups.copy_state(s)
    t_ref, ns_ref, _, _ = oracle.run_2d(s, ref, steps)
    got = setups.copy_state(s)
    run = drivers.make_run(s, tile=tile)
    try:
        t, ns, merr, nexec = drivers.run_resident(s, got, steps, run=run)
    finally:
        run.close()
    assert merr == 0 and ns == ns_ref and nexec == ns
    for k, a, b in zip(s["names"], got, ref):
        assert rel_linf(a, b) <= TOL_FAST, (k, rel_linf(a, b))


def test_marching_tile_falls_back_for_exact_and_mlw_m(gpu, oracle_lib):
    """Asked of the exact policy or of mlw_m, tiles 6 and 7 run the 32x9
    tile: still bit for bit."""
    for solver in ("mlw_m3", "mlw_m"):
        s = setups.random_state(70, 45, seed=9, solver=solver)
        ref = setups.copy_state(s)
        dt, _ = oracle.cfl_2d(s, ref, 0.4)
        oracle.step_2d(s, ref, dt)
        run = drivers.make_run(s, exact=True, tile=MARCH_TILES[1])
        try:
            run.push(setups.copy_state(s))
            run.step(dt, apply_bc=False)
            got = run.pull()
        finally:
            run.close()
        assert_same(s["names"], got, ref, solver)
