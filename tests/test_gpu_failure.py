"""Failure detection of the device-resident loops, tested without a GPU fault:
the failure is made on the host, in the input state (a NaN or a negative
pressure in one interior cell), and the GPU only does arithmetic on it.

The reference's CFL scan skips a cell whose time step is not a number
(cfl_m.f: `if (dtq .lt. dt)`), and its loop carries on.  The resident loop
does the same by default and counts the warps whose CFL met a cell
with a non-positive density or pressure or a non-finite value
(cans_run_state.n_bad); with stop_on_bad the loop ends at the start of the
next iteration with merr = CANS_ERR_NONFINITE."""
import numpy as np
import pytest

from utrip_gb300 import capi, drivers, setups

pytestmark = pytest.mark.gpu

CASES = {
    "mlw_m3_2d": lambda: setups.orszag_tang(32),
    "roe_m3_2d": lambda: setups.orszag_tang(32, solver="roe_m3"),
    "mlw_m_3d": lambda: setups.turbulence_3d(16),
    "roe_m_3d": lambda: setups.turbulence_3d(16, solver="roe_m_3d"),
    "hlld_3d": lambda: setups.turbulence_3d(16, solver="hlld_3d"),
    "mlw_m_1d": lambda: setups.shock_tube_1d(64),
}


def poison(s, value, var="pr"):
    st = setups.copy_state(s)
    a = st[s["names"].index(var)]
    idx = tuple(n // 2 for n in a.shape)
    a[idx] = value
    return st


def run(s, st, nstop, stop):
    r = drivers.make_run(s, stop_on_bad=stop)
    try:
        r.push(st)
        r.start(t0=0.0, tend=1e30, nstop=nstop, safety=s["safety"], dtmin=s["dtmin"])
        r.advance(nstop + 1)
        q = r.query()
        return q.ns, q.merr, q.n_bad
    finally:
        r.close()


@pytest.mark.parametrize("case", sorted(CASES))
def test_healthy_run_counts_nothing(gpu, case):
    s = CASES[case]()
    ns, merr, nbad = run(s, setups.copy_state(s), 20, stop=True)
    assert (ns, merr, nbad) == (20, 0, 0)


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("value", [float("nan"), -1.0e3])
def test_bad_cell_is_counted_and_the_loop_goes_on(gpu, case, value):
    s = CASES[case]()
    ns, merr, nbad = run(s, poison(s, value), 5, stop=False)
    assert ns == 5 and merr == 0 and nbad > 0


@pytest.mark.parametrize("case", sorted(CASES))
def test_stop_on_bad_ends_the_loop(gpu, case):
    s = CASES[case]()
    ns, merr, nbad = run(s, poison(s, float("nan")), 5, stop=True)
    assert merr == capi.CANS_ERR_NONFINITE and nbad > 0 and ns == 1


def test_batch_counts_per_run(gpu):
    runs = [setups.shear_layer(32, beta=b, seed=k) for k, b in enumerate((0.5, 1.0))]
    b = capi.Batch(runs)
    try:
        b.push(0, setups.copy_state(runs[0]))
        b.push(1, poison(runs[1], float("nan")))
        b.start(nstop=4, safety=0.4, dtmin=1e-10)
        b.advance(5)
        q0, q1 = b.query(0), b.query(1)
        assert q0.n_bad == 0 and q1.n_bad > 0 and q0.ns == q1.ns == 4
    finally:
        b.close()
