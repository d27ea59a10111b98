"""Many 1-D runs advanced together (cans_run_advance_group): the spicule
model of cans1d/md_spicule/hdmlw at several plasma betas, as the
reference's parameter studies run it, and MHD shock tubes of several sizes.
The group only changes which SMs a run's cells live on, so in the exact
policy every run of a group ends bit for bit where the same run advanced
alone ends (state and loop state).  In the fast policy the group kernel is
another instance of the same loop, and the compiler may fuse its
multiply-adds differently: there the runs agree to the fast policy's
tolerances (1e-10 relative; vx of the spicule 1e-4, whose corona amplifies
one rounding of the energy that much, as its fast-policy test states) and
take the same number of steps."""
import numpy as np
import pytest

from utrip_gb300 import capi, drivers, setups

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.int64)


def rel_linf(a, b):
    scale = float(np.max(np.abs(b))) or 1.0
    return float(np.max(np.abs(a - b))) / scale


def loop_state(st):
    return (st.t, st.dt, st.ns, st.nexec, st.merr, st.done, st.pause, st.n_floor, st.n_bad)


def start(s, exact):
    run = drivers.make_run(s, exact=exact)
    run.push(setups.copy_state(s))
    run.start(tend=s["tend"], nstop=s.get("nstop", 10 ** 9), safety=s["safety"],
              dtmin=s["dtmin"])
    return run


def compare_group_with_single(setups_list, iters, exact, chunks=1):
    alone = []
    for s in setups_list:
        run = start(s, exact)
        try:
            for _ in range(chunks):
                run.advance(iters)
            alone.append((run.pull(), loop_state(run.query())))
        finally:
            run.close()
    runs = [start(s, exact) for s in setups_list]
    try:
        for _ in range(chunks):
            capi.Run.advance_group(runs, iters)
        grouped = [(r.pull(), loop_state(r.query())) for r in runs]
    finally:
        for r in runs:
            r.close()
    for k, (s, (ga, gs), (aa, as_)) in enumerate(zip(setups_list, grouped, alone)):
        if exact:
            assert gs == as_, (k, gs, as_)
            for name, a, b in zip(s["names"], ga, aa):
                assert np.array_equal(bits(a), bits(b)), (k, name)
            continue
        # ns, nexec, merr, done, pause, chkdav events, bad warps; t and dt
        assert gs[2:] == as_[2:], (k, gs, as_)
        assert abs(gs[0] - as_[0]) <= 1e-10 * abs(as_[0]), (k, gs[0], as_[0])
        for name, a, b in zip(s["names"], ga, aa):
            tol = 1e-4 if (name == "vx" and s["solver"] == "mlw_m_bg_1d") else 1e-10
            assert rel_linf(a, b) <= tol, (k, name, rel_linf(a, b))
    return alone


@pytest.mark.parametrize("exact", [False, True])
def test_spicule_beta_group_equals_runs_alone(gpu, exact):
    """Five spicule runs (plasma beta 0.3, 1, 3 at the base, two grid sizes,
    torque and floor on), 300 loop iterations in two group calls."""
    group = [setups.spicule_1d(1024, beta=b, seed=k, torque=30.0 + 5 * k)
             for k, b in enumerate((0.3, 1.0, 3.0))]
    group += [setups.spicule_1d(n, beta=2.0, seed=7) for n in (512, 700)]
    alone = compare_group_with_single(group, 150, exact, chunks=2)
    assert all(st[3] == 300 for _, st in alone)  # every run took 300 iterations


@pytest.mark.parametrize("exact", [False, True])
def test_shock_tube_group_to_tend_equals_runs_alone(gpu, exact):
    """MHD shock tubes of 1024, 300 and 2000 cells run to t = 0.1 in one group
    call: runs of different lengths end at their own tend."""
    group = [setups.shock_tube_1d(n) for n in (1024, 300, 2000)]
    alone = compare_group_with_single(group, 10 ** 6, exact)
    steps = [st[2] for _, st in alone]
    assert len(set(steps)) == 3 and all(st[5] == 1 for _, st in alone)
    assert all(st[0] >= 0.1 for _, st in alone)


def test_group_rejects_mixed_or_repeated_runs(gpu):
    bg = start(setups.spicule_1d(256), False)
    mhd = start(setups.shock_tube_1d(256), False)
    two = start(setups.orszag_tang(16), False)
    exact = start(setups.spicule_1d(256), True)
    try:
        for runs in ([bg, mhd], [mhd, two], [bg, bg], [bg, exact]):
            with pytest.raises(capi.CansError) as e:
                capi.Run.advance_group(runs, 5)
            assert e.value.code == capi.CANS_ERR_ARG
        with pytest.raises(ValueError):
            capi.Run.advance_group([], 5)
    finally:
        for r in (bg, mhd, two, exact):
            r.close()
