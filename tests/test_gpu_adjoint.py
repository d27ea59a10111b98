"""GPU tests of the discrete adjoint of the 2-D mlw_m3 run (the reverse sweep
with binomial checkpointing, cans_run_adjoint): the transposed boundary fill
passes the dot-product test, the gradient does not depend on the number of
stored states, and directional derivatives match FP64 central finite
differences of both the GPU forward and the CPU oracle (frozen dt sequence)."""
import numpy as np
import pytest

import oracle
from utrip_gb300 import capi, drivers, setups

pytestmark = pytest.mark.gpu
H = 1e-6
EPS = float(np.finfo(np.float64).eps)


def _close(ad, fd, J, h=H):
    """Within 1e-6 of the central difference, beyond the difference's own
    rounding error (a few ulps of J divided by 2h)."""
    return abs(ad - fd) <= 1e-6 * abs(fd) + 8.0 * EPS * abs(J) / (2.0 * h)


def _setup(n=32, ny=28, beta=1.0, seed=4, qav=0.0):
    """Shear layer whose ghost cells already obey its boundary program (the
    set-up fills them from the analytic profile), so that a perturbation of
    the interior extended by the same program moves along a straight line.

    The artificial viscosity q = qav dxm max(0, |dv| - 1e-4) switches on
    where a velocity jump crosses 1e-4; the shear layer has jumps passing
    through that value, so J has kinks close to the base point and a
    central difference with h = 1e-6 can straddle one.  The smooth checks
    therefore run with qav = 0; the viscosity path is checked on a state
    whose jumps are far from the switch, and the kinks by their own test."""
    s = setups.shear_layer(n, beta=beta, ny=ny, seed=seed)
    s["qav"] = qav
    oracle.apply_bc_program(s["state"], s["bc"], s["margin"], s)
    return s


def _fd(s, z, dts, h):
    Js = []
    for sg in (h, -h):
        r = _run(s, [np.asfortranarray(a + sg * b) for a, b in zip(s["state"], z)])
        try:
            Js.append(r.objective(dts))
        finally:
            r.close()
    return (Js[0] - Js[1]) / (2 * h), Js


def _run(s, state=None, exact=False):
    run = drivers.make_run(s, exact=exact)
    run.push(state if state is not None else s["state"])
    return run


def _directional_state(s, d, h):
    """P_0 + h d on the interior vy, ghosts refilled by the boundary program."""
    st = setups.copy_state(s)
    st[3][1:-1, 1:-1] += h * d
    oracle.apply_bc_program(st, s["bc"], s["margin"], s)
    return st


def _extend(s, d):
    """The direction d on the interior vy as a full state (ghosts by the same
    linear boundary program)."""
    z = [np.zeros_like(a) for a in s["state"]]
    z[3][1:-1, 1:-1] = d
    oracle.apply_bc_program(z, s["bc"], s["margin"], s)
    return z


def test_bc_transpose_dot_product(gpu, oracle_lib):
    s = _setup()
    rng = np.random.default_rng(1)
    lam = [np.asfortranarray(rng.standard_normal(a.shape)) for a in s["state"]]
    d = [np.asfortranarray(rng.standard_normal(a.shape)) for a in s["state"]]
    bd = [a.copy(order="F") for a in d]
    oracle.apply_bc_program(bd, s["bc"], s["margin"], s)
    run = _run(s)
    try:
        lt = [a.copy(order="F") for a in lam]
        run.bc_transpose(lt)
    finally:
        run.close()
    lhs = sum(float(np.sum(a * b)) for a, b in zip(lt, d))
    rhs = sum(float(np.sum(a * b)) for a, b in zip(lam, bd))
    assert abs(lhs - rhs) <= 1e-12 * abs(rhs)


def test_gradient_independent_of_stored_states(gpu):
    s = _setup()
    run = _run(s)
    try:
        dts, J0 = run.record_dts(24)
        ref = None
        nf_prev = None
        for nsnap in (2, 3, 5, 25):
            J, g, nf = run.adjoint(dts, nsnap=nsnap)
            assert J == J0
            if ref is None:
                ref = g
            else:
                for a, b in zip(g, ref):
                    assert np.array_equal(a, b)
            if nf_prev is not None:
                assert nf <= nf_prev  # more snapshots never cost more steps
            nf_prev = nf
        # one stored state per step: each step runs forward once, and the raw
        # output of the step being reversed comes from the state after it,
        # except for the last step, which runs once more
        assert nf_prev == 24
    finally:
        run.close()


def test_directional_derivative_matches_gpu_finite_differences(gpu):
    s = _setup()
    nsteps = 40
    run = _run(s)
    try:
        dts, _ = run.record_dts(nsteps)
        J, grad, _ = run.adjoint(dts, nsnap=6)
    finally:
        run.close()
    rng = np.random.default_rng(5)
    for _ in range(4):
        d = rng.standard_normal((s["state"][0].shape[0] - 2, s["state"][0].shape[1] - 2))
        ad = sum(float(np.sum(g * e)) for g, e in zip(grad, _extend(s, d)))
        Js = []
        for h in (H, -H):
            r = _run(s, _directional_state(s, d, h))
            try:
                Js.append(r.objective(dts))
            finally:
                r.close()
        fd = (Js[0] - Js[1]) / (2 * H)
        assert _close(ad, fd, J), (ad, fd)


def test_directional_derivative_matches_oracle_finite_differences(gpu, oracle_lib):
    s = _setup(n=24, ny=20)
    nsteps = 20
    run = _run(s)
    try:
        dts, _ = run.record_dts(nsteps)
        _, grad, _ = run.adjoint(dts, nsnap=4)
    finally:
        run.close()

    def oracle_J(st):
        for dt in dts:
            oracle.step_2d(s, st, dt)
            oracle.apply_bc_program(st, s["bc"], s["margin"], s)
        bx, by, bz = st[5], st[6], st[7]
        w = np.outer(s["dx"], s["dy"])[1:-1, 1:-1]
        e = (bx * bx + by * by + bz * bz)[1:-1, 1:-1]
        return float(np.sum(e * w)) / np.pi / 8.0

    rng = np.random.default_rng(9)
    for _ in range(2):
        d = rng.standard_normal((24, 20))
        ad = sum(float(np.sum(g * e)) for g, e in zip(grad, _extend(s, d)))
        jp, jm = oracle_J(_directional_state(s, d, H)), oracle_J(_directional_state(s, d, -H))
        fd = (jp - jm) / (2 * H)
        assert _close(ad, fd, jp), (ad, fd)


def test_beta_derivative(gpu):
    """p = 0.625 beta in every cell, so dJ/dbeta = 0.625 sum(dJ/dp)."""
    beta = 1.0
    s = _setup(beta=beta)
    nsteps = 30
    run = _run(s)
    try:
        dts, _ = run.record_dts(nsteps)
        _, grad, _ = run.adjoint(dts, nsnap=8)
    finally:
        run.close()
    ad = 0.625 * float(np.sum(grad[1]))
    Js = []
    for h in (H, -H):
        sb = _setup(beta=beta + h)
        r = _run(sb)
        try:
            Js.append(r.objective(dts))
        finally:
            r.close()
    fd = (Js[0] - Js[1]) / (2 * H)
    assert _close(ad, fd, Js[0]), (ad, fd)


def test_viscosity_path_matches_finite_differences(gpu):
    """A random state whose velocity jumps are all far above 1e-4: every AV
    face is on and stays on, the objective is smooth there."""
    s = setups.random_state(30, 26, seed=3)
    oracle.apply_bc_program(s["state"], s["bc"], s["margin"], s)
    run = _run(s)
    try:
        dts, _ = run.record_dts(5)
        _, grad, _ = run.adjoint(dts, nsnap=3)
    finally:
        run.close()
    rng = np.random.default_rng(2)
    for v in range(8):
        z = [np.zeros_like(a) for a in s["state"]]
        z[v][1:-1, 1:-1] = rng.standard_normal((28, 24))
        oracle.apply_bc_program(z, s["bc"], s["margin"], s)
        ad = sum(float(np.sum(g * e)) for g, e in zip(grad, z))
        fd, (jp, _) = _fd(s, z, dts, H)
        assert _close(ad, fd, jp), (s["names"][v], ad, fd)


def test_viscosity_kinks_on_the_shear_layer(gpu):
    """With qav = 3 the shear-layer objective has kinks within 1e-6 of the
    base point: the one-sided differences at h = 1e-6 disagree, the adjoint
    (the derivative of the branches taken at the base point) lies between
    them, and a central difference with h = 1e-8 recovers it."""
    s = _setup(qav=3.0)
    run = _run(s)
    try:
        dts, J0 = run.record_dts(40)
        _, grad, _ = run.adjoint(dts, nsnap=6)
    finally:
        run.close()
    d = np.random.default_rng(5).standard_normal((32, 28))
    z = _extend(s, d)
    ad = sum(float(np.sum(g * e)) for g, e in zip(grad, z))
    _, (jp, jm) = _fd(s, z, dts, H)
    fwd, bwd = (jp - J0) / H, (J0 - jm) / H
    assert abs(fwd - bwd) > 1e-3 * abs(ad)
    assert min(fwd, bwd) <= ad <= max(fwd, bwd)
    fd8, _ = _fd(s, z, dts, 1e-8)
    assert abs(fd8 - ad) <= 1e-5 * abs(ad)


def _frozen_fd(run, s, z, dts, h):
    """Central differences of the held-branch objective along z: second
    order at h, and fourth order from h and 2h (Richardson), with the
    switch crossings counted at +h and -h."""
    J, fl = {}, {}
    for m in (1, -1, 2, -2):
        run.push([np.asfortranarray(a + m * h * b) for a, b in zip(s["state"], z)])
        J[m], fl[m] = run.objective_frozen_av(dts)
    run.push(s["state"])
    d1 = (J[1] - J[-1]) / (2 * h)
    d2 = (J[2] - J[-2]) / (4 * h)
    return d1, (4.0 * d1 - d2) / 3.0, fl[1], fl[-1]


def test_frozen_branch_record_leaves_the_run_unchanged(gpu):
    """Recording the viscosity branches runs the same step: holding them at
    the base point reproduces J bit for bit with no switch crossed."""
    s = _setup(n=64, ny=64, qav=3.0)
    run = _run(s)
    try:
        dts, J = run.record_dts(60)
        run.av_record(dts)
        assert run.objective(dts) == J
        Jf, nflip = run.objective_frozen_av(dts)
        assert Jf == J and nflip == 0
    finally:
        run.close()


def test_frozen_branch_finite_differences_reduced_c5(gpu):
    """The adjoint configuration reduced to 64^2 and 200 steps at qav = 3:
    with every viscosity face held at its base-point branch the objective is
    smooth, and the adjoint matches its central differences (h = 1e-6,
    fourth order) within 1e-6 on smooth seeded directions of the vy field,
    and dJ/dbeta the same way.  The unheld objective crosses switches
    within h on these directions (counted), which is why its own central
    differences miss the adjoint there."""
    s = _setup(n=64, ny=64, qav=3.0)
    run = _run(s)
    try:
        dts, J = run.record_dts(200)
        _, grad, _ = run.adjoint(dts, nsnap=12)
        run.av_record(dts)
        rng = np.random.default_rng(5)
        k = np.fft.fftfreq(64, d=1.0 / 64)
        KX, KY = np.meshgrid(k, k, indexing="ij")
        mask = (KX ** 2 + KY ** 2) <= 64.0
        for _ in range(4):
            spec = np.where(mask, rng.standard_normal((64, 64)) +
                            1j * rng.standard_normal((64, 64)), 0.0)
            d = np.real(np.fft.ifft2(spec))
            d /= np.sqrt(np.mean(d ** 2))
            z = _extend(s, d)
            ad = sum(float(np.sum(g * e)) for g, e in zip(grad, z))
            fd2, fd4, fp, fm = _frozen_fd(run, s, z, dts, H)
            assert _close(ad, fd4, J), (ad, fd4, fd2, fp, fm)
        # dJ/dbeta: p = 0.625 beta in every cell, held branches
        ad = 0.625 * float(np.sum(grad[1]))
        Jb = {}
        for m in (1, -1, 2, -2):
            run.push(_setup(n=64, ny=64, beta=1.0 + m * H, qav=3.0)["state"])
            Jb[m], _ = run.objective_frozen_av(dts)
        d1 = (Jb[1] - Jb[-1]) / (2 * H)
        fd4 = (4.0 * d1 - (Jb[2] - Jb[-2]) / (4 * H)) / 3.0
        assert _close(ad, fd4, J), (ad, fd4, d1)
    finally:
        run.close()


def test_recorded_branches_hold_the_oracle_to_the_same_run(gpu, oracle_lib):
    """The branches the GPU records (cans_run_av_branches) in the format the
    oracle holds: a 64^2 shear layer at qav = 3, 40 steps in the exact
    policy; the oracle's run holding the GPU's branches equals the GPU's
    held run bit for bit, and so does the oracle's plain run (on the base
    trajectory the held branches are its own)."""
    s = _setup(n=64, ny=64, qav=3.0)
    run = _run(s, exact=True)
    try:
        dts, J = run.record_dts(40)
        run.av_record(dts)
        Jh, nflip = run.objective_frozen_av(dts)
        rec = [run.av_branches(k) for k in range(40)]
    finally:
        run.close()
    assert Jh == J and nflip == 0
    assert any(int(np.count_nonzero(r & 1)) for r in rec)  # viscosity faces active
    final = {}
    for mode in (0, 2):
        st = setups.copy_state(s)
        try:
            for k, dt in enumerate(dts):
                oracle_lib.set_av_branch(mode, rec[k])
                oracle_lib.step_2d(s, st, dt)
                oracle_lib.apply_bc_program(st, s["bc"], s["margin"], s)
        finally:
            oracle_lib.set_av_branch(0)
        final[mode] = st
        w = np.outer(s["dx"], s["dy"])[1:-1, 1:-1]
        e = (st[5] ** 2 + st[6] ** 2 + st[7] ** 2)[1:-1, 1:-1]
        Jo = float(np.sum(e * w)) / np.pi / 8.0
        assert abs(Jo - J) <= 1e-13 * abs(J), (mode, Jo, J)  # summation order only
    for a, b in zip(final[2], final[0]):
        assert np.array_equal(a, b)


def test_frozen_branch_needs_a_record(gpu):
    s = _setup(qav=3.0)
    run = _run(s)
    try:
        dts, _ = run.record_dts(10)
        with pytest.raises(capi.CansError):
            run.objective_frozen_av(dts)
        run.av_record(dts[:5])
        with pytest.raises(capi.CansError):  # longer than the record
            run.objective_frozen_av(dts)
        Jf, _ = run.objective_frozen_av(dts[:5])
        assert np.isfinite(Jf)
    finally:
        run.close()


def test_reverse_sweep_in_fp64_and_double_float_agree(gpu):
    """The reverse arithmetic (double-float by default, FP64 on request)
    changes the gradient only at the level of its rounding: within 1e-11 of
    the largest component, with qav = 3 (every viscosity path live)."""
    s = _setup(n=40, ny=36, qav=3.0)
    run = _run(s)
    try:
        dts, J = run.record_dts(60)
        Jd, gd, _ = run.adjoint(dts, nsnap=8)
        run.set_adjoint_df64(False)
        J6, g6, _ = run.adjoint(dts, nsnap=8)
    finally:
        run.close()
    assert Jd == J6 == J
    for a, b in zip(gd, g6):
        scale = max(float(np.max(np.abs(b))), 1e-300)
        assert float(np.max(np.abs(a - b))) <= 1e-11 * scale


def test_adjoint_rejects_other_solvers(gpu):
    s = setups.random_state_3d(12, 12, 12, seed=1)
    run = drivers.make_run(s)
    try:
        with pytest.raises(capi.CansError):
            run.record_dts(3)
    finally:
        run.close()
