"""CPU oracle of the CANS mLW step -- TEST INFRASTRUCTURE ONLY.

ctypes binding of the C restatement in this directory (libcansoracle.so) with
the same Python signatures as utrip_gb300.capi, plus a restatement of the
model-package time loop (cans2d/md_mhdkh/hdmlw/main.f:160-219).  Only the
tests, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use it.

Parity status: the 1-D spicule loop (mlw_m_bg, chkdav, torque, bnd) is
pinned against the output the reference ships for its spicule run
(tests/golden/spicule_reference.npz, checked in tests/test_oracle.py and
tests/test_dac.py).  The mLW step in 1-D, 2-D and 3-D (mlw_m, mlw_m3), the
Roe-MUSCL step in 1-D, 2-D and 3-D and the HLLD engine are pinned against
the reference's own known answer for its shock-tube model, the exact
solution of cans1d/md_shktb/hdmlw/shktb_analytic.pro (shktb_analytic.py
here; tests/test_sod.py).  No output of the Fortran itself exists for these
(no Fortran compiler is available and the reference ships no golden vectors
for them); beyond the known answer they are pinned by invariants and frozen
fixtures in tests/golden/.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libcansoracle.so"
_lib = None
_dp = C.POINTER(C.c_double)
_ldp = C.POINTER(C.c_longdouble)
_ip = C.POINTER(C.c_int)
BD_PER, BD_SPP, BD_SPN, BD_SMP, BD_SMN, BD_FRE, BD_CNS, BD_FRD = range(8)


def build() -> Path:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        lib = C.CDLL(str(LIB))
        d, i = C.c_double, C.c_int
        lib.oracle_mlw_m3_2d.argtypes = [_dp] * 9 + [d, d, d, _dp, _dp, i, _dp, _dp, i]
        lib.oracle_mlw_m_2d.argtypes = [_dp] * 7 + [d, d, d, _dp, _dp, i, _dp, _dp, i]
        lib.oracle_mlw_m3_g_2d.argtypes = [_dp] * 9 + [d, d, d] + [_dp] * 6 + [i, _dp, _dp, i]
        lib.oracle_mlw_m_g_2d.argtypes = [_dp] * 7 + [d, d, d] + [_dp] * 6 + [i, _dp, _dp, i]
        lib.oracle_cfl_m3_2d.argtypes = [_dp, d, d, _ip, d] + [_dp] * 8 + [_dp, i, _dp, i]
        lib.oracle_mlw_m3_ge_2d.argtypes = [_dp] * 9 + [d, d, d] + [_dp] * 8 + [i, _dp, _dp, i]
        lib.oracle_mlw_m_ge_2d.argtypes = [_dp] * 7 + [d, d, d] + [_dp] * 8 + [i, _dp, _dp, i]
        lib.oracle_cfl_m3_e_2d.argtypes = [_dp, d, d, _ip, d] + [_dp] * 9 + [_dp, i, _dp, i]
        lib.oracle_cfl_m_2d.argtypes = [_dp, d, d, _ip, d] + [_dp] * 6 + [_dp, i, _dp, i]
        lib.oracle_bd_2d.argtypes = [i, i, i, i, _dp, d, _dp, i, i]
        lib.oracle_bd_1d.argtypes = [i, i, i, _dp, d, _dp, i]
        lib.oracle_bd_3d.argtypes = [i, i, i, i, _dp, d, _dp, i, i, i]
        lib.oracle_bbtoaa_2d.argtypes = [_dp, _dp, _dp, _dp, _dp, i, i, i]
        lib.oracle_grdrdy.argtypes = [_dp, _dp, _dp, _dp, i]
        lib.oracle_mlw_m_1d.argtypes = [_dp] * 7 + [d, d, d, _dp, _dp, i]
        lib.oracle_cfl_m_1d.argtypes = [_dp, d, d, _ip, d] + [_dp] * 6 + [_dp, i]
        lib.oracle_mlw_m_3d.argtypes = [_dp] * 8 + [d, d, d, _dp, _dp, i, _dp, _dp, i, _dp, _dp, i]
        lib.oracle_mlw_m_g_3d.argtypes = ([_dp] * 8 + [d, d, d] + [_dp] * 6 +
                                          [_dp, _dp, i, _dp, _dp, i, _dp, _dp, i])
        lib.oracle_mlw_m_e_3d.argtypes = ([_dp] * 8 + [d, d, d] + [_dp] * 2 +
                                          [_dp, _dp, i, _dp, _dp, i, _dp, _dp, i])
        lib.oracle_cfl_m_e_3d.argtypes = [_dp, d, d, _ip, d] + [_dp] * 9 + [_dp, i, _dp, i,
                                                                              _dp, i]
        lib.oracle_cfl_m_3d.argtypes = [_dp, d, d, _ip, d] + [_dp] * 8 + [_dp, i, _dp, i, _dp, i]
        lib.oracle_roe_m_3d.argtypes = [_dp] * 8 + [d, d, _dp, i, _dp, i, _dp, i]
        lib.oracle_roe_m3_2d.argtypes = [_dp] * 9 + [d, d, _dp, i, _dp, i]
        lib.oracle_roe_m_1d.argtypes = [_dp] * 7 + [d, d, _dp, i]
        lib.oracle_hlld_engine_3d.argtypes = [_dp] * 8 + [d, d, d, _dp, i, _dp, i, _dp, i, _ip]
        lib.oracle_mlw_m_bg_1d.argtypes = [_dp] * 7 + [d, d, d] + [_dp] * 12 + [i]
        lib.oracle_chkdav.argtypes = [_dp, _dp, d, i]
        lib.oracle_chkdav.restype = i
        lib.oracle_torque_uniform.argtypes = [C.c_ulonglong, C.c_longlong, i, i]
        lib.oracle_torque_uniform.restype = d
        lib.oracle_trqalfven.argtypes = [_dp, d, _dp, _dp, d, C.c_ulonglong, C.c_longlong, i]
        lib.oracle_spicule_run.argtypes = ([_dp] * 7 + [d, d] + [_dp] * 13 +
                                           [d, C.c_ulonglong, i, d, i, _ip, i, d, d,
                                            C.c_longlong, d, d, C.c_longlong, i, _dp,
                                            C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)])
        lib.oracle_spicule_run.restype = i
        lib.oracle_set_threads.argtypes = [i]
        lib.oracle_get_threads.restype = i
        lib.oracle_set_av_branch.argtypes = [i, C.c_void_p]
        ld = C.c_longdouble
        lib.oracle_ld_set_av_branch.argtypes = [i, C.c_void_p]
        lib.oracle_ld_mlw_m3_2d.argtypes = [_ldp] * 9 + [ld, ld, ld, _ldp, _ldp, i, _ldp, _ldp, i]
        _lib = lib
    return _lib


def P(a):
    assert a.dtype == np.float64 and (a.flags.f_contiguous or a.ndim == 1)
    return a.ctypes.data_as(_dp)


def PL(a):
    assert a.dtype == np.longdouble and (a.flags.f_contiguous or a.ndim == 1)
    return a.ctypes.data_as(_ldp)


def set_av_branch(mode: int, rec=None, long_double: bool = False) -> None:
    """The artificial viscosity's branch in the mlw_m3 step (not a
    reference routine; for the finite-difference check of the adjoint):
    mode 0 as mlw_m3.f, 1 records each face's branch into rec (uint8,
    2 ix jx bytes: x faces then y faces), 2 holds every face at the branch
    rec holds.  long_double: the setting of the long-double build."""
    if mode:
        assert rec is not None and rec.dtype == np.uint8 and rec.flags.c_contiguous
    ptr = rec.ctypes.data if mode else None
    f = load().oracle_ld_set_av_branch if long_double else load().oracle_set_av_branch
    f(int(mode), ptr)


def mlw_m3_ld(ro, pr, vx, vy, vz, bx, by, bz, az, dt, qav, gm, dx, dxm, dy, dym):
    """cans2d/hdmlw/mlw_m3.f:1, the restatement evaluated in long double
    (mlw2d_ld.c): every array np.longdouble, Fortran order."""
    ix, jx = ro.shape
    ld = np.longdouble
    load().oracle_ld_mlw_m3_2d(*[PL(a) for a in (ro, pr, vx, vy, vz, bx, by, bz, az)],
                               ld(dt), ld(qav), ld(gm), PL(dx), PL(dxm), ix, PL(dy), PL(dym),
                               jx)


_oplib = None


def opcount_mlw_m3(setup, state, dt):
    """Floating-point operations of one reference mlw_m3 step and one cfl_m3
    of `state` (updated in place by the step), counted by the oracle's
    restatement compiled with a counting number type (opcount.cpp):
    {"step": {...}, "cfl": {...}}, each with add (and subtract), mul, div,
    sqrt and cmp."""
    global _oplib
    if _oplib is None:
        if not (HERE / "_build" / "libcansopcount.so").exists():
            build()
        lib = C.CDLL(str(HERE / "_build" / "libcansopcount.so"))
        d, i = C.c_double, C.c_int
        lib.oracle_opcount_mlw_m3_2d.argtypes = [C.POINTER(_dp), d, d, d, _dp, _dp, i, _dp,
                                                 _dp, i, _dp]
        _oplib = lib
    ix, jx = state[0].shape
    arr = (_dp * 9)(*[P(a) for a in state])
    out = np.zeros(10)
    _oplib.oracle_opcount_mlw_m3_2d(arr, dt, setup["qav"], setup["gm"], P(setup["dx"]),
                                    P(setup["dxm"]), ix, P(setup["dy"]), P(setup["dym"]), jx,
                                    P(out))
    keys = ("add", "mul", "div", "sqrt", "cmp")
    return {"step": dict(zip(keys, out[:5].astype(int).tolist())),
            "cfl": dict(zip(keys, out[5:].astype(int).tolist()))}


def set_threads(n: int) -> None:
    load().oracle_set_threads(int(n))


def get_threads() -> int:
    return int(load().oracle_get_threads())


def mlw_m3(ro, pr, vx, vy, vz, bx, by, bz, az, dt, qav, gm, dx, dxm, dy, dym):
    ix, jx = ro.shape
    load().oracle_mlw_m3_2d(*[P(a) for a in (ro, pr, vx, vy, vz, bx, by, bz, az)],
                            dt, qav, gm, P(dx), P(dxm), ix, P(dy), P(dym), jx)


def mlw_m(ro, pr, vx, vy, bx, by, az, dt, qav, gm, dx, dxm, dy, dym):
    ix, jx = ro.shape
    load().oracle_mlw_m_2d(*[P(a) for a in (ro, pr, vx, vy, bx, by, az)],
                           dt, qav, gm, P(dx), P(dxm), ix, P(dy), P(dym), jx)


def cfl_m3(safety, dtmin, gm, ro, pr, vx, vy, vz, bx, by, bz, dx, dy):
    ix, jx = ro.shape
    dt, merr = C.c_double(), C.c_int()
    load().oracle_cfl_m3_2d(C.byref(dt), safety, dtmin, C.byref(merr), gm,
                            *[P(a) for a in (ro, pr, vx, vy, vz, bx, by, bz)],
                            P(dx), ix, P(dy), jx)
    return dt.value, merr.value


def cfl_m(safety, dtmin, gm, ro, pr, vx, vy, bx, by, dx, dy):
    ix, jx = ro.shape
    dt, merr = C.c_double(), C.c_int()
    load().oracle_cfl_m_2d(C.byref(dt), safety, dtmin, C.byref(merr), gm,
                           *[P(a) for a in (ro, pr, vx, vy, bx, by)], P(dx), ix, P(dy), jx)
    return dt.value, merr.value


def bd(kind, axis, mbnd, margin, qq, q0=0.0, dxm=None):
    """One bd* call on a 2-D array; BD_PER does both faces like bdper?."""
    ix, jx = qq.shape
    lib = load()
    dp = P(dxm) if dxm is not None else None
    if kind == BD_PER:
        lib.oracle_bd_2d(kind, axis, 0, margin, P(qq), q0, dp, ix, jx)
        lib.oracle_bd_2d(kind, axis, 1, margin, P(qq), q0, dp, ix, jx)
    else:
        lib.oracle_bd_2d(kind, axis, mbnd, margin, P(qq), q0, dp, ix, jx)


def bbtoaa(bx, by, dxm, dym, margin):
    ix, jx = bx.shape
    az = np.zeros((ix, jx), order="F")
    load().oracle_bbtoaa_2d(P(az), P(bx), P(by), P(dxm), P(dym), margin, ix, jx)
    return az


def apply_bc_program(state, program, margin, grid=None):
    """Apply a boundary program axis by axis (all x faces, then all y faces),
    as cans2d/md_mhdkh/hdmlw/bnd.f:11-39 orders its bd* calls."""
    for axis in (0, 1):
        for var, face, kind, q0 in program:
            if face // 2 != axis or kind < 0:
                continue
            dxm = None
            if grid is not None:
                dxm = grid["dxm"] if axis == 0 else grid["dym"]
            if kind == BD_PER:
                load().oracle_bd_2d(kind, axis, face % 2, margin, P(state[var]), q0,
                                    P(dxm) if dxm is not None else None, *state[var].shape)
            else:
                bd(kind, axis, face % 2, margin, state[var], q0, dxm)


def roe_m3(ro, pr, vx, vy, vz, bx, by, bz, az, dt, gm, dx, dy):
    """cans2d/hdroe/roe_m3.f:1"""
    ix, jx = ro.shape
    load().oracle_roe_m3_2d(*[P(a) for a in (ro, pr, vx, vy, vz, bx, by, bz, az)], dt, gm,
                            P(dx), ix, P(dy), jx)


def mlw_m3_g(ro, pr, vx, vy, vz, bx, by, bz, az, dt, qav, gm, gx, gxm, gy, gym,
             dx, dxm, dy, dym):
    """cans2d/hdmlw/mlw_m3_g.f:1"""
    ix, jx = ro.shape
    load().oracle_mlw_m3_g_2d(*[P(a) for a in (ro, pr, vx, vy, vz, bx, by, bz, az)], dt, qav,
                              gm, *[P(a) for a in (gx, gxm, gy, gym, dx, dxm)], ix, P(dy),
                              P(dym), jx)


def mlw_m_g(ro, pr, vx, vy, bx, by, az, dt, qav, gm, gx, gxm, gy, gym, dx, dxm, dy, dym):
    """cans2d/hdmlw/mlw_m_g.f:1"""
    ix, jx = ro.shape
    load().oracle_mlw_m_g_2d(*[P(a) for a in (ro, pr, vx, vy, bx, by, az)], dt, qav, gm,
                             *[P(a) for a in (gx, gxm, gy, gym, dx, dxm)], ix, P(dy), P(dym),
                             jx)


def _Pn(a):
    return None if a is None else P(a)


def mlw_m3_e(ro, pr, vx, vy, vz, bx, by, bz, az, dt, qav, gm, et, etm, dx, dxm, dy, dym,
             gx=None, gxm=None, gy=None, gym=None):
    """cans2d/hdmlw/mlw_m3_e.f:2 (with gx..gym: mlw_m3_ge.f:2)"""
    ix, jx = ro.shape
    load().oracle_mlw_m3_ge_2d(*[P(a) for a in (ro, pr, vx, vy, vz, bx, by, bz, az)], dt,
                               qav, gm, *[_Pn(a) for a in (gx, gxm, gy, gym)], P(et),
                               P(etm), P(dx), P(dxm), ix, P(dy), P(dym), jx)


def mlw_m_e(ro, pr, vx, vy, bx, by, az, dt, qav, gm, et, etm, dx, dxm, dy, dym,
            gx=None, gxm=None, gy=None, gym=None):
    """cans2d/hdmlw/mlw_m_e.f:2 (with gx..gym: mlw_m_ge.f:2)"""
    ix, jx = ro.shape
    load().oracle_mlw_m_ge_2d(*[P(a) for a in (ro, pr, vx, vy, bx, by, az)], dt, qav, gm,
                              *[_Pn(a) for a in (gx, gxm, gy, gym)], P(et), P(etm), P(dx),
                              P(dxm), ix, P(dy), P(dym), jx)


def cfl_m3_e(safety, dtmin, gm, ro, pr, vx, vy, vz, bx, by, bz, et, dx, dy):
    """cans2d/common/cfl_m3_e.f:2"""
    ix, jx = ro.shape
    dt, merr = C.c_double(), C.c_int()
    load().oracle_cfl_m3_e_2d(C.byref(dt), safety, dtmin, C.byref(merr), gm,
                              *[P(a) for a in (ro, pr, vx, vy, vz, bx, by, bz, et)],
                              P(dx), ix, P(dy), jx)
    return dt.value, merr.value


def cfl_m_e(safety, dtmin, gm, ro, pr, vx, vy, bx, by, et, dx, dy):
    """cans2d/common/cfl_m_e.f:2"""
    ix, jx = ro.shape
    dt, merr = C.c_double(), C.c_int()
    load().oracle_cfl_m3_e_2d(C.byref(dt), safety, dtmin, C.byref(merr), gm,
                              P(ro), P(pr), P(vx), P(vy), None, P(bx), P(by), None, P(et),
                              P(dx), ix, P(dy), jx)
    return dt.value, merr.value


def step_2d(setup, state, dt):
    if setup.get("et") is not None:
        e = [np.asfortranarray(setup[k]) for k in ("et", "etm")]
        g = ([np.asfortranarray(setup[k]) for k in ("gx", "gxm", "gy", "gym")]
             if setup.get("gravity") else [None] * 4)
        (mlw_m3_e if setup["solver"] == "mlw_m3" else mlw_m_e)(
            *state, dt, setup["qav"], setup["gm"], *e, setup["dx"], setup["dxm"], setup["dy"],
            setup["dym"], *g)
        return
    if setup.get("gravity"):
        g = [np.asfortranarray(setup[k]) for k in ("gx", "gxm", "gy", "gym")]
        args = (setup["qav"], setup["gm"], *g, setup["dx"], setup["dxm"], setup["dy"],
                setup["dym"])
        (mlw_m3_g if setup["solver"] == "mlw_m3" else mlw_m_g)(*state, dt, *args)
        return
    if setup["solver"] == "roe_m3":
        roe_m3(*state, dt, setup["gm"], setup["dx"], setup["dy"])
        return
    args = (setup["qav"], setup["gm"], setup["dx"], setup["dxm"], setup["dy"], setup["dym"])
    if setup["solver"] == "mlw_m3":
        mlw_m3(*state, dt, *args)
    else:
        mlw_m(*state, dt, *args)


def cfl_2d(setup, state, safety):
    if setup.get("et") is not None:
        et = np.asfortranarray(setup["et"])
        if setup["solver"] == "mlw_m3":
            return cfl_m3_e(safety, setup["dtmin"], setup["gm"], *state[:8], et, setup["dx"],
                            setup["dy"])
        return cfl_m_e(safety, setup["dtmin"], setup["gm"], *state[:6], et, setup["dx"],
                       setup["dy"])
    if setup["solver"] in ("mlw_m3", "roe_m3"):
        return cfl_m3(safety, setup["dtmin"], setup["gm"], *state[:8], setup["dx"], setup["dy"])
    return cfl_m(safety, setup["dtmin"], setup["gm"], *state[:6], setup["dx"], setup["dy"])


def mlw_m_1d(ro, pr, vx, vy, by, bx, bxm, dt, qav, gm, dx, dxm):
    load().oracle_mlw_m_1d(*[P(a) for a in (ro, pr, vx, vy, by, bx, bxm)], dt, qav, gm,
                           P(dx), P(dxm), ro.size)


def roe_m_1d(ro, pr, vx, vy, by, bx, bxm, dt, gm, dx):
    """cans1d/hdroe/roe_m.f:2"""
    load().oracle_roe_m_1d(*[P(a) for a in (ro, pr, vx, vy, by, bx, bxm)], dt, gm, P(dx),
                           ro.size)


def cfl_m_1d(safety, dtmin, gm, bx, ro, pr, vx, vy, by, dx):
    dt, merr = C.c_double(), C.c_int()
    load().oracle_cfl_m_1d(C.byref(dt), safety, dtmin, C.byref(merr), gm, P(bx),
                           *[P(a) for a in (ro, pr, vx, vy, by)], P(dx), ro.size)
    return dt.value, merr.value


def bd_1d(kind, mbnd, margin, qq, q0=0.0, dxm=None):
    lib = load()
    dp = P(dxm) if dxm is not None else None
    if kind == BD_PER:
        lib.oracle_bd_1d(kind, 0, margin, P(qq), q0, dp, qq.size)
        lib.oracle_bd_1d(kind, 1, margin, P(qq), q0, dp, qq.size)
    else:
        lib.oracle_bd_1d(kind, mbnd, margin, P(qq), q0, dp, qq.size)


def apply_bc_program_1d(state, program, margin, grid):
    """cans1d/md_mhdshktb/hdmlw/bnd.f:9-19: every lower-face rule, then every
    upper-face rule."""
    for side in (0, 1):
        for var, face, kind, q0 in program:
            if face != side or kind < 0:
                continue
            load().oracle_bd_1d(kind, side, margin, P(state[var]), q0, P(grid["dxm"]),
                                state[var].size)


def run_1d(setup, state, nstop, tend=None, safety=None, t0=0.0):
    """The 1-D model-package loop (cans1d/md_mhdshktb/hdmlw/main.f:139-199),
    with the set-up's step: mlw_m, roe_m or mlw_m_bg (the md_mhdwind loop,
    cans1d/md_mhdwind/hdmlw/main.f:160-176; the spicule loop with its torque
    and floor is run_spicule)."""
    tend = setup.get("tend", 1e30) if tend is None else tend
    safety = setup["safety"] if safety is None else safety
    bx, bxm = setup["bx"], setup["bxm"]
    t, ns, dts = t0, 0, []
    while True:
        ns += 1
        dt, merr = cfl_m_1d(safety, setup["dtmin"], setup["gm"], bx, *state, setup["dx"])
        if merr:
            return t, ns, merr, dts
        t = t + dt
        dts.append(dt)
        if setup["solver"] == "roe_m_1d":
            roe_m_1d(*state, bx, bxm, dt, setup["gm"], setup["dx"])
        elif setup["solver"] == "mlw_m_bg_1d":
            step_bg(setup, state, dt)
        else:
            mlw_m_1d(*state, bx, bxm, dt, setup["qav"], setup["gm"], setup["dx"], setup["dxm"])
        apply_bc_program_1d(state, setup["bc"], setup["margin"], setup)
        if setup.get("floor") is not None:
            chkdav_state(setup, state)
        if not (ns < nstop and t < tend):
            return t, ns, 0, dts


def mlw_m_bg(ro, pr, vx, vy, by, bx, bxm, dt, qav, gm, gx, gxm, sc, dsc, scm, dscm,
             rr, rrm, drr, drrm, dx, dxm):
    """cans1d/hdmlw/mlw_m_bg.f:2 (argument order of the reference)."""
    load().oracle_mlw_m_bg_1d(*[P(a) for a in (ro, pr, vx, vy, by, bx, bxm)], dt, qav, gm,
                              *[P(a) for a in (gx, gxm, sc, dsc, scm, dscm, rr, rrm, drr,
                                               drrm, dx, dxm)], ro.size)


def chkdav(da, vx, floor):
    """cans1d/common/chkdav.f:2; returns n_events."""
    return int(load().oracle_chkdav(P(da), P(vx), floor, da.size))


def chkdav_nd(da, vels, floor):
    """cans2d/common/chkdav.f:33-44 and cans3d/common/chkdav.f: da below floor
    is raised to it and the velocity components set to zero there (a
    pointwise rule, so the array order of the scan does not matter); returns
    n_events."""
    mask = da < floor
    da[mask] = floor
    for v in vels:
        v[mask] = 0.0
    return int(np.count_nonzero(mask))


def chkdav_state(setup, state):
    """chkdav of ro, then pr, as the model packages call it after bnd
    (cans2d/md_efr/hdmlw/main.f:183-185); velocities vx, vy (and vz in 3-D,
    vx alone in 1-D)."""
    floor = setup["floor"]
    names = setup["names"]
    if state[0].ndim == 1:
        return (chkdav(state[0], state[2], floor) + chkdav(state[1], state[2], floor))
    vel = [state[names.index(k)] for k in (("vx", "vy", "vz") if state[0].ndim == 3
                                            else ("vx", "vy"))]
    return chkdav_nd(state[0], vel, floor) + chkdav_nd(state[1], vel, floor)


def torque_uniform(seed, ns, g, ix):
    return float(load().oracle_torque_uniform(seed, ns, g, ix))


def trqalfven(vy, dt, trq, rr, trq0, seed, ns):
    load().oracle_trqalfven(P(vy), dt, P(trq), P(rr), trq0, seed, ns, vy.size)


def step_bg(setup, state, dt):
    s = setup
    mlw_m_bg(*state, s["bx"], s["bxm"], dt, s["qav"], s["gm"], s["gx"], s["gxm"], s["sc"],
             s["dsc"], s["scm"], s["dscm"], s["rr"], s["rrm"], s["drr"], s["drrm"], s["dx"],
             s["dxm"])


def run_spicule_c(setup, state, nstop, tend=None, safety=None, t0=0.0, ns0=0, torque=True,
                  floor=True):
    """run_spicule without output pauses, the whole loop in C.  Returns
    (t, ns, merr, n_floor_events)."""
    s = setup
    tend = s.get("tend", 1e30) if tend is None else tend
    safety = s["safety"] if safety is None else safety
    kind = np.full(10, -1, dtype=np.int32)
    for var, face, k, q0 in s["bc"]:
        if q0 != 0.0 or k in (BD_CNS, BD_FRD, BD_PER):
            raise ValueError("the C loop takes the zero-constant bd kinds only")
        kind[2 * var + face] = k
    t, ns, nev = C.c_double(), C.c_longlong(), C.c_longlong()
    merr = load().oracle_spicule_run(
        *[P(a) for a in state], P(s["bx"]), P(s["bxm"]), s["qav"], s["gm"],
        *[P(s[k]) for k in ("gx", "gxm", "sc", "dsc", "scm", "dscm", "rr", "rrm", "drr",
                             "drrm", "dx", "dxm", "trq")],
        s["trq0"], s["seed"], 1 if torque else 0, s["floor"], 1 if floor else 0,
        kind.ctypes.data_as(_ip), s["margin"], safety, s["dtmin"], nstop, tend, t0, ns0,
        state[0].size, C.byref(t), C.byref(ns), C.byref(nev))
    return t.value, ns.value, int(merr), nev.value


def run_spicule(setup, state, nstop, tend=None, safety=None, t0=0.0, ns0=0, torque=True,
                floor=True, on_output=None):
    """The spicule loop (cans1d/md_spicule/hdmlw/main.f:160-219): cfl_m,
    t += dt, mlw_m_bg, trqalfven, bnd, chkdav of ro then pr, the output test
    (on_output(ns, t) when int(tp/dtout) < int(t/dtout)) and the loop test.
    Returns (t, ns, merr, dts, n_floor_events)."""
    s = setup
    tend = s.get("tend", 1e30) if tend is None else tend
    safety = s["safety"] if safety is None else safety
    fl = s["floor"] if floor else None
    t, ns, dts, nev = t0, ns0, [], 0
    while True:
        ns += 1
        dt, merr = cfl_m_1d(safety, s["dtmin"], s["gm"], s["bx"], *state, s["dx"])
        if merr:
            return t, ns, merr, dts, nev
        tp = t
        t = t + dt
        dts.append(dt)
        step_bg(s, state, dt)
        if torque:
            trqalfven(state[3], dt, s["trq"], s["rr"], s["trq0"], s["seed"], ns)
        apply_bc_program_1d(state, s["bc"], s["margin"], s)
        if fl is not None:
            nev += chkdav(state[0], state[2], fl)
            nev += chkdav(state[1], state[2], fl)
        if on_output is not None and s.get("dtout", 0) > 0 and int(tp / s["dtout"]) < int(t / s["dtout"]):
            on_output(ns, t)
        if not (ns < nstop and t < tend):
            return t, ns, 0, dts, nev


def mlw_m_3d(ro, pr, vx, vy, vz, bx, by, bz, dt, qav, gm, dx, dxm, dy, dym, dz, dzm):
    ix, jx, kx = ro.shape
    load().oracle_mlw_m_3d(*[P(a) for a in (ro, pr, vx, vy, vz, bx, by, bz)], dt, qav, gm,
                           P(dx), P(dxm), ix, P(dy), P(dym), jx, P(dz), P(dzm), kx)


def mlw_m_g_3d(ro, pr, vx, vy, vz, bx, by, bz, dt, qav, gm, gx, gxm, gy, gym, gz, gzm,
               dx, dxm, dy, dym, dz, dzm):
    """cans3d/hdmlw/mlw_m_g.f:2"""
    ix, jx, kx = ro.shape
    load().oracle_mlw_m_g_3d(*[P(a) for a in (ro, pr, vx, vy, vz, bx, by, bz)], dt, qav, gm,
                             *[P(a) for a in (gx, gxm, gy, gym, gz, gzm)], P(dx), P(dxm), ix,
                             P(dy), P(dym), jx, P(dz), P(dzm), kx)


def mlw_m_e_3d(ro, pr, vx, vy, vz, bx, by, bz, dt, qav, gm, et, etm, dx, dxm, dy, dym,
               dz, dzm):
    """cans3d/hdmlw/mlw_m_e.f:2"""
    ix, jx, kx = ro.shape
    load().oracle_mlw_m_e_3d(*[P(a) for a in (ro, pr, vx, vy, vz, bx, by, bz)], dt, qav, gm,
                             P(et), P(etm), P(dx), P(dxm), ix, P(dy), P(dym), jx, P(dz),
                             P(dzm), kx)


def cfl_m_e_3d(safety, dtmin, gm, ro, pr, vx, vy, vz, bx, by, bz, et, dx, dy, dz):
    """cans3d/common/cfl_m_e.f:2"""
    ix, jx, kx = ro.shape
    dt, merr = C.c_double(), C.c_int()
    load().oracle_cfl_m_e_3d(C.byref(dt), safety, dtmin, C.byref(merr), gm,
                             *[P(a) for a in (ro, pr, vx, vy, vz, bx, by, bz, et)],
                             P(dx), ix, P(dy), jx, P(dz), kx)
    return dt.value, merr.value


def cfl_m_3d(safety, dtmin, gm, ro, pr, vx, vy, vz, bx, by, bz, dx, dy, dz):
    ix, jx, kx = ro.shape
    dt, merr = C.c_double(), C.c_int()
    load().oracle_cfl_m_3d(C.byref(dt), safety, dtmin, C.byref(merr), gm,
                           *[P(a) for a in (ro, pr, vx, vy, vz, bx, by, bz)],
                           P(dx), ix, P(dy), jx, P(dz), kx)
    return dt.value, merr.value


def bd_3d(kind, axis, mbnd, margin, qq, q0=0.0, dxm=None):
    """One bd* call on a 3-D array; BD_PER does both faces like bdper?."""
    lib = load()
    dp = P(dxm) if dxm is not None else None
    if kind == BD_PER:
        lib.oracle_bd_3d(kind, axis, 0, margin, P(qq), q0, dp, *qq.shape)
        lib.oracle_bd_3d(kind, axis, 1, margin, P(qq), q0, dp, *qq.shape)
    else:
        lib.oracle_bd_3d(kind, axis, mbnd, margin, P(qq), q0, dp, *qq.shape)


def apply_bc_program_3d(state, program, margin, grid):
    """Boundary program axis by axis (x, y, z), as the 3-D bnd routines do."""
    for axis in (0, 1, 2):
        dxm = grid["d" + "xyz"[axis] + "m"]
        for var, face, kind, q0 in program:
            if face // 2 != axis or kind < 0:
                continue
            load().oracle_bd_3d(kind, axis, face % 2, margin, P(state[var]), q0, P(dxm),
                                *state[var].shape)


def roe_m_3d(ro, pr, vx, vy, vz, bx, by, bz, dt, gm, dx, dy, dz):
    ix, jx, kx = ro.shape
    load().oracle_roe_m_3d(*[P(a) for a in (ro, pr, vx, vy, vz, bx, by, bz)], dt, gm,
                           P(dx), ix, P(dy), jx, P(dz), kx)


def hlld_engine_3d(ro, pr, vx, vy, vz, bx, by, bz, gm, mu, dt, dx, dy, dz, mfdim):
    ix, jx, kx = ro.shape
    md = (C.c_int * 3)(*mfdim)
    load().oracle_hlld_engine_3d(*[P(a) for a in (ro, pr, vx, vy, vz, bx, by, bz)], gm, mu,
                                 dt, P(dx), ix, P(dy), jx, P(dz), kx,
                                 C.cast(md, _ip))


def step_3d(setup, state, dt):
    if setup.get("solver") == "hlld_3d":
        hlld_engine_3d(*state, setup["gm"], setup["mu"], dt, setup["dx"], setup["dy"],
                       setup["dz"], setup["mfdim"])
        return
    if setup.get("solver") == "roe_m_3d":
        roe_m_3d(*state, dt, setup["gm"], setup["dx"], setup["dy"], setup["dz"])
        return
    if setup.get("et") is not None:
        mlw_m_e_3d(*state, dt, setup["qav"], setup["gm"], np.asfortranarray(setup["et"]),
                   np.asfortranarray(setup["etm"]), setup["dx"], setup["dxm"], setup["dy"],
                   setup["dym"], setup["dz"], setup["dzm"])
        return
    if setup.get("gravity"):
        g = [np.asfortranarray(setup[k]) for k in ("gx", "gxm", "gy", "gym", "gz", "gzm")]
        mlw_m_g_3d(*state, dt, setup["qav"], setup["gm"], *g, setup["dx"], setup["dxm"],
                   setup["dy"], setup["dym"], setup["dz"], setup["dzm"])
        return
    mlw_m_3d(*state, dt, setup["qav"], setup["gm"], setup["dx"], setup["dxm"], setup["dy"],
             setup["dym"], setup["dz"], setup["dzm"])


def cfl_3d(setup, state, safety):
    if setup.get("et") is not None:
        return cfl_m_e_3d(safety, setup["dtmin"], setup["gm"], *state,
                          np.asfortranarray(setup["et"]), setup["dx"], setup["dy"], setup["dz"])
    return cfl_m_3d(safety, setup["dtmin"], setup["gm"], *state, setup["dx"], setup["dy"],
                    setup["dz"])


def run_3d(setup, state, nstop, tend=None, safety=None, t0=0.0):
    """The 3-D model-package loop (cans3d/md_mhdshktb/hdmlw/main.f:167-182;
    hdroe/main.f:167-180 for the Roe solver)."""
    tend = setup.get("tend", 1e30) if tend is None else tend
    safety = setup["safety"] if safety is None else safety
    t, ns, dts = t0, 0, []
    while True:
        ns += 1
        dt, merr = cfl_3d(setup, state, safety)
        if merr:
            return t, ns, merr, dts
        t = t + dt
        dts.append(dt)
        step_3d(setup, state, dt)
        apply_bc_program_3d(state, setup["bc"], setup["margin"], setup)
        if setup.get("floor") is not None:
            chkdav_state(setup, state)
        if not (ns < nstop and t < tend):
            return t, ns, 0, dts


def run_2d(setup, state, nstop, tend=None, safety=None, t0=0.0):
    """Restatement of the model-package loop (md_mhdkh/hdmlw/main.f:160-219):
    ns+=1; cfl; merr test; t+=dt; step; bnd; loop while ns<nstop and t<tend.
    Returns (t, ns, merr, dts)."""
    tend = setup.get("tend", 1e30) if tend is None else tend
    safety = setup["safety"] if safety is None else safety
    t, ns, dts = t0, 0, []
    while True:
        ns += 1
        dt, merr = cfl_2d(setup, state, safety)
        if merr:
            return t, ns, merr, dts
        t = t + dt
        dts.append(dt)
        step_2d(setup, state, dt)
        apply_bc_program(state, setup["bc"], setup["margin"], setup)
        if setup.get("floor") is not None:
            chkdav_state(setup, state)
        if not (ns < nstop and t < tend):
            return t, ns, 0, dts
