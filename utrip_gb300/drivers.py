"""Time loops of the reference model packages on top of the C ABI.

run_literal  -- the reference driver shape (cans2d/md_mhdkh/hdmlw/main.f:
                160-219) calling the drop-in entry points once per step:
                cfl_m3 -> t += dt -> mlw_m3 -> bnd (and the 1-D, 3-D
                and Roe forms of the same loop).  With `resident=True` the
                arrays are registered first, so the calls run on device
                mirrors and only dt crosses to the host each step.
run_resident -- the same loop kept on the device by the run handle and
                replayed as a CUDA graph; the host waits once at the end.
run_spicule  -- the spicule model package (cans1d/md_spicule/hdmlw/main.f)
                on the device, with its DAC output files and restart.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from . import capi, dac, setups


def _bnd(setup, state):
    """bnd.f: every x-face rule for all variables, then every y-face rule."""
    margin = setup["margin"]
    for axis in (0, 1):
        for var, face, kind, q0 in setup["bc"]:
            if face // 2 != axis or kind < 0:
                continue
            dxm = setup["dxm"] if axis == 0 else setup["dym"]
            if kind == capi.BD_PER:
                # bdper? fills both faces in one call; issue it once (lower face)
                if face % 2 == 0:
                    capi.bd(kind, axis, 0, margin, state[var])
            else:
                capi.bd(kind, axis, face % 2, margin, state[var], q0, dxm)


def _bnd3(setup, state):
    """3-D bnd: every x-face rule, then y, then z."""
    margin = setup["margin"]
    for axis in (0, 1, 2):
        dxm = setup["d" + "xyz"[axis] + "m"]
        for var, face, kind, q0 in setup["bc"]:
            if face // 2 != axis or kind < 0:
                continue
            if kind == capi.BD_PER:
                if face % 2 == 0:
                    capi.bd_3d(kind, axis, 0, margin, state[var])
            else:
                capi.bd_3d(kind, axis, face % 2, margin, state[var], q0, dxm)


def _chkdav(setup, state):
    """chkdav of ro, then pr, after bnd (cans2d/md_efr/hdmlw/main.f:183-185)."""
    fl, names = setup["floor"], setup["names"]
    if state[0].ndim == 1:
        capi.chkdav(state[0], state[2], fl)
        capi.chkdav(state[1], state[2], fl)
        return
    three = state[0].ndim == 3
    v = [state[names.index(k)] for k in (("vx", "vy", "vz") if three else ("vx", "vy"))]
    for q in (0, 1):
        if three:
            capi.chkdav_3d(state[q], v[0], v[1], v[2], fl)
        else:
            capi.chkdav_2d(state[q], v[0], v[1], fl)


def _bnd1(setup, state):
    """cans1d/md_mhdshktb/hdmlw/bnd.f:9-19: lower-face rules, then upper."""
    margin = setup["margin"]
    for side in (0, 1):
        for var, face, kind, q0 in setup["bc"]:
            if face != side or kind < 0:
                continue
            if kind == capi.BD_PER:
                if side == 0:
                    capi.bd_1d(kind, 0, margin, state[var])
            else:
                capi.bd_1d(kind, side, margin, state[var], q0, setup["dxm"])


def _cfl(setup, state, safety):
    if setup["solver"] in ("mlw_m_1d", "mlw_m_bg_1d", "roe_m_1d"):
        return capi.cfl_m_1d(safety, setup["dtmin"], setup["gm"], setup["bx"], *state,
                             setup["dx"])
    if setup["solver"] == "mlw_m_3d" and setup.get("et") is not None:  # cfl_m_e 3-D
        return capi.cfl_m_e_3d(safety, setup["dtmin"], setup["gm"], *state,
                               np.asfortranarray(setup["et"]), setup["dx"], setup["dy"],
                               setup["dz"])
    if setup["solver"] in ("mlw_m_3d", "roe_m_3d", "hlld_3d"):
        return capi.cfl_m_3d(safety, setup["dtmin"], setup["gm"], *state, setup["dx"],
                             setup["dy"], setup["dz"])
    if setup.get("et") is not None:  # cfl_m3_e / cfl_m_e
        et = np.asfortranarray(setup["et"])
        if setup["solver"] == "mlw_m3":
            return capi.cfl_m3_e(safety, setup["dtmin"], setup["gm"], *state[:8], et,
                                 setup["dx"], setup["dy"])
        return capi.cfl_m_e(safety, setup["dtmin"], setup["gm"], *state[:6], et, setup["dx"],
                            setup["dy"])
    if setup["solver"] in ("mlw_m3", "roe_m3"):
        return capi.cfl_m3(safety, setup["dtmin"], setup["gm"], *state[:8], setup["dx"],
                           setup["dy"])
    return capi.cfl_m(safety, setup["dtmin"], setup["gm"], *state[:6], setup["dx"], setup["dy"])


def _step(setup, state, dt):
    if setup["solver"] == "mlw_m_bg_1d":
        s = setup
        capi.mlw_m_bg(*state, s["bx"], s["bxm"], dt, s["qav"], s["gm"], s["gx"], s["gxm"],
                      s["sc"], s["dsc"], s["scm"], s["dscm"], s["rr"], s["rrm"], s["drr"],
                      s["drrm"], s["dx"], s["dxm"])
        return
    if setup["solver"] == "roe_m_1d":
        capi.roe_m_1d(*state, setup["bx"], setup["bxm"], dt, setup["gm"], setup["dx"])
        return
    if setup["solver"] == "mlw_m_1d":
        capi.mlw_m_1d(*state, setup["bx"], setup["bxm"], dt, setup["qav"], setup["gm"],
                      setup["dx"], setup["dxm"])
        return
    if setup["solver"] == "roe_m3":
        capi.roe_m3(*state, dt, setup["gm"], setup["dx"], setup["dy"])
        return
    if setup["solver"] == "roe_m_3d":
        capi.roe_m_3d(*state, dt, setup["gm"], setup["dx"], setup["dy"], setup["dz"])
        return
    if setup["solver"] == "hlld_3d":
        capi.hlld_engine_3d(*state, setup["gm"], setup["mu"], dt, setup["dx"], setup["dxm"],
                            setup["dy"], setup["dym"], setup["dz"], setup["dzm"],
                            setup["mfdim"])
        return
    if setup.get("et") is not None and setup["solver"] == "mlw_m_3d":  # 3-D mlw_m_e
        e = [np.asfortranarray(setup[k]) for k in ("et", "etm")]
        capi.mlw_m_e_3d(*state, dt, setup["qav"], setup["gm"], *e, setup["dx"], setup["dxm"],
                        setup["dy"], setup["dym"], setup["dz"], setup["dzm"])
        return
    if setup.get("et") is not None:  # mlw_m3_e / mlw_m_e, with gravity _ge
        e = [np.asfortranarray(setup[k]) for k in ("et", "etm")]
        g = ([np.asfortranarray(setup[k]) for k in ("gx", "gxm", "gy", "gym")]
             if setup.get("gravity") else [None] * 4)
        (capi.mlw_m3_e if setup["solver"] == "mlw_m3" else capi.mlw_m_e)(
            *state, dt, setup["qav"], setup["gm"], *e, setup["dx"], setup["dxm"], setup["dy"],
            setup["dym"], *g)
        return
    if setup.get("gravity") and setup["solver"] == "mlw_m_3d":  # 3-D mlw_m_g
        g = [np.asfortranarray(setup[k]) for k in ("gx", "gxm", "gy", "gym", "gz", "gzm")]
        capi.mlw_m_g_3d(*state, dt, setup["qav"], setup["gm"], *g, setup["dx"], setup["dxm"],
                        setup["dy"], setup["dym"], setup["dz"], setup["dzm"])
        return
    if setup.get("gravity"):
        g = [setup[k] for k in ("gx", "gxm", "gy", "gym")]
        args = (setup["qav"], setup["gm"], *g, setup["dx"], setup["dxm"], setup["dy"],
                setup["dym"])
        (capi.mlw_m3_g if setup["solver"] == "mlw_m3" else capi.mlw_m_g)(*state, dt, *args)
        return
    args = (setup["qav"], setup["gm"], setup["dx"], setup["dxm"], setup["dy"], setup["dym"])
    if setup["solver"] == "mlw_m_3d":
        capi.mlw_m_3d(*state, dt, *args, setup["dz"], setup["dzm"])
    elif setup["solver"] == "mlw_m3":
        capi.mlw_m3(*state, dt, *args)
    else:
        capi.mlw_m(*state, dt, *args)


def run_literal(setup, state, nstop, tend=None, safety=None, t0=0.0, resident=False):
    """Reference loop through the drop-in entry points.  Returns
    (t, ns, merr, dts); `state` holds the final state on return."""
    tend = setup.get("tend", 1e30) if tend is None else tend
    safety = setup["safety"] if safety is None else safety
    if resident:
        capi.register(state)
    try:
        t, ns, dts = t0, 0, []
        while True:
            ns += 1
            dt, merr = _cfl(setup, state, safety)
            if merr:
                return t, ns, merr, dts
            t = t + dt
            dts.append(dt)
            _step(setup, state, dt)
            {"mlw_m_3d": _bnd3, "roe_m_3d": _bnd3, "hlld_3d": _bnd3,
             "mlw_m_1d": _bnd1, "mlw_m_bg_1d": _bnd1,
             "roe_m_1d": _bnd1}.get(setup["solver"], _bnd)(setup, state)
            if setup.get("floor") is not None:
                _chkdav(setup, state)
            if not (ns < nstop and t < tend):
                return t, ns, 0, dts
    finally:
        if resident:
            capi.pull(state[0])
            capi.release(state[0])


def make_run(setup, exact=False, tile=-1, stream=None, floor=True, torque=True,
             stop_on_bad=False, df64=False) -> capi.Run:
    """Run handle for a set-up; a set-up with a "floor" gets the chkdav
    option and one with a "trq" profile the torque source (each can be
    switched off here).  df64 selects the double-float policy of the step
    (cans_run_set_df64)."""
    fl = setup.get("floor") if floor else None
    tq = None
    if torque and setup.get("trq") is not None:
        tq = {"trq": setup["trq"], "trq0": setup["trq0"], "seed": setup.get("seed", 0)}
    run = capi.Run(setup["solver_id"], setup, setup["gm"], setup["qav"], setup["margin"],
                   exact=exact, tile=tile, stream=stream, mu=setup.get("mu", 1.0),
                   mfdim=setup.get("mfdim", (0, 0, 0)), floor=fl, torque=tq,
                   stop_on_bad=stop_on_bad)
    run.set_bc_program(setup["bc"])
    if df64:
        run.set_df64(True)
        if tile >= 0:
            run.set_tile(tile)
    return run


def run_resident(setup, state, nstop, tend=None, safety=None, t0=0.0, exact=False,
                 chunk=256, run: capi.Run | None = None, df64=False):
    """Reference loop on the device.  Returns (t, ns, merr, nexec)."""
    tend = setup.get("tend", 1e30) if tend is None else tend
    safety = setup["safety"] if safety is None else safety
    own = run is None
    if own:
        run = make_run(setup, exact=exact, df64=df64)
    try:
        run.push(state)
        run.start(t0=t0, tend=tend, nstop=nstop, safety=safety, dtmin=setup["dtmin"])
        while True:
            st = run.query()
            if st.done:
                break
            run.advance(min(chunk, max(1, nstop - st.ns + 1)))
        run.pull(state)
        return st.t, st.ns, st.merr, st.nexec
    finally:
        if own:
            run.close()


# ---- the spicule model package ------------------------------------------------

def _e10_3(v: float) -> str:
    """Fortran E10.3: 0.ddd with a two-digit exponent, right-justified."""
    v = float(v)
    if v == 0.0:
        body = "0.000E+00"
    else:
        digits, ex = ("%.2e" % abs(v)).split("e")
        body = "0." + digits.replace(".", "") + "E%+03d" % (int(ex) + 1)
        if v < 0:
            body = "-" + body
    return body.rjust(10)


def _out_line(kind: str, ns: int, t: float, nd: int | None = None) -> str:
    """main.f formats 913 / 915: (1x,' write    ','step=',i8,' time=',e10.3,' nd =',i3)."""
    line = " " + (" write    " if kind == "write" else " stop     ") + "step=" + "%8d" % ns
    line += " time=" + _e10_3(t)
    if nd is not None:
        line += " nd =" + "%3d" % nd
    return line


def run_spicule(out_dir, nx: int = 1024, tend: float = 100.0, dtout: float = 0.5,
                nstop: int = 100000, mcont: int = 0, in_dir=None, exact: bool = False,
                seed: int = 0, chunk: int = 20000, torque: bool = True):
    """cans1d/md_spicule/hdmlw/main.f on the device.

    Writes what the reference writes into out_dir: params.txt (ix, margin,
    ztr, tcor, gm), the static profiles x, bx, bxm, sc, scm, gx, gxm, rr, rrm
    (dacdef1d), the time series t, ro, pr, vx, vy, by (dacdef0s / dacdef1s)
    with a record at the start, at every crossing of a multiple of dtout and
    at the end (unless the last step wrote one), and out.txt.  With mcont=1
    the state and time are the last record (at most the 1000th) of
    in_dir/{t,ro,pr,vx,vy,by}.dac, as main.f:78-102 reads them.  The loop
    runs as the 1-D cluster kernel, pausing on the device at output times.
    Returns a dict with t, ns, merr, the number of records written and the
    chkdav event count."""
    s = setups.spicule_1d(nx, seed=seed, tend=tend, nstop=nstop, dtout=dtout)
    ix, names = s["x"].size, s["names"]
    out = Path(out_dir)
    out.mkdir(parents=True, exist_ok=True)
    outtxt = out / "out.txt"
    outtxt.write_text("")

    def say(line: str) -> None:
        with open(outtxt, "a") as f:
            f.write(line + "\n")

    params = dac.DacParams(out / "params.txt")
    ft = dac.dacdef0s(out / "t.dac")
    fs = {k: dac.dacdef1s(out / f"{k}.dac", ix) for k in names}
    params.puti("ix", ix)
    params.puti("margin", s["margin"])
    params.putd("ztr", s["ztr"])
    params.putd("tcor", s["tcor"])
    state = setups.copy_state(s)
    t = 0.0
    if mcont == 1:
        src = Path(in_dir) if in_dir is not None else Path("in")
        tt = dac.dacopnr(src / "t.dac", 0)
        nrec = min(tt.nx, 1000)
        if nrec > 0:
            t = float(tt.records[nrec - 1])
            for k, name in enumerate(names):
                f = dac.dacopnr(src / f"{name}.dac", 1)
                if f.dims != (ix,):
                    raise dac.DacError(f"{name}.dac holds {f.dims[0]} cells, the model {ix}")
                state[k][:] = f.records[min(nrec, f.nx) - 1]
    for k in ("x", "bx", "bxm", "sc", "scm", "gx", "gxm", "rr", "rrm"):
        dac.write_1d(out / f"{k}.dac", s[k])
    params.putd("gm", s["gm"])
    nd = 1

    def write_records(ns_: int, t_: float) -> None:
        nonlocal nd
        ft.write(np.float64(t_))
        for k, name in enumerate(names):
            fs[name].write(state[k])
        say(_out_line("write", ns_, t_, nd))
        nd += 1

    write_records(0, t)
    run = make_run(s, exact=exact, torque=torque)
    try:
        run.push(state)
        run.start(t0=t, tend=tend, nstop=nstop, safety=s["safety"], dtmin=s["dtmin"],
                  dtout=dtout, pause_on_output=True)
        wrote_last = False
        while True:
            st = run.query()
            if st.pause:
                run.pull(state)
                write_records(int(st.ns), st.t)
                wrote_last = True
                if st.done:
                    break
                run.resume()
                continue
            if st.done:
                break
            wrote_last = False
            run.advance(min(chunk, max(1, nstop - int(st.ns) + 1)))
        st = run.query()
        run.pull(state)
        if not wrote_last or st.merr:
            write_records(int(st.ns), st.t)
        say(_out_line("stop", int(st.ns), st.t))
        if st.merr == 0:
            say("   ### normal stop ###")
        else:
            say("   ### abnormal stop ###")
            say("   merr = %11d" % st.merr)
        return {"t": st.t, "ns": int(st.ns), "merr": int(st.merr), "records": nd - 1,
                "n_floor": int(st.n_floor), "state": state}
    finally:
        run.close()
        ft.close()
        for f in fs.values():
            f.close()
        params.close()
