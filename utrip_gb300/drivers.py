"""Time loops of the reference model packages on top of the C ABI.

run_literal  -- the reference driver shape (cans2d/md_mhdkh/hdmlw/main.f:
                160-219) calling the drop-in entry points once per step:
                cfl_m3 -> t += dt -> mlw_m3 -> bnd (and the 1-D, 3-D
                and Roe forms of the same loop).  With `resident=True` the
                arrays are registered first, so the calls run on device
                mirrors and only dt crosses to the host each step.
run_resident -- the same loop kept on the device by the run handle and
                replayed as a CUDA graph; the host waits once at the end.
"""
from __future__ import annotations

from . import capi


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
    if setup["solver"] == "mlw_m_1d":
        return capi.cfl_m_1d(safety, setup["dtmin"], setup["gm"], setup["bx"], *state,
                             setup["dx"])
    if setup["solver"] in ("mlw_m_3d", "roe_m_3d", "hlld_3d"):
        return capi.cfl_m_3d(safety, setup["dtmin"], setup["gm"], *state, setup["dx"],
                             setup["dy"], setup["dz"])
    if setup["solver"] == "mlw_m3":
        return capi.cfl_m3(safety, setup["dtmin"], setup["gm"], *state[:8], setup["dx"],
                           setup["dy"])
    return capi.cfl_m(safety, setup["dtmin"], setup["gm"], *state[:6], setup["dx"], setup["dy"])


def _step(setup, state, dt):
    if setup["solver"] == "mlw_m_1d":
        capi.mlw_m_1d(*state, setup["bx"], setup["bxm"], dt, setup["qav"], setup["gm"],
                      setup["dx"], setup["dxm"])
        return
    if setup["solver"] == "roe_m_3d":
        capi.roe_m_3d(*state, dt, setup["gm"], setup["dx"], setup["dy"], setup["dz"])
        return
    if setup["solver"] == "hlld_3d":
        capi.hlld_engine_3d(*state, setup["gm"], setup["mu"], dt, setup["dx"], setup["dxm"],
                            setup["dy"], setup["dym"], setup["dz"], setup["dzm"],
                            setup["mfdim"])
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
             "mlw_m_1d": _bnd1}.get(setup["solver"], _bnd)(setup, state)
            if not (ns < nstop and t < tend):
                return t, ns, 0, dts
    finally:
        if resident:
            capi.pull(state[0])
            capi.release(state[0])


def make_run(setup, exact=False, tile=-1, stream=None) -> capi.Run:
    run = capi.Run(setup["solver_id"], setup, setup["gm"], setup["qav"], setup["margin"],
                   exact=exact, tile=tile, stream=stream, mu=setup.get("mu", 1.0),
                   mfdim=setup.get("mfdim", (0, 0, 0)))
    run.set_bc_program(setup["bc"])
    return run


def run_resident(setup, state, nstop, tend=None, safety=None, t0=0.0, exact=False,
                 chunk=256, run: capi.Run | None = None):
    """Reference loop on the device.  Returns (t, ns, merr, nexec)."""
    tend = setup.get("tend", 1e30) if tend is None else tend
    safety = setup["safety"] if safety is None else safety
    own = run is None
    if own:
        run = make_run(setup, exact=exact)
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
