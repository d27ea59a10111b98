"""Generate the frozen oracle fixtures in this directory.

Run from the repository root:  python tests/golden/make_golden.py [name ...]
The fixtures freeze the CPU oracle's outputs on small seeded inputs so that a
change to the oracle (and through it the exact-mode GPU parity) is caught.
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from utrip_gb300 import setups  # noqa: E402

OUT = Path(__file__).resolve().parent


def case_2d(solver, ix, jx, seed, nsteps):
    s = setups.random_state(ix, jx, seed=seed, solver=solver)
    # inputs are stored too: the NumPy transcendental functions that build
    # them may differ in the last bit between machines
    out = {"in_" + k: a for k, a in zip(s["names"], s["state"])}
    for k in ("dx", "dxm", "dy", "dym"):
        out["grid_" + k] = s[k]
    st = setups.copy_state(s)
    dt0, _ = oracle.cfl_2d(s, st, 0.4)
    one = setups.copy_state(s)
    oracle.step_2d(s, one, dt0)
    t, ns, merr, dts = oracle.run_2d(s, st, nsteps)
    out.update({"dt0": np.array(dt0), "t": np.array(t), "ns": np.array(ns),
                "dts": np.array(dts)})
    for k, a in zip(s["names"], one):
        out["step1_" + k] = a
    for k, a in zip(s["names"], st):
        out["loop_" + k] = a
    return out


def case_roe(ix, jx, kx, seed):
    """One Roe-MUSCL step (cans3d/hdroe/roe_m.f) of a seeded 3-D state."""
    s = setups.random_state_3d(ix, jx, kx, seed=seed, solver="roe_m_3d")
    out = {"in_" + k: a for k, a in zip(s["names"], s["state"])}
    for k in ("dx", "dy", "dz"):
        out["grid_" + k] = s[k]
    st = setups.copy_state(s)
    dt, _ = oracle.cfl_3d(s, st, 0.4)
    oracle.roe_m_3d(*st, dt, s["gm"], s["dx"], s["dy"], s["dz"])
    out.update({"dt": np.array(dt), "gm": np.array(s["gm"])})
    for k, a in zip(s["names"], st):
        out["out_" + k] = a
    return out


def case_hlld(ix, jx, kx, seed):
    """One HLLD step (cansxx-nosupport/md_mhdshktb/hdhlld-x/engine.f) of a
    seeded 3-D state in Heaviside units, every axis active."""
    s = setups.random_state_3d(ix, jx, kx, seed=seed, solver="hlld_3d")
    out = {"in_" + k: a for k, a in zip(s["names"], s["state"])}
    for k in ("dx", "dy", "dz"):
        out["grid_" + k] = s[k]
    st = setups.copy_state(s)
    dt, _ = oracle.cfl_3d(s, st, 0.4)
    oracle.hlld_engine_3d(*st, s["gm"], s["mu"], dt, s["dx"], s["dy"], s["dz"], (1, 1, 1))
    out.update({"dt": np.array(dt), "gm": np.array(s["gm"]), "mu": np.array(s["mu"])})
    for k, a in zip(s["names"], st):
        out["out_" + k] = a
    return out


def case_roe2(ix, jx, seed):
    """One 2-D Roe-MUSCL step (cans2d/hdroe/roe_m3.f) of a seeded state,
    margin 2 as the md_mhdkh Roe package."""
    s = setups.random_state(ix, jx, seed=seed, solver="roe_m3")
    out = {"in_" + k: a for k, a in zip(s["names"], s["state"])}
    for k in ("dx", "dy"):
        out["grid_" + k] = s[k]
    st = setups.copy_state(s)
    dt, _ = oracle.cfl_2d(s, st, 0.4)
    oracle.roe_m3(*st, dt, s["gm"], s["dx"], s["dy"])
    out.update({"dt": np.array(dt), "gm": np.array(s["gm"])})
    for k, a in zip(s["names"], st):
        out["out_" + k] = a
    return out


def case_roe1(ix, seed):
    """One 1-D Roe-MUSCL step (cans1d/hdroe/roe_m.f) of a seeded state."""
    s = setups.random_state_1d(ix, seed=seed)
    out = {"in_" + k: a for k, a in zip(s["names"], s["state"])}
    out.update(bx=s["bx"], bxm=s["bxm"], dx=s["dx"])
    st = setups.copy_state(s)
    dt, _ = oracle.cfl_m_1d(0.5, 1e-10, 2.0, s["bx"], *st, s["dx"])
    oracle.roe_m_1d(*st, s["bx"], s["bxm"], dt, 2.0, s["dx"])
    out.update({"dt": np.array(dt), "gm": np.array(2.0)})
    for k, a in zip(s["names"], st):
        out["out_" + k] = a
    return out


def case_grav(solver, ix, jx, seed):
    """One 2-D step with gravity (mlw_m_g / mlw_m3_g) of a seeded state with
    seeded non-uniform gravity fields."""
    s = setups.random_gravity(setups.random_state(ix, jx, seed=seed, solver=solver), seed + 1)
    out = {"in_" + k: a for k, a in zip(s["names"], s["state"])}
    for k in ("dx", "dxm", "dy", "dym"):
        out["grid_" + k] = s[k]
    for k in ("gx", "gxm", "gy", "gym"):
        out["grav_" + k] = s[k]
    st = setups.copy_state(s)
    dt, _ = oracle.cfl_2d(s, st, 0.4)
    oracle.step_2d(s, st, dt)
    out["dt"] = np.array(dt)
    for k, a in zip(s["names"], st):
        out["out_" + k] = a
    return out


def case_res(solver, ix, jx, seed, grav):
    """One resistive 2-D step (mlw_m_e / mlw_m3_e, with gravity mlw_m_ge /
    mlw_m3_ge) of a seeded state with seeded resistivity, dt from cfl_m_e /
    cfl_m3_e."""
    s = setups.random_resistivity(
        setups.random_state(ix, jx, seed=seed, solver=solver, margin=2), seed + 1)
    if grav:
        s = setups.random_gravity(s, seed + 2)
    out = {"in_" + k: a for k, a in zip(s["names"], s["state"])}
    for k in ("dx", "dxm", "dy", "dym"):
        out["grid_" + k] = s[k]
    for k in ("et", "etm") + (("gx", "gxm", "gy", "gym") if grav else ()):
        out["src_" + k] = s[k]
    st = setups.copy_state(s)
    dt, _ = oracle.cfl_2d(s, st, 0.4)
    oracle.step_2d(s, st, dt)
    out["dt"] = np.array(dt)
    for k, a in zip(s["names"], st):
        out["out_" + k] = a
    return out


def case_grav3(ix, jx, kx, seed):
    """One 3-D step with gravity (cans3d/hdmlw/mlw_m_g.f) of a seeded state
    with seeded non-uniform gravity fields."""
    s = setups.random_gravity(setups.random_state_3d(ix, jx, kx, seed=seed), seed + 1)
    out = {"in_" + k: a for k, a in zip(s["names"], s["state"])}
    for k in ("dx", "dxm", "dy", "dym", "dz", "dzm"):
        out["grid_" + k] = s[k]
    for k in ("gx", "gxm", "gy", "gym", "gz", "gzm"):
        out["grav_" + k] = s[k]
    st = setups.copy_state(s)
    dt, _ = oracle.cfl_3d(s, st, 0.4)
    oracle.step_3d(s, st, dt)
    out["dt"] = np.array(dt)
    for k, a in zip(s["names"], st):
        out["out_" + k] = a
    return out


def case_res3(ix, jx, kx, seed):
    """One resistive 3-D step (cans3d/hdmlw/mlw_m_e.f) of a seeded state with
    seeded resistivity, dt from cfl_m_e (cans3d/common/cfl_m_e.f)."""
    s = setups.random_resistivity(setups.random_state_3d(ix, jx, kx, seed=seed), seed + 1)
    out = {"in_" + k: a for k, a in zip(s["names"], s["state"])}
    for k in ("dx", "dxm", "dy", "dym", "dz", "dzm"):
        out["grid_" + k] = s[k]
    for k in ("et", "etm"):
        out["src_" + k] = s[k]
    st = setups.copy_state(s)
    dt, _ = oracle.cfl_3d(s, st, 0.4)
    oracle.step_3d(s, st, dt)
    out["dt"] = np.array(dt)
    for k, a in zip(s["names"], st):
        out["out_" + k] = a
    return out


def bd_case():
    rng = np.random.default_rng(13)
    q = np.asfortranarray(rng.standard_normal((9, 7)))
    dxm = np.linspace(0.1, 0.2, 9)
    dym = np.linspace(0.1, 0.3, 7)
    bc = {}
    for kind in range(8):
        for axis in (0, 1):
            for mbnd in (0, 1):
                a = q.copy(order="F")
                oracle.bd(kind, axis, mbnd, 2, a, q0=0.75, dxm=dxm if axis == 0 else dym)
                bc[f"k{kind}_a{axis}_m{mbnd}"] = a
    return dict(q=q, dxm=dxm, dym=dym, **bc)


FIXTURES = {
    "mlw_m3_2d_18x14": lambda: case_2d("mlw_m3", 18, 14, 11, 10),
    "mlw_m_2d_16x20": lambda: case_2d("mlw_m", 16, 20, 12, 10),
    "bd_2d_9x7": bd_case,
    "roe_m_3d_14x12x13": lambda: case_roe(14, 12, 13, 21),
    "hlld_3d_13x11x12": lambda: case_hlld(13, 11, 12, 22),
    "roe_m3_2d_17x15": lambda: case_roe2(17, 15, 23),
    "roe_m_1d_70": lambda: case_roe1(70, 24),
    "mlw_m_g_2d_19x16": lambda: case_grav("mlw_m", 19, 16, 25),
    "mlw_m3_g_2d_17x18": lambda: case_grav("mlw_m3", 17, 18, 26),
    "mlw_m_e_2d_18x17": lambda: case_res("mlw_m", 18, 17, 27, False),
    "mlw_m3_ge_2d_17x19": lambda: case_res("mlw_m3", 17, 19, 28, True),
    "mlw_m_g_3d_13x12x14": lambda: case_grav3(13, 12, 14, 29),
    "mlw_m_e_3d_12x13x11": lambda: case_res3(12, 13, 11, 30),
}


def main(names):
    """Write the named fixtures (all of them when none is named)."""
    oracle.build()
    for name in names or FIXTURES:
        np.savez_compressed(OUT / f"{name}.npz", **FIXTURES[name]())
        print("wrote", OUT / f"{name}.npz")


if __name__ == "__main__":
    main(sys.argv[1:])
