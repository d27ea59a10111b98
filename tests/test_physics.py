"""Physics checks of the mLW path against known answers (the reference's
own validation is by model runs with analytic overlays, e.g.
cans2d/md_mhdwave/hdmlw/mhdwave_analytic.pro):

- linear sound, fast and Alfven waves travel at the phase speeds of the
  ideal-MHD dispersion relation (c_s^2 = gm p/rho, c_a^2 = B^2/(4 pi rho) in
  CANS units, c_f^2 = c_s^2 + c_a^2 across the field);
- the 1-D shock tube mirrored about x = 0 gives the mirrored solution.

The oracle runs them on the CPU; the GPU tests run the same waves through
the device-resident loop."""
import math

import numpy as np
import pytest

import oracle
from utrip_gb300 import capi, drivers, setups


def wave_setup(kind: str, n: int = 128, amp: float = 1e-6):
    """A periodic 2-D box [0,1] x [0, 4/n] (4 cells across), uniform rho = 1,
    p = 0.6, gm = 5/3 (c_s = 1), and one linear eigenmode of wavelength 1
    along x:
      sound   B = (ca sqrt(4 pi), 0, 0) along k; (d rho, d vx, d p) acoustic
      fast    B = (0, ca sqrt(4 pi), 0) across k; the fast mode with d by
      alfven  (mlw_m3) B = (ca sqrt(4 pi), 0, 0); d vz = -ca e, d bz = e sqrt(4 pi) ca
    with ca = 0.5.  Returns (setup, phase speed of the mode)."""
    solver = "mlw_m3" if kind == "alfven" else "mlw_m"
    m = 1
    x, dx, dxm = setups.uniform_axis(n, 1.0, m)
    y, dy, dym = setups.uniform_axis(4, 4.0 / n, m)
    X, _ = np.meshgrid(x, y, indexing="ij")
    gm, ro0, pr0, ca = 5.0 / 3.0, 1.0, 0.6, 0.5
    cs = math.sqrt(gm * pr0 / ro0)
    b0 = ca * math.sqrt(4.0 * math.pi * ro0)
    s = np.sin(2.0 * math.pi * X)
    z = np.zeros(X.shape)
    f = dict(ro=ro0 + z, pr=pr0 + z, vx=z.copy(), vy=z.copy(), vz=z.copy(), bx=z.copy(),
             by=z.copy(), bz=z.copy(), az=z.copy())
    if kind == "sound":
        c = cs
        f["bx"] = b0 + z
        f["ro"] = ro0 * (1 + amp * s)
        f["vx"] = c * amp * s
        f["pr"] = pr0 * (1 + gm * amp * s)
    elif kind == "fast":
        c = math.sqrt(cs * cs + ca * ca)
        f["by"] = b0 * (1 + amp * s)
        f["ro"] = ro0 * (1 + amp * s)
        f["vx"] = c * amp * s
        f["pr"] = pr0 * (1 + gm * amp * s)
    else:
        c = ca
        f["bx"] = b0 + z
        f["vz"] = -ca * amp * s
        f["bz"] = b0 * amp * s
    bc = []
    for v in range(len(setups.VARS[solver])):
        bc += [(v, face, setups.BD_PER, 0.0) for face in range(4)]
    st = setups._pack(solver, x, dx, dxm, y, dy, dym, f, gm, 3.0, bc, safety=0.4,
                      dtmin=1e-10, tend=0.25, margin=m, name=f"{kind}_wave_{n}")
    return st, c


def phase_speed(setup, state, var, t):
    """Phase speed of the wavelength-1 mode of `var` between the set-up and
    `state` at time t (interior cells, mean over y)."""
    m = setup["margin"]
    x = setup["x"][m:-m]
    k = 2.0 * math.pi

    def phase(a):
        row = a[m:-m, m:-m].mean(axis=1)
        row = row - row.mean()
        return math.atan2(np.sum(row * np.cos(k * x)), np.sum(row * np.sin(k * x)))

    i = setup["names"].index(var)
    dphi = phase(state[i]) - phase(setup["state"][i])
    dphi = (dphi + math.pi) % (2 * math.pi) - math.pi
    return -dphi / (k * t)


WAVES = [("sound", "ro"), ("fast", "ro"), ("alfven", "vz")]


@pytest.mark.parametrize("kind,var", WAVES)
def test_linear_wave_phase_speed_oracle(oracle_lib, kind, var):
    s, c = wave_setup(kind)
    st = setups.copy_state(s)
    t, ns, merr, _ = oracle_lib.run_2d(s, st, 10 ** 6, tend=0.25)
    assert merr == 0 and t >= 0.25
    got = phase_speed(s, st, var, t)
    # second-order scheme, 128 cells per wavelength: phase error ~1e-4
    assert abs(got - c) < 2e-3 * c, (kind, got, c)


def test_shock_tube_mirror_symmetry_oracle(oracle_lib):
    """x -> -x maps (rho, p, vx, vy, by) to (rho, p, -vx, vy, -by) with bx
    unchanged (B is a pseudovector); the mirrored tube evolves into the
    mirror image of the solution."""
    s = setups.shock_tube_1d(256)
    a = setups.copy_state(s)
    oracle_lib.run_1d(s, a, 200)
    sign = {"ro": 1, "pr": 1, "vx": -1, "vy": 1, "by": -1}
    mir = dict(s, state=[sign[k] * v[::-1].copy() for k, v in zip(s["names"], s["state"])])
    b = setups.copy_state(mir)
    oracle_lib.run_1d(mir, b, 200)
    for k, x, y in zip(s["names"], a, b):
        scale = max(float(np.max(np.abs(x))), 1e-300)
        assert np.max(np.abs(sign[k] * y[::-1] - x)) <= 1e-12 * scale, k


@pytest.mark.gpu
@pytest.mark.parametrize("kind,var", WAVES)
def test_linear_wave_phase_speed_gpu(gpu, oracle_lib, kind, var):
    s, c = wave_setup(kind)
    st = setups.copy_state(s)
    t, ns, merr, nexec = drivers.run_resident(s, st, 10 ** 6, tend=0.25)
    assert merr == 0 and t >= 0.25
    got = phase_speed(s, st, var, t)
    assert abs(got - c) < 2e-3 * c, (kind, got, c)


def friedrichs_ratios(s, state, t):
    """Outermost pressure peak along rays from the pulse centre (every 15
    degrees) divided by the fast-mode distance c_f(theta) t, theta the angle
    to the field: the fronts of cans2d/md_mhdwave trace the Friedrichs
    diagram of mhdwave_analytic.pro."""
    from scipy.interpolate import RegularGridInterpolator
    gm = s["gm"]
    cs2 = 1.0                                        # gm p / rho
    ca2 = (8 * math.pi / gm * float(np.float32(0.5))) / (4 * math.pi)
    f = RegularGridInterpolator((s["x"], s["y"]), state[1] - 1 / gm)
    out = []
    for deg in range(0, 180, 15):
        phi = math.radians(deg)
        r = np.linspace(0.05, 0.45, 1601)
        v = f(np.stack([r * math.cos(phi), r * math.sin(phi)], axis=1))
        peaks = [k for k in range(1, r.size - 1)
                 if v[k] >= v[k - 1] and v[k] >= v[k + 1] and v[k] > 0.2 * v.max()]
        c = math.cos(phi - s["thini"])
        cf = math.sqrt(0.5 * (cs2 + ca2 + math.sqrt((cs2 + ca2) ** 2 - 4 * cs2 * ca2 * c * c)))
        out.append(r[peaks[-1]] / (cf * t))
    return np.array(out)


def test_friedrichs_diagram_oracle(oracle_lib):
    pytest.importorskip("scipy")
    s = setups.mhd_wave_2d(128)
    st = setups.copy_state(s)
    t, ns, merr, _ = oracle_lib.run_2d(s, st, 10 ** 6, tend=0.25)
    ratios = friedrichs_ratios(s, st, t)
    assert np.all(np.abs(ratios - 1) < 0.05), ratios


@pytest.mark.gpu
def test_friedrichs_diagram_gpu(gpu):
    pytest.importorskip("scipy")
    s = setups.mhd_wave_2d(256)
    st = setups.copy_state(s)
    t, ns, merr, _ = drivers.run_resident(s, st, 10 ** 6, tend=0.25)
    ratios = friedrichs_ratios(s, st, t)
    assert np.all(np.abs(ratios - 1) < 0.03), ratios
