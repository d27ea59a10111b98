"""Model set-ups: grids, initial states and boundary programs.

These play the part of the reference model packages (md_*/hdmlw/model.f,
bnd.f and the grdrdy / bbtoaa calls of main.f) for the benchmark
configurations.  Everything is computed once on the host in NumPy and shared
by the GPU path and the CPU oracle, so transcendental functions in the
initial conditions never differ between them.

Field values are in CANS units: magnetic pressure is B^2/8pi, so a field
given in Heaviside-Lorentz form (B^2/2) is multiplied by sqrt(4 pi), as the
reference shock-tube set-up does (cans1d/md_mhdshktb/hdmlw/model.f:45-54).
"""
from __future__ import annotations

import math

import numpy as np

from .capi import (BD_CNS, BD_FRD, BD_FRE, BD_PER, BD_SMN, BD_SMP, BD_SPN, BD_SPP,
                   SOLVER_HLLD_3D,
                   SOLVER_MLW_M_2D, SOLVER_MLW_M3_2D, SOLVER_ROE_M3_2D, SOLVER_ROE_M_3D)

SQ4PI = math.sqrt(4.0 * math.pi)

# variable order of each solver (the order of the reference arguments)
VARS = {
    "mlw_m3": ["ro", "pr", "vx", "vy", "vz", "bx", "by", "bz", "az"],
    "mlw_m": ["ro", "pr", "vx", "vy", "bx", "by", "az"],
}
VARS["roe_m3"] = VARS["mlw_m3"]
SOLVER_ID = {"mlw_m": SOLVER_MLW_M_2D, "mlw_m3": SOLVER_MLW_M3_2D, "roe_m3": SOLVER_ROE_M3_2D}
# ghost layers of each 2-D solver (md_mhdkh/hdmlw/main.f:5 and
# md_mhdkh/hdroe/main.f:5)
MARGIN_2D = {"mlw_m": 1, "mlw_m3": 1, "roe_m3": 2}


def grdrdy(x: np.ndarray):
    """cans2d/common/grdrdy.f:28-42: dx, xm, dxm from the cell positions."""
    ix = x.size
    dxm = np.empty(ix)
    dxm[: ix - 1] = x[1:] - x[:-1]
    dxm[ix - 1] = dxm[ix - 2]
    dx = np.empty(ix)
    dx[1: ix - 1] = (dxm[: ix - 2] + dxm[1: ix - 1]) / 2.0
    dx[0] = dx[1]
    dx[ix - 1] = dx[ix - 2]
    xm = np.empty(ix)
    xm[: ix - 1] = (x[: ix - 1] + x[1:]) / 2.0
    xm[ix - 1] = xm[ix - 2] + dx[ix - 2]
    return dx, xm, dxm


def uniform_axis(n: int, length: float, margin: int = 1, origin: float = 0.0):
    """Cell positions built the way the model packages build them
    (cans2d/md_mhdkh/hdmlw/model.f:64-76): constant dxm, the first interior
    cell centred half a cell from `origin`, positions accumulated outward."""
    ix = n + 2 * margin
    d0 = length / n
    x = np.empty(ix)
    iz = margin  # 0-based index of the first interior cell
    x[iz] = origin + d0 / 2.0
    for i in range(iz + 1, ix):
        x[i] = x[i - 1] + d0
    for i in range(iz - 1, -1, -1):
        x[i] = x[i + 1] - d0
    dx, xm, dxm = grdrdy(x)
    return x, dx, dxm


def bbtoaa(bx: np.ndarray, by: np.ndarray, dxm: np.ndarray, dym: np.ndarray,
           margin: int) -> np.ndarray:
    """cans2d/common/bbtoaa.f:28-49: az by line integration from
    (margin+1, margin+1); the recurrences run in the reference order."""
    ix, jx = bx.shape
    az = np.zeros((ix, jx), order="F")
    m = margin  # 0-based index of Fortran index margin+1
    az[m, m] = 0.0
    for j in range(m + 1, jx):
        az[m, j] = az[m, j - 1] + 0.5 * (bx[m, j - 1] + bx[m, j]) * dym[j - 1]
    for j in range(m - 1, -1, -1):
        az[m, j] = az[m, j + 1] - 0.5 * (bx[m, j] + bx[m, j + 1]) * dym[j]
    # the i recurrences are independent per j: vectorised over j
    for i in range(m + 1, ix):
        az[i, :] = az[i - 1, :] - 0.5 * (by[i - 1, :] + by[i, :]) * dxm[i - 1]
    for i in range(m - 1, -1, -1):
        az[i, :] = az[i + 1, :] + 0.5 * (by[i, :] + by[i + 1, :]) * dxm[i]
    return az


def _farr(shape):
    return np.zeros(shape, order="F")


def _bc_all(nvar: int, x_kind: int, y_kind: int):
    prog = []
    for v in range(nvar):
        prog += [(v, 0, x_kind, 0.0), (v, 1, x_kind, 0.0),
                 (v, 2, y_kind, 0.0), (v, 3, y_kind, 0.0)]
    return prog


def _pack(solver, x, dx, dxm, y, dy, dym, fields, gm, qav, bc, **extra):
    names = VARS[solver]
    state = [np.asfortranarray(fields[k], dtype=np.float64) for k in names]
    d = dict(solver=solver, solver_id=SOLVER_ID[solver], names=names, x=x, dx=dx,
             dxm=dxm, y=y, dy=dy, dym=dym, state=state, gm=gm, qav=qav,
             margin=MARGIN_2D[solver], bc=bc)
    d.update(extra)
    return d


def orszag_tang(n: int = 512, solver: str = "mlw_m3", margin: int | None = None):
    """2-D Orszag-Tang vortex: [0, 2pi]^2 periodic, gamma=5/3,
    rho=25/(36 pi), p=5/(12 pi), v=(-sin y, sin x), B=(-sin y, sin 2x)/sqrt(4pi)
    in Heaviside-Lorentz units, i.e. (-sin y, sin 2x) in CANS units.  margin
    defaults to the solver's."""
    L = 2.0 * math.pi
    m = margin or MARGIN_2D[solver]
    x, dx, dxm = uniform_axis(n, L, m)
    y, dy, dym = uniform_axis(n, L, m)
    X, Y = np.meshgrid(x, y, indexing="ij")
    shape = X.shape
    f = {
        "ro": np.full(shape, 25.0 / (36.0 * math.pi)),
        "pr": np.full(shape, 5.0 / (12.0 * math.pi)),
        "vx": -np.sin(Y), "vy": np.sin(X), "vz": np.zeros(shape),
        "bx": SQ4PI * (-np.sin(Y) / SQ4PI), "by": SQ4PI * (np.sin(2.0 * X) / SQ4PI),
        "bz": np.zeros(shape),
    }
    f["az"] = bbtoaa(np.asfortranarray(f["bx"]), np.asfortranarray(f["by"]), dxm, dym, m)
    nvar = len(VARS[solver])
    return _pack(solver, x, dx, dxm, y, dy, dym, f, 5.0 / 3.0, 3.0,
                 _bc_all(nvar, BD_PER, BD_PER), safety=0.4, dtmin=1e-10, margin=m,
                 tend=math.pi / 2.0, name=f"orszag_tang_{n}")


def shear_layer(n: int = 256, beta: float = 1.0, seed: int = 4, ny: int | None = None,
                solver: str = "mlw_m3"):
    """Magnetised shear layer on [0,1]^2 (the md_mhdkh set-up shape,
    cans2d/md_mhdkh/hdmlw/model.f:94-165): vx = 0.5 tanh((y-0.5)/0.05),
    vy = 1e-3 sin(2 pi x + phase) with a seeded phase, rho=1, gamma=5/3,
    B0 = sqrt(4pi)(1, 0.5, 0) and p = beta |B0_HL|^2 / 2.  Periodic in x,
    bdsppy in y (md_mhdkh/hdmlw/bnd.f:11-39)."""
    ny = ny or n
    rng = np.random.default_rng(seed)
    phase = float(rng.uniform(0.0, 2.0 * math.pi))
    m = MARGIN_2D[solver]
    x, dx, dxm = uniform_axis(n, 1.0, m)
    y, dy, dym = uniform_axis(ny, 1.0, m)
    X, Y = np.meshgrid(x, y, indexing="ij")
    shape = X.shape
    b0 = np.array([1.0, 0.5, 0.0])
    f = {
        "ro": np.ones(shape),
        "pr": np.full(shape, beta * float(b0 @ b0) / 2.0),
        "vx": 0.5 * np.tanh((Y - 0.5) / 0.05),
        "vy": 1e-3 * np.sin(2.0 * math.pi * X + phase),
        "vz": np.zeros(shape),
        "bx": np.full(shape, SQ4PI * b0[0]), "by": np.full(shape, SQ4PI * b0[1]),
        "bz": np.zeros(shape),
    }
    f["az"] = bbtoaa(np.asfortranarray(f["bx"]), np.asfortranarray(f["by"]), dxm, dym, m)
    nvar = len(VARS[solver])
    return _pack(solver, x, dx, dxm, y, dy, dym, f, 5.0 / 3.0, 3.0,
                 _bc_all(nvar, BD_PER, BD_SPP), safety=0.4, dtmin=1e-10,
                 tend=1e30, beta=beta, phase=phase, name=f"shear_layer_{n}x{ny}_b{beta:g}")


def random_state(ix: int, jx: int, seed: int = 0, solver: str = "mlw_m3", amp: float = 0.05,
                 margin: int | None = None):
    """Smooth state with seeded random perturbations on every variable, for
    parity tests that exercise all terms of the step (non-uniform fields in
    every component, including vz, bz and az).  margin defaults to the
    solver's."""
    rng = np.random.default_rng(seed)
    m = margin or MARGIN_2D[solver]
    x, dx, dxm = uniform_axis(ix - 2 * m, 1.0, m)
    y, dy, dym = uniform_axis(jx - 2 * m, 1.0, m)
    X, Y = np.meshgrid(x, y, indexing="ij")

    def smooth(scale):
        kx, ky = rng.integers(1, 4, size=2)
        ph = rng.uniform(0, 2 * math.pi, size=2)
        base = np.sin(2 * math.pi * kx * X + ph[0]) * np.cos(2 * math.pi * ky * Y + ph[1])
        return scale * (base + amp * rng.standard_normal(X.shape))

    f = {
        "ro": 1.0 + 0.3 * np.abs(smooth(1.0)),
        "pr": 0.6 + 0.2 * np.abs(smooth(1.0)),
        "vx": smooth(0.3), "vy": smooth(0.3), "vz": smooth(0.2),
        "bx": SQ4PI * (0.8 + smooth(0.2)), "by": SQ4PI * smooth(0.3),
        "bz": SQ4PI * smooth(0.2), "az": smooth(0.1),
    }
    nvar = len(VARS[solver])
    return _pack(solver, x, dx, dxm, y, dy, dym, f, 5.0 / 3.0, 3.0,
                 _bc_all(nvar, BD_PER, BD_SPP), safety=0.4, dtmin=1e-10,
                 tend=1e30, margin=m, name=f"random_{ix}x{jx}_s{seed}")


VARS["mlw_m_3d"] = ["ro", "pr", "vx", "vy", "vz", "bx", "by", "bz"]
SOLVER_ID["mlw_m_3d"] = 2
VARS["roe_m_3d"] = VARS["mlw_m_3d"]
SOLVER_ID["roe_m_3d"] = SOLVER_ROE_M_3D
VARS["hlld_3d"] = VARS["mlw_m_3d"]
SOLVER_ID["hlld_3d"] = SOLVER_HLLD_3D
# ghost layers of each 3-D solver (hdmlw/main.f:5, hdroe/main.f:5,
# cansxx-nosupport/md_mhdshktb/hdhlld-x/main.f:5)
MARGIN_3D = {"mlw_m_3d": 1, "roe_m_3d": 3, "hlld_3d": 3}
# the HLLD engine works in Heaviside units (B^2/2): fields given in CANS units
# (B^2/8pi) are divided by sqrt(4 pi) for it
B_UNIT = {"mlw_m_3d": 1.0, "roe_m_3d": 1.0, "hlld_3d": 1.0 / math.sqrt(4.0 * math.pi)}


def _bc_all3(nvar: int, kinds=(BD_PER, BD_PER, BD_PER)):
    prog = []
    for v in range(nvar):
        for axis, kind in enumerate(kinds):
            prog += [(v, 2 * axis, kind, 0.0), (v, 2 * axis + 1, kind, 0.0)]
    return prog


def _pack3(x, dx, dxm, y, dy, dym, z, dz, dzm, fields, gm, qav, bc, solver="mlw_m_3d",
           **extra):
    names = VARS[solver]
    state = [np.asfortranarray(fields[k], dtype=np.float64) for k in names]
    d = dict(solver=solver, solver_id=SOLVER_ID[solver], names=names, x=x, dx=dx,
             dxm=dxm, y=y, dy=dy, dym=dym, z=z, dz=dz, dzm=dzm, state=state, gm=gm, qav=qav,
             margin=MARGIN_3D[solver], bc=bc)
    if solver == "hlld_3d":
        d.update(mu=1.0, mfdim=(1, 1, 1))
    d.update(extra)
    return d


def _periodic_pad(a: np.ndarray, margin: int = 1) -> np.ndarray:
    return np.asfortranarray(np.pad(a, margin, mode="wrap"))


def turbulence_3d(n: int = 256, seed: int = 3, kmax: float = 8.0, rms: float = 1e-2,
                  solver: str = "mlw_m_3d", b0=(1.0, 0.0, 0.0)):
    """3-D MHD at plasma beta 1 on [0,1]^3, periodic: rho=1, p=0.5,
    B = sqrt(4pi)(1,0,0) (beta = 8 pi p / B^2 = 1), gamma=5/3, and a seeded
    Gaussian random velocity whose Fourier modes are limited to integer
    wavenumbers |k| <= kmax, rescaled to an rms speed of `rms`.  The interior
    is the same for both 3-D solvers; the ghost layers are 1 (mlw_m_3d) or 3
    (roe_m_3d, hlld_3d) cells wide; hlld_3d takes the field in Heaviside
    units.  b0 is the unit direction of the mean field."""
    m = MARGIN_3D[solver]
    rng = np.random.default_rng(seed)
    k = np.fft.fftfreq(n, d=1.0 / n)
    kz = np.fft.rfftfreq(n, d=1.0 / n)
    KX, KY, KZ = np.meshgrid(k, k, kz, indexing="ij")
    mask = (KX ** 2 + KY ** 2 + KZ ** 2) <= kmax ** 2
    mask[0, 0, 0] = False
    comps = []
    for _ in range(3):
        spec = np.zeros(mask.shape, dtype=np.complex128)
        cnt = int(mask.sum())
        spec[mask] = rng.standard_normal(cnt) + 1j * rng.standard_normal(cnt)
        comps.append(np.fft.irfftn(spec, s=(n, n, n), axes=(0, 1, 2)))
    v2 = sum(c ** 2 for c in comps)
    scale = rms / math.sqrt(float(np.mean(v2)))
    x, dx, dxm = uniform_axis(n, 1.0, margin=m)
    shape = (n + 2 * m,) * 3
    f = {
        "ro": np.ones(shape), "pr": np.full(shape, 0.5),
        "vx": _periodic_pad(comps[0] * scale, m), "vy": _periodic_pad(comps[1] * scale, m),
        "vz": _periodic_pad(comps[2] * scale, m),
        "bx": np.full(shape, SQ4PI * B_UNIT[solver] * b0[0]),
        "by": np.full(shape, SQ4PI * B_UNIT[solver] * b0[1]),
        "bz": np.full(shape, SQ4PI * B_UNIT[solver] * b0[2]),
    }
    return _pack3(x, dx, dxm, x.copy(), dx.copy(), dxm.copy(), x.copy(), dx.copy(), dxm.copy(),
                  f, 5.0 / 3.0, 3.0, _bc_all3(8), solver=solver, safety=0.4, dtmin=1e-10,
                  tend=1e30, name=f"turbulence_{n}^3")


def random_state_3d(ix: int, jx: int, kx: int, seed: int = 0, amp: float = 0.05,
                    solver: str = "mlw_m_3d"):
    """Seeded smooth-plus-noise 3-D state with every component non-zero, for
    parity tests; periodic in x, bdspp in y, bdfre in z.  ix, jx, kx include
    the ghost layers of the solver."""
    rng = np.random.default_rng(seed)
    m = MARGIN_3D[solver]
    x, dx, dxm = uniform_axis(ix - 2 * m, 1.0, margin=m)
    y, dy, dym = uniform_axis(jx - 2 * m, 1.0, margin=m)
    z, dz, dzm = uniform_axis(kx - 2 * m, 1.0, margin=m)
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")

    def smooth(scale):
        kk = rng.integers(1, 4, size=3)
        ph = rng.uniform(0, 2 * math.pi, size=3)
        base = (np.sin(2 * math.pi * kk[0] * X + ph[0]) * np.cos(2 * math.pi * kk[1] * Y + ph[1])
                * np.cos(2 * math.pi * kk[2] * Z + ph[2]))
        return scale * (base + amp * rng.standard_normal(X.shape))

    f = {
        "ro": 1.0 + 0.3 * np.abs(smooth(1.0)), "pr": 0.6 + 0.2 * np.abs(smooth(1.0)),
        "vx": smooth(0.3), "vy": smooth(0.3), "vz": smooth(0.3),
        "bx": SQ4PI * (0.8 + smooth(0.2)), "by": SQ4PI * smooth(0.3), "bz": SQ4PI * smooth(0.3),
    }
    for k in ("bx", "by", "bz"):
        f[k] = f[k] * B_UNIT[solver]
    return _pack3(x, dx, dxm, y, dy, dym, z, dz, dzm, f, 5.0 / 3.0, 3.0,
                  _bc_all3(8, (BD_PER, BD_SPP, 5)), solver=solver, safety=0.4, dtmin=1e-10,
                  tend=1e30, name=f"random3d_{ix}x{jx}x{kx}_s{seed}")


def _r4(v: float) -> float:
    """A Fortran real*4 literal or real*4 result, widened to double."""
    return float(np.float32(v))


def shock_tube_3d(n: int = 32, solver: str = "roe_m_3d", tend: float = 0.1):
    """Oblique 3-D MHD shock tube as cans3d/md_mhdshktb/{hdroe,hdmlw}/model.f
    sets it up: n^3 interior cells of size 1/n, izero = ix/2+1 centred at
    dxm/2, gamma = 2; the discontinuity is the plane n.x = 0 with the normal
    at theta = 60, phi = 30 degrees (real*4 60./180.); left rho=1, p=1, right
    rho=0.125, p=0.1 (real*4 0.1); B = b0 (0.75 n +/- e) with e a unit vector
    normal to n; v = 0.  bnd.f: bdfre on every face, margin 3 (hdroe) or 1
    (hdmlw); tend = 0.1, safety 0.4 (main.f:25,167)."""
    m = MARGIN_3D[solver]
    ix = n + 2 * m
    pi = math.acos(-1.0)

    def axis():
        dx0 = 1.0 / _r4(ix - 2 * m)
        dxm = np.full(ix, dx0)
        x = np.empty(ix)
        iz = ix // 2  # 0-based index of izero = ix/2+1
        x[iz] = dxm[iz] / 2.0
        for i in range(iz + 1, ix):
            x[i] = x[i - 1] + dxm[i - 1]
        for i in range(iz - 1, -1, -1):
            x[i] = x[i + 1] - dxm[i]
        dx, _, dxm2 = grdrdy(x)
        return x, dx, dxm2

    x, dx, dxm = axis()
    b0 = math.sqrt(4 * pi)
    thini = _r4(_r4(60.0) / _r4(180.0)) * pi
    phini = _r4(_r4(30.0) / _r4(180.0)) * pi
    ux, uy, uz = math.sin(thini) * math.cos(phini), math.sin(thini) * math.sin(phini), \
        math.cos(thini)
    ebx0, eby0 = 1.0, 2.0
    ebz0 = -(ebx0 * ux + eby0 * uy) / uz
    ebb0 = math.sqrt(ebx0 ** 2 + eby0 ** 2 + ebz0 ** 2)
    ebx, eby, ebz = ebx0 / ebb0, eby0 / ebb0, ebz0 / ebb0
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    left = (ux * X + uy * Y + uz * Z) <= 0.0
    shape = (ix,) * 3
    f = {
        "ro": np.where(left, 1.0, 0.125), "pr": np.where(left, 1.0, _r4(0.1)),
        "vx": np.zeros(shape), "vy": np.zeros(shape), "vz": np.zeros(shape),
        "bx": np.where(left, b0 * 0.75 * ux + b0 * ebx, b0 * 0.75 * ux - b0 * ebx),
        "by": np.where(left, b0 * 0.75 * uy + b0 * eby, b0 * 0.75 * uy - b0 * eby),
        "bz": np.where(left, b0 * 0.75 * uz + b0 * ebz, b0 * 0.75 * uz - b0 * ebz),
    }
    return _pack3(x, dx, dxm, x.copy(), dx.copy(), dxm.copy(), x.copy(), dx.copy(), dxm.copy(),
                  f, 2.0, 3.0, _bc_all3(8, (5, 5, 5)), solver=solver, safety=0.4, dtmin=1e-10,
                  tend=tend, name=f"shock_tube_3d_{n}^3_{solver}")


VARS["mlw_m_1d"] = ["ro", "pr", "vx", "vy", "by"]
SOLVER_ID["mlw_m_1d"] = 3


def shock_tube_1d(n: int = 1024, safety: float | None = None, tend: float = 0.1,
                  solver: str = "mlw_m_1d"):
    """Brio-Wu-type MHD shock tube as cans1d/md_mhdshktb/hdmlw/model.f sets
    it up: margin 1, dx0 = 1/n, cell izero = ix/2 centred at -dx0/2 (the
    interface between cells ix/2 and ix/2+1 at x = 0; the box is [-0.5, 0.5],
    a translation of [0, 1] with the interface at 0.5), gamma = 2.  Left
    (x <= 0): rho=1, p=1, By=+sqrt(4pi); right: rho=0.125, p=0.1,
    By=-sqrt(4pi); Bx = 0.75 sqrt(4pi).  bnd.f: bdsppx for ro, pr, vy, by and
    bdsmnx for vx on both faces.  qav = 1 (main.f:149).  solver "roe_m_1d"
    is the Roe package of the same model (md_mhdshktb/hdroe: margin 3, cfl
    safety 1.0, main.f:5,139); the mLW package uses margin 1, safety 0.4."""
    margin = 3 if solver == "roe_m_1d" else 1
    if safety is None:
        safety = 1.0 if solver == "roe_m_1d" else 0.4
    ix = n + 2 * margin
    dx0 = 1.0 / float(np.float32(ix - 2 * margin))
    dxm0 = np.full(ix, dx0)
    x = np.empty(ix)
    iz = ix // 2 - 1  # 0-based index of Fortran izero = ix/2
    x[iz] = -dxm0[iz] / 2
    for i in range(iz + 1, ix):
        x[i] = x[i - 1] + dxm0[i - 1]
    for i in range(iz - 1, -1, -1):
        x[i] = x[i + 1] - dxm0[i]
    dx, _, dxm = grdrdy(x)
    left = x <= 0
    f = {
        "ro": np.where(left, 1.0, 0.125), "pr": np.where(left, 1.0, 0.1),
        "vx": np.zeros(ix), "vy": np.zeros(ix),
        "by": np.where(left, math.sqrt(4.0 * math.pi), -math.sqrt(4.0 * math.pi)),
    }
    bx = np.full(ix, 0.75 * math.sqrt(4.0 * math.pi))
    bc = []
    for v, name in enumerate(VARS["mlw_m_1d"]):
        kind = BD_SMN if name == "vx" else BD_SPP
        bc += [(v, 0, kind, 0.0), (v, 1, kind, 0.0)]
    state = [np.ascontiguousarray(f[k], dtype=np.float64) for k in VARS["mlw_m_1d"]]
    return dict(solver=solver, solver_id=3, names=VARS["mlw_m_1d"], x=x, dx=dx, dxm=dxm,
                bx=bx, bxm=bx.copy(), state=state, gm=2.0, qav=1.0, margin=margin, bc=bc,
                safety=safety, dtmin=1e-10, tend=tend, dtout=0.01,
                name=f"shock_tube_{n}" if solver == "mlw_m_1d" else f"shock_tube_{solver}_{n}")


def _shktb_axis(n: int, margin: int = 1):
    """cans1d/md_shktb/hdmlw/model.f:18-31: dx0 = 1/real(ix - 2 margin),
    cell izero = ix/2 centred at -dx0/2, positions accumulated outward."""
    ix = n + 2 * margin
    dx0 = 1.0 / float(np.float32(ix - 2 * margin))
    dxm0 = np.full(ix, dx0)
    x = np.empty(ix)
    iz = ix // 2 - 1  # 0-based index of Fortran izero = ix/2
    x[iz] = -dxm0[iz] / 2
    for i in range(iz + 1, ix):
        x[i] = x[i - 1] + dxm0[i - 1]
    for i in range(iz - 1, -1, -1):
        x[i] = x[i + 1] - dxm0[i]
    dx, _, dxm = grdrdy(x)
    return x, dx, dxm


def sod_shock_tube(n: int = 1024, ndim: int = 1, ncross: int = 4,
                   safety: float | None = None):
    """The hydrodynamic shock tube of cans1d/md_shktb/hdmlw (model.f:33-53,
    main.f:20-23,136-146) run by the ideal-MHD mLW step with B = 0: gamma =
    1.4; left (x <= 0) rho = 1, p = 1, right rho = 0.125, p = 0.1, at rest;
    qav = 0.3; tend = 0.14154.  The x axis is model.f's (n cells, the
    interface at x = 0 on a cell edge); bnd.f: bdsppx for rho and p, bdspnx
    for vx (the waves do not reach the walls by tend).

    ndim 1 runs the 1-D mlw_m (bx = by = 0) with safety 1.0 as main.f does;
    ndim 2 and 3 run mlw_m3 and the 3-D mlw_m on an x-aligned tube of
    ncross cells across (periodic, spacing dx) with the 2-D/3-D drivers'
    safety 0.4: their cfl_m divides by sqrt(v^2 + c^2), not |v| + c, so
    safety 1 would put the x Courant number above 1.  The exact answer is
    oracle/shktb_analytic.py, the restatement of md_shktb's
    shktb_analytic.pro."""
    x, dx, dxm = _shktb_axis(n)
    left = x <= 0.0
    ro1d = np.where(left, 1.0, 0.125)
    pr1d = np.where(left, 1.0, 0.1)
    common = dict(tend=0.14154, dtmin=1e-10, sod=dict(gm=1.4, ro1=0.125, pr1=0.1, ro4=1.0,
                                                      pr4=1.0, x0=0.0))
    if ndim == 1:
        f = {"ro": ro1d, "pr": pr1d, "vx": np.zeros(x.size), "vy": np.zeros(x.size),
             "by": np.zeros(x.size)}
        bc = []
        for v, name in enumerate(VARS["mlw_m_1d"]):
            kind = BD_SPN if name == "vx" else BD_SPP
            bc += [(v, 0, kind, 0.0), (v, 1, kind, 0.0)]
        state = [np.ascontiguousarray(f[k], dtype=np.float64) for k in VARS["mlw_m_1d"]]
        return dict(solver="mlw_m_1d", solver_id=3, names=VARS["mlw_m_1d"], x=x, dx=dx,
                    dxm=dxm, bx=np.zeros(x.size), bxm=np.zeros(x.size), state=state, gm=1.4,
                    qav=0.3, margin=1, bc=bc, safety=1.0 if safety is None else safety,
                    dtout=0.01, name=f"sod_{n}_1d", **common)
    yc, dyc, dymc = uniform_axis(ncross, ncross * float(dxm[1]))
    sf = 0.4 if safety is None else safety
    if ndim == 2:
        shape = (x.size, ncross + 2)
        ro = np.repeat(ro1d[:, None], shape[1], axis=1)
        pr = np.repeat(pr1d[:, None], shape[1], axis=1)
        z = np.zeros(shape)
        f = {"ro": ro, "pr": pr, "vx": z, "vy": z, "vz": z, "bx": z, "by": z, "bz": z,
             "az": z}
        bc = []
        for v, name in enumerate(VARS["mlw_m3"]):
            kind = BD_SPN if name == "vx" else BD_SPP
            bc += [(v, 0, kind, 0.0), (v, 1, kind, 0.0), (v, 2, BD_PER, 0.0),
                   (v, 3, BD_PER, 0.0)]
        return _pack("mlw_m3", x, dx, dxm, yc, dyc, dymc, f, 1.4, 0.3, bc, safety=sf,
                     name=f"sod_{n}x{ncross}_mlw_m3", **common)
    shape = (x.size, ncross + 2, ncross + 2)
    ro = np.broadcast_to(ro1d[:, None, None], shape).copy()
    pr = np.broadcast_to(pr1d[:, None, None], shape).copy()
    z = np.zeros(shape)
    f = {"ro": ro, "pr": pr, "vx": z, "vy": z, "vz": z, "bx": z, "by": z, "bz": z}
    bc = []
    for v, name in enumerate(VARS["mlw_m_3d"]):
        kind = BD_SPN if name == "vx" else BD_SPP
        bc += [(v, 0, kind, 0.0), (v, 1, kind, 0.0)]
        for face in (2, 3, 4, 5):
            bc.append((v, face, BD_PER, 0.0))
    return _pack3(x, dx, dxm, yc, dyc, dymc, yc.copy(), dyc.copy(), dymc.copy(), f, 1.4, 0.3,
                  bc, solver="mlw_m_3d", safety=sf,
                  name=f"sod_{n}x{ncross}x{ncross}_mlw_m_3d", **common)


def sod_shock_tube_riemann(n: int = 1024, solver: str = "roe_m_3d", ncross: int = 4,
                           safety: float | None = None):
    """The md_shktb hydrodynamic shock tube (model.f:18-53: gamma = 1.4, left
    rho = 1, p = 1, right rho = 0.125, p = 0.1, at rest, the interface at
    x = 0 on a cell edge; tend = 0.14154) run by the ideal-MHD Riemann-solver
    steps with B = 0, with their packages' three ghost layers:
    - "roe_m_1d": the 1-D roe_m, safety 1.0 (md_shktb/hdroe/main.f:92, whose
      1-D CFL divides by |v| + c as this one does);
    - "roe_m3": the 2-D roe_m3 on an x-aligned tube ncross cells across;
    - "roe_m_3d": the 3-D roe_m on an x-aligned tube ncross x ncross across;
    - "hlld_3d": the HLLD engine along x alone (jx = kx = 1, mfdim = 1,0,0,
      as the hdhlld-x package runs its shock tube).
    The 2-D/3-D CFL divides by sqrt(v^2 + c^2), so those take the 0.4 of
    their drivers.  x faces: bdsppx for every variable but vx, bdspnx for vx
    (md_shktb bnd.f); cross axes periodic.  The exact answer is
    oracle/shktb_analytic.py."""
    m = 3
    x, dx, dxm = _shktb_axis(n, margin=m)
    left = x <= 0.0
    ro1d = np.where(left, 1.0, 0.125)
    pr1d = np.where(left, 1.0, 0.1)
    common = dict(tend=0.14154, dtmin=1e-10, dtout=0.01, margin=m,
                  sod=dict(gm=1.4, ro1=0.125, pr1=0.1, ro4=1.0, pr4=1.0, x0=0.0))

    def xfaces(names, cross_faces=()):
        bc = []
        for v, name in enumerate(names):
            kind = BD_SPN if name == "vx" else BD_SPP
            bc += [(v, 0, kind, 0.0), (v, 1, kind, 0.0)]
            bc += [(v, f, BD_PER, 0.0) for f in cross_faces]
        return bc

    if solver == "roe_m_1d":
        names = VARS["mlw_m_1d"]
        f = {"ro": ro1d, "pr": pr1d, "vx": np.zeros(x.size), "vy": np.zeros(x.size),
             "by": np.zeros(x.size)}
        state = [np.ascontiguousarray(f[k], dtype=np.float64) for k in names]
        return dict(solver=solver, solver_id=3, names=names, x=x, dx=dx, dxm=dxm,
                    bx=np.zeros(x.size), bxm=np.zeros(x.size), state=state, gm=1.4, qav=0.0,
                    bc=xfaces(names), safety=1.0 if safety is None else safety,
                    name=f"sod_{n}_roe_m_1d", **common)
    sf = 0.4 if safety is None else safety
    if solver == "roe_m3":
        yc, dyc, dymc = uniform_axis(ncross, ncross * float(dxm[m]), margin=m)
        shape = (x.size, yc.size)
        f = {k: np.zeros(shape) for k in VARS["roe_m3"]}
        f["ro"] = np.repeat(ro1d[:, None], shape[1], axis=1)
        f["pr"] = np.repeat(pr1d[:, None], shape[1], axis=1)
        return _pack("roe_m3", x, dx, dxm, yc, dyc, dymc, f, 1.4, 0.0,
                     xfaces(VARS["roe_m3"], (2, 3)), safety=sf,
                     name=f"sod_{n}x{ncross}_roe_m3", **common)
    if solver == "roe_m_3d":
        yc, dyc, dymc = uniform_axis(ncross, ncross * float(dxm[m]), margin=m)
        shape = (x.size, yc.size, yc.size)
        f = {k: np.zeros(shape) for k in VARS["roe_m_3d"]}
        f["ro"] = np.broadcast_to(ro1d[:, None, None], shape).copy()
        f["pr"] = np.broadcast_to(pr1d[:, None, None], shape).copy()
        return _pack3(x, dx, dxm, yc, dyc, dymc, yc.copy(), dyc.copy(), dymc.copy(), f, 1.4,
                      0.0, xfaces(VARS["roe_m_3d"], (2, 3, 4, 5)), solver="roe_m_3d",
                      safety=sf, name=f"sod_{n}x{ncross}x{ncross}_roe_m_3d", **common)
    if solver == "hlld_3d":
        one = (np.array([0.5]), np.array([1.0]), np.array([1.0]))  # an inactive axis
        shape = (x.size, 1, 1)
        f = {k: np.zeros(shape) for k in VARS["hlld_3d"]}
        f["ro"] = ro1d[:, None, None].copy()
        f["pr"] = pr1d[:, None, None].copy()
        return _pack3(x, dx, dxm, *one, *one, f, 1.4, 0.0, xfaces(VARS["hlld_3d"]),
                      solver="hlld_3d", mu=1.0, mfdim=(1, 0, 0), safety=sf,
                      name=f"sod_{n}_hlld", **common)
    raise ValueError(f"no Riemann-solver shock tube for {solver!r}")


def sod_interior_profile(setup: dict, state) -> tuple:
    """(x, dx, ro, pr, vx) along the tube's interior cells; for a 2-D or 3-D
    tube the first interior row (every row holds the same profile)."""
    m = setup["margin"]
    sl = slice(m, -m)
    # the first interior cell across the tube (an inactive axis has one cell)
    j = m if state[0].ndim > 1 and state[0].shape[1] > 2 * m else 0
    pick = {1: lambda a: a[sl], 2: lambda a: a[sl, j], 3: lambda a: a[sl, j, j]}[state[0].ndim]
    names = setup["names"]
    return (setup["x"][sl], setup["dx"][sl], pick(state[names.index("ro")]),
            pick(state[names.index("pr")]), pick(state[names.index("vx")]))


def random_state_1d(ix: int, seed: int = 0):
    """Smooth-plus-noise 1-D state for parity tests (every variable varies)."""
    rng = np.random.default_rng(seed)
    x, dx, dxm = uniform_axis(ix - 2, 1.0)
    k = rng.integers(1, 4, size=5)
    ph = rng.uniform(0, 2 * math.pi, size=5)
    s = [np.sin(2 * math.pi * k[i] * x + ph[i]) + 0.05 * rng.standard_normal(ix) for i in range(5)]
    f = {"ro": 1.0 + 0.3 * np.abs(s[0]), "pr": 0.6 + 0.2 * np.abs(s[1]), "vx": 0.3 * s[2],
         "vy": 0.3 * s[3], "by": SQ4PI * 0.4 * s[4]}
    bx = SQ4PI * (0.7 + 0.05 * np.sin(2 * math.pi * x))
    bxm = SQ4PI * (0.7 + 0.05 * np.sin(2 * math.pi * (x + dxm / 2)))
    bc = [(v, f_, BD_PER, 0.0) for v in range(5) for f_ in (0, 1)]
    state = [np.ascontiguousarray(f[k], dtype=np.float64) for k in VARS["mlw_m_1d"]]
    return dict(solver="mlw_m_1d", solver_id=3, names=VARS["mlw_m_1d"], x=x, dx=dx, dxm=dxm,
                bx=bx, bxm=bxm, state=state, gm=5.0 / 3.0, qav=3.0, margin=1, bc=bc,
                safety=0.4, dtmin=1e-10, tend=1e30, name=f"random1d_{ix}_s{seed}")


def copy_state(setup: dict):
    return [a.copy(order="F") for a in setup["state"]]


def shock_tube_hlld_1d(n: int = 1024, tend: float = 0.1):
    """The HLLD shock tube of cansxx-nosupport/md_mhdshktb/hdhlld-x
    (model.f, bnd.f, main.f): ix = n + 6 (margin 3), jx = kx = 1, active axis
    x only (mfdim = 1,0,0); gamma = 2, mu = 1, Heaviside units with
    b0 = sqrt(2 mu/gm) = 1: left rho=1, p=1, B=(0.75, 1, 0), right rho=0.125,
    p=0.1, B=(0.75, -1, 0), v=0, the interface at x=0 (izero = ix/2+1 centred
    at dxm/2).  The cell size is 1/dble(max(ix-2*margin, ix)) = 1/ix, as the
    model writes it; grdrdy2 gives dx = dxm.  bdfrex on both faces, margin 3;
    the loop calls the 3-D cfl_m with safety 0.4, tend = 0.1."""
    m = 3
    ix, jx, kx = n + 2 * m, 1, 1

    def axis(nx):
        d0 = 1.0 / float(max(nx - 2 * m, nx))
        dxm = np.full(nx, d0)
        x = np.empty(nx)
        iz = nx // 2  # 0-based index of izero = nx/2+1
        x[iz] = dxm[iz] / 2.0
        for i in range(iz + 1, nx):
            x[i] = x[i - 1] + dxm[i - 1]
        for i in range(iz - 1, -1, -1):
            x[i] = x[i + 1] - dxm[i]
        dx = np.empty(nx)
        dx[1:] = 0.5 * (dxm[:-1] + dxm[1:])  # grdrdy2.f
        dx[0] = dxm[0]
        return x, dx, dxm

    x, dx, dxm = axis(ix)
    y, dy, dym = axis(jx)
    z, dz, dzm = axis(kx)
    gm, mu = 2.0, 1.0
    b0 = math.sqrt(2.0 * mu / gm)
    left = (x <= 0.0)[:, None, None] * np.ones((ix, jx, kx), dtype=bool)
    f = {
        "ro": np.where(left, 1.0, 0.125), "pr": np.where(left, 1.0, 0.1),
        "vx": np.zeros((ix, jx, kx)), "vy": np.zeros((ix, jx, kx)), "vz": np.zeros((ix, jx, kx)),
        "bx": np.where(left, b0 * 0.75 * 1.0 + b0 * 0.0, b0 * 0.75 * 1.0 - b0 * 0.0),
        "by": np.where(left, b0 * 0.75 * 0.0 + b0 * 1.0, b0 * 0.75 * 0.0 - b0 * 1.0),
        "bz": np.where(left, b0 * 0.75 * 0.0 + b0 * 0.0, b0 * 0.75 * 0.0 - b0 * 0.0),
    }
    bc = [(v, f_, 5, 0.0) for v in range(8) for f_ in (0, 1)]
    return _pack3(x, dx, dxm, y, dy, dym, z, dz, dzm, f, gm, 0.0, bc, solver="hlld_3d",
                  mu=mu, mfdim=(1, 0, 0), safety=0.4, dtmin=1e-10, tend=tend,
                  name=f"shock_tube_hlld_{n}")


# ---- the spicule model (cans1d/md_spicule/hdmlw) ------------------------------

VARS["mlw_m_bg_1d"] = ["ro", "pr", "vx", "vy", "by"]
SOLVER_ID["mlw_m_bg_1d"] = 6
# static profiles of mlw_m_bg (cans1d/hdmlw/mlw_m_bg.f:2-3), in the order the
# run descriptor takes them
BG_PROFILES = ["gx", "gxm", "sc", "scm", "dsc", "dscm", "rr", "rrm", "drr", "drrm"]


def bd_host_1d(kind: int, mbnd: int, m: int, q: np.ndarray) -> None:
    """One bd* rule on a host line in place (cans1d/bc/bdsppx.f, bdspnx.f,
    bdsmpx.f, bdsmnx.f, bdfrex.f), for the set-up's static profiles.  The
    indices below are the reference's 1-based ones."""
    n = q.size

    def get(i):
        return q[i - 1]

    def put(i, v):
        q[i - 1] = v

    if mbnd == 0:
        b = 1 + m
        for i in range(1, m + 1):
            if kind == BD_SPP:
                put(b - i, get(b - 1 + i))
            elif kind == BD_SPN:
                put(b - i, -get(b - 1 + i))
            elif kind == BD_SMP:
                put(b - i, get(b + i))
            elif kind == BD_SMN:
                put(b - i, -get(b + i))
            elif kind == BD_FRE:
                put(b - i, get(b))
        if kind == BD_SMN:
            put(b, 0.0)
    else:
        b = n - m
        for i in range(1, m + 1):
            if kind == BD_SPP:
                put(b + i, get(b + 1 - i))
            elif kind == BD_SPN:
                put(b + i, -get(b + 1 - i))
            elif kind == BD_SMP:
                put(b + i, get(b - i))
            elif kind == BD_SMN:
                put(b + i, -get(b - i))
            elif kind == BD_FRE:
                put(b + i, get(b))
        if kind == BD_SMN:
            put(b, 0.0)


def scrdy(sc: np.ndarray, scm: np.ndarray, dx: np.ndarray, dxm: np.ndarray):
    """cans1d/common/scrdy.f:28-34: dsc(2..ix-1) and dscm(2..ix-2).  The
    other entries are left at zero, the value the reference main program's
    static arrays hold there."""
    ix = sc.size
    dsc = np.zeros(ix)
    dscm = np.zeros(ix)
    for i in range(2, ix):          # 1-based i = 2..ix-1
        dsc[i - 1] = (scm[i - 1] - scm[i - 2]) / dx[i - 1]
    for i in range(2, ix - 1):      # 1-based i = 2..ix-2
        dscm[i - 1] = (sc[i] - sc[i - 1]) / dxm[i - 1]
    return dsc, dscm


def chkdav_host(da: np.ndarray, vx: np.ndarray, floor: float) -> int:
    """cans1d/common/chkdav.f:68-76 on host arrays: values below `floor` are
    raised to it and the velocity there set to zero; returns the count."""
    low = da < floor
    da[low] = floor
    vx[low] = 0.0
    return int(low.sum())


def spicule_1d(nx: int = 1024, torque: float = 30.0, seed: int = 0, tend: float = 100.0,
               nstop: int = 100000, dtout: float = 0.5, beta: float = 1.0):
    """The spicule model: cans1d/md_spicule/hdmlw/model.f with the set-up
    part of main.f (grdrdy, bnd, scrdy twice, bndsc, chkdav of ro and pr),
    margin 1, ix = nx + 2.

    Grid: dxm = 0.04 up to cell i1 = aint(2 ztr/dx0), then growing by 2 %
    per cell up to 50 dx0; cell izero = 2 centred at dxm/2.  Gravity
    -1/gm (1 - tanh((x-400)/10))/2 on cells and faces (both evaluated at the
    cell position, model.f:104-110), then bdspnx / bdsmnx.  A temperature
    step of width 0.5 at ztr = 15 from 1 to 300, hydrostatic density built
    outward from the base cell with ro0 = 1, p = ro T / gm.  Flux tube:
    rr = 1, bx uniform with plasma beta `beta` at the bottom (model.f's
    onebeta, 1.0 in the package; the studies' parameter), cross section 1/bx.
    Boundaries (bnd.f): bdsppx (vx: bdspnx) at the bottom, bdfrex at the top.
    The loop (main.f:160-219): cfl_m with safety 0.8 and dtmin 1e-10,
    mlw_m_bg with qav = 1, the torque source of trqalfven.f, bnd, chkdav of
    ro and pr with floor 1e-9."""
    margin = 1
    ix = nx + 2 * margin
    ztr = 15.0
    gm = 5.0 / 3.0
    # ---- grid (model.f:36-68) -------------------------------------------------
    dx0 = 0.04
    i1 = int(2.0 * ztr / dx0)
    apx1 = 1.02
    dxmax1 = 50.0 * dx0
    dxm0 = np.full(ix, dx0)
    if i1 < ix:
        for i in range(i1 + 1, ix + 1):          # 1-based i1+1..ix
            v = apx1 * dxm0[i - 2]
            dxm0[i - 1] = dxmax1 if v > dxmax1 else v
    bd_host_1d(BD_SMP, 0, margin - 1, dxm0)
    izero = margin + 1
    x = np.empty(ix)
    x[izero - 1] = dxm0[izero - 1] / 2
    for i in range(izero + 1, ix + 1):
        x[i - 1] = x[i - 2] + dxm0[i - 2]
    for i in range(izero - 1, 0, -1):
        x[i - 1] = x[i] - dxm0[i - 1]
    # ---- gravity (model.f:86-101) ---------------------------------------------
    gl0 = 1.0 / gm
    ro0, pr0, te0 = 1.0, 1.0 / gm, 1.0
    tpho, wtr = te0, 0.5
    zg0, wg0 = 400.0, 10.0
    gx = -(gl0 * (1.0 - np.tanh((x - zg0) / wg0)) / 2)
    gxm = gx.copy()
    bd_host_1d(BD_SPN, 0, margin, gx)
    bd_host_1d(BD_SMN, 0, margin - 1, gxm)
    rr = np.ones(ix)
    rrm = np.ones(ix)
    # ---- hydrostatic atmosphere (model.f:113-148) ------------------------------
    ac = 300.0
    te = tpho * (1 + 0.5 * (ac - 1) * (np.tanh((x - ztr) / wtr) + 1.0))
    ro1 = np.empty(ix)
    i = izero + 1
    h = 0.5 * gm * gxm[i - 2] * dxm0[i - 2] / 2
    ro1[i - 1] = (te[i - 2] + h) / (te[i - 1] - h) * ro0
    for i in range(izero + 2, ix + 1):
        h = 0.5 * gm * gxm[i - 2] * dxm0[i - 2]
        ro1[i - 1] = (te[i - 2] + h) / (te[i - 1] - h) * ro1[i - 2]
    i = izero
    h = 0.5 * gm * gxm[i - 1] * dxm0[i - 1] / 2
    ro1[i - 1] = (te[i] - h) / (te[i - 1] + h) * ro0
    for i in range(izero - 1, 0, -1):
        h = 0.5 * gm * gxm[i - 1] * dxm0[i - 1]
        ro1[i - 1] = ro1[i] * (te[i] - h) / (te[i - 1] + h)
    pr1 = pr0 * (ro1 / ro0) * (te / te0)
    # ---- field and flux tube (model.f:150-185) -------------------------------
    pi = math.acos(-1.0)
    onebeta = float(beta)
    bx = np.empty(ix)
    bx[0] = math.sqrt(onebeta * 8 * pi * pr1[0])
    bx[1:] = bx[0] * (rr[0] / rr[1:]) ** 2
    bxm = np.empty(ix)
    bxm[: ix - 1] = 0.5 * (bx[: ix - 1] + bx[1:])
    bxm[ix - 1] = bxm[ix - 2]
    sc = 1.0 / bx
    scm = 1.0 / bxm
    # ---- main.f:78-90: metrics, boundaries, cross-section derivatives ---------
    dx, _, dxm = grdrdy(x)
    f = {"ro": ro1.copy(), "pr": pr1.copy(), "vx": np.zeros(ix), "vy": np.zeros(ix),
         "by": np.zeros(ix)}
    bc = []
    for v, name in enumerate(VARS["mlw_m_bg_1d"]):
        bc.append((v, 0, BD_SPN if name == "vx" else BD_SPP, 0.0))
    for v in range(5):
        bc.append((v, 1, BD_FRE, 0.0))
    for v, face, kind, _ in bc:
        bd_host_1d(kind, face, margin, f[VARS["mlw_m_bg_1d"][v]])
    dsc, dscm = scrdy(sc, scm, dx, dxm)
    drr, drrm = scrdy(rr, rrm, dx, dxm)
    # bndsc.f:9-19
    bd_host_1d(BD_SPP, 0, margin, sc)
    bd_host_1d(BD_SPN, 0, margin, dsc)
    bd_host_1d(BD_SMP, 0, margin - 1, scm)
    bd_host_1d(BD_SMN, 0, margin - 1, dscm)
    bd_host_1d(BD_SPP, 1, margin, sc)
    bd_host_1d(BD_SPN, 1, margin, dsc)
    bd_host_1d(BD_SMP, 1, margin, scm)
    bd_host_1d(BD_SMN, 1, margin, dscm)
    floor = 1e-9
    chkdav_host(f["ro"], f["vx"], floor)
    chkdav_host(f["pr"], f["vx"], floor)
    # torque profile of trqalfven.f:25-29 (the 0.075 is a real*4 literal)
    trq = np.tanh((x - 0.75) / float(np.float32(0.075))) - 1
    trq[ix - 1] = trq[ix - 3]
    state = [np.ascontiguousarray(f[k], dtype=np.float64) for k in VARS["mlw_m_bg_1d"]]
    prof = dict(gx=gx, gxm=gxm, sc=sc, scm=scm, dsc=dsc, dscm=dscm, rr=rr, rrm=rrm,
                drr=drr, drrm=drrm)
    return dict(solver="mlw_m_bg_1d", solver_id=6, names=VARS["mlw_m_bg_1d"], x=x, dx=dx,
                dxm=dxm, bx=bx, bxm=bxm, state=state, gm=gm, qav=1.0, margin=margin, bc=bc,
                safety=0.8, dtmin=1e-10, tend=tend, nstop=nstop, dtout=dtout, floor=floor,
                trq=trq, trq0=float(torque), seed=int(seed), ztr=ztr, tcor=200.0,
                beta=float(beta), name=f"spicule_{nx}", **prof)


# ---- 2-D steps with gravity (mlw_m_g / mlw_m3_g) -------------------------------

def mhd_gravity_wave(n: int = 64, solver: str = "mlw_m", amp: float = 0.5):
    """The MHD gravity-wave model of cans2d/md_mhdgwave/hdmlw (model.f, bnd.f,
    main.f:161-176): x in [0, 5], y in [-2, 6], margin 1, gamma 5/3,
    uniform gravity gy = -1/gm on cells and corners, an isothermal
    hydrostatic atmosphere built outward from the cell jzero with the
    discrete balance of model.f, a vertical field with 1/beta = 0.05, and a
    Gaussian pressure pulse of relative amplitude amp and width 0.2 at the
    origin.  Boundaries: x symmetric (vx, bx odd), y free with constant
    gradient for ro and pr and odd vy.  cfl_m safety 0.4, qav 3, tend 7.
    solver "mlw_m3" adds vz = bz = 0."""
    margin = 1
    ix = jx = n + 2 * margin
    gm = 5.0 / 3.0
    ymax, ymin, xmax = 6.0, -2.0, 5.0
    pi = math.acos(-1.0)
    dx0 = xmax / float(ix - margin * 2)
    dxm0 = np.full(ix, dx0)
    izero = margin + 1
    x = np.empty(ix)
    x[izero - 1] = dxm0[izero - 1] / 2.0
    for i in range(izero + 1, ix + 1):
        x[i - 1] = x[i - 2] + dxm0[i - 2]
    for i in range(izero - 1, 0, -1):
        x[i - 1] = x[i] - dxm0[i - 1]
    dy0 = (ymax - ymin) / float(jx - margin * 2)
    dym0 = np.full(jx, dy0)
    jzero = int(-ymin / dy0) + margin + 1
    y = np.empty(jx)
    y[jzero - 1] = dym0[jzero - 1] / 2.0
    for j in range(jzero + 1, jx + 1):
        y[j - 1] = y[j - 2] + dym0[j - 2]
    for j in range(jzero - 1, 0, -1):
        y[j - 1] = y[j] - dym0[j - 1]
    g0 = -1.0 / gm
    gym0 = np.full(jx, g0)
    tem0 = np.ones(jx)
    den0 = np.empty(jx)
    pre0 = np.empty(jx)
    den0[jzero - 1] = 1.0
    pre0[jzero - 1] = 1.0 / gm * tem0[jzero - 1]
    for j in range(jzero + 1, jx + 1):
        h = 0.5 * gm * gym0[j - 2] * dym0[j - 2]
        den0[j - 1] = den0[j - 2] * (tem0[j - 2] + h) / (tem0[j - 1] - h)
        pre0[j - 1] = pre0[jzero - 1] * (den0[j - 1] / den0[jzero - 1]) * \
            (tem0[j - 1] / tem0[jzero - 1])
    for j in range(jzero - 1, 0, -1):
        h = 0.5 * gm * gym0[j - 1] * dym0[j - 1]
        den0[j - 1] = den0[j] * (tem0[j] - h) / (tem0[j - 1] + h)
        pre0[j - 1] = pre0[jzero - 1] * (den0[j - 1] / den0[jzero - 1]) * \
            (tem0[j - 1] / tem0[jzero - 1])
    betai = float(np.float32(0.05))
    bb0 = math.sqrt(8 * pi * 1 / gm * betai)
    X, Y = np.meshgrid(x, y, indexing="ij")
    shape = (ix, jx)
    wexp = float(np.float32(0.2))
    ss = np.sqrt(X ** 2 + Y ** 2)
    f = {"ro": np.broadcast_to(den0, shape).copy(),
         "pr": np.broadcast_to(pre0, shape) * (1 + amp * np.exp(-(ss / wexp) ** 2)),
         "vx": np.zeros(shape), "vy": np.zeros(shape), "vz": np.zeros(shape),
         "bx": np.zeros(shape), "by": np.full(shape, bb0), "bz": np.zeros(shape)}
    dx, _, dxm = grdrdy(x)
    dy, _, dym = grdrdy(y)
    f["az"] = bbtoaa(np.asfortranarray(f["bx"]), np.asfortranarray(f["by"]), dxm, dym, margin)
    names = VARS[solver]
    bc = []
    for v, name in enumerate(names):
        bc.append((v, 0, BD_SPN if name in ("vx", "bx") else BD_SPP, 0.0))
        bc.append((v, 1, BD_SPN if name in ("vx", "bx") else BD_SPP, 0.0))
    for v, name in enumerate(names):
        kind = BD_FRD if name in ("ro", "pr") else (BD_SPN if name == "vy" else BD_FRE)
        bc.append((v, 2, kind, 0.0))
        bc.append((v, 3, kind, 0.0))
    grav = dict(gx=np.zeros(shape, order="F"), gxm=np.zeros(shape, order="F"),
                gy=np.full(shape, g0, order="F"), gym=np.full(shape, g0, order="F"))
    return _pack(solver, x, dx, dxm, y, dy, dym, f, gm, 3.0, bc, safety=0.4, dtmin=1e-10,
                 tend=7.0, gravity=True, name=f"mhd_gravity_wave_{n}_{solver}", **grav)


def random_gravity(s: dict, seed: int = 0, scale: float = 0.3) -> dict:
    """Seeded non-uniform gravity fields on a 2-D or 3-D set-up (every source
    term of mlw_m_g / mlw_m3_g, or of the 3-D mlw_m_g, non-zero): returns a
    copy with gx, gxm, gy, gym (and gz, gzm in 3-D)."""
    rng = np.random.default_rng(seed)
    shape = s["state"][0].shape
    out = dict(s)
    keys = ("gx", "gxm", "gy", "gym") + (("gz", "gzm") if len(shape) == 3 else ())
    for k in keys:
        out[k] = np.asfortranarray(scale * rng.standard_normal(shape))
    out["gravity"] = True
    return out


def random_resistivity(s: dict, seed: int = 0, scale: float = 0.02) -> dict:
    """Seeded non-negative resistivity on a 2-D or 3-D set-up (et at the
    cells, etm at the corners, every resistive term of mlw_m_e / mlw_m3_e or
    of the 3-D mlw_m_e non-zero): returns a copy with et and etm."""
    rng = np.random.default_rng(seed)
    shape = s["state"][0].shape
    out = dict(s)
    for k in ("et", "etm"):
        out[k] = np.asfortranarray(scale * (0.5 + rng.random(shape)))
    return out


def magnetic_reconnection(n: int = 128):
    """The magnetic-reconnection model of cans2d/md_recon/hdmlw (model.f,
    bnd.f, main.f:161-176): x in [0, 5], y in [0, 20] on n x n cells with two
    ghost layers, gamma 5/3, a Harris-type current sheet by =
    sqrt(8 pi betai/gm) tanh(x/0.5) with betai = 10 in pressure balance, and
    a localised resistivity etai (2 r^3 - 3 retai r^2)/retai^3 + etai inside
    r < retai = 0.8 of the origin (et at the cells, etm at the corners; zero
    elsewhere).  Boundaries: symmetric about x = 0 and y = 0 (vx, by odd at
    x = 0; vy, bx odd at y = 0), the same rules at the outer faces with bx
    odd at the outer x face.  cfl_m_e safety 0.4, qav 3, tend 23."""
    margin = 2
    ix = jx = n + 2 * margin
    gm = 5.0 / 3.0
    pi = math.acos(-1.0)
    xmax, ymax = 5.0, 20.0

    def axis(length, nn):
        d0 = length / float(nn - margin * 2)
        dm = np.full(nn, d0)
        iz = margin + 1
        x = np.empty(nn)
        x[iz - 1] = dm[iz - 1] / 2.0
        for i in range(iz + 1, nn + 1):
            x[i - 1] = x[i - 2] + dm[i - 2]
        for i in range(iz - 1, 0, -1):
            x[i - 1] = x[i] - dm[i - 1]
        return x, dm

    x, dxm0 = axis(xmax, ix)
    y, dym0 = axis(ymax, jx)
    X, Y = np.meshgrid(x, y, indexing="ij")
    etai, retai = 0.03, 0.8

    def eta(rr):
        # etai*(2*rr**3-3*retai*rr**2)/retai**3+etai (model.f), integer
        # powers as repeated products
        r3 = rr * rr * rr
        v = etai * (2.0 * r3 - (3.0 * retai) * (rr * rr)) / (retai * retai * retai) + etai
        return np.where(rr < retai, v, 0.0)

    rr = np.sqrt(X * X + Y * Y)
    et = eta(rr)
    Xm = X + (dxm0 / 2.0)[:, None]
    Ym = Y + (dym0 / 2.0)[None, :]
    etm = eta(np.sqrt(Xm * Xm + Ym * Ym))
    betai = 10.0
    by = np.sqrt(betai * pi * 8 / gm) * np.tanh(X / 0.5)
    pr = 1 / gm * (1 + betai) - by * by / pi / 8.0
    f = {"ro": pr * gm, "pr": pr, "vx": np.zeros(X.shape), "vy": np.zeros(X.shape),
         "bx": np.zeros(X.shape), "by": by}
    dx, _, dxm = grdrdy(x)
    dy, _, dym = grdrdy(y)
    f["az"] = bbtoaa(np.asfortranarray(f["bx"]), np.asfortranarray(f["by"]), dxm, dym, margin)
    names = VARS["mlw_m"]
    # bnd.f: per face, the rule of each variable (SPN = odd about the face)
    odd = {0: ("vx", "by"), 1: ("vx", "bx"), 2: ("vy", "bx"), 3: ("vy", "bx")}
    bc = []
    for face in range(4):
        for v, name in enumerate(names):
            bc.append((v, face, BD_SPN if name in odd[face] else BD_SPP, 0.0))
    s = _pack("mlw_m", x, dx, dxm, y, dy, dym, f, gm, 3.0, bc, safety=0.4, dtmin=1e-10,
              tend=23.0, dtout=1.0, margin=margin, name=f"magnetic_reconnection_{n}")
    s["et"] = np.asfortranarray(et)
    s["etm"] = np.asfortranarray(etm)
    return s


def magnetic_reconnection_3d(n: int = 128, nz: int = 4):
    """The 3-D magnetic-reconnection model of cans3d/md_recon/hdmlw (model.f,
    bnd.f, main.f:167-186): the current sheet of the 2-D model (x in [0, 5],
    y in [0, 20]) extended over z in [0, 2], n x n x nz cells with two ghost
    layers, the same localised resistivity in every z plane, cfl_m_e ->
    mlw_m_e -> bnd with safety 0.4, qav 3, tend 23.  Boundaries (bnd.f): at
    x = 0 vx, by, bz odd; at the outer x face vx, bx odd; at y = 0 vy, bx, bz
    odd; at the outer y face vy, vz, bx odd; at both z faces vz, bz odd; the
    other variables even."""
    margin = 2
    ix = jx = n + 2 * margin
    kx = nz + 2 * margin
    gm = 5.0 / 3.0
    pi = math.acos(-1.0)

    def axis(length, nn):
        d0 = length / float(nn - margin * 2)
        dm = np.full(nn, d0)
        iz = margin + 1
        c = np.empty(nn)
        c[iz - 1] = dm[iz - 1] / 2.0
        for i in range(iz + 1, nn + 1):
            c[i - 1] = c[i - 2] + dm[i - 2]
        for i in range(iz - 1, 0, -1):
            c[i - 1] = c[i] - dm[i - 1]
        return c, dm

    x, dxm0 = axis(5.0, ix)
    y, dym0 = axis(20.0, jx)
    z, _ = axis(2.0, kx)
    X, Y, _ = np.meshgrid(x, y, z, indexing="ij")
    etai, retai = 0.03, 0.8

    def eta(rr):
        # etai*(2*rr**3-3*retai*rr**2)/retai**3+etai (model.f:67-74), integer
        # powers as repeated products
        r3 = rr * rr * rr
        v = etai * (2.0 * r3 - (3.0 * retai) * (rr * rr)) / (retai * retai * retai) + etai
        return np.where(rr < retai, v, 0.0)

    et = eta(np.sqrt(X * X + Y * Y))
    Xm = X + (dxm0 / 2.0)[:, None, None]
    Ym = Y + (dym0 / 2.0)[None, :, None]
    etm = eta(np.sqrt(Xm * Xm + Ym * Ym))
    betai = 10.0
    by = np.sqrt(betai * pi * 8 / gm) * np.tanh(X / 0.5)
    pr = 1 / gm * (1 + betai) - by * by / pi / 8.0
    zero = np.zeros(X.shape)
    f = {"ro": pr * gm, "pr": pr, "vx": zero, "vy": zero, "vz": zero, "bx": zero, "by": by,
         "bz": zero}
    dx, _, dxm = grdrdy(x)
    dy, _, dym = grdrdy(y)
    dz, _, dzm = grdrdy(z)
    names = VARS["mlw_m_3d"]
    odd = {0: ("vx", "by", "bz"), 1: ("vx", "bx"), 2: ("vy", "bx", "bz"),
           3: ("vy", "vz", "bx"), 4: ("vz", "bz"), 5: ("vz", "bz")}
    bc = [(v, face, BD_SPN if name in odd[face] else BD_SPP, 0.0)
          for face in range(6) for v, name in enumerate(names)]
    s = _pack3(x, dx, dxm, y, dy, dym, z, dz, dzm, f, gm, 3.0, bc, safety=0.4, dtmin=1e-10,
               tend=23.0, dtout=1.0, margin=margin,
               name=f"magnetic_reconnection_{n}x{n}x{nz}")
    s["et"] = np.asfortranarray(et)
    s["etm"] = np.asfortranarray(etm)
    return s


def _efr_column(z, dzm0, kzero, gm, nz):
    """The vertical structure of the md_efr models (model.f): temperature
    tem0 of the convection zone, photosphere and corona, the flux-sheet
    profile rbeta0 = 1/beta, and density, pressure and field bmx0 in the
    discrete magnetohydrostatic balance built outward from cell kzero."""
    pi = math.acos(-1.0)
    ztr = 10.0
    g0 = -1.0 / gm
    gzm0 = np.full(z.size, g0)
    wtr, tcor, tadg, zcnv = 0.5, 25.0, 2.0, 0.0
    tem0 = (1.0 - tadg * (gm - 1.0) / gm * (z - zcnv) * 0.5 * (1 - np.tanh(z - zcnv))
            + 0.5 * (tcor - 1.0) * (np.tanh((z - ztr) / wtr) + 1.0))
    zf1, zf2, rbetaf = -2.0, -0.0, 1 / 4.0
    af1 = (np.tanh((z - zf1) / 0.5) + 1.0) / 2
    af2 = (-np.tanh((z - zf2) / 0.5) + 1.0) / 2
    rbeta0 = rbetaf * af1 * af2
    kx = z.size
    den0 = np.empty(kx)
    pre0 = np.empty(kx)
    kz = kzero - 1
    den0[kz] = 1.0
    pre0[kz] = 1.0 / gm * tem0[kz]
    for k in range(kz + 1, kx):
        h = 0.5 * gm * gzm0[k - 1] * dzm0[k - 1]
        den0[k] = den0[k - 1] * ((1 + rbeta0[k - 1]) * tem0[k - 1] + h) / \
            ((1 + rbeta0[k]) * tem0[k] - h)
        pre0[k] = pre0[kz] * (den0[k] / den0[kz]) * (tem0[k] / tem0[kz])
    for k in range(kz - 1, -1, -1):
        h = 0.5 * gm * gzm0[k] * dzm0[k]
        den0[k] = den0[k + 1] * ((1 + rbeta0[k + 1]) * tem0[k + 1] - h) / \
            ((1 + rbeta0[k]) * tem0[k] + h)
        pre0[k] = pre0[kz] * (den0[k] / den0[kz]) * (tem0[k] / tem0[kz])
    if not (np.all(den0 > 0) and np.all(pre0 > 0)):
        # the discrete balance needs tem0 > 0.5 gm |g| dz across the
        # photosphere: about 48 cells or more along the vertical
        raise ValueError(f"{nz} cells are too coarse for the stratification of md_efr")
    bmx0 = np.sqrt(8 * pi * pre0 * rbeta0)
    return den0, pre0, bmx0


def _efr_perturbation(X, Z):
    """pertub.f: amp = 0.05 (single precision), xptb = 20, between z = -2
    and 0, on the vertical velocity."""
    pi = math.acos(-1.0)
    amp, xptb, zptb1, zptb2, wptb = float(np.float32(0.05)), 20.0, -2.0, 0.0, 0.5
    return (amp * np.cos(2 * pi * X / xptb) * 0.5
            * (np.tanh((X + 0.75 * xptb) / wptb) - np.tanh((X - 0.75 * xptb) / wptb)) * 0.5
            * (np.tanh((Z - zptb1) / wptb) - np.tanh((Z - zptb2) / wptb)))


def _efr_axis(n, d0, iz):
    dm = np.full(n, d0)
    x = np.empty(n)
    x[iz - 1] = dm[iz - 1] / 2.0
    for i in range(iz + 1, n + 1):
        x[i - 1] = x[i - 2] + dm[i - 2]
    for i in range(iz - 1, 0, -1):
        x[i - 1] = x[i] - dm[i - 1]
    return x, dm


def emerging_flux_2d(nx: int = 64, ny: int = 128):
    """The 2-D emerging-flux model of cans2d/md_efr/hdmlw (model.f, pertub.f,
    bnd.f, main.f:160-183): the vertical structure of the 3-D model along y
    in [-4, 40], x in [0, 40], nx x ny cells (the reference runs 64 x 128)
    with one ghost layer, gravity gy = -1/gm, the flux sheet bx, a vy
    perturbation, az from bbtoaa.  Boundaries: x symmetric (vx, by odd); at
    the y faces vy, by odd, vx, bx, az even, and ro, pr held at their initial
    ghost values (bdiniy, the constant rule bdcnsy for this horizontally
    uniform state).  mlw_m_g, cfl_m safety 0.4, qav 3, tend 80, and chkdav
    of ro and pr with floor 1e-9 after every boundary fill."""
    margin = 1
    ix, jx = nx + 2 * margin, ny + 2 * margin
    gm = 5.0 / 3.0
    ymax, ymin, xmax = 40.0, -4.0, 40.0
    x, _ = _efr_axis(ix, xmax / float(ix - 2 * margin), margin + 1)
    dy0 = (ymax - ymin) / float(jx - 2 * margin)
    jzero = int(-ymin / dy0) + margin + 1
    y, dym0 = _efr_axis(jx, dy0, jzero)
    den0, pre0, bmx0 = _efr_column(y, dym0, jzero, gm, ny)
    shape = (ix, jx)
    X, Y = np.meshgrid(x, y, indexing="ij")
    f = {"ro": np.broadcast_to(den0, shape).copy(), "pr": np.broadcast_to(pre0, shape).copy(),
         "vx": np.zeros(shape), "vy": 0.0 + _efr_perturbation(X, Y),
         "bx": np.broadcast_to(bmx0, shape).copy(), "by": np.zeros(shape)}
    dx, _, dxm = grdrdy(x)
    dy, _, dym = grdrdy(y)
    f["az"] = bbtoaa(np.asfortranarray(f["bx"]), np.asfortranarray(f["by"]), dxm, dym, margin)
    names = VARS["mlw_m"]
    bc = []
    for face in (0, 1):
        for v, name in enumerate(names):
            bc.append((v, face, BD_SPN if name in ("vx", "by") else BD_SPP, 0.0))
    for face in (2, 3):
        for v, name in enumerate(names):
            if name in ("ro", "pr"):
                base = den0 if name == "ro" else pre0
                bc.append((v, face, BD_CNS, float(base[0 if face == 2 else jx - 1])))
            else:
                bc.append((v, face, BD_SPN if name in ("vy", "by") else BD_SPP, 0.0))
    g0 = -1.0 / gm
    grav = dict(gx=np.zeros(shape, order="F"), gxm=np.zeros(shape, order="F"),
                gy=np.full(shape, g0, order="F"), gym=np.full(shape, g0, order="F"))
    # main.f:183-185: chkdav of ro and pr with floor 1e-9 after every bnd
    return _pack("mlw_m", x, dx, dxm, y, dy, dym, f, gm, 3.0, bc, safety=0.4, dtmin=1e-10,
                 tend=80.0, dtout=1.0, gravity=True, floor=1e-9,
                 name=f"emerging_flux_{nx}x{ny}", **grav)


def emerging_flux_3d(nx: int = 128, ny: int = 2, nz: int = 128):
    """The 3-D emerging-flux model of cans3d/md_efr/hdmlw (model.f, pertub.f,
    bnd.f, main.f:174-191): x in [0, 40], y in [0, 2], z in [-4, 40] on
    nx x ny x nz cells with one ghost layer (the reference runs 128 x 2 x
    128), gamma 5/3, uniform gravity gz = -1/gm on cells and corners, a
    convection zone / photosphere / corona temperature profile, a horizontal
    flux sheet bx = sqrt(8 pi p rbeta) with 1/beta = rbetaf = 1/4 between
    z = -2 and 0 in magnetohydrostatic balance (the discrete balance of
    model.f), and a vz perturbation of amplitude 0.05 (pertub.f).
    Boundaries: x and y symmetric (vx, by, bz odd at the x faces; vy, by odd
    at the y faces); at the z faces vz and bz odd, vx, vy, bx, by even, and
    ro, pr held at their initial ghost values (bdiniz, which for this
    horizontally uniform state is the constant rule bdcnsz).  cfl_m safety
    0.4, qav 3, tend 80, dtout 1."""
    margin = 1
    ix, jx, kx = nx + 2 * margin, ny + 2 * margin, nz + 2 * margin
    gm = 5.0 / 3.0
    zmax, zmin, xmax, ymax = 40.0, -4.0, 40.0, 2.0
    # dx0 = xmax/real(ix-margin*2): the count converted in single precision
    x, _ = _efr_axis(ix, xmax / float(np.float32(ix - 2 * margin)), margin + 1)
    y, _ = _efr_axis(jx, ymax / float(np.float32(jx - 2 * margin)), margin + 1)
    dz0 = (zmax - zmin) / float(np.float32(kx - 2 * margin))
    kzero = int(-zmin / dz0) + margin + 1
    z, dzm0 = _efr_axis(kx, dz0, kzero)
    den0, pre0, bmx0 = _efr_column(z, dzm0, kzero, gm, nz)
    g0 = -1.0 / gm
    shape = (ix, jx, kx)
    X = np.broadcast_to(x[:, None, None], shape)
    Z = np.broadcast_to(z[None, None, :], shape)
    f = {"ro": np.broadcast_to(den0, shape).copy(), "pr": np.broadcast_to(pre0, shape).copy(),
         "vx": np.zeros(shape), "vy": np.zeros(shape), "vz": 0.0 + _efr_perturbation(X, Z),
         "bx": np.broadcast_to(bmx0, shape).copy(), "by": np.zeros(shape),
         "bz": np.zeros(shape)}
    dx, _, dxm = grdrdy(x)
    dy, _, dym = grdrdy(y)
    dz, _, dzm = grdrdy(z)
    names = VARS["mlw_m_3d"]
    odd = {0: ("vx", "by", "bz"), 1: ("vy", "by"), 2: ("vz", "bz")}
    bc = []
    for axis_ in range(3):
        for face in (2 * axis_, 2 * axis_ + 1):
            for v, name in enumerate(names):
                if axis_ == 2 and name in ("ro", "pr"):
                    base = den0 if name == "ro" else pre0
                    bc.append((v, face, BD_CNS, float(base[0 if face == 4 else kx - 1])))
                else:
                    bc.append((v, face, BD_SPN if name in odd[axis_] else BD_SPP, 0.0))
    grav = dict(gx=np.zeros(shape, order="F"), gxm=np.zeros(shape, order="F"),
                gy=np.zeros(shape, order="F"), gym=np.zeros(shape, order="F"),
                gz=np.full(shape, g0, order="F"), gzm=np.full(shape, g0, order="F"))
    return _pack3(x, dx, dxm, y, dy, dym, z, dz, dzm, f, gm, 3.0, bc, safety=0.4,
                  dtmin=1e-10, tend=80.0, dtout=1.0, gravity=True,
                  name=f"emerging_flux_{nx}x{ny}x{nz}", **grav)


def mhd_wind_1d(nx: int = 1024):
    """The magnetised stellar-wind model of cans1d/md_mhdwind/hdmlw (model.f,
    bnd.f, bndsc.f, main.f:70-80, 160-176), the Weber-Davis problem: a
    rotating star of radius rstar = 6, gamma 1.2, point-mass gravity
    gx = -(1/gm) rstar^2/x^2, a radial field bx ~ 1/x^2 with 1/beta = 0.1 at
    the base, a flux tube of cross section sc = 1/bx, distance from the axis
    rr = x, an exponential atmosphere to x = 12 and a tenuous ISM beyond, on a
    grid stretched by 1.006 per cell (nx cells from x = 6, dx0 = 10/nx).
    Boundaries: at the base ro = 1, pr = 1/gm and the rotation vy = vstar =
    0.15 held, vx and by free; the outer face free.  mlw_m_bg with qav 2,
    cfl_m safety 1.0, tend 2000 (the wind settles to a steady state)."""
    margin = 1
    ix = nx + 2 * margin
    gm, rstar, vstar = 1.2, 6.0, 0.15
    pi = math.acos(-1.0)
    dx0 = 10.0 / float(np.float32(ix - 2 * margin))
    ratx = 1.006
    dxm0 = np.full(ix, dx0)
    for i in range(1, ix):
        dxm0[i] = dxm0[i - 1] * ratx
    izero = margin + 1
    x = np.empty(ix)
    x[izero - 1] = rstar + dxm0[izero - 1] / 2.0
    for i in range(izero + 1, ix + 1):
        x[i - 1] = x[i - 2] + dxm0[i - 2]
    for i in range(izero - 1, 0, -1):
        x[i - 1] = x[i] - dxm0[i - 1]
    gx = -1 / gm * (rstar * rstar) / (x * x)
    xh = x + 0.5 * dxm0
    gxm = -1 / gm * (rstar * rstar) / (xh * xh)
    rr = x.copy()
    rrm = x + dxm0 / 2
    rhs = 2.0 * rstar
    roism, teism = 1.0e-8, 1.0e-2
    ro = (np.exp(rstar * (rstar / x - 1)) * (1 - np.tanh((x - rhs) / 0.5)) / 2
          + roism * (1 + np.tanh((x - rhs) / 0.5)) / 2)
    te = teism + (1 - teism) * (1 - (x - rhs) / (x[ix - margin - 1] - rhs))
    te = np.where(x <= rhs, 1.0, te)
    pr = ro * te / gm
    betai = float(np.float32(0.1))
    bx0 = math.sqrt(betai * pr[izero - 1] * 8 * pi)
    x0 = x[izero - 1]
    bx = bx0 * (x0 * x0) / (x * x)
    bxm = bx0 * (x0 * x0) / ((x + dxm0 / 2) * (x + dxm0 / 2))
    sc = 1.0 / bx
    scm = 1.0 / bxm
    dx, _, dxm = grdrdy(x)
    f = {"ro": ro, "pr": pr, "vx": np.zeros(ix), "vy": np.zeros(ix), "by": np.zeros(ix)}
    names = VARS["mlw_m_bg_1d"]
    # bnd.f: base ro = 1, pr = 1/gm, vy = vstar held, vx and by free; outer free
    held = {"ro": 1.0, "pr": 1.0 / gm, "vy": vstar}
    bc = []
    for v, name in enumerate(names):
        bc.append((v, 0, BD_CNS, held[name]) if name in held else (v, 0, BD_FRE, 0.0))
        bc.append((v, 1, BD_FRE, 0.0))
    for v, face, kind, q0 in bc:
        a = f[names[v]]
        if kind == BD_CNS:
            a[:margin] = q0
        else:
            bd_host_1d(kind, face, margin, a)
    dsc, dscm = scrdy(sc, scm, dx, dxm)
    drr, drrm = scrdy(rr, rrm, dx, dxm)
    # bndsc.f: dsc free at both faces, dscm free at the outer face
    bd_host_1d(BD_FRE, 0, margin, dsc)
    bd_host_1d(BD_FRE, 1, margin, dsc)
    bd_host_1d(BD_FRE, 1, margin, dscm)
    state = [np.ascontiguousarray(f[k], dtype=np.float64) for k in names]
    prof = dict(gx=gx, gxm=gxm, sc=sc, scm=scm, dsc=dsc, dscm=dscm, rr=rr, rrm=rrm,
                drr=drr, drrm=drrm)
    return dict(solver="mlw_m_bg_1d", solver_id=6, names=names, x=x, dx=dx, dxm=dxm,
                bx=bx, bxm=bxm, state=state, gm=gm, qav=2.0, margin=margin, bc=bc,
                safety=1.0, dtmin=1e-10, tend=2000.0, dtout=100.0, vstar=vstar,
                name=f"mhd_wind_{nx}", **prof)


def mhd_wave_2d(n: int = 64):
    """The MHD wave model of cans2d/md_mhdwave/hdmlw (model.f, bnd.f,
    main.f:155-171): a Gaussian pressure pulse (relative amplitude 0.1,
    width 0.02) at the centre of [-0.5, 0.5]^2 (n x n cells, one ghost
    layer), rho = 1, gamma 5/3, c_s = 1, a uniform field at 60 degrees to x
    with 1/beta = 0.5 (c_a^2 = 0.6), free boundaries, mlw_m with qav 3, cfl_m
    safety 0.4, tend 1.  Its fronts trace the Friedrichs diagram of the
    reference's mhdwave_analytic.pro."""
    margin = 1
    ix = jx = n + 2 * margin
    gm = 5.0 / 3.0
    pi = math.acos(-1.0)

    def axis(nn):
        d0 = 1.0 / float(nn - 2 * margin)
        dm = np.full(nn, d0)
        iz = nn // 2 + 1
        x = np.empty(nn)
        x[iz - 1] = dm[iz - 1] / 2.0
        for i in range(iz + 1, nn + 1):
            x[i - 1] = x[i - 2] + dm[i - 2]
        for i in range(iz - 1, 0, -1):
            x[i - 1] = x[i] - dm[i - 1]
        return x

    x, y = axis(ix), axis(jx)
    X, Y = np.meshgrid(x, y, indexing="ij")
    betai = float(np.float32(0.5))
    b0 = math.sqrt(8 * pi / gm * betai)
    thini = float(np.float32(60.0)) / float(np.float32(180.0)) * pi
    wexp = float(np.float32(0.02))
    amp = 0.1
    ss = np.sqrt(X * X + Y * Y)
    f = {"ro": np.ones(X.shape), "pr": 1 / gm + amp / gm * np.exp(-((ss / wexp) ** 2)),
         "bx": np.full(X.shape, b0 * math.cos(thini)),
         "by": np.full(X.shape, b0 * math.sin(thini)),
         "vx": np.zeros(X.shape), "vy": np.zeros(X.shape)}
    dx, _, dxm = grdrdy(x)
    dy, _, dym = grdrdy(y)
    f["az"] = bbtoaa(np.asfortranarray(f["bx"]), np.asfortranarray(f["by"]), dxm, dym, margin)
    bc = _bc_all(len(VARS["mlw_m"]), BD_FRE, BD_FRE)
    return _pack("mlw_m", x, dx, dxm, y, dy, dym, f, gm, 3.0, bc, safety=0.4, dtmin=1e-10,
                 tend=1.0, margin=margin, thini=thini, name=f"mhd_wave_{n}")


def parker_instability(nx: int = 64, ny: int = 128):
    """The Parker-instability model of cans2d/md_parkerinst/hdmlw (model.f,
    pertub.f, bnd.f, main.f:160-180): a gravitationally stratified disk on
    [-50, 50] x [-25, 25] (nx x ny cells, one ghost layer) with gravity
    gy = -(1/gm) tanh(y/0.5) towards the midplane, a cool layer (T = 1)
    under a corona (T = 25) beyond |y| = 6, a horizontal field with
    1/beta = 5 inside |y| < 2.5 in the discrete magnetohydrostatic balance
    of model.f, and a vy perturbation of amplitude 0.1 (pertub.f).
    Boundaries: x periodic, y symmetric (vy, by odd).  mlw_m_g with qav 3,
    cfl_m safety 0.4, chkdav of ro and pr with floor 1e-9, tend 60."""
    margin = 1
    ix, jx = nx + 2 * margin, ny + 2 * margin
    gm = 5.0 / 3.0
    pi = math.acos(-1.0)
    f32 = lambda v: float(np.float32(v))  # noqa: E731  (real*4 literals)

    def axis(nn, lo, hi):
        d0 = (hi - lo) / float(nn - 2 * margin)
        dm = np.full(nn, d0)
        iz = nn // 2 + 1
        x = np.empty(nn)
        x[iz - 1] = dm[iz - 1] / 2.0
        for i in range(iz + 1, nn + 1):
            x[i - 1] = x[i - 2] + dm[i - 2]
        for i in range(iz - 1, 0, -1):
            x[i - 1] = x[i] - dm[i - 1]
        return x, dm

    x, _ = axis(ix, -50.0, 50.0)
    y, dym0 = axis(jx, -25.0, 25.0)
    g0 = -1.0 / gm
    wg0 = f32(0.5)
    gym0 = g0 * np.tanh((y + 0.5 * dym0) / wg0)
    ytr, wtr, tcor = f32(6.0), f32(0.5), f32(25.0)
    tem0 = 1.0 + 0.5 * (tcor - 1.0) * (np.tanh((np.abs(y) - ytr) / wtr) + 1.0)
    yf1, yf2, wf0 = f32(-2.5), f32(2.5), f32(0.5)
    rbetaf = f32(f32(1.0) / np.float32(0.2))  # 1.0/0.2 evaluated in single precision
    af1 = (np.tanh((y - yf1) / wf0) + 1.0) / 2
    af2 = (-np.tanh((y - yf2) / wf0) + 1.0) / 2
    rbeta0 = np.abs(rbetaf * af1 * af2)
    jz = jx // 2  # 0-based index of Fortran jzero = jx/2+1
    den0, pre0 = np.empty(jx), np.empty(jx)
    den0[jz] = 1.0
    pre0[jz] = 1.0 / gm * tem0[jz]
    for j in range(jz + 1, jx):
        h = 0.5 * gm * gym0[j - 1] * dym0[j - 1]
        den0[j] = den0[j - 1] * ((1 + rbeta0[j - 1]) * tem0[j - 1] + h) / \
            ((1 + rbeta0[j]) * tem0[j] - h)
        pre0[j] = pre0[jz] * (den0[j] / den0[jz]) * (tem0[j] / tem0[jz])
    for j in range(jz - 1, -1, -1):
        h = 0.5 * gm * gym0[j] * dym0[j]
        den0[j] = den0[j + 1] * ((1 + rbeta0[j + 1]) * tem0[j + 1] - h) / \
            ((1 + rbeta0[j]) * tem0[j] + h)
        pre0[j] = pre0[jz] * (den0[j] / den0[jz]) * (tem0[j] / tem0[jz])
    bmx0 = np.sqrt(8 * pi * pre0 * rbeta0)
    shape = (ix, jx)
    X, Y = np.meshgrid(x, y, indexing="ij")
    amp, xptb, yptb1, yptb2, wptb = f32(0.1), f32(20.0), f32(-4.0), f32(4.0), f32(0.5)
    vy = (amp * np.cos(2 * pi * X / xptb) * 0.5
          * (np.tanh((X + 0.75 * xptb) / wptb) - np.tanh((X - 0.75 * xptb) / wptb)) * 0.5
          * (np.tanh((Y - yptb1) / wptb) - np.tanh((Y - yptb2) / wptb)))
    f = {"ro": np.broadcast_to(den0, shape).copy(), "pr": np.broadcast_to(pre0, shape).copy(),
         "vx": np.zeros(shape), "vy": 0.0 + vy,
         "bx": np.broadcast_to(bmx0, shape).copy(), "by": np.zeros(shape)}
    dx, _, dxm = grdrdy(x)
    dy, _, dym = grdrdy(y)
    f["az"] = bbtoaa(np.asfortranarray(f["bx"]), np.asfortranarray(f["by"]), dxm, dym, margin)
    names = VARS["mlw_m"]
    bc = []
    for v, name in enumerate(names):
        bc += [(v, 0, BD_PER, 0.0), (v, 1, BD_PER, 0.0)]
    for v, name in enumerate(names):
        kind = BD_SPN if name in ("vy", "by") else BD_SPP
        bc += [(v, 2, kind, 0.0), (v, 3, kind, 0.0)]
    grav = dict(gx=np.zeros(shape, order="F"), gxm=np.zeros(shape, order="F"),
                gy=np.asfortranarray(np.broadcast_to(g0 * np.tanh(y / wg0), shape)),
                gym=np.asfortranarray(np.broadcast_to(gym0, shape)))
    return _pack("mlw_m", x, dx, dxm, y, dy, dym, f, gm, 3.0, bc, safety=0.4, dtmin=1e-10,
                 tend=60.0, dtout=2.0, gravity=True, floor=1e-9,
                 name=f"parker_instability_{nx}x{ny}", **grav)


def oblique_shock_tube_2d(n: int = 64):
    """The oblique MHD shock tube of cans2d/md_mhd3shktb/hdmlw (model.f,
    bnd.f, main.f:165-180): the Brio-Wu states (rho 1 / 0.125, p 1 / 0.1,
    bz +-b0) joined by a tanh of width 0.02 across the line
    x cos(60 deg) + y sin(60 deg) = 0 of [-0.5, 0.5]^2 (n x n cells, one
    ghost layer), an in-plane field 0.75 b0 along that normal,
    b0 = sqrt(8 pi/gm), gamma 2, free boundaries; mlw_m3 with qav 3, cfl_m3
    safety 0.4, tend 0.1."""
    margin = 1
    ix = jx = n + 2 * margin
    gm = 2.0
    pi = math.acos(-1.0)
    f32 = lambda v: float(np.float32(v))  # noqa: E731  (real*4 literals)

    def axis(nn):
        d0 = 1.0 / float(nn - 2 * margin)
        dm = np.full(nn, d0)
        iz = nn // 2 + 1
        x = np.empty(nn)
        x[iz - 1] = dm[iz - 1] / 2.0
        for i in range(iz + 1, nn + 1):
            x[i - 1] = x[i - 2] + dm[i - 2]
        for i in range(iz - 1, 0, -1):
            x[i - 1] = x[i] - dm[i - 1]
        return x

    x, y = axis(ix), axis(jx)
    X, Y = np.meshgrid(x, y, indexing="ij")
    b0 = math.sqrt(8 * pi / gm)
    thini = f32(60.0) / f32(180.0) * pi
    b00 = f32(0.75) * b0
    wtr = f32(0.02)
    ro0, ro1, pr0, pr1 = 1.0, f32(0.125), 1.0, f32(0.1)
    bz0, bz1 = +b0, -b0
    ss = X * math.cos(thini) + Y * math.sin(thini)
    w = (1 + np.tanh(ss / wtr)) / 2
    f = {"ro": ro0 + (ro1 - ro0) * w, "pr": pr0 + (pr1 - pr0) * w,
         "bx": np.full(X.shape, b00 * math.cos(thini)),
         "by": np.full(X.shape, b00 * math.sin(thini)), "bz": bz0 + (bz1 - bz0) * w,
         "vx": np.zeros(X.shape), "vy": np.zeros(X.shape), "vz": np.zeros(X.shape)}
    dx, _, dxm = grdrdy(x)
    dy, _, dym = grdrdy(y)
    f["az"] = bbtoaa(np.asfortranarray(f["bx"]), np.asfortranarray(f["by"]), dxm, dym, margin)
    bc = _bc_all(len(VARS["mlw_m3"]), BD_FRE, BD_FRE)
    return _pack("mlw_m3", x, dx, dxm, y, dy, dym, f, gm, 3.0, bc, safety=0.4, dtmin=1e-10,
                 tend=0.1, margin=margin, name=f"oblique_shock_tube_{n}")
