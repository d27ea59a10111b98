"""ctypes binding of libcansgpu.so (the C ABI declared in include/cans_gpu.h).

The Python functions keep the reference routine names and argument meaning
(cans2d/hdmlw/mlw_m3.f:2, cans2d/common/cfl_m3.f:2, cans2d/bc/bd*.f:2, ...):
arrays are NumPy float64 arrays in Fortran (column-major) order with their
ghost cells, updated in place; scalars are plain Python numbers.  Every call
goes to the GPU library; there is no CPU path, and a missing or unusable
library raises CansError.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

LIB_PATH = _build.LIBDIR / _build.LIBNAME

CANS_OK = 0
CANS_ERR_DTMIN = 9001
CANS_ERR_NONFINITE = 9100
CANS_ERR_CUDA = 9200
CANS_ERR_ARG = 9400

SOLVER_MLW_M_2D = 0
SOLVER_MLW_M3_2D = 1
SOLVER_MLW_M_3D = 2
SOLVER_MLW_M_1D = 3
SOLVER_ROE_M_3D = 4
SOLVER_HLLD_3D = 5
SOLVER_MLW_M_BG_1D = 6
SOLVER_ROE_M3_2D = 7

BD_NONE, BD_PER, BD_SPP, BD_SPN, BD_SMP, BD_SMN, BD_FRE, BD_CNS, BD_FRD = range(-1, 8)

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lib = None


class CansError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str = ""):
        super().__init__(f"{where} returned {code}" + (f": {detail}" if detail else ""))
        self.code = code


def load() -> C.CDLL:
    """Load libcansgpu.so (built by __graft_entry__.build()); raise if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise CansError(CANS_ERR_CUDA, "load",
                        f"{LIB_PATH} is missing; build it with __graft_entry__.build()")
    lib = C.CDLL(str(LIB_PATH))
    i, d, vp = C.c_int, C.c_double, C.c_void_p
    sig = {
        "cans_set_exact": (i, [i]), "cans_get_exact": (i, []),
        "cans_set_stream": (i, [vp]), "cans_last_error": (C.c_char_p, []),
        "cans_launch_count": (C.c_ulonglong, []), "cans_device_ok": (i, []),
        "cans_mlw_m3_2d": (i, [_dp] * 9 + [_dp, _dp, _dp, _dp, _dp, _ip, _dp, _dp, _ip]),
        "cans_mlw_m_2d": (i, [_dp] * 7 + [_dp, _dp, _dp, _dp, _dp, _ip, _dp, _dp, _ip]),
        "cans_cfl_m3_2d": (i, [_dp, _dp, _dp, _ip, _dp] + [_dp] * 8 + [_dp, _ip, _dp, _ip]),
        "cans_cfl_m_2d": (i, [_dp, _dp, _dp, _ip, _dp] + [_dp] * 6 + [_dp, _ip, _dp, _ip]),
        "cans_gpu_register": (i, [C.POINTER(_dp), _ip, _ip, _ip, _ip]),
        "cans_gpu_pull": (i, [_dp]), "cans_gpu_push": (i, [_dp]),
        "cans_gpu_release": (i, [_dp]),
        "cans_run_create": (i, [C.POINTER(vp), vp]), "cans_run_destroy": (i, [vp]),
        "cans_run_set_bc": (i, [vp, i, i, i, d]),
        "cans_run_push": (i, [vp, C.POINTER(_dp)]), "cans_run_pull": (i, [vp, C.POINTER(_dp)]),
        "cans_run_start": (i, [vp, d, d, C.c_longlong, d, d, d, i]),
        "cans_run_advance": (i, [vp, i]), "cans_run_query": (i, [vp, vp]),
        "cans_run_advance_group": (i, [C.POINTER(vp), i, i]),
        "cans_run_resume": (i, [vp]), "cans_run_step": (i, [vp, _dp, i]),
        "cans_run_cfl": (i, [vp, d, _dp]), "cans_run_autotune": (i, [vp, i, _ip]),
        "cans_run_device_state": (i, [vp, C.POINTER(_dp)]),
        "cans_run_profile": (i, [vp, i, _dp, _dp]),
        "cans_cfl_m3_2d_noalloc": (i, [_dp, _dp, _dp, _ip, _dp] + [vp] * 8 + [vp, _ip, vp, _ip]),
        "cans_run_set_graph": (i, [vp, i]),
        "cans_run_set_df64": (i, [vp, i]), "cans_run_set_tile": (i, [vp, i]),
        "cans_run_set_adjoint_df64": (i, [vp, i]),
        "cans_run_record_dts": (i, [vp, C.c_longlong, d, _dp, _dp]),
        "cans_run_objective": (i, [vp, C.c_longlong, _dp, _dp]),
        "cans_run_adjoint": (i, [vp, C.c_longlong, _dp, i, _dp, C.POINTER(_dp),
                                 C.POINTER(C.c_longlong)]),
        "cans_run_bc_transpose": (i, [vp, C.POINTER(_dp)]),
        "cans_run_av_record": (i, [vp, C.c_longlong, _dp]),
        "cans_run_av_branches": (i, [vp, C.c_longlong, vp]),
        "cans_run_objective_frozen_av": (i, [vp, C.c_longlong, _dp, _dp,
                                             C.POINTER(C.c_longlong)]),
        "cans_batch_create": (i, [C.POINTER(vp), i, vp]), "cans_batch_destroy": (i, [vp]),
        "cans_batch_set_bc": (i, [vp, i, i, i, i, d]),
        "cans_batch_push": (i, [vp, i, C.POINTER(_dp)]),
        "cans_batch_pull": (i, [vp, i, C.POINTER(_dp)]),
        "cans_batch_start": (i, [vp, d, d, C.c_longlong, d, d]),
        "cans_batch_advance": (i, [vp, i, i]), "cans_batch_query": (i, [vp, i, vp]),
        "cans_batch_configs": (i, []), "cans_batch_set_config": (i, [vp, i]),
        "cans_batch_autotune": (i, [vp, i, _ip]),
    }
    sig["cans_mlw_m_3d"] = (i, [_dp] * 8 + [_dp, _dp, _dp, _dp, _dp, _ip, _dp, _dp, _ip,
                                             _dp, _dp, _ip])
    sig["cans_cfl_m_3d"] = (i, [_dp, _dp, _dp, _ip, _dp] + [_dp] * 8 +
                            [_dp, _ip, _dp, _ip, _dp, _ip])
    sig["cans_roe_m_3d"] = (i, [_dp] * 8 + [_dp, _dp, _dp, _ip, _dp, _ip, _dp, _ip])
    sig["cans_mlw_m3_g_2d"] = (i, [_dp] * 9 + [_dp] * 7 + [_dp, _dp, _ip, _dp, _dp, _ip])
    sig["cans_mlw_m_g_3d"] = (i, [_dp] * 8 + [_dp] * 9 + [_dp, _dp, _ip, _dp, _dp, _ip,
                                                           _dp, _dp, _ip])
    sig["cans_mlw_m_g_2d"] = (i, [_dp] * 7 + [_dp] * 7 + [_dp, _dp, _ip, _dp, _dp, _ip])
    sig["cans_mlw_m3_e_2d"] = (i, [_dp] * 9 + [_dp] * 5 + [_dp, _dp, _ip, _dp, _dp, _ip])
    sig["cans_mlw_m_e_2d"] = (i, [_dp] * 7 + [_dp] * 5 + [_dp, _dp, _ip, _dp, _dp, _ip])
    sig["cans_mlw_m3_ge_2d"] = (i, [_dp] * 9 + [_dp] * 9 + [_dp, _dp, _ip, _dp, _dp, _ip])
    sig["cans_mlw_m_ge_2d"] = (i, [_dp] * 7 + [_dp] * 9 + [_dp, _dp, _ip, _dp, _dp, _ip])
    sig["cans_cfl_m3_e_2d"] = (i, [_dp, _dp, _dp, _ip, _dp] + [_dp] * 9 + [_dp, _ip, _dp, _ip])
    sig["cans_cfl_m_e_2d"] = (i, [_dp, _dp, _dp, _ip, _dp] + [_dp] * 7 + [_dp, _ip, _dp, _ip])
    sig["cans_roe_m3_2d"] = (i, [_dp] * 9 + [_dp, _dp, _dp, _ip, _dp, _ip])
    sig["cans_hlld_engine_3d"] = (i, [_dp] * 8 + [_dp] * 9 + [_ip] * 4)
    sig["cans_mlw_m_1d"] = (i, [_dp] * 7 + [_dp, _dp, _dp, _dp, _dp, _ip])
    sig["cans_cfl_m_1d"] = (i, [_dp, _dp, _dp, _ip, _dp, _dp] + [_dp] * 5 + [_dp, _ip])
    sig["cans_mlw_m_bg"] = (i, [_dp] * 7 + [_dp, _dp, _dp] + [_dp] * 12 + [_ip])
    sig["cans_chkdav"] = (i, [_ip, _dp, _dp, _dp, _ip])
    sig["cans_chkdav_2d"] = (i, [_ip, _dp, _dp, _dp, _dp, _ip, _ip])
    sig["cans_chkdav_3d"] = (i, [_ip, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _ip])
    sig["cans_roe_m_1d"] = (i, [_dp] * 7 + [_dp, _dp, _dp, _ip])
    sig["cans_bdperx_1d"] = (i, [_ip, _ip, _dp, _ip])
    for fam in ("spp", "spn", "smp", "smn", "fre"):
        sig[f"cans_bd{fam}x_1d"] = (i, [_ip, _ip, _dp, _ip])
    sig["cans_bdcnsx_1d"] = (i, [_ip, _ip, _dp, _dp, _ip])
    sig["cans_bdfrdx_1d"] = (i, [_ip, _ip, _dp, _dp, _ip])
    for ax in "xyz":
        sig[f"cans_bdper{ax}_3d"] = (i, [_ip, _ip, _dp, _ip, _ip, _ip])
        for fam in ("spp", "spn", "smp", "smn", "fre"):
            sig[f"cans_bd{fam}{ax}_3d"] = (i, [_ip, _ip, _dp, _ip, _ip, _ip])
        sig[f"cans_bdcns{ax}_3d"] = (i, [_ip, _ip, _dp, _dp, _ip, _ip, _ip])
        sig[f"cans_bdfrd{ax}_3d"] = (i, [_ip, _ip, _dp, _dp, _ip, _ip, _ip])
    for name in ("bdperx", "bdpery"):
        sig[f"cans_{name}_2d"] = (i, [_ip, _ip, _dp, _ip, _ip])
    for fam in ("spp", "spn", "smp", "smn", "fre"):
        for ax in "xy":
            sig[f"cans_bd{fam}{ax}_2d"] = (i, [_ip, _ip, _dp, _ip, _ip])
    for ax in "xy":
        sig[f"cans_bdcns{ax}_2d"] = (i, [_ip, _ip, _dp, _dp, _ip, _ip])
        sig[f"cans_bdfrd{ax}_2d"] = (i, [_ip, _ip, _dp, _dp, _ip, _ip])
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    """Names declared in include/cans_gpu.h (for the export check)."""
    import re
    hdr = (_build.ROOT / "include" / "cans_gpu.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*|unsigned long long)\s*\*?\s*(cans_\w+)\s*\(",
                                 hdr, flags=re.M)))


def _check(rc: int, where: str) -> int:
    if rc not in (CANS_OK,):
        detail = load().cans_last_error().decode() if rc == CANS_ERR_CUDA else ""
        raise CansError(rc, where, detail)
    return rc


def _ptr(a: np.ndarray | None):
    if a is None:  # a NULL argument: the library rejects it
        return None
    if a.dtype != np.float64 or not (a.flags.f_contiguous or a.ndim == 1):
        raise CansError(CANS_ERR_ARG, "array", "float64 Fortran-ordered arrays are required")
    return a.ctypes.data_as(_dp)


def _dref(x: float):
    return C.byref(C.c_double(float(x)))


def _iref(x: int):
    return C.byref(C.c_int(int(x)))


def set_exact(flag: bool) -> None:
    load().cans_set_exact(1 if flag else 0)


def launch_count() -> int:
    return int(load().cans_launch_count())


def device_ok() -> bool:
    return bool(load().cans_device_ok())


# ---- drop-in routines (2-D) ------------------------------------------------

def mlw_m3(ro, pr, vx, vy, vz, bx, by, bz, az, dt, qav, gm, dx, dxm, dy, dym):
    """cans2d/hdmlw/mlw_m3.f:2 -- one mLW step of the 2.5-D state, in place."""
    ix, jx = ro.shape
    lib = load()
    return _check(lib.cans_mlw_m3_2d(*[_ptr(a) for a in (ro, pr, vx, vy, vz, bx, by, bz, az)],
                                     _dref(dt), _dref(qav), _dref(gm), _ptr(dx), _ptr(dxm),
                                     _iref(ix), _ptr(dy), _ptr(dym), _iref(jx)), "mlw_m3")


def mlw_m3_g(ro, pr, vx, vy, vz, bx, by, bz, az, dt, qav, gm, gx, gxm, gy, gym,
             dx, dxm, dy, dym):
    """cans2d/hdmlw/mlw_m3_g.f:1 -- mlw_m3 with gravity, in place."""
    ix, jx = ro.shape
    return _check(load().cans_mlw_m3_g_2d(
        *[_ptr(a) for a in (ro, pr, vx, vy, vz, bx, by, bz, az)], _dref(dt), _dref(qav),
        _dref(gm), *[_ptr(a) for a in (gx, gxm, gy, gym)], _ptr(dx), _ptr(dxm), _iref(ix),
        _ptr(dy), _ptr(dym), _iref(jx)), "mlw_m3_g")


def mlw_m_g(ro, pr, vx, vy, bx, by, az, dt, qav, gm, gx, gxm, gy, gym, dx, dxm, dy, dym):
    """cans2d/hdmlw/mlw_m_g.f:1 -- mlw_m with gravity, in place."""
    ix, jx = ro.shape
    return _check(load().cans_mlw_m_g_2d(
        *[_ptr(a) for a in (ro, pr, vx, vy, bx, by, az)], _dref(dt), _dref(qav), _dref(gm),
        *[_ptr(a) for a in (gx, gxm, gy, gym)], _ptr(dx), _ptr(dxm), _iref(ix), _ptr(dy),
        _ptr(dym), _iref(jx)), "mlw_m_g")


def mlw_m3_e(ro, pr, vx, vy, vz, bx, by, bz, az, dt, qav, gm, et, etm, dx, dxm, dy, dym,
             gx=None, gxm=None, gy=None, gym=None):
    """cans2d/hdmlw/mlw_m3_e.f:2 -- mlw_m3 with resistivity et (cells) and
    etm (corners), in place; with gx..gym mlw_m3_ge (mlw_m3_ge.f:2)."""
    ix, jx = ro.shape
    st = [_ptr(a) for a in (ro, pr, vx, vy, vz, bx, by, bz, az)]
    tail = (_ptr(et), _ptr(etm), _ptr(dx), _ptr(dxm), _iref(ix), _ptr(dy), _ptr(dym),
            _iref(jx))
    if gx is None:
        return _check(load().cans_mlw_m3_e_2d(*st, _dref(dt), _dref(qav), _dref(gm), *tail),
                      "mlw_m3_e")
    return _check(load().cans_mlw_m3_ge_2d(*st, _dref(dt), _dref(qav), _dref(gm),
                                           *[_ptr(a) for a in (gx, gxm, gy, gym)], *tail),
                  "mlw_m3_ge")


def mlw_m_e(ro, pr, vx, vy, bx, by, az, dt, qav, gm, et, etm, dx, dxm, dy, dym,
            gx=None, gxm=None, gy=None, gym=None):
    """cans2d/hdmlw/mlw_m_e.f:2 -- mlw_m with resistivity, in place; with
    gx..gym mlw_m_ge (mlw_m_ge.f:2)."""
    ix, jx = ro.shape
    st = [_ptr(a) for a in (ro, pr, vx, vy, bx, by, az)]
    tail = (_ptr(et), _ptr(etm), _ptr(dx), _ptr(dxm), _iref(ix), _ptr(dy), _ptr(dym),
            _iref(jx))
    if gx is None:
        return _check(load().cans_mlw_m_e_2d(*st, _dref(dt), _dref(qav), _dref(gm), *tail),
                      "mlw_m_e")
    return _check(load().cans_mlw_m_ge_2d(*st, _dref(dt), _dref(qav), _dref(gm),
                                          *[_ptr(a) for a in (gx, gxm, gy, gym)], *tail),
                  "mlw_m_ge")


def cfl_m3_e(safety, dtmin, gm, ro, pr, vx, vy, vz, bx, by, bz, et, dx, dy):
    """cans2d/common/cfl_m3_e.f:2 -- returns (dt, merr)."""
    ix, jx = ro.shape
    dt, merr = C.c_double(0.0), C.c_int(0)
    _check(load().cans_cfl_m3_e_2d(C.byref(dt), _dref(safety), _dref(dtmin), C.byref(merr),
                                   _dref(gm),
                                   *[_ptr(a) for a in (ro, pr, vx, vy, vz, bx, by, bz, et)],
                                   _ptr(dx), _iref(ix), _ptr(dy), _iref(jx)), "cfl_m3_e")
    return dt.value, merr.value


def cfl_m_e(safety, dtmin, gm, ro, pr, vx, vy, bx, by, et, dx, dy):
    """cans2d/common/cfl_m_e.f:2 -- returns (dt, merr)."""
    ix, jx = ro.shape
    dt, merr = C.c_double(0.0), C.c_int(0)
    _check(load().cans_cfl_m_e_2d(C.byref(dt), _dref(safety), _dref(dtmin), C.byref(merr),
                                  _dref(gm), *[_ptr(a) for a in (ro, pr, vx, vy, bx, by, et)],
                                  _ptr(dx), _iref(ix), _ptr(dy), _iref(jx)), "cfl_m_e")
    return dt.value, merr.value


def mlw_m(ro, pr, vx, vy, bx, by, az, dt, qav, gm, dx, dxm, dy, dym):
    """cans2d/hdmlw/mlw_m.f:2 -- one mLW step of the 2-D state, in place."""
    ix, jx = ro.shape
    lib = load()
    return _check(lib.cans_mlw_m_2d(*[_ptr(a) for a in (ro, pr, vx, vy, bx, by, az)],
                                    _dref(dt), _dref(qav), _dref(gm), _ptr(dx), _ptr(dxm),
                                    _iref(ix), _ptr(dy), _ptr(dym), _iref(jx)), "mlw_m")


def cfl_m3(safety, dtmin, gm, ro, pr, vx, vy, vz, bx, by, bz, dx, dy):
    """cans2d/common/cfl_m3.f:2 -- returns (dt, merr)."""
    ix, jx = ro.shape
    dt, merr = C.c_double(0.0), C.c_int(0)
    _check(load().cans_cfl_m3_2d(C.byref(dt), _dref(safety), _dref(dtmin), C.byref(merr),
                                 _dref(gm), *[_ptr(a) for a in (ro, pr, vx, vy, vz, bx, by, bz)],
                                 _ptr(dx), _iref(ix), _ptr(dy), _iref(jx)), "cfl_m3")
    return dt.value, merr.value


def cfl_m3_noalloc(safety, dtmin, gm, dev_arrays, dev_dx, dev_dy, ix, jx):
    """cfl_m3 on device arrays for callers that cannot allocate: dev_arrays
    are the device addresses (ints) of ro,pr,vx,vy,vz,bx,by,bz (each ix*jx,
    column-major), dev_dx / dev_dy those of dx(ix), dy(jx).  Returns
    (dt, merr).  The library allocates nothing for this call."""
    dt, merr = C.c_double(0.0), C.c_int(0)
    _check(load().cans_cfl_m3_2d_noalloc(C.byref(dt), _dref(safety), _dref(dtmin),
                                         C.byref(merr), _dref(gm),
                                         *[C.c_void_p(int(p)) for p in dev_arrays],
                                         C.c_void_p(int(dev_dx)), _iref(ix),
                                         C.c_void_p(int(dev_dy)), _iref(jx)),
           "cfl_m3_noalloc")
    return dt.value, merr.value


def cfl_m(safety, dtmin, gm, ro, pr, vx, vy, bx, by, dx, dy):
    """cans2d/common/cfl_m.f:2 -- returns (dt, merr)."""
    ix, jx = ro.shape
    dt, merr = C.c_double(0.0), C.c_int(0)
    _check(load().cans_cfl_m_2d(C.byref(dt), _dref(safety), _dref(dtmin), C.byref(merr),
                                _dref(gm), *[_ptr(a) for a in (ro, pr, vx, vy, bx, by)],
                                _ptr(dx), _iref(ix), _ptr(dy), _iref(jx)), "cfl_m")
    return dt.value, merr.value


_BD_NAMES = {BD_SPP: "spp", BD_SPN: "spn", BD_SMP: "smp", BD_SMN: "smn",
             BD_FRE: "fre", BD_CNS: "cns", BD_FRD: "frd"}


def bd(kind: int, axis: int, mbnd: int, margin: int, qq: np.ndarray,
       q0: float = 0.0, dxm: np.ndarray | None = None) -> int:
    """One reference bd* call on a 2-D array (cans2d/bc/bd*.f).

    For BD_PER, mbnd is ignored and the call is bdper?(margin, margin, ...)."""
    lib = load()
    ix, jx = qq.shape
    a = "xy"[axis]
    if kind == BD_PER:
        f = getattr(lib, f"cans_bdper{a}_2d")
        return _check(f(_iref(margin), _iref(margin), _ptr(qq), _iref(ix), _iref(jx)), f"bdper{a}")
    name = f"cans_bd{_BD_NAMES[kind]}{a}_2d"
    f = getattr(lib, name)
    if kind == BD_CNS:
        return _check(f(_iref(mbnd), _iref(margin), _ptr(qq), _dref(q0), _iref(ix), _iref(jx)), name)
    if kind == BD_FRD:
        return _check(f(_iref(mbnd), _iref(margin), _ptr(qq), _ptr(dxm), _iref(ix), _iref(jx)), name)
    return _check(f(_iref(mbnd), _iref(margin), _ptr(qq), _iref(ix), _iref(jx)), name)


# ---- drop-in routines (1-D) ------------------------------------------------

def mlw_m_1d(ro, pr, vx, vy, by, bx, bxm, dt, qav, gm, dx, dxm):
    """cans1d/hdmlw/mlw_m.f:2 -- one mLW step of the 1-D state, in place."""
    ix = ro.size
    return _check(load().cans_mlw_m_1d(*[_ptr(a) for a in (ro, pr, vx, vy, by, bx, bxm)],
                                       _dref(dt), _dref(qav), _dref(gm), _ptr(dx), _ptr(dxm),
                                       _iref(ix)), "mlw_m_1d")


def mlw_m_bg(ro, pr, vx, vy, by, bx, bxm, dt, qav, gm, gx, gxm, sc, dsc, scm, dscm,
             rr, rrm, drr, drrm, dx, dxm):
    """cans1d/hdmlw/mlw_m_bg.f:2 -- one mLW step with gravity, flux-tube
    cross section and rotation, in place (reference argument order)."""
    ix = ro.size
    return _check(load().cans_mlw_m_bg(*[_ptr(a) for a in (ro, pr, vx, vy, by, bx, bxm)],
                                       _dref(dt), _dref(qav), _dref(gm),
                                       *[_ptr(a) for a in (gx, gxm, sc, dsc, scm, dscm, rr,
                                                           rrm, drr, drrm, dx, dxm)],
                                       _iref(ix)), "mlw_m_bg")


def roe_m_1d(ro, pr, vx, vy, by, bx, bxm, dt, gm, dx):
    """cans1d/hdroe/roe_m.f:2 -- one 1-D Roe-MUSCL step, in place."""
    return _check(load().cans_roe_m_1d(*[_ptr(a) for a in (ro, pr, vx, vy, by, bx, bxm)],
                                       _dref(dt), _dref(gm), _ptr(dx), _iref(ro.size)),
                  "roe_m_1d")


def chkdav_2d(da, vx, vy, floor):
    """cans2d/common/chkdav.f:2 -- floor da, zero vx, vy there; returns n_events."""
    n = C.c_int(0)
    ix, jx = da.shape
    _check(load().cans_chkdav_2d(C.byref(n), _ptr(da), _ptr(vx), _ptr(vy), _dref(floor),
                                 _iref(ix), _iref(jx)), "chkdav_2d")
    return n.value


def chkdav_3d(da, vx, vy, vz, floor):
    """cans3d/common/chkdav.f:2 -- floor da, zero vx, vy, vz there."""
    n = C.c_int(0)
    ix, jx, kx = da.shape
    _check(load().cans_chkdav_3d(C.byref(n), _ptr(da), _ptr(vx), _ptr(vy), _ptr(vz),
                                 _dref(floor), _iref(ix), _iref(jx), _iref(kx)), "chkdav_3d")
    return n.value


def chkdav(da, vx, floor):
    """cans1d/common/chkdav.f:2 -- floor da, zero vx there; returns n_events."""
    n = C.c_int(0)
    _check(load().cans_chkdav(C.byref(n), _ptr(da), _ptr(vx), _dref(floor), _iref(da.size)),
           "chkdav")
    return n.value


def cfl_m_1d(safety, dtmin, gm, bx, ro, pr, vx, vy, by, dx):
    """cans1d/common/cfl_m.f:2 -- returns (dt, merr)."""
    dt, merr = C.c_double(0.0), C.c_int(0)
    _check(load().cans_cfl_m_1d(C.byref(dt), _dref(safety), _dref(dtmin), C.byref(merr),
                                _dref(gm), _ptr(bx), *[_ptr(a) for a in (ro, pr, vx, vy, by)],
                                _ptr(dx), _iref(ro.size)), "cfl_m_1d")
    return dt.value, merr.value


def bd_1d(kind: int, mbnd: int, margin: int, qq: np.ndarray, q0: float = 0.0,
          dxm: np.ndarray | None = None) -> int:
    """One reference bd* call on a 1-D array (cans1d/bc/bd*.f)."""
    lib = load()
    ix = qq.size
    if kind == BD_PER:
        return _check(lib.cans_bdperx_1d(_iref(margin), _iref(margin), _ptr(qq), _iref(ix)),
                      "bdperx")
    name = f"cans_bd{_BD_NAMES[kind]}x_1d"
    f = getattr(lib, name)
    if kind == BD_CNS:
        return _check(f(_iref(mbnd), _iref(margin), _ptr(qq), _dref(q0), _iref(ix)), name)
    if kind == BD_FRD:
        return _check(f(_iref(mbnd), _iref(margin), _ptr(qq), _ptr(dxm), _iref(ix)), name)
    return _check(f(_iref(mbnd), _iref(margin), _ptr(qq), _iref(ix)), name)


# ---- drop-in routines (3-D) ------------------------------------------------

def mlw_m_g_3d(ro, pr, vx, vy, vz, bx, by, bz, dt, qav, gm, gx, gxm, gy, gym, gz, gzm,
               dx, dxm, dy, dym, dz, dzm):
    """cans3d/hdmlw/mlw_m_g.f:2 -- the 3-D step with gravity, in place."""
    ix, jx, kx = ro.shape
    return _check(load().cans_mlw_m_g_3d(
        *[_ptr(a) for a in (ro, pr, vx, vy, vz, bx, by, bz)], _dref(dt), _dref(qav),
        _dref(gm), *[_ptr(a) for a in (gx, gxm, gy, gym, gz, gzm)], _ptr(dx), _ptr(dxm),
        _iref(ix), _ptr(dy), _ptr(dym), _iref(jx), _ptr(dz), _ptr(dzm), _iref(kx)),
        "mlw_m_g_3d")


def mlw_m_e_3d(ro, pr, vx, vy, vz, bx, by, bz, dt, qav, gm, et, etm, dx, dxm, dy, dym, dz,
               dzm):
    """cans3d/hdmlw/mlw_m_e.f:2 -- the 3-D resistive step, in place."""
    ix, jx, kx = ro.shape
    return _check(load().cans_mlw_m_e_3d(
        *[_ptr(a) for a in (ro, pr, vx, vy, vz, bx, by, bz)], _dref(dt), _dref(qav),
        _dref(gm), _ptr(et), _ptr(etm), _ptr(dx), _ptr(dxm), _iref(ix), _ptr(dy), _ptr(dym),
        _iref(jx), _ptr(dz), _ptr(dzm), _iref(kx)), "mlw_m_e_3d")


def cfl_m_e_3d(safety, dtmin, gm, ro, pr, vx, vy, vz, bx, by, bz, et, dx, dy, dz):
    """cans3d/common/cfl_m_e.f:2 -- returns (dt, merr)."""
    ix, jx, kx = ro.shape
    dt, merr = C.c_double(0.0), C.c_int(0)
    _check(load().cans_cfl_m_e_3d(C.byref(dt), _dref(safety), _dref(dtmin), C.byref(merr),
                                  _dref(gm),
                                  *[_ptr(a) for a in (ro, pr, vx, vy, vz, bx, by, bz, et)],
                                  _ptr(dx), _iref(ix), _ptr(dy), _iref(jx), _ptr(dz),
                                  _iref(kx)), "cfl_m_e_3d")
    return dt.value, merr.value


def mlw_m_3d(ro, pr, vx, vy, vz, bx, by, bz, dt, qav, gm, dx, dxm, dy, dym, dz, dzm):
    """cans3d/hdmlw/mlw_m.f:2 -- one mLW step of the 3-D state, in place."""
    ix, jx, kx = ro.shape
    return _check(load().cans_mlw_m_3d(*[_ptr(a) for a in (ro, pr, vx, vy, vz, bx, by, bz)],
                                       _dref(dt), _dref(qav), _dref(gm), _ptr(dx), _ptr(dxm),
                                       _iref(ix), _ptr(dy), _ptr(dym), _iref(jx), _ptr(dz),
                                       _ptr(dzm), _iref(kx)), "mlw_m_3d")


def cfl_m_3d(safety, dtmin, gm, ro, pr, vx, vy, vz, bx, by, bz, dx, dy, dz):
    """cans3d/common/cfl_m.f:2 -- returns (dt, merr)."""
    ix, jx, kx = ro.shape
    dt, merr = C.c_double(0.0), C.c_int(0)
    _check(load().cans_cfl_m_3d(C.byref(dt), _dref(safety), _dref(dtmin), C.byref(merr),
                                _dref(gm), *[_ptr(a) for a in (ro, pr, vx, vy, vz, bx, by, bz)],
                                _ptr(dx), _iref(ix), _ptr(dy), _iref(jx), _ptr(dz),
                                _iref(kx)), "cfl_m_3d")
    return dt.value, merr.value


def hlld_engine_3d(ro, pr, vx, vy, vz, bx, by, bz, gm, mu, dt, dx, dxm, dy, dym, dz, dzm,
                   mfdim=(1, 1, 1)):
    """cansxx-nosupport/md_mhdshktb/hdhlld-x/engine.f:2 -- one HLLD step of the
    3-D state in Heaviside units, in place; mfdim marks the active axes."""
    ix, jx, kx = ro.shape
    md = (C.c_int * 3)(*mfdim)
    return _check(load().cans_hlld_engine_3d(
        *[_ptr(a) for a in (ro, pr, vx, vy, vz, bx, by, bz)], _dref(gm), _dref(mu), _dref(dt),
        _ptr(dx), _ptr(dxm), _ptr(dy), _ptr(dym), _ptr(dz), _ptr(dzm), _iref(ix), _iref(jx),
        _iref(kx), C.cast(md, _ip)), "hlld_engine_3d")


def roe_m3(ro, pr, vx, vy, vz, bx, by, bz, az, dt, gm, dx, dy):
    """cans2d/hdroe/roe_m3.f:1 -- one 2-D Roe-MUSCL step of the nine arrays,
    in place."""
    ix, jx = ro.shape
    return _check(load().cans_roe_m3_2d(*[_ptr(a) for a in (ro, pr, vx, vy, vz, bx, by, bz, az)],
                                        _dref(dt), _dref(gm), _ptr(dx), _iref(ix), _ptr(dy),
                                        _iref(jx)), "roe_m3")


def roe_m_3d(ro, pr, vx, vy, vz, bx, by, bz, dt, gm, dx, dy, dz):
    """cans3d/hdroe/roe_m.f:2 -- one Roe-MUSCL step of the 3-D state, in place
    (cells 3..n-2 updated, the others kept)."""
    ix, jx, kx = ro.shape
    return _check(load().cans_roe_m_3d(*[_ptr(a) for a in (ro, pr, vx, vy, vz, bx, by, bz)],
                                       _dref(dt), _dref(gm), _ptr(dx), _iref(ix), _ptr(dy),
                                       _iref(jx), _ptr(dz), _iref(kx)), "roe_m_3d")


def bd_3d(kind: int, axis: int, mbnd: int, margin: int, qq: np.ndarray,
          q0: float = 0.0, dxm: np.ndarray | None = None) -> int:
    """One reference bd* call on a 3-D array (cans3d/bc/bd*.f)."""
    lib = load()
    ix, jx, kx = qq.shape
    a = "xyz"[axis]
    dims = (_iref(ix), _iref(jx), _iref(kx))
    if kind == BD_PER:
        f = getattr(lib, f"cans_bdper{a}_3d")
        return _check(f(_iref(margin), _iref(margin), _ptr(qq), *dims), f"bdper{a}")
    name = f"cans_bd{_BD_NAMES[kind]}{a}_3d"
    f = getattr(lib, name)
    if kind == BD_CNS:
        return _check(f(_iref(mbnd), _iref(margin), _ptr(qq), _dref(q0), *dims), name)
    if kind == BD_FRD:
        return _check(f(_iref(mbnd), _iref(margin), _ptr(qq), _ptr(dxm), *dims), name)
    return _check(f(_iref(mbnd), _iref(margin), _ptr(qq), *dims), name)


# ---- residency registry ----------------------------------------------------

def register(arrays) -> None:
    arr = (_dp * len(arrays))(*[_ptr(a) for a in arrays])
    shp = arrays[0].shape + (1,) * (3 - arrays[0].ndim)
    _check(load().cans_gpu_register(arr, _iref(len(arrays)), _iref(shp[0]), _iref(shp[1]),
                                    _iref(shp[2])), "cans_gpu_register")


def pull(any_array) -> None:
    _check(load().cans_gpu_pull(_ptr(any_array)), "cans_gpu_pull")


def push(any_array) -> None:
    _check(load().cans_gpu_push(_ptr(any_array)), "cans_gpu_push")


def release(any_array) -> None:
    _check(load().cans_gpu_release(_ptr(any_array)), "cans_gpu_release")


# ---- device-resident run handle --------------------------------------------

def arr_of(keep: list, a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    keep.append(a)
    return a.ctypes.data_as(_dp)


class _Desc(C.Structure):
    _fields_ = [("solver", C.c_int), ("ix", C.c_int), ("jx", C.c_int), ("kx", C.c_int),
                ("margin", C.c_int), ("gm", C.c_double), ("qav", C.c_double),
                ("dx", _dp), ("dxm", _dp), ("dy", _dp), ("dym", _dp), ("dz", _dp), ("dzm", _dp),
                ("exact", C.c_int), ("tile", C.c_int), ("stream", C.c_void_p),
                ("bx", _dp), ("bxm", _dp), ("mu", C.c_double), ("mfdim", C.c_int * 3),
                ("gx", _dp), ("gxm", _dp), ("sc", _dp), ("scm", _dp), ("dsc", _dp),
                ("dscm", _dp), ("rr", _dp), ("rrm", _dp), ("drr", _dp), ("drrm", _dp),
                ("chkdav", C.c_int), ("floor", C.c_double), ("trq", _dp),
                ("trq0", C.c_double), ("seed", C.c_ulonglong), ("gy", _dp), ("gym", _dp),
                ("et", _dp), ("etm", _dp), ("gz", _dp), ("gzm", _dp),
                ("stop_on_bad", C.c_int)]


class RunState(C.Structure):
    _fields_ = [("t", C.c_double), ("dt", C.c_double), ("ns", C.c_longlong),
                ("nexec", C.c_longlong), ("merr", C.c_int), ("done", C.c_int),
                ("pause", C.c_int), ("n_floor", C.c_longlong), ("n_bad", C.c_longlong)]


class Run:
    """Device-resident run of the reference time loop (cans_run_* API)."""

    def __init__(self, solver: int, grid: dict, gm: float, qav: float, margin: int = 1,
                 exact: bool = False, tile: int = -1, stream: int | None = None,
                 mu: float = 1.0, mfdim=(0, 0, 0), floor: float | None = None,
                 torque: dict | None = None, stop_on_bad: bool = False):
        """grid holds dx, dxm (dy, dym, dz, dzm by dimension; bx, bxm in 1-D;
        the ten BG_PROFILES of mlw_m_bg for SOLVER_MLW_M_BG_1D).  1-D loops
        take floor (chkdav of ro and pr after each boundary fill) and, with
        mlw_m_bg, torque = {"trq": profile, "trq0": amplitude, "seed": key}."""
        self.lib = load()
        self.solver = solver
        self.nvar = {SOLVER_MLW_M_2D: 7, SOLVER_MLW_M3_2D: 9, SOLVER_MLW_M_3D: 8,
                     SOLVER_MLW_M_1D: 5, SOLVER_ROE_M_3D: 8, SOLVER_HLLD_3D: 8,
                     SOLVER_MLW_M_BG_1D: 5, SOLVER_ROE_M3_2D: 9}[solver]
        three = solver in (SOLVER_MLW_M_3D, SOLVER_ROE_M_3D, SOLVER_HLLD_3D)
        one = solver in (SOLVER_MLW_M_1D, SOLVER_MLW_M_BG_1D)
        bgv = solver == SOLVER_MLW_M_BG_1D

        def arr(k):
            a = np.ascontiguousarray(grid[k], dtype=np.float64)
            self._keep.append(a)
            return a.ctypes.data_as(_dp)

        self._keep = []
        nx = np.asarray(grid["dx"]).size
        ny = 1 if one else np.asarray(grid["dy"]).size
        nz = np.asarray(grid["dz"]).size if three else 1
        d = _Desc(solver, nx, ny, nz, margin, gm, qav, arr("dx"), arr("dxm"),
                  None if one else arr("dy"), None if one else arr("dym"),
                  arr("dz") if three else None, arr("dzm") if three else None,
                  1 if exact else 0, tile, C.c_void_p(stream) if stream else None,
                  arr("bx") if one else None, arr("bxm") if one else None,
                  mu, (C.c_int * 3)(*mfdim))
        if not one and grid.get("gx") is not None:
            # step with gravity: four fields (2-D) or six (3-D), Fortran order
            shape = (nx, ny, nz) if three else (nx, ny)
            for k in ("gx", "gxm", "gy", "gym") + (("gz", "gzm") if three else ()):
                if grid.get(k) is None:  # NULL: the library rejects the set-up
                    continue
                a = np.asfortranarray(grid[k], dtype=np.float64)
                if a.shape != shape:
                    raise CansError(CANS_ERR_ARG, k, f"{k} must have shape {shape}")
                self._keep.append(a)
                setattr(d, k, a.ctypes.data_as(_dp))
        if not one and grid.get("et") is not None:
            # resistive step: et at the cells, etm at the corners (a missing
            # etm stays NULL and the library rejects the set-up)
            shape = (nx, ny, nz) if three else (nx, ny)
            for k in ("et", "etm"):
                if grid.get(k) is None:
                    continue
                a = np.asfortranarray(grid[k], dtype=np.float64)
                if a.shape != shape:
                    raise CansError(CANS_ERR_ARG, k, f"{k} must have shape {shape}")
                self._keep.append(a)
                setattr(d, k, a.ctypes.data_as(_dp))
        if bgv:
            for k in ("gx", "gxm", "sc", "scm", "dsc", "dscm", "rr", "rrm", "drr", "drrm"):
                if grid.get(k) is not None:  # a missing profile is rejected by the library
                    setattr(d, k, arr(k))
        if floor is not None:
            d.chkdav, d.floor = 1, float(floor)
        d.stop_on_bad = 1 if stop_on_bad else 0
        if torque is not None:
            d.trq = arr_of(self._keep, torque["trq"])
            d.trq0 = float(torque["trq0"])
            d.seed = int(torque.get("seed", 0))
        self.shape = (nx,) if one else ((nx, ny) + ((nz,) if three else ()))
        h = C.c_void_p()
        _check(self.lib.cans_run_create(C.byref(h), C.byref(d)), "cans_run_create")
        self.h = h

    def close(self):
        if self.h:
            self.lib.cans_run_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_bc(self, var: int, face: int, kind: int, q0: float = 0.0):
        _check(self.lib.cans_run_set_bc(self.h, var, face, kind, q0), "cans_run_set_bc")

    def set_bc_program(self, program):
        """program: iterable of (var, face, kind, q0)."""
        for var, face, kind, q0 in program:
            self.set_bc(var, face, kind, q0)

    def push(self, arrays):
        arr = (_dp * self.nvar)(*[_ptr(a) for a in arrays])
        _check(self.lib.cans_run_push(self.h, arr), "cans_run_push")

    def pull(self, arrays=None):
        if arrays is None:
            arrays = [np.zeros(self.shape, order="F") for _ in range(self.nvar)]
        arr = (_dp * self.nvar)(*[_ptr(a) for a in arrays])
        _check(self.lib.cans_run_pull(self.h, arr), "cans_run_pull")
        return arrays

    def start(self, t0=0.0, tend=1e30, nstop=10 ** 12, safety=0.4, dtmin=1e-10,
              dtout=0.0, pause_on_output=False):
        _check(self.lib.cans_run_start(self.h, t0, tend, nstop, safety, dtmin, dtout,
                                       1 if pause_on_output else 0), "cans_run_start")

    def advance(self, iters: int):
        _check(self.lib.cans_run_advance(self.h, iters), "cans_run_advance")

    @staticmethod
    def advance_group(runs, iters: int):
        """Up to `iters` loop iterations of every run in `runs` (started 1-D
        runs of one solver family and policy), in one launch
        (cans_run_advance_group)."""
        runs = list(runs)
        if not runs:
            raise ValueError("advance_group needs at least one run")
        arr = (C.c_void_p * len(runs))(*[r.h.value for r in runs])
        _check(runs[0].lib.cans_run_advance_group(arr, len(runs), iters),
               "cans_run_advance_group")

    def query(self) -> RunState:
        st = RunState()
        rc = self.lib.cans_run_query(self.h, C.byref(st))
        if rc not in (CANS_OK, CANS_ERR_DTMIN, CANS_ERR_NONFINITE):
            _check(rc, "cans_run_query")
        return st

    def resume(self):
        _check(self.lib.cans_run_resume(self.h), "cans_run_resume")

    def step(self, dt: float, apply_bc: bool = True):
        _check(self.lib.cans_run_step(self.h, _dref(dt), 1 if apply_bc else 0), "cans_run_step")

    def cfl(self, safety: float) -> float:
        dt = C.c_double(0.0)
        _check(self.lib.cans_run_cfl(self.h, safety, C.byref(dt)), "cans_run_cfl")
        return dt.value

    def autotune(self, trial_steps: int = 5) -> int:
        t = C.c_int(0)
        _check(self.lib.cans_run_autotune(self.h, trial_steps, C.byref(t)), "cans_run_autotune")
        return t.value

    def set_graph(self, use_graph: bool):
        _check(self.lib.cans_run_set_graph(self.h, 1 if use_graph else 0), "cans_run_set_graph")

    def set_tile(self, tile: int):
        _check(self.lib.cans_run_set_tile(self.h, tile), "cans_run_set_tile")

    def set_df64(self, on: bool = True):
        """The double-float policy of the step: 2-D mlw_m3, 3-D mlw_m, the
        1-D mlw_m and mlw_m_bg loops, the Roe-MUSCL and HLLD face fluxes
        (see cans_run_set_df64)."""
        _check(self.lib.cans_run_set_df64(self.h, 1 if on else 0), "cans_run_set_df64")

    def profile(self, iters: int):
        """(summed step-kernel ms, summed iteration ms) over `iters` un-graphed
        iterations timed with CUDA events on the run's stream."""
        a, b = C.c_double(0.0), C.c_double(0.0)
        _check(self.lib.cans_run_profile(self.h, iters, C.byref(a), C.byref(b)),
               "cans_run_profile")
        return a.value, b.value

    # ---- discrete adjoint (2-D mlw_m3 runs) ----
    def record_dts(self, nsteps: int, safety: float = 0.4):
        """Forward run from the current state with the CFL time step; returns
        (dts, J) -- the frozen dt sequence and the final magnetic energy."""
        dts = np.zeros(nsteps)
        J = C.c_double(0.0)
        _check(self.lib.cans_run_record_dts(self.h, nsteps, safety, _ptr(dts), C.byref(J)),
               "cans_run_record_dts")
        return dts, J.value

    def objective(self, dts) -> float:
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        J = C.c_double(0.0)
        _check(self.lib.cans_run_objective(self.h, dts.size, _ptr(dts), C.byref(J)),
               "cans_run_objective")
        return J.value

    def av_record(self, dts) -> None:
        """Run the frozen dts from the current state and keep every face's
        artificial-viscosity branch (active or not, sign of dv) on the
        device, for objective_frozen_av."""
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        _check(self.lib.cans_run_av_record(self.h, dts.size, _ptr(dts)), "cans_run_av_record")

    def av_branches(self, step: int):
        """The branches av_record kept for one step: uint8, 2 ix jx (x faces,
        then y faces; bit 0 active, bit 1 dv < 0)."""
        out = np.zeros(2 * int(np.prod(self.shape)), dtype=np.uint8)
        _check(self.lib.cans_run_av_branches(self.h, int(step), out.ctypes.data),
               "cans_run_av_branches")
        return out

    def objective_frozen_av(self, dts):
        """The objective of the frozen dts with every viscosity face held at
        its recorded branch; returns (J, nflip), nflip the face-steps whose
        own branch differs from the recorded one."""
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        J = C.c_double(0.0)
        nf = C.c_longlong(0)
        _check(self.lib.cans_run_objective_frozen_av(self.h, dts.size, _ptr(dts), C.byref(J),
                                                     C.byref(nf)),
               "cans_run_objective_frozen_av")
        return J.value, nf.value

    def set_adjoint_df64(self, on: bool = True):
        """Reverse sweep in double-float (default) or FP64."""
        _check(self.lib.cans_run_set_adjoint_df64(self.h, 1 if on else 0),
               "cans_run_set_adjoint_df64")

    def adjoint(self, dts, nsnap: int = 32):
        """Reverse sweep with binomial checkpointing in nsnap stored states:
        returns (J, grad, nfwd), grad the list of dJ/dP_0 arrays (ghosts
        included) in the state's variable order."""
        dts = np.ascontiguousarray(dts, dtype=np.float64)
        grad = [np.zeros(self.shape, order="F") for _ in range(self.nvar)]
        arr = (_dp * self.nvar)(*[_ptr(g) for g in grad])
        J = C.c_double(0.0)
        nf = C.c_longlong(0)
        _check(self.lib.cans_run_adjoint(self.h, dts.size, _ptr(dts), nsnap, C.byref(J), arr,
                                         C.byref(nf)), "cans_run_adjoint")
        return J.value, grad, nf.value

    def bc_transpose(self, arrays):
        """Transpose of the boundary program, in place on host arrays."""
        arr = (_dp * self.nvar)(*[_ptr(a) for a in arrays])
        _check(self.lib.cans_run_bc_transpose(self.h, arr), "cans_run_bc_transpose")


def _desc_for(solver: int, grid: dict, gm: float, qav: float, margin: int, exact: bool,
              tile: int, stream, keep: list):
    def arr(k):
        a = np.ascontiguousarray(grid[k], dtype=np.float64)
        keep.append(a)
        return a.ctypes.data_as(_dp)
    d = _Desc(solver, np.asarray(grid["dx"]).size, np.asarray(grid["dy"]).size, 1, margin,
              gm, qav, arr("dx"), arr("dxm"), arr("dy"), arr("dym"), None, None,
              1 if exact else 0, tile, C.c_void_p(stream) if stream else None, None, None)
    # source-term fields are passed on so that a solver without them (the
    # batch) refuses the set-up instead of running the plain step
    for k in ("gx", "gxm", "gy", "gym", "et", "etm"):
        if grid.get(k) is not None and (k[0] != "g" or grid.get("gravity")):
            a = np.asfortranarray(grid[k], dtype=np.float64)
            keep.append(a)
            setattr(d, k, a.ctypes.data_as(_dp))
    return d


class Batch:
    """Many independent 2-D runs advanced together (cans_batch_* API).

    setups: list of set-up dicts of one solver (utrip_gb300.setups)."""

    def __init__(self, setups_, exact: bool = False, stream: int | None = None):
        self.lib = load()
        self._keep = []
        solver = setups_[0]["solver_id"]
        self.nvar = 9 if solver == SOLVER_MLW_M3_2D else 7
        descs = (_Desc * len(setups_))(*[
            _desc_for(solver, s, s["gm"], s["qav"], s["margin"], exact, -1, stream, self._keep)
            for s in setups_])
        self.shapes = [s["state"][0].shape for s in setups_]
        h = C.c_void_p()
        _check(self.lib.cans_batch_create(C.byref(h), len(setups_), descs), "cans_batch_create")
        self.h = h
        for g, s in enumerate(setups_):
            for var, face, kind, q0 in s["bc"]:
                _check(self.lib.cans_batch_set_bc(self.h, g, var, face, kind, q0),
                       "cans_batch_set_bc")

    def close(self):
        if self.h:
            self.lib.cans_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def push(self, grid: int, arrays):
        arr = (_dp * self.nvar)(*[_ptr(a) for a in arrays])
        _check(self.lib.cans_batch_push(self.h, grid, arr), "cans_batch_push")

    def pull(self, grid: int, arrays=None):
        if arrays is None:
            arrays = [np.zeros(self.shapes[grid], order="F") for _ in range(self.nvar)]
        arr = (_dp * self.nvar)(*[_ptr(a) for a in arrays])
        _check(self.lib.cans_batch_pull(self.h, grid, arr), "cans_batch_pull")
        return arrays

    def start(self, t0=0.0, tend=1e30, nstop=10 ** 12, safety=0.4, dtmin=1e-10):
        _check(self.lib.cans_batch_start(self.h, t0, tend, nstop, safety, dtmin),
               "cans_batch_start")

    def advance(self, iters: int, use_graph: bool = True):
        _check(self.lib.cans_batch_advance(self.h, iters, 1 if use_graph else 0),
               "cans_batch_advance")

    def query(self, grid: int) -> RunState:
        st = RunState()
        _check(self.lib.cans_batch_query(self.h, grid, C.byref(st)), "cans_batch_query")
        return st

    def set_config(self, config: int):
        _check(self.lib.cans_batch_set_config(self.h, config), "cans_batch_set_config")

    def autotune(self, trial_steps: int = 3) -> int:
        c = C.c_int(0)
        _check(self.lib.cans_batch_autotune(self.h, trial_steps, C.byref(c)),
               "cans_batch_autotune")
        return c.value


def batch_configs() -> int:
    return int(load().cans_batch_configs())
