"""CPU-side checks of the C ABI: the library builds, loads, exports every
symbol include/cans_gpu.h declares, and rejects bad arguments before it
touches a device.  No compute call is made here (there is no GPU)."""
import ctypes as C

import numpy as np
import pytest

from utrip_gb300 import build, capi


@pytest.fixture(scope="module")
def lib():
    build.build()
    return capi.load()


def test_every_declared_symbol_is_exported(lib):
    names = capi.exported_symbols()
    assert len(names) >= 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_header_declares_the_drop_in_routines():
    names = set(capi.exported_symbols())
    for n in ("cans_mlw_m3_2d", "cans_mlw_m_2d", "cans_cfl_m3_2d", "cans_cfl_m_2d",
              "cans_bdperx_2d", "cans_bdsppy_2d", "cans_bdsmnx_2d", "cans_gpu_register",
              "cans_gpu_pull", "cans_run_create", "cans_run_advance"):
        assert n in names, n


def test_bad_sizes_are_rejected_without_a_device(lib):
    a = np.zeros((2, 5), order="F")
    z = C.c_double(0.1)
    with pytest.raises(capi.CansError) as e:
        capi.mlw_m3(*([a] * 9), 0.1, 3.0, 5 / 3, np.ones(2), np.ones(2), np.ones(5), np.ones(5))
    assert e.value.code == capi.CANS_ERR_ARG
    # bd with a margin larger than the axis
    q = np.zeros((3, 3), order="F")
    with pytest.raises(capi.CansError) as e:
        capi.bd(capi.BD_SPP, 0, 0, 4, q)
    assert e.value.code == capi.CANS_ERR_ARG
    del z


def test_run_desc_layout_matches_header(tmp_path):
    # the ctypes mirror of cans_run_desc must keep the C field order, offsets
    # and size: compile the header with the host compiler and compare
    fields = [f[0] for f in capi._Desc._fields_]
    assert fields == ["solver", "ix", "jx", "kx", "margin", "gm", "qav", "dx", "dxm", "dy",
                      "dym", "dz", "dzm", "exact", "tile", "stream", "bx", "bxm", "mu",
                      "mfdim", "gx", "gxm", "sc", "scm", "dsc", "dscm", "rr", "rrm", "drr",
                      "drrm", "chkdav", "floor", "trq", "trq0", "seed", "gy", "gym", "et", "etm", "gz", "gzm",
                      "stop_on_bad"]
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    src = tmp_path / "layout.c"
    body = "".join(f'  printf("%zu ", offsetof(cans_run_desc, {f}));\n' for f in fields)
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "cans_gpu.h"\n'
                   "int main(void) {\n" + body +
                   '  printf("%zu\\n", sizeof(cans_run_desc));\n  return 0;\n}\n')
    exe = tmp_path / "layout"
    inc = build.ROOT / "include"
    subprocess.run([cc, f"-I{inc}", str(src), "-o", str(exe)], check=True)
    out = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True,
                                          text=True).stdout.split()]
    want = [getattr(capi._Desc, f).offset for f in fields] + [C.sizeof(capi._Desc)]
    assert out == want


def test_run_state_layout_matches_header(tmp_path):
    import shutil
    import subprocess
    fields = [f[0] for f in capi.RunState._fields_]
    assert fields[-1] == "n_bad"
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no host C compiler")
    src = tmp_path / "state.c"
    body = "".join(f'  printf("%zu ", offsetof(cans_run_state, {f}));\n' for f in fields)
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "cans_gpu.h"\n'
                   "int main(void) {\n" + body +
                   '  printf("%zu\\n", sizeof(cans_run_state));\n  return 0;\n}\n')
    exe = tmp_path / "state"
    subprocess.run([cc, f"-I{build.ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    out = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True,
                                          text=True).stdout.split()]
    assert out == [getattr(capi.RunState, f).offset for f in fields] + [C.sizeof(capi.RunState)]


def test_mlw_m_bg_run_arguments_rejected_without_a_device(lib):
    from utrip_gb300 import setups
    s = setups.shock_tube_1d(64)
    # the torque source needs the mlw_m_bg profiles
    with pytest.raises(capi.CansError) as e:
        capi.Run(capi.SOLVER_MLW_M_1D, s, s["gm"], s["qav"],
                 torque={"trq": np.zeros(s["x"].size), "trq0": 1.0})
    assert e.value.code == capi.CANS_ERR_ARG
    # mlw_m_bg without its profiles
    with pytest.raises(capi.CansError) as e:
        capi.Run(capi.SOLVER_MLW_M_BG_1D, dict(s, gx=None), s["gm"], s["qav"])
    assert e.value.code in (capi.CANS_ERR_ARG,)


def test_hlld_and_roe_run_arguments_rejected_without_a_device(lib):
    from utrip_gb300 import setups
    s = setups.random_state_3d(12, 11, 10, seed=1, solver="roe_m_3d")
    with pytest.raises(capi.CansError) as e:  # Roe needs three boundary layers
        capi.Run(capi.SOLVER_ROE_M_3D, s, s["gm"], 0.0, margin=2)
    assert e.value.code == capi.CANS_ERR_ARG
    s = setups.shock_tube_hlld_1d(32)
    with pytest.raises(capi.CansError) as e:  # y is one cell long: cannot be active
        capi.Run(capi.SOLVER_HLLD_3D, s, s["gm"], 0.0, margin=3, mfdim=(1, 1, 0))
    assert e.value.code == capi.CANS_ERR_ARG


def test_advance_group_arguments_rejected_without_a_device(lib):
    """cans_run_advance_group refuses an empty group, a null list and null
    handles before any device work."""
    assert lib.cans_run_advance_group(None, 1, 5) == capi.CANS_ERR_ARG
    arr = (C.c_void_p * 2)(None, None)
    assert lib.cans_run_advance_group(arr, 0, 5) == capi.CANS_ERR_ARG
    assert lib.cans_run_advance_group(arr, 2, 5) == capi.CANS_ERR_ARG
    assert lib.cans_run_advance_group(arr, 2, -1) == capi.CANS_ERR_ARG
    with pytest.raises(ValueError):
        capi.Run.advance_group([], 5)


def test_av_branches_rejects_a_null_handle(lib):
    out = np.zeros(8, dtype=np.uint8)
    assert lib.cans_run_av_branches(None, 0, out.ctypes.data) == capi.CANS_ERR_ARG
