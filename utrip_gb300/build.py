"""Build the sm_103a CUDA library (libcansgpu.so) in-tree, and beside it the
benchmark's peak probe (libcansprobe.so, not part of the solver's ABI).

Each .cu translation unit is compiled by its own nvcc process (in parallel),
then linked into utrip_gb300/_lib/libcansgpu.so.  Host code is compiled with
-ffp-contract=off so the metric arrays computed on the host keep the
reference's separately rounded operations.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
OBJDIR = PKG / "_build"
LIBNAME = "libcansgpu.so"
PROBE = PKG / "probe" / "peaks.cu"
PROBELIB = "libcansprobe.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"),
                 "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcansgpu.so")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def common_flags() -> list[str]:
    return [ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
            "-Xcompiler", "-ffp-contract=off", f"-I{ROOT / 'include'}",
            f"-I{CSRC}"]


def _compile(src: Path, extra: list[str]) -> Path:
    obj = OBJDIR / (src.stem + ".o")
    deps = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + \
        list((ROOT / "include").glob("*.h")) + [src]
    if obj.exists() and all(obj.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return obj
    cmd = [nvcc(), *common_flags(), *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile every .cu under csrc/ and link libcansgpu.so; returns its path."""
    OBJDIR.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    extra = list(extra or [])
    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    lib = LIBDIR / LIBNAME
    if not lib.exists() or any(o.stat().st_mtime > lib.stat().st_mtime for o in objs):
        tmp = LIBDIR / (LIBNAME + ".tmp")
        cmd = [nvcc(), ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    probe = LIBDIR / PROBELIB
    if not probe.exists() or probe.stat().st_mtime < PROBE.stat().st_mtime:
        cmd = [nvcc(), ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
               str(PROBE), "-o", str(probe)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"probe build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {lib} and {probe.name}")
    return lib


def build_oracle() -> Path:
    """Compile the CPU oracle (test infrastructure) with its Makefile."""
    odir = ROOT / "oracle"
    r = subprocess.run(["make", "-s", "-C", str(odir)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return odir / "_build" / "libcansoracle.so"


if __name__ == "__main__":
    build(verbose=True)
    print(build_oracle())
