"""Build recipe for libmagma_lu.so (the C-ABI library with the sm_103a kernels).

Each .cu file under csrc/ is compiled by nvcc for sm_103a in parallel, then
linked into magma_gb300/libmagma_lu.so.  Objects go to magma_gb300/_build/.
A rebuild only happens when a source or header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libmagma_lu.so"
BUILD_BC = PKG / "_build_bc"
LIB_BC = PKG / "libmagma_lu_bc.so"
PROBE_SRC = PKG / "probe" / "peaks.cu"
PROBE_LIB = PKG / "libmlu_probe.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmagma_lu.so")
    return cand


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _deps() -> list[Path]:
    return sources() + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "magma_lu.h", Path(__file__)]


def up_to_date() -> bool:
    if not LIB.exists() or not PROBE_LIB.exists():
        return False
    t = min(LIB.stat().st_mtime, PROBE_LIB.stat().st_mtime)
    return all(p.stat().st_mtime <= t for p in _deps() + [PROBE_SRC])


def _compile(src: Path, extra: list[str], outdir: Path = BUILD) -> Path:
    obj = outdir / (src.stem + ".o")
    cmd = [nvcc_path(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-O2", "--expt-relaxed-constexpr", "-I", str(ROOT / "include"),
           *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and "-Xptxas" in " ".join(extra):
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    """Compile every kernel source for sm_103a and link libmagma_lu.so."""
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    srcs = sources() + [PROBE_SRC]
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    _link(objs[:-1], LIB)
    _link(objs[-1:], PROBE_LIB)
    return LIB


def build_bounds_check(force: bool = False) -> Path:
    """The bounds-check build (-DMLU_BOUNDS_CHECK): the same sources with every
    instrumented global access checked against its operand's logical extent, the
    first violation recorded in a device word (mlu_bounds_check_read).  Separate
    objects and library (libmagma_lu_bc.so); relocatable device code, so that
    every translation unit records into the one word.  Its function-local statics (the
    per-device caches of kernel attributes) are ordinary weak symbols bound inside the
    library (-fno-gnu-unique, -Bsymbolic): as GNU-unique symbols the dynamic linker would
    merge them with the normal library's in a process that loads both, and one library's
    filled cache would keep the other from setting its kernels' attributes."""
    if not force and LIB_BC.exists() and all(p.stat().st_mtime <= LIB_BC.stat().st_mtime for p in _deps()):
        return LIB_BC
    BUILD_BC.mkdir(exist_ok=True)
    extra = ["-rdc=true", "-DMLU_BOUNDS_CHECK", "-Xcompiler", "-fno-gnu-unique"]
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, BUILD_BC), srcs))
    _link(objs, LIB_BC, ["-rdc=true", "-Xlinker", "-Bsymbolic"])
    return LIB_BC


def _link(objs: list[Path], out: Path, extra: list[str] | None = None) -> None:
    tmp = out.with_suffix(".so.tmp")
    cmd = [nvcc_path(), *ARCH, "-shared", *(extra or []), "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    print(LIB)
