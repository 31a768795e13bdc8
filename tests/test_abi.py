"""C-ABI checks that need no GPU: the library builds, loads and exports every
routine include/magma_lu.h declares; argument errors are reported the MAGMA
way (negative return, no device work) before any CUDA call."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = "\n".join(l for l in text.splitlines() if not l.lstrip().startswith("#"))
        for m in re.finditer(r"\b(magma\w*)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from magma_gb300 import lib as L
    return L.load()


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("magma_dgetrf_batched", "magma_dgetrs_batched", "magma_dgesv_batched",
                     "magma_queue_create_internal", "magma_sgetrf_batched"):
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from magma_gb300 import lib as L
    assert set(declared_functions()) <= set(L.exported_names())


@pytest.mark.parametrize("args,code", [
    ((-1, 1, 1, 1), -1),
    ((4, -1, 4, 4), -2),
    ((4, 1, 3, 4), -4),
    ((4, 1, 4, 3), -6),
])
def test_gesv_argument_errors(lib, args, code, capfd):
    n, nrhs, ldda, lddb = args
    rc = lib.magma_dgesv_batched(n, nrhs, None, ldda, None, None, lddb, None, 1, None)
    assert rc == code
    assert "magma_dgesv_batched" in capfd.readouterr().err


@pytest.mark.parametrize("args,code", [((-1, 1, 1), -1), ((1, -1, 1), -2), ((5, 5, 4), -4)])
def test_getrf_argument_errors(lib, args, code):
    m, n, ldda = args
    assert lib.magma_dgetrf_batched(m, n, None, ldda, None, None, 1, None) == code
    assert lib.magma_sgetrf_batched(m, n, None, ldda, None, None, 1, None) == code


@pytest.mark.parametrize("args,code", [
    ((110, 4, 1, 4, 4), -1), ((111, -1, 1, 4, 4), -2), ((112, 4, -1, 4, 4), -3),
    ((111, 4, 1, 3, 4), -5), ((113, 4, 1, 4, 3), -8)])
def test_getrs_argument_errors(lib, args, code):
    trans, n, nrhs, ldda, lddb = args
    assert lib.magma_dgetrs_batched(trans, n, nrhs, None, ldda, None, None, lddb, 1, None) == code


def test_quick_returns_do_no_work(lib):
    # n == 0 or batchCount == 0 return 0 without touching any pointer
    assert lib.magma_dgesv_batched(0, 1, None, 1, None, None, 1, None, 5, None) == 0
    assert lib.magma_dgetrf_batched(4, 4, None, 4, None, None, 0, None) == 0
    assert lib.magma_dgetrs_batched(111, 4, 0, None, 4, None, None, 4, 3, None) == 0


def test_small_path_declines_large_sizes(lib):
    # magma_?gesv_batched_small returns -100 ("not applicable") like MAGMA
    assert lib.magma_dgesv_batched_small(33, 1, None, 33, None, None, 33, None, 1, None) == -100
    assert lib.magma_dgesv_batched_small(8, 17, None, 8, None, None, 8, None, 1, None) == -100


def test_vbatched_tuning_table_roundtrip(lib):
    """The tuning table of the variable-size kernel: host-only get/set, validation."""
    import ctypes as C
    for p in "ds":
        get = getattr(lib, f"magma_{p}vbatched_tuning_get")
        put = getattr(lib, f"magma_{p}vbatched_tuning_set")
        nb0, t0 = (C.c_int * 8)(), (C.c_int * 8)()
        assert get(nb0, t0) == 0
        assert all(x in (8, 16, 32) for x in nb0) and all(0 <= x <= 2 for x in t0)
        nb = (C.c_int * 8)(8, 16, 32, 16, 32, 16, 32, 32)
        tile = (C.c_int * 8)(2, 1, 0, 2, 1, 0, 2, 0)
        assert put(nb, tile) == 0
        nb1, t1 = (C.c_int * 8)(), (C.c_int * 8)()
        assert get(nb1, t1) == 0
        assert list(nb1) == list(nb) and list(t1) == list(tile)
        assert put((C.c_int * 8)(12, 16, 32, 16, 32, 16, 32, 32), tile) == -1
        assert put(nb, (C.c_int * 8)(0, 0, 0, 3, 0, 0, 0, 0)) == -2
        assert put(nb0, t0) == 0                       # restore
        # autotune argument errors need no GPU
        assert getattr(lib, f"magma_{p}getrf_vbatched_autotune")(-1, None, None, None) == -1
        assert getattr(lib, f"magma_{p}getrf_vbatched_autotune")(64, None, None, None) == -4


def test_header_is_c99_and_links(lib, tmp_path):
    """A C caller: the header compiles as ISO C99 (-pedantic -Werror) and a program that
    takes the addresses of the entry points links against libmagma_lu.so."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "caller.c"
    src.write_text(
        '#include "magma_lu.h"\n'
        "typedef magma_int_t (*gesv_fn)(magma_int_t, magma_int_t, double **, magma_int_t,\n"
        "                               magma_int_t **, double **, magma_int_t, magma_int_t *,\n"
        "                               magma_int_t, magma_queue_t);\n"
        "static void (*volatile keep[3])(void);\n"
        "int main(void) {\n"
        "    gesv_fn f = magma_dgesv_batched;\n"
        "    keep[0] = (void (*)(void))f;\n"
        "    keep[1] = (void (*)(void))magma_dgetrf_batched;\n"
        "    keep[2] = (void (*)(void))magma_dsposv_batched;\n"
        "    return 0;\n"
        "}\n")
    from magma_gb300 import lib as L
    inc = ROOT / "include"
    libdir = L.LIB_PATH.parent
    out = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", f"-I{inc}",
                          str(src), f"-L{libdir}", "-lmagma_lu", f"-Wl,-rpath,{libdir}", "-o",
                          str(tmp_path / "caller")], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr


def _dynamic_symbol_bindings(path):
    """(binding, name) of every dynamic symbol of a shared library, from readelf."""
    import shutil
    import subprocess
    if shutil.which("readelf") is None:
        pytest.skip("readelf is not installed")
    out = subprocess.run(["readelf", "-W", "--dyn-syms", str(path)], capture_output=True, text=True).stdout
    rows = []
    for line in out.splitlines():
        f = line.split()
        if len(f) >= 8 and f[0].rstrip(":").isdigit():
            rows.append((f[4], f[7]))
    return rows


def test_bounds_check_build_exports_and_binds_locally():
    """The bounds-check library (tests/test_gpu_bounds_check.py loads it beside the normal
    one) exports every declared entry point and its record reader, and holds no GNU-unique
    symbols: those the dynamic linker would merge with the normal library's, sharing its
    per-device kernel-attribute caches across the two libraries."""
    from magma_gb300 import build as B
    path = B.build_bounds_check()
    bc = C.CDLL(str(path))
    missing = [n for n in declared_functions() + ["mlu_bounds_check_read"] if not hasattr(bc, n)]
    assert not missing, missing
    unique = [name for binding, name in _dynamic_symbol_bindings(path) if binding == "UNIQUE"]
    assert not unique, unique[:5]
