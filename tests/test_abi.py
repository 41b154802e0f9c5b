"""The C ABI boundary, checked without a GPU: the library builds, loads and
exports every function include/g6.h declares; host-side argument checks
return error codes.  No kernel is launched here."""
import ctypes
import os
import re
import subprocess

import pytest

import amuse_gb300 as ag

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "g6.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?(?:int|void|double|char)\s*\*?\s*(\w+)\s*\(",
                                 src, flags=re.M)))


def exported(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    return {line.split()[-1]: line.split()[-2] for line in out.splitlines() if line.strip()}


def test_header_lists_the_16_grape6_symbols():
    fns = declared_functions()
    for s in ag.ABI_SYMBOLS:
        assert s in fns
    assert len(ag.ABI_SYMBOLS) == 16


def test_every_declared_symbol_is_exported(lib_built):
    syms = exported(ag.LIB_PATH)
    missing = [f for f in declared_functions() if f not in syms]
    assert not missing, missing
    # by-value forms are weak so that ph4's grape.cc copies take precedence
    for s in ag.BYVALUE_SYMBOLS:
        assert syms[s] in ("W", "V"), (s, syms[s])
    for s in ag.ABI_SYMBOLS + ag.EXT_SYMBOLS:
        assert syms[s] == "T", s


def test_library_loads_and_binds(lib_built):
    lib = ag.load()
    for s in ag.ABI_SYMBOLS + ag.BYVALUE_SYMBOLS + ag.EXT_SYMBOLS:
        assert hasattr(lib, s)
    drv = ag.driver()
    for s in ("drv_load", "drv_update", "drv_force"):
        assert hasattr(drv, s)


def test_no_cpu_force_path_in_library(lib_built):
    # The product library must not carry the oracle's symbols.
    syms = exported(ag.LIB_PATH)
    assert not any(s.startswith(("orc_", "ph4ref_")) for s in syms)


def test_calls_before_open_fail_cleanly(lib_built):
    lib = ag.load()
    if lib.g6x_get_precision() is None:
        pytest.skip()
    ti = ctypes.c_double(0.0)
    cid = ctypes.c_int(0)
    # not opened in this process (no GPU here): negative code, no crash
    if os.environ.get("CUDA_VISIBLE_DEVICES", None) == "" or not _has_gpu():
        assert lib.g6_set_ti_(ctypes.byref(cid), ctypes.byref(ti)) == -1
        assert lib.g6_open_(ctypes.byref(cid)) in (-5, -3)
        assert lib.g6_npipes_() == 16384
        # extension calls: G6_ERR_NOT_OPEN before any device work
        slots = (ctypes.c_int * 1)(0)
        ids = (ctypes.c_int * 12)()
        d2 = (ctypes.c_double * 12)()
        assert lib.g6x_set_encounters(ag.ENC_STOP_COLLISION, 0.0) == -1
        assert lib.g6x_set_radius(0, None) == -1
        assert lib.g6x_encounter(None, None) == -1
        assert lib.g6x_knn(12, 10, 0.0, 1, slots, ids, d2) == -1
        assert lib.g6x_run(1.0, None, None) == -1


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_driver_ffi_stub_compiles(tmp_path, lib_built):
    """The binding a ph4 maintainer adds: grape.cc's by-value calls resolve
    against libsapporo.so with nothing but the header and -lsapporo."""
    src = tmp_path / "caller.c"
    src.write_text(
        '#include "g6.h"\n'
        "int main(void){ int id=0; double t=0; if (g6_open(0)) return 0;\n"
        " g6_set_ti_(&id,&t); return g6_npipes() > 0 ? 0 : 1; }\n")
    exe = tmp_path / "caller"
    subprocess.run(["gcc", str(src), "-I", os.path.dirname(HEADER), "-L", ag.LIB_DIR,
                    "-lsapporo", "-Wl,-rpath," + ag.LIB_DIR, "-o", str(exe)], check=True)
    assert exe.exists()


def test_ph4_gpu_mode_links_against_libsapporo(lib_built):
    """The real drop-in: the UNMODIFIED ph4 sources built in GPU mode
    (-DGPU -DNOMPI: src/amuse_ph4/src/gpu.cc:36-492 and grape.cc:6-147 call
    the GRAPE-6 API) link against libsapporo.so.  ph4's own by-value wrappers
    (grape.cc) are the definitions in the executable; every trailing-
    underscore ABI symbol they call is left to libsapporo.so.  Needs the
    reference checkout (AMUSE_REF); compile and link only."""
    import oracle
    if oracle.ref_root() is None:
        pytest.skip("AMUSE_REF does not name a reference checkout")
    here = os.path.dirname(oracle.__file__)
    subprocess.run(["make", "-s", "-C", here, "link", "-j8"], check=True)
    exe = os.path.join(here, "_ref", "ph4_gpu_run")
    syms = subprocess.run(["nm", exe], capture_output=True, text=True, check=True).stdout
    defined = {ln.split()[-1] for ln in syms.splitlines() if " T " in ln}
    undefined = {ln.split()[-1] for ln in syms.splitlines() if ln.strip().startswith("U ")}
    for s in ag.ABI_SYMBOLS:
        assert s in undefined, s           # resolved by libsapporo.so at run time
        assert s[:-1] in defined, s[:-1]   # ph4's strong wrapper, not the library's weak one
    dyn = subprocess.run(["readelf", "-d", exe], capture_output=True, text=True,
                         check=True).stdout
    assert "[libsapporo.so]" in dyn
