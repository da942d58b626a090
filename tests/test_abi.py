"""The C-ABI library: builds, loads without a GPU, exports every symbol that
include/*.h declares, and rejects bad arguments before touching CUDA."""
import ctypes as C
import glob
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        txt = re.sub(r"//[^\n]*", "", txt)
        if "extern \"C\"" not in txt and "fastload_compat" in h:
            continue
        for name in re.findall(r"\b(fl_[a-z0-9_]+)\s*\(", txt):
            syms.add(name)
    return syms


def exported_symbols(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if ln.strip()}


def test_library_exports_every_declared_symbol(built_lib):
    from fastload_gb300 import _build, _lib

    declared = declared_symbols()
    assert "fl_fastload_spmv" in declared and "fl_plan_spmv" in declared
    exported = exported_symbols(_build.lib_path())
    missing = sorted(declared - exported)
    assert not missing, f"declared but not exported: {missing}"
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert declared <= bound | {"fl_plan_info_get"}, sorted(declared - bound)


def test_library_exports_only_the_c_api(built_lib):
    """Built with hidden visibility: no C function beyond the header's, and no
    GNU-unique symbol (the static state of a template instantiation, which the
    dynamic linker shares across every library in the process that defines
    it)."""
    from fastload_gb300 import _build

    out = subprocess.run(["nm", "-D", "--defined-only", _build.lib_path()], capture_output=True, text=True,
                         check=True).stdout
    rows = [ln.split() for ln in out.splitlines() if ln.strip()]
    unique = [r[-1] for r in rows if r[-2] == "u"]
    assert not unique, f"GNU-unique exports: {unique[:5]}"
    c_funcs = {r[-1] for r in rows if r[-2] == "T" and not r[-1].startswith("_Z")}
    extra = sorted(c_funcs - declared_symbols())
    assert not extra, f"exported but not declared in include/: {extra}"
    # C++ exports: only standard-library template instances (default
    # visibility in libstdc++'s own headers), none of the library's types
    own = [r[-1] for r in rows if r[-1].startswith("_Z") and not r[-1].startswith(("_ZNSt", "_ZSt", "_ZNKSt"))]
    assert not own, f"library C++ symbols exported: {own[:5]}"


def test_library_is_built_for_sm_103a_only(built_lib):
    from fastload_gb300 import _build

    assert ["-gencode", "arch=compute_103a,code=sm_103a"] == _build.ARCH


def test_version_and_device_count(built_lib):
    assert b"sm_103a" in built_lib.fl_version()
    assert built_lib.fl_device_count() >= 0


def _vp(a):
    return C.c_void_p(a.ctypes.data)


def test_argument_errors_without_gpu(built_lib):
    from fastload_gb300 import _lib

    t = C.c_double()
    rc = built_lib.fl_csr_to_csc(C.byref(t), -1, 3, 0, None, None, None, None, None, None, None)
    assert rc == -1
    assert b"negative size" in built_lib.fl_last_error()
    rc = built_lib.fl_csr_to_csc(C.byref(t), 3, 3, 2, None, None, None, None, None, None, None)
    assert rc == -1 and b"NULL" in built_lib.fl_last_error()
    rc = built_lib.fl_csr_to_csc(C.byref(t), 3, 3, 0x7fffffff, None, None, None, None, None, None, None)
    assert rc == -4  # FL_ERR_OVERFLOW
    m = _lib.SlideMatrixC()
    rc = built_lib.fl_format_transform(None, None, None, None, None, None, 0, 1, 1, None)
    assert rc == -1
    rc = built_lib.fl_fastload_spmv(C.byref(m), 1, 1, 1, None, None, None, 1, None, None)
    assert rc == -1
    x = np.zeros(1)
    rc = built_lib.fl_fastload_spmv(C.byref(m), 0, 1, 1, _vp(x), _vp(x), None, -3, None, None)
    assert rc == -1 and b"reps" in built_lib.fl_last_error()
    h = C.c_void_p()
    rc = built_lib.fl_plan_create_csr(C.byref(h), 2, 2, 1, None, None, None, 0, None)
    assert rc == -1 and not h.value
    # the calls added beside the reference's: argument checks before any GPU work
    assert built_lib.fl_convert_values(0, 4, None, None, None) == -1  # FP64 is not a storage conversion
    assert built_lib.fl_convert_values(1, -1, None, None, None) == -1
    assert built_lib.fl_convert_values(2, 0, None, None, None) == 0  # nothing to convert
    fid = C.c_int(-1)
    assert built_lib.fl_plan_add_form_opts(None, None, C.byref(fid)) == -1
    assert built_lib.fl_plan_form_set_launch(None, 0, 1, 0) == -1
    assert built_lib.fl_plan_add_tuned_form(None, b"model", 1, 0, C.byref(fid), None) == -1
    assert built_lib.fl_tuner_variants(None, 0) > 0


def test_python_wrappers_raise(built_lib):
    from fastload_gb300 import FastLoadError, csr_to_csc

    with pytest.raises(FastLoadError):
        csr_to_csc(3, 3, 2, np.zeros(2), np.zeros(3, np.int32), np.zeros(2, np.int32))  # rowptr too short


def test_tile_destroy_accepts_empty(built_lib):
    from fastload_gb300 import _lib

    m = _lib.SlideMatrixC()
    built_lib.fl_tile_destroy(C.byref(m))
    built_lib.fl_tile_destroy(None)


def test_dropin_program_links_against_the_library(built_lib, tmp_path):
    """tests/dropin/main_dropin.cpp (the reference main.cu's call sequence on
    fastload_compat.h) compiles with g++ and links: every fl_ symbol it needs
    is exported.  Running it needs the GPU (test_gpu_parity.py)."""
    import shutil

    from fastload_gb300 import _build

    if not shutil.which("g++"):
        pytest.skip("no g++")
    exe = str(tmp_path / "dropin")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "dropin", "main_dropin.cpp"), "-o", exe,
                    "-L", _build.LIBDIR, "-lfastload_gb300", f"-Wl,-rpath,{_build.LIBDIR}"], check=True)
    out = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True, text=True, check=True).stdout
    needed = {ln.split()[-1] for ln in out.splitlines() if ln.split() and ln.split()[-1].startswith("fl_")}
    assert needed, "the drop-in program calls no library function"
    assert needed <= exported_symbols(_build.lib_path())
