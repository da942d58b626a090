"""The reference's own driver program, src/main.cu, compiles and links
against this library with no change but its include lines: the four GPU
headers it includes (src/main.cu:4 FastLoad_GPU.h, :6 csr2csc_cuda.h, :7
formatTransform_GPU.h, :8 ColSort_GPU.h) are replaced by fastload_compat.h,
and everything else -- its CPU headers (coo2csc.h, FastLoad_CPU.h,
auxiliary.h, mmio.h), its comparators (CSCSpMV.h, cusparse_cuda.h) and every
call it makes -- comes from the reference checkout unchanged, compiled here
as test infrastructure in a temporary directory (nothing is copied into the
repository).  Running it needs a GPU and the checkout's matrix files, which
only this machine has, so the test stops at the link: every fl_ symbol the
program needs must be exported by the library."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT, reference_checkout
from test_abi import exported_symbols

REPLACED = {4: "FastLoad_GPU.h", 6: "csr2csc_cuda.h", 7: "formatTransform_GPU.h", 8: "ColSort_GPU.h"}


def test_reference_main_cu_links_against_the_library(built_lib, tmp_path):
    ref = reference_checkout()
    if ref is None:
        pytest.skip("the reference checkout is not on this machine")
    if not shutil.which("nvcc"):
        pytest.skip("no nvcc")
    from fastload_gb300 import _build

    src = open(os.path.join(ref, "src", "main.cu")).read().split("\n")
    out = list(src)
    for line, header in REPLACED.items():
        assert src[line - 1].strip() == f'#include "{header}"', (line, src[line - 1])
        out[line - 1] = '#include "fastload_compat.h"' if line == 4 else ""
    changed = [i + 1 for i, (a, b) in enumerate(zip(src, out)) if a != b]
    assert changed == sorted(REPLACED)  # the include lines and nothing else
    main = tmp_path / "main.cu"
    main.write_text("\n".join(out))
    exe = str(tmp_path / "fastload_main")
    r = subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-w",
                        "-I", os.path.join(ref, "src"), "-I", os.path.join(ROOT, "include"), str(main), "-o", exe,
                        "-L", _build.LIBDIR, "-lfastload_gb300", "-lcusparse", "-Xlinker", f"-rpath={_build.LIBDIR}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    nm = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True, text=True, check=True).stdout
    needed = {ln.split()[-1] for ln in nm.splitlines() if ln.split() and ln.split()[-1].startswith("fl_")}
    # main.cu's four replaced calls: csr_to_csc, ColSort, formatTransform, FastLoad_spmv
    assert {"fl_csr_to_csc", "fl_col_sort", "fl_format_transform", "fl_fastload_spmv"} <= needed
    assert needed <= exported_symbols(_build.lib_path())
