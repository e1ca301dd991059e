"""Drop-in at the C++ level: the reference's own benchmark programs
(SpMM/SpMM/spmm_benchmark.cpp, SDDMM/SDDMM/sddmm_benchmark.cpp), compiled from
their unmodified sources, link against libmagicube_gb300.so in place of the
reference's kernel sources (every spmm:: / sddmm:: symbol they call resolves
to this library).  CPU only; skipped where no reference checkout is known
(MAGICUBE_REFERENCE, or the one recorded by the build of oracle/_ref)."""
import shutil
import subprocess
from pathlib import Path

import pytest

from magicube_gb300 import build

from oracle.reference import location

REF = location() or Path("/nonexistent")
PROGRAMS = ["SpMM/SpMM/spmm_benchmark.cpp", "SDDMM/SDDMM/sddmm_benchmark.cpp"]


@pytest.mark.skipif(not REF.exists() or shutil.which("g++") is None, reason="reference sources not present")
@pytest.mark.parametrize("prog", PROGRAMS)
def test_reference_program_links_against_library(tmp_path, prog):
    src = REF / prog
    if not src.exists():
        pytest.skip(f"{src} missing")
    if not build.LIB.exists():
        build.build()
    cuda = Path(build._cuda_include()).parent
    exe = tmp_path / src.stem
    res = subprocess.run(
        ["g++", "-std=c++17", "-O1", "-w", "-include", "typeinfo", "-include", "numeric", "-include", "cstring",
         "-I", str(cuda / "include"), str(src), "-o", str(exe), "-L", str(build.PKG), "-lmagicube_gb300",
         "-L", str(cuda / "lib64"), "-lcudart", "-Wl,--no-undefined"],
        capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    assert exe.exists()
