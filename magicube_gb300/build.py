"""In-tree build of libmagicube_gb300.so (sm_103a) and the C++ tools.

Each CUDA translation unit is compiled by its own nvcc process (in parallel),
then linked into ``magicube_gb300/libmagicube_gb300.so``.  Objects go to
``magicube_gb300/_build``.  A translation unit is rebuilt when it or any header
under ``csrc``/``include`` is newer than its object.

Run ``python -m magicube_gb300.build`` or call :func:`build`.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libmagicube_gb300.so"
PROBE_LIB = PKG / "libmagicube_gb300_probe.so"  # diagnostics (probe.cu), linked against LIB
PROBE_SRCS = ("probe.cu",)
CLI = PKG / "cli"
BIN = PKG / "bin"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmagicube_gb300.so")
    return cand


def _cuda_include() -> str:
    return str(Path(_nvcc()).resolve().parent.parent / "include")


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h")))


def _stale(src: Path, obj: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps])


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build command failed ({res.returncode}):\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _compile(src: Path, verbose: bool) -> Path:
    obj = BUILD / (src.name + ".o")
    deps = _headers()
    if not _stale(src, obj, deps):
        return obj
    if src.suffix == ".cu":
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "--expt-relaxed-constexpr", "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I", str(INCLUDE), "-I", _cuda_include(),
               "-c", str(src), "-o", str(obj)]
    _run(cmd)
    return obj


def _cuda_lib() -> str:
    return str(Path(_nvcc()).resolve().parent.parent / "lib64")


def build_cli() -> list[Path]:
    """The command-line benchmark programs (magicube_gb300/bin), linked
    against the library."""
    BIN.mkdir(exist_ok=True)
    outs = []
    for src in sorted(CLI.glob("*.cpp")):
        exe = BIN / src.stem
        if not exe.exists() or any(p.stat().st_mtime > exe.stat().st_mtime
                                      for p in [src, LIB, *INCLUDE.glob("*.h"), *CLI.glob("*.h")]):
            _run(["g++", "-O2", "-std=c++17", "-Wall", "-I", str(INCLUDE), "-I", _cuda_include(), str(src),
                  "-o", str(exe), "-L", str(PKG), "-lmagicube_gb300", "-L", _cuda_lib(), "-lcudart",
                  "-Wl,-rpath,$ORIGIN/..", "-Wl,-rpath," + _cuda_lib()])
        outs.append(exe)
    return outs


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile and link the library and the CLI programs; returns the path of
    the shared object."""
    BUILD.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    jobs = jobs or max(1, min(len(srcs), os.cpu_count() or 4))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    lib_objs = [o for o, src in zip(objs, srcs) if src.name not in PROBE_SRCS]
    probe_objs = [o for o, src in zip(objs, srcs) if src.name in PROBE_SRCS]
    if not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in lib_objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, lib_objs)])
        os.replace(tmp, LIB)
    if not PROBE_LIB.exists() or any(o.stat().st_mtime > PROBE_LIB.stat().st_mtime for o in [*probe_objs, LIB]):
        tmp = PROBE_LIB.with_suffix(".so.tmp")
        _run([_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, probe_objs), "-L", str(PKG), "-lmagicube_gb300",
              "-Xlinker", "-rpath,$ORIGIN"])
        os.replace(tmp, PROBE_LIB)
    build_cli()
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
