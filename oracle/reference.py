"""Build of the reference's own host routines under oracle/_ref (test
infrastructure only, like the rest of this package).

`build_if_available(default)` compiles them with `make -C oracle ref` from the
reference sources where they lie -- the directory named by the
MAGICUBE_REFERENCE environment variable, else `default` (the build script's
choice) -- and records that directory in oracle/_ref/reference_path.txt so
the tests that drive the reference find it.  Where neither exists (the GPU
machines carry no reference checkout) it does nothing.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
RECORD = HERE / "_ref" / "reference_path.txt"


def location() -> Path | None:
    """The reference checkout: MAGICUBE_REFERENCE, else the one recorded by
    the last build; None when neither names an existing directory."""
    env = os.environ.get("MAGICUBE_REFERENCE")
    cands = [Path(env)] if env else []
    if RECORD.exists():
        cands.append(Path(RECORD.read_text().strip()))
    for c in cands:
        if c.is_dir():
            return c
    return None


def build_if_available(default: str | None = None) -> Path | None:
    env = os.environ.get("MAGICUBE_REFERENCE") or default
    if not env or not Path(env).is_dir():
        return None
    ref = Path(env).resolve()
    if not (ref / "SpMM" / "SpMM" / "spmm_benchmark.cpp").exists():
        return None
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={ref}"], check=True)
    RECORD.parent.mkdir(exist_ok=True)
    RECORD.write_text(str(ref) + "\n")
    return ref
