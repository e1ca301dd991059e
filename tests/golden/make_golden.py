"""Generate the golden fixtures under tests/golden/ from the reference itself.

Needs the reference checkout (--ref, or MAGICUBE_REFERENCE) and builds
oracle/_ref (``make -C oracle ref``): the reference's own host benchmark
programs and verification routines compiled from its source files against a
host-memory fake of the CUDA runtime.  Two kinds of fixture are written:

* ``ref_spmm_*.npz`` / ``ref_sddmm_*.npz`` -- a run of the reference program
  (``spmm_benchmark`` / ``sddmm_benchmark``, same command line as the
  reference's) on a small synthetic ``.smtx`` matrix: the device arrays its
  host packer produced (aligned row offsets, padded / shuffled column
  indices, transposed / bit-plane value layout, rhs), the result, and the
  reference's own verification verdict.  The stand-in kernels compute the
  result with the oracle's device-layout decoder, so "PASS" means the
  reference host routine agrees with that decoder on the reference's data.
* ``routine_*.npz`` -- the reference's compute_ref_integers /
  Host_sddmm_integers called directly on full-range random data (where the
  top-lane sign extension of the reference routines matters), with inputs
  and outputs.

Run:  python tests/golden/make_golden.py --ref <reference checkout>
"""
from __future__ import annotations

import argparse
import ctypes
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from magicube_gb300 import smtx, synth  # noqa: E402

SPMM_PAIRS = [(4, 4), (8, 4), (16, 4), (8, 8), (16, 8), (12, 4), (12, 8), (16, 16)]
SPMM_CASES = [(pa, pb, V) for (pa, pb) in SPMM_PAIRS for V in (2, 4, 8)]
SDDMM_CASES = [(b, V) for b in (4, 8, 16) for V in (2, 4, 8)]
# (TypeA bytes, scaleA) per (preA, preB, V): the dispatch table of the
# reference's main (SpMM/SpMM/spmm_benchmark.cpp:805-831).
TYPEA = {(4, 4, 8): (4, 1), (4, 4, 4): (2, 1), (4, 4, 2): (1, 1),
         (8, 4, 8): (8, 1), (8, 4, 4): (4, 1), (8, 4, 2): (2, 1),
         (16, 4, 8): (8, 2), (16, 4, 4): (8, 1), (16, 4, 2): (4, 1),
         (8, 8, 8): (8, 1), (8, 8, 4): (4, 1), (8, 8, 2): (2, 1),
         (16, 8, 8): (8, 2), (16, 8, 4): (8, 1), (16, 8, 2): (4, 1),
         (12, 4, 8): (8, 2), (12, 4, 4): (8, 1), (12, 4, 2): (4, 1),
         (12, 8, 8): (8, 2), (12, 8, 4): (8, 1), (12, 8, 2): (4, 1),
         (16, 16, 8): (2, 8), (16, 16, 4): (2, 4), (16, 16, 2): (2, 2)}


def lane_bits(pa: int) -> int:
    """Bits per stored lane: the reference keeps 12-bit values in 16-bit containers."""
    return 16 if pa == 12 else pa


def _read(d: Path, name: str, dtype) -> np.ndarray:
    return np.fromfile(d / name, dtype=dtype)


def run_spmm(ref_bin: Path, pa: int, pb: int, V: int, seed: int) -> dict:
    K, N = 128, 128
    lengths = [0, 1, 15, 16, 17, 31, 33, 64, 100, 5, 128, 2]
    mask = synth.lengths_mask(lengths, K, V, seed=seed)
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        smtx.write(td / "m.smtx", mask)
        env = dict(os.environ, MC_REF_DUMP=str(td))
        args = [str(ref_bin), str(td / "m.smtx"), str(N), str(V), "0", "1", "1", "1", str(pa), str(pb)]
        res = subprocess.run(args, capture_output=True, text=True, env=env, timeout=120)
        verdict = "PASS" if "Results verification: PASS" in res.stdout else "FAIL"
        out = {
            "cmd": np.array(" ".join(["spmm_benchmark", "m.smtx"] + args[2:])),
            "verdict": np.array(verdict),
            "m_vec": mask.m_vec, "V": V, "K": K, "N": N, "preA": pa, "preB": pb,
            "csr_row_offsets": mask.row_offsets, "csr_col_indices": mask.col_indices,
            "row_indices": _read(td, "row_indices.bin", np.int32),
            "row_offsets": _read(td, "row_offsets.bin", np.int32),
            "col_indices": _read(td, "col_indices.bin", np.int32),
            "values": _read(td, "values.bin", np.uint8),
            "rhs": _read(td, "rhs.bin", np.uint8),
            "out": _read(td, "out.bin", np.int32),
        }
    return out


def run_sddmm(ref_bin: Path, bits: int, V: int, seed: int) -> dict:
    K, N = 64, 256
    lengths = [0, 1, 7, 8, 9, 16, 17, 40, 100, 3, 256, 12]
    mask = synth.lengths_mask(lengths, N, V, seed=seed)
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        smtx.write(td / "m.smtx", mask)
        env = dict(os.environ, MC_REF_DUMP=str(td))
        args = [str(ref_bin), str(td / "m.smtx"), str(K), str(V), "1", "1", "1", str(bits), str(bits)]
        res = subprocess.run(args, capture_output=True, text=True, env=env, timeout=120)
        verdict = "PASS" if "SDDMM results verification: PASS" in res.stdout else "FAIL"
        out = {
            "cmd": np.array(" ".join(["sddmm_benchmark", "m.smtx"] + args[2:])),
            "verdict": np.array(verdict),
            "m_vec": mask.m_vec, "V": V, "K": K, "N": N, "bits": bits,
            "csr_row_offsets": mask.row_offsets, "csr_col_indices": mask.col_indices,
            "row_indices": _read(td, "row_indices.bin", np.int32),
            "row_offsets": _read(td, "row_offsets.bin", np.int32),
            "col_indices": _read(td, "col_indices.bin", np.int32),
            "lhs": _read(td, "lhs.bin", np.uint8),
            "rhs": _read(td, "rhs.bin", np.uint8),
            "out": _read(td, "out.bin", np.int32),
        }
    return out


def routine_spmm(lib: ctypes.CDLL, pa: int, pb: int, V: int, seed: int) -> dict:
    """compute_ref_integers on full-range random bits."""
    K, N = 64, 64
    mask = synth.lengths_mask([0, 3, 17, 40, 64, 9], K, V, seed=seed)
    tb, scaleA = TYPEA[(pa, pb, V)]
    lb = lane_bits(pa)
    vals = synth.random_bytes(mask.nnz_vec * V * lb // 8, seed + 1)
    rhs = synth.random_bytes(K * N * pb // 8, seed + 2)
    C = np.zeros(mask.rows * N, dtype=np.int32)
    buf = np.ascontiguousarray(vals.copy())
    rb = np.ascontiguousarray(rhs.copy())
    ro = np.ascontiguousarray(mask.row_offsets.copy())
    ci = np.ascontiguousarray(mask.col_indices.copy())
    lib.mcref_compute_ref_integers(tb, buf.ctypes.data, rb.ctypes.data, C.ctypes.data, mask.rows, K, N, lb, pa, pb, V,
                                   ro.ctypes.data, ci.ctypes.data if ci.size else None, mask.m_vec, scaleA)
    return {"m_vec": mask.m_vec, "V": V, "K": K, "N": N, "preA": pa, "preB": pb,
            "row_offsets": mask.row_offsets, "col_indices": mask.col_indices, "values": vals, "rhs": rhs, "out": C}


def routine_sddmm(lib: ctypes.CDLL, bits: int, V: int, seed: int) -> dict:
    """Host_sddmm_integers on full-range random bits (blocked layout, alignment 8)."""
    from magicube_gb300 import formats
    K, N = 64, 128
    mask = synth.lengths_mask([0, 5, 8, 30, 128, 1], N, V, seed=seed)
    pairs, n = formats.align_row_offsets(mask, 8)
    cols = formats.pad_column_indices(mask, pairs, n, shuffle8=False)
    lhs = synth.random_bytes(mask.rows * K * bits // 8, seed + 1)
    rhs = synth.random_bytes(N * K * bits // 8, seed + 2)
    C = np.zeros(n * V, dtype=np.int32)
    a, b = np.ascontiguousarray(lhs.copy()), np.ascontiguousarray(rhs.copy())
    p, c = np.ascontiguousarray(pairs.copy()), np.ascontiguousarray(cols.copy())
    lib.mcref_host_sddmm_integers(a.ctypes.data, b.ctypes.data, C.ctypes.data, mask.rows, K, N, bits, bits, V,
                                  p.ctypes.data, c.ctypes.data, mask.m_vec, 8)
    return {"m_vec": mask.m_vec, "V": V, "K": K, "N": N, "bits": bits, "row_offsets": pairs, "col_indices": cols,
            "lhs": lhs, "rhs": rhs, "out": C}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("MAGICUBE_REFERENCE"))
    args = ap.parse_args()
    if not args.ref:
        ap.error("give --ref <reference checkout> or set MAGICUBE_REFERENCE")
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "all", "ref", f"REF={args.ref}"], check=True)
    rdir = ROOT / "oracle" / "_ref"
    for i, (pa, pb, V) in enumerate(SPMM_CASES):
        d = run_spmm(rdir / "spmm_benchmark", pa, pb, V, seed=100 + i)
        assert str(d["verdict"]) == "PASS", (pa, pb, V)
        np.savez_compressed(HERE / f"ref_spmm_L{pa}R{pb}_V{V}.npz", **d)
    for i, (bits, V) in enumerate(SDDMM_CASES):
        d = run_sddmm(rdir / "sddmm_benchmark", bits, V, seed=200 + i)
        assert str(d["verdict"]) == "PASS", (bits, V)
        np.savez_compressed(HERE / f"ref_sddmm_{bits}b_V{V}.npz", **d)
    lib_s = ctypes.CDLL(str(rdir / "libref_spmm.so"))
    lib_s.mcref_compute_ref_integers.restype = ctypes.c_double
    lib_s.mcref_compute_ref_integers.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 3 + [ctypes.c_int] * 7 + \
        [ctypes.c_void_p] * 2 + [ctypes.c_int] * 2
    lib_d = ctypes.CDLL(str(rdir / "libref_sddmm.so"))
    lib_d.mcref_host_sddmm_integers.restype = ctypes.c_double
    lib_d.mcref_host_sddmm_integers.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 6 + [ctypes.c_void_p] * 2 + \
        [ctypes.c_int] * 2
    for i, (pa, pb, V) in enumerate(SPMM_CASES):
        np.savez_compressed(HERE / f"routine_spmm_L{pa}R{pb}_V{V}.npz", **routine_spmm(lib_s, pa, pb, V, 300 + i))
    for i, (bits, V) in enumerate(SDDMM_CASES):
        np.savez_compressed(HERE / f"routine_sddmm_{bits}b_V{V}.npz", **routine_sddmm(lib_d, bits, V, 400 + i))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
