"""CPU oracle of the quantized vector-sparse SpMM / SDDMM path.

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` as the checker; the library never
uses it.  ``mc_oracle.c`` restates the reference's host verification routines
(compute_ref_integers, SpMM/SpMM/spmm_benchmark.cpp:69-120; Host_sddmm_integers,
SDDMM/SDDMM/sddmm_benchmark.cpp:24-60); this module wraps it for numpy.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libmc_oracle.so"

LITERAL, UNSIGNED, SIGNED = 0, 1, 2
OUT_BLOCKED, OUT_VECMAJOR = 0, 1

_handle = None


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    return LIB_PATH


def lib() -> ctypes.CDLL:
    global _handle
    if _handle is None:
        if not LIB_PATH.exists():
            build()
        h = ctypes.CDLL(str(LIB_PATH))
        vp, ci = ctypes.c_void_p, ctypes.c_int
        h.mco_spmm_host.argtypes = [vp, vp, vp] + [ci] * 7 + [vp, vp, ci]
        h.mco_spmm_host.restype = None
        h.mco_sddmm_host.argtypes = [vp, vp, vp] + [ci] * 6 + [vp, vp, ci, ci, ci]
        h.mco_sddmm_host.restype = None
        h.mco_spmm_device.argtypes = [vp, vp, vp, vp, vp] + [ci] * 8
        h.mco_spmm_device.restype = None
        _handle = h
    return _handle


def _p(a: np.ndarray):
    return a.ctypes.data if a.size else None


def spmm_host(values: np.ndarray, rhs: np.ndarray, row_offsets: np.ndarray, col_indices: np.ndarray,
              m_vec: int, V: int, K: int, N: int, preA: int, preB: int, mode: int,
              preA_cut: int | None = None) -> np.ndarray:
    """C (M x N int32) from the original operand layout (compute_ref_integers)."""
    values = np.ascontiguousarray(values, dtype=np.uint8)
    rhs = np.ascontiguousarray(rhs).view(np.uint8)
    ro = np.ascontiguousarray(row_offsets, dtype=np.int32)
    ci = np.ascontiguousarray(col_indices, dtype=np.int32)
    out = np.empty((m_vec * V, N), dtype=np.int32)
    lib().mco_spmm_host(_p(values), _p(rhs), _p(out), m_vec, V, K, N, preA, preA_cut or preA, preB,
                        _p(ro), _p(ci), mode)
    return out


def sddmm_host(lhs: np.ndarray, rhs: np.ndarray, pairs: np.ndarray, cols: np.ndarray, m_vec: int, V: int,
               K: int, N: int, preA: int, preB: int, mode: int, alignment: int = 8,
               layout: int = OUT_BLOCKED, out_size: int | None = None) -> np.ndarray:
    """SDDMM output over the aligned slots (Host_sddmm_integers); padding stays 0."""
    lhs = np.ascontiguousarray(lhs).view(np.uint8)
    rhs = np.ascontiguousarray(rhs).view(np.uint8)
    pr = np.ascontiguousarray(pairs, dtype=np.int32)
    cc = np.ascontiguousarray(cols, dtype=np.int32)
    size = out_size if out_size is not None else cc.size * V
    out = np.zeros(size, dtype=np.int32)
    lib().mco_sddmm_host(_p(lhs), _p(rhs), _p(out), m_vec, V, K, N, preA, preB, _p(pr), _p(cc),
                         alignment, layout, mode)
    return out


def align_pairs(row_offsets: np.ndarray, alignment: int) -> tuple[np.ndarray, int]:
    """Aligned [start, end) pairs of a plain vector CSR, numpy only.

    Restates the reference's host conversion (SpMM/SpMM/spmm_benchmark.cpp:196-206):
    each vector-row starts at the running total of the previous rows' lengths
    rounded up to a multiple of `alignment`; its end is start + true length.
    Returns (pairs int32[2 m_vec], aligned slot count)."""
    ro = np.asarray(row_offsets, dtype=np.int64)
    lengths = np.diff(ro)
    padded = (lengths + alignment - 1) // alignment * alignment
    starts = np.zeros(lengths.size, dtype=np.int64)
    if lengths.size > 1:
        np.cumsum(padded[:-1], out=starts[1:])
    pairs = np.empty(2 * lengths.size, dtype=np.int32)
    pairs[0::2] = starts
    pairs[1::2] = starts + lengths
    return pairs, int(padded.sum())


def pad_columns(row_offsets: np.ndarray, col_indices: np.ndarray, pairs: np.ndarray, aligned_nnz: int) -> np.ndarray:
    """Column indices in the aligned slots, -1 in the padding slots (numpy
    restatement of SpMM/SpMM/spmm_benchmark.cpp:209-216, without the 4-bit
    8-shuffle)."""
    ro = np.asarray(row_offsets, dtype=np.int64)
    ci = np.asarray(col_indices, dtype=np.int32)
    out = np.full(aligned_nnz, -1, dtype=np.int32)
    lengths = np.diff(ro)
    # destination slot of source nonzero j of row i: pairs[2 i] + (j - ro[i])
    dst = np.repeat(np.asarray(pairs[0::2], dtype=np.int64) - ro[:-1], lengths) + np.arange(int(ro[-1]))
    out[dst] = ci[:int(ro[-1])]
    return out


def spmm_device(pairs: np.ndarray, cols: np.ndarray, dev_values: np.ndarray, rhs: np.ndarray, m_vec: int,
                V: int, K: int, N: int, preA: int, preB: int, mode: int, layout: int = 0) -> np.ndarray:
    """C (M x N int32) decoded from the SpMM device operand layout."""
    pr = np.ascontiguousarray(pairs, dtype=np.int32)
    cc = np.ascontiguousarray(cols, dtype=np.int32)
    dv = np.ascontiguousarray(dev_values).view(np.uint8)
    rhs = np.ascontiguousarray(rhs).view(np.uint8)
    out = np.empty((m_vec * V, N), dtype=np.int32)
    lib().mco_spmm_device(_p(pr), _p(cc), _p(dv), _p(rhs), _p(out), m_vec, V, K, N, preA, preB, mode, layout)
    return out
