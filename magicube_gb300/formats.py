"""Vector-sparse storage: plain CSR of column vectors and its device layout.

A sparse M x K matrix with vector length V is stored as m_vec = M / V
vector-rows.  ``row_offsets`` (m_vec + 1 entries) and ``col_indices`` describe
the plain CSR of vectors (one column index per nonzero vector, the layout of
the reference's ``.smtx`` files, SpMM/SpMM/spmm_benchmark.cpp:126-175).  The
kernels consume the aligned device layout built here by the library's C++
packer (``mcAlignRowOffsets`` / ``mcPadColumnIndices`` / ``mcPackSpmmValues``).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib


def _ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


@dataclass
class VectorSparse:
    """Plain CSR of column vectors (host arrays)."""

    m_vec: int
    vec_length: int
    ncols: int
    row_offsets: np.ndarray  # int32[m_vec + 1]
    col_indices: np.ndarray  # int32[nnz_vec]

    @property
    def nnz_vec(self) -> int:
        return int(self.row_offsets[-1])

    @property
    def rows(self) -> int:
        return self.m_vec * self.vec_length

    def row_lengths(self) -> np.ndarray:
        return np.diff(self.row_offsets)


def spmm_chunk(lhs_bits: int, rhs_bits: int) -> int:
    """Vector slots per value chunk (and row alignment) of the SpMM layout."""
    return 32 if (lhs_bits == 4 or rhs_bits == 4) else 16


def lane_bits(lhs_bits: int) -> int:
    """Bits per stored value lane: 12-bit values live in 16-bit lanes (the
    reference's 12-bit containers, SpMM/SpMM/spmm_benchmark.cpp:810-822)."""
    return 16 if lhs_bits == 12 else lhs_bits


def align_row_offsets(mask: VectorSparse, alignment: int) -> tuple[np.ndarray, int]:
    ro = np.ascontiguousarray(mask.row_offsets, dtype=np.int32)
    pairs = np.zeros(2 * mask.m_vec, dtype=np.int32)
    n = _lib.lib().mcAlignRowOffsets(mask.m_vec, _ptr(ro), alignment, _ptr(pairs))
    if n < 0:
        _lib.check(1, "mcAlignRowOffsets")
    return pairs, int(n)


def pad_column_indices(mask: VectorSparse, pairs: np.ndarray, aligned_nnz: int, shuffle8: bool) -> np.ndarray:
    ro = np.ascontiguousarray(mask.row_offsets, dtype=np.int32)
    ci = np.ascontiguousarray(mask.col_indices, dtype=np.int32)
    out = np.empty(max(aligned_nnz, 1), dtype=np.int32)
    _lib.check(_lib.lib().mcPadColumnIndices(mask.m_vec, _ptr(ro), _ptr(ci) if ci.size else None,
                                             _ptr(pairs), aligned_nnz, int(shuffle8), _ptr(out)),
               "mcPadColumnIndices")
    return out[:aligned_nnz]


VALUES_PACKED, VALUES_SOFTMAX, VALUES_SLOT_MAJOR = 0, 1, 2


def pack_spmm_values(mask: VectorSparse, pairs: np.ndarray, aligned_nnz: int, values: np.ndarray,
                     lhs_bits: int, rhs_bits: int, layout: int = VALUES_PACKED) -> np.ndarray:
    """values: uint8 array of nnz_vec * V * lane_bits(lhs_bits) / 8 bytes (lane v
    at bit v * lane_bits(lhs_bits))."""
    ro = np.ascontiguousarray(mask.row_offsets, dtype=np.int32)
    v = np.ascontiguousarray(values, dtype=np.uint8)
    nbytes = aligned_nnz * mask.vec_length * lane_bits(lhs_bits) // 8
    out = np.empty(max(nbytes, 4), dtype=np.uint8)
    _lib.check(_lib.lib().mcPackSpmmValuesEx(mask.m_vec, mask.vec_length, lhs_bits, rhs_bits, _ptr(ro),
                                             _ptr(pairs), aligned_nnz, _ptr(v) if v.size else None, _ptr(out), layout),
               "mcPackSpmmValuesEx")
    return out[:nbytes]


def sorted_row_swizzle(mask: VectorSparse) -> np.ndarray:
    ro = np.ascontiguousarray(mask.row_offsets, dtype=np.int32)
    out = np.empty(max(mask.m_vec, 1), dtype=np.int32)
    _lib.check(_lib.lib().mcSortedRowSwizzle(mask.m_vec, _ptr(ro), _ptr(out)), "mcSortedRowSwizzle")
    return out[:mask.m_vec]


def identity_row_swizzle(m_vec: int) -> np.ndarray:
    return np.arange(m_vec, dtype=np.int32)


@dataclass
class SpmmLhs:
    """Host arrays of a sparse lhs in the SpMM device layout."""

    mask: VectorSparse
    lhs_bits: int
    rhs_bits: int
    row_indices: np.ndarray
    row_offsets: np.ndarray  # aligned [start, end) pairs
    col_indices: np.ndarray  # aligned, -1 padded (8-shuffled for 4-bit operands)
    values: np.ndarray       # uint8 device value layout
    aligned_nnz: int


def prepare_spmm(mask: VectorSparse, values: np.ndarray, lhs_bits: int, rhs_bits: int,
                 sort_rows: bool = True, layout: int = VALUES_PACKED) -> SpmmLhs:
    chunk = spmm_chunk(lhs_bits, rhs_bits)
    pairs, n = align_row_offsets(mask, chunk)
    cols = pad_column_indices(mask, pairs, n, shuffle8=(chunk == 32 and layout == VALUES_PACKED))
    vals = pack_spmm_values(mask, pairs, n, values, lhs_bits, rhs_bits, layout)
    ri = sorted_row_swizzle(mask) if sort_rows else identity_row_swizzle(mask.m_vec)
    return SpmmLhs(mask, lhs_bits, rhs_bits, ri, pairs, cols, vals, n)


@dataclass
class SddmmMask:
    """Host arrays of an SDDMM output mask in the aligned layout."""

    mask: VectorSparse
    alignment: int
    row_indices: np.ndarray
    row_offsets: np.ndarray
    col_indices: np.ndarray
    aligned_nnz: int


def prepare_sddmm(mask: VectorSparse, alignment: int = 8, sort_rows: bool = True) -> SddmmMask:
    if alignment % 8:
        raise ValueError("SDDMM alignment must be a multiple of 8")
    pairs, n = align_row_offsets(mask, alignment)
    cols = pad_column_indices(mask, pairs, n, shuffle8=False)
    ri = sorted_row_swizzle(mask) if sort_rows else identity_row_swizzle(mask.m_vec)
    return SddmmMask(mask, alignment, ri, pairs, cols, n)
