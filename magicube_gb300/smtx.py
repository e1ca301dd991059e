"""Reader / writer of the reference's ``.smtx`` sparse-matrix text format.

Layout (as parsed by SpMM/SpMM/spmm_benchmark.cpp:126-175 and
SDDMM/SDDMM/sddmm_benchmark.cpp:73-96):

    line 1: ``m_vec, ncols, nnz_vec``
    line 2: the m_vec + 1 CSR row offsets, space separated
    line 3: the nnz_vec column indices, space separated

For a vector-sparse matrix the rows of the file are vector-rows (the
vector length V is a command-line argument of the reference programs).
The DLMC benchmark matrices use this format, so a DLMC checkout can be read
directly.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from .formats import VectorSparse


def write(path: str | Path, mask: VectorSparse) -> None:
    ro = np.asarray(mask.row_offsets, dtype=np.int64)
    ci = np.asarray(mask.col_indices, dtype=np.int64)
    with open(path, "w") as f:
        f.write(f"{mask.m_vec}, {mask.ncols}, {int(ro[-1])}\n")
        f.write(" ".join(map(str, ro.tolist())) + "\n")
        f.write(" ".join(map(str, ci.tolist())) + "\n")


def read(path: str | Path, vec_length: int) -> VectorSparse:
    text = Path(path).read_text()
    head, rest = text.split("\n", 1)
    m_vec, ncols, nnz = (int(x) for x in head.split(","))
    if m_vec < 0 or ncols <= 0 or nnz < 0:
        raise ValueError(f"{path}: header out of range (rows >= 0, columns > 0, nonzeros >= 0)")
    toks = rest.split()
    if len(toks) < m_vec + 1 + nnz:
        raise ValueError(f"{path}: expected {m_vec + 1} offsets and {nnz} column indices")
    ro = np.asarray(toks[:m_vec + 1], dtype=np.int64).astype(np.int32)
    ci = np.asarray(toks[m_vec + 1:m_vec + 1 + nnz], dtype=np.int64).astype(np.int32)
    if ro[0] != 0 or ro[-1] != nnz or np.any(np.diff(ro) < 0):
        raise ValueError(f"{path}: malformed row offsets")
    if nnz and (ci.min() < 0 or ci.max() >= ncols):
        raise ValueError(f"{path}: column index out of range")
    return VectorSparse(m_vec, vec_length, ncols, ro, ci)
