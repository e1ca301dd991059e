"""Seeded synthetic vector-sparse inputs.

The reference measures on the DLMC pruned-weight matrices (``.smtx`` files),
which are not available; these generators produce masks and operands with the
shapes, sparsities and value distributions of the benchmark configurations:
uniform column placement per vector-row, per-row lengths drawn from a normal
distribution (magnitude-pruning-like), banded-plus-random attention masks, and
uniformly random packed integers (every bit pattern equally likely, i.e.
int8 uniform in [-128, 127], int4 uniform in [-8, 7], int16 uniform).
"""
from __future__ import annotations

import numpy as np

from .formats import VectorSparse


def _from_lengths(lengths: np.ndarray, ncols: int, V: int, rng: np.random.Generator) -> VectorSparse:
    lengths = np.clip(np.asarray(lengths, dtype=np.int64), 0, ncols)
    offsets = np.zeros(len(lengths) + 1, dtype=np.int64)
    np.cumsum(lengths, out=offsets[1:])
    cols = np.empty(int(offsets[-1]), dtype=np.int32)
    for i, n in enumerate(lengths):
        if n:
            c = rng.choice(ncols, size=int(n), replace=False)
            c.sort()
            cols[offsets[i]:offsets[i] + n] = c
    return VectorSparse(len(lengths), V, ncols, offsets.astype(np.int32), cols)


def uniform_mask(m_vec: int, ncols: int, V: int, sparsity: float, seed: int = 42) -> VectorSparse:
    """Every vector-row holds floor((1 - sparsity) * ncols) distinct uniformly placed columns."""
    rng = np.random.default_rng(seed)
    n = int((1.0 - sparsity) * ncols)
    return _from_lengths(np.full(m_vec, n), ncols, V, rng)


def normal_mask(m_vec: int, ncols: int, V: int, sparsity: float, cv: float = 0.3, seed: int = 42) -> VectorSparse:
    """Row lengths ~ Normal(mu, cv * mu), mu = (1 - sparsity) * ncols, clipped to [0, ncols]."""
    rng = np.random.default_rng(seed)
    mu = (1.0 - sparsity) * ncols
    lengths = np.rint(rng.normal(mu, cv * mu, size=m_vec)).astype(np.int64)
    return _from_lengths(lengths, ncols, V, rng)


def lengths_mask(lengths, ncols: int, V: int, seed: int = 42) -> VectorSparse:
    """Mask with the given per-vector-row lengths (ragged test cases)."""
    return _from_lengths(np.asarray(lengths), ncols, V, np.random.default_rng(seed))


def band_random_mask(seq_len: int, V: int, band: int, sparsity: float, seed: int = 42) -> VectorSparse:
    """Attention mask over seq_len x seq_len: a `band`-wide diagonal band of
    vectors plus uniformly random extra vectors, `sparsity` overall."""
    rng = np.random.default_rng(seed)
    m_vec = seq_len // V
    target = max(1, int(round((1.0 - sparsity) * seq_len)))
    offsets = [0]
    cols_all = []
    for i in range(m_vec):
        center = i * V + V // 2
        lo = max(0, center - band // 2)
        hi = min(seq_len, lo + band)
        lo = max(0, hi - band)
        band_cols = np.arange(lo, hi)
        extra = max(0, target - band_cols.size)
        if extra:
            pool = np.setdiff1d(np.arange(seq_len), band_cols, assume_unique=True)
            extra_cols = rng.choice(pool, size=min(extra, pool.size), replace=False)
            c = np.concatenate([band_cols, extra_cols])
        else:
            c = band_cols[:target]
        c = np.sort(c).astype(np.int32)
        cols_all.append(c)
        offsets.append(offsets[-1] + c.size)
    cols = np.concatenate(cols_all) if cols_all else np.zeros(0, np.int32)
    return VectorSparse(m_vec, V, seq_len, np.asarray(offsets, dtype=np.int32), cols.astype(np.int32))


def random_bytes(nbytes: int, seed: int) -> np.ndarray:
    """Uniformly random packed integer payload."""
    return np.random.default_rng(seed).integers(0, 256, size=nbytes, dtype=np.uint8)
