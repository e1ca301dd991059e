"""Attention masks in the layout the sparse-attention path expects.

static_random_mask_aligned mirrors the reference's mask generator
(end2end_eval/sparse_transformer_magicube/verify/static_mask.py:29-76):
a random vector-sparse pattern over (m = seq_len / V) x n with density
1 - sparsity, row offsets aligned to mma_k_dim as [start, end) pairs, column
indices padded with -1 (plain and 8-shuffled), row order by ascending length.
It takes a seed (the reference draws unseeded).  banded_random_mask builds
the band-plus-random masks of the batched attention configuration.
"""
from __future__ import annotations

import numpy as np
import torch

from . import formats, synth
from .formats import VectorSparse


def _to_attention_layout(mask: VectorSparse, mma_k_dim: int, device):
    pairs, n = formats.align_row_offsets(mask, mma_k_dim)
    cols = formats.pad_column_indices(mask, pairs, n, shuffle8=False)
    cols_sh = formats.pad_column_indices(mask, pairs, n, shuffle8=True) if n % 8 == 0 else cols.copy()
    row_indices = np.argsort(mask.row_lengths(), kind="stable").astype(np.int32)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)  # noqa: E731
    return t(cols), t(cols_sh), t(pairs), t(row_indices), n


def static_random_mask_aligned(m: int, n: int, sparsity: float, mma_k_dim: int, seed: int = 0,
                               vec_length: int = 1, device="cuda"):
    """Returns (column_indices, column_indices_shuffle, row_offsets, row_indices, aligned_num_item)."""
    rng = np.random.default_rng(seed)
    density = 1.0 - sparsity
    lengths = rng.binomial(n, density, size=m)
    mask = synth.lengths_mask(lengths, n, vec_length, seed=seed + 1)
    return _to_attention_layout(mask, mma_k_dim, device)


def banded_random_mask(seq_len: int, vec_length: int, band: int, sparsity: float, mma_k_dim: int, seed: int = 0,
                       device="cuda"):
    """Band of `band` columns around the diagonal plus uniformly random column
    vectors, `sparsity` overall, in the attention layout."""
    mask = synth.band_random_mask(seq_len, vec_length, band, sparsity, seed=seed)
    return _to_attention_layout(mask, mma_k_dim, device), mask
