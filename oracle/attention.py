"""CPU oracle of the quantized sparse-attention steps.

TEST INFRASTRUCTURE ONLY (the checker of tests/, smoke and the benchmark's
CPU leg).  numpy restatements of:
  * quantization_kernel.cu:14-131 (sparse_transformer_magicube/src/cuda):
    q = trunc(clamp(float32(x) * scale)), packed little-endian;
  * q_softmax_kernel.cu:181-271: per vector-row and lane, p = exp(x*s - max)
    / sum over the row's nonzeros, q = trunc(clamp(p * scale)), written in
    the softmax value layout ([v][16] per 16 slots for 8 bits, lo/hi byte
    halves per lane for 16 bits, nibbles [v][32] per 32 slots for 4 bits);
  * the library's row-max requantization (q = round(127 exp(x - max)) and a
    divisor 127 * sum * scale per row and lane), which has no reference
    counterpart;
  * the unquantized sparse attention in float64 (the accuracy reference of
    the quantized pipeline): softmax(Q K^T * s) restricted to the vector mask,
    times V.
"""
from __future__ import annotations

import numpy as np


def quantize(x: np.ndarray, bits: int, scale: float) -> np.ndarray:
    """float16 array (last dim n) -> packed uint8 bytes, flattened."""
    lo, hi = (-128.0, 127.0) if bits == 8 else (-8.0, 7.0)
    f = x.astype(np.float32) * np.float32(scale)
    q = np.trunc(np.clip(f, lo, hi)).astype(np.int64).ravel()
    if bits == 8:
        return (q & 0xFF).astype(np.uint8)
    q = (q & 0xF).astype(np.uint8)
    return (q[0::2] | (q[1::2] << 4)).astype(np.uint8)


def softmax_quant(scores: np.ndarray, pairs: np.ndarray, row_indices: np.ndarray, V: int, bits: int,
                  scaling: float, scale: float, out_bytes: int) -> tuple[np.ndarray, np.ndarray]:
    """Returns (packed bytes in the softmax layout, the unquantized p*scale as
    float64 per (slot, lane) for tolerance checks).  scores: float16
    [aligned_nnz * V] vector-major."""
    lo, hi = {4: (-8.0, 7.0), 8: (-128.0, 127.0), 16: (-32768.0, 32767.0)}[bits]
    out = np.zeros(out_bytes, dtype=np.uint8)
    exact = np.zeros(scores.size, dtype=np.float64)
    for r in row_indices:
        s, e = int(pairs[2 * r]), int(pairs[2 * r + 1])
        n = e - s
        if n == 0:
            continue
        x = scores[s * V:e * V].reshape(n, V).astype(np.float32) * np.float32(scaling)
        m = x.max(axis=0)
        ex = np.exp(x - m)
        p = ex / ex.sum(axis=0, dtype=np.float32) * np.float32(scale)
        exact[s * V:e * V] = p.ravel()
        q = np.trunc(np.clip(p, lo, hi)).astype(np.int64)
        base = s * V * bits // 8
        for j in range(n):
            for v in range(V):
                val = int(q[j, v])
                if bits == 8:
                    out[base + (j // 16) * V * 16 + v * 16 + j % 16] = val & 0xFF
                elif bits == 16:
                    o = base + (j // 16) * V * 32 + v * 32 + j % 16
                    out[o] = val & 0xFF
                    out[o + 16] = (val >> 8) & 0xFF
                else:
                    o = base + (j // 32) * V * 16 + v * 16 + (j % 32) // 2
                    out[o] |= (val & 0xF) << (4 * (j % 2))
    return out, exact


def softmax_rowmax(scores: np.ndarray, pairs: np.ndarray, row_indices: np.ndarray, V: int, scaling: float,
                   scale: float, out_bytes: int, m_vec: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """The library's row-max requantization (no reference counterpart): per
    vector-row and lane, x = float32(score) * scaling, q = round(127 exp(x -
    max)) in the 8-bit softmax layout, divisor 127 * sum(exp) * scale.
    Returns (packed bytes, divisors [m_vec * V], the unrounded 127 exp(x - max)
    per (slot, lane) for tolerance checks)."""
    out = np.zeros(out_bytes, dtype=np.uint8)
    div = np.zeros(m_vec * V, dtype=np.float32)
    exact = np.zeros(scores.size, dtype=np.float64)
    for r in row_indices:
        s, e = int(pairs[2 * r]), int(pairs[2 * r + 1])
        n = e - s
        if n == 0:
            continue
        x = scores[s * V:e * V].reshape(n, V).astype(np.float32) * np.float32(scaling)
        ex = np.exp(x - x.max(axis=0))
        div[r * V:(r + 1) * V] = np.float32(127.0) * ex.sum(axis=0, dtype=np.float32) * np.float32(scale)
        p = np.float32(127.0) * ex
        exact[s * V:e * V] = p.ravel()
        q = np.rint(p).astype(np.int64)
        base = s * V
        for j in range(n):
            for v in range(V):
                out[base + (j // 16) * V * 16 + v * 16 + j % 16] = int(q[j, v]) & 0xFF
    return out, div, exact


def dense_mask(pairs: np.ndarray, cols: np.ndarray, m_vec: int, V: int, ncols: int) -> np.ndarray:
    """Boolean [m_vec*V, ncols] mask of a vector-sparse pattern."""
    mk = np.zeros((m_vec * V, ncols), dtype=bool)
    for i in range(m_vec):
        c = cols[int(pairs[2 * i]):int(pairs[2 * i + 1])]
        mk[i * V:(i + 1) * V, c] = True
    return mk


def sparse_attention_fp64(q: np.ndarray, k: np.ndarray, v: np.ndarray, mask: np.ndarray,
                          scaling: float) -> np.ndarray:
    """[H, L, d] float inputs, [L, L] bool mask -> [H, L, d] float64 output."""
    q, k, v = (a.astype(np.float64) for a in (q, k, v))
    s = np.einsum("hld,hmd->hlm", q, k) * scaling
    s = np.where(mask[None], s, -np.inf)
    mx = s.max(axis=-1, keepdims=True)
    mx = np.where(np.isfinite(mx), mx, 0.0)
    p = np.exp(s - mx)
    den = p.sum(axis=-1, keepdims=True)
    p = np.where(den > 0, p / np.where(den > 0, den, 1.0), 0.0)
    return np.einsum("hlm,hmd->hld", p, v)


def sparse_attention_fp64_rows(q: np.ndarray, k: np.ndarray, v: np.ndarray, row_offsets: np.ndarray,
                               col_indices: np.ndarray, V: int, scaling: float) -> np.ndarray:
    """The same unquantized attention as sparse_attention_fp64, computed
    vector-row by vector-row on the gathered K and V rows of the row's
    columns (no dense L x L scores).  q, k, v: [H, L, d]; row_offsets /
    col_indices: the plain vector CSR (m_vec + 1 offsets).  Rows without
    nonzeros give 0."""
    q, k, v = (np.asarray(a, dtype=np.float64) for a in (q, k, v))
    H, L, d = q.shape
    out = np.zeros((H, L, d), dtype=np.float64)
    m_vec = len(row_offsets) - 1
    for i in range(m_vec):
        c = col_indices[int(row_offsets[i]):int(row_offsets[i + 1])]
        if c.size == 0:
            continue
        s = np.matmul(q[:, i * V:(i + 1) * V, :], k[:, c, :].transpose(0, 2, 1)) * scaling  # [H, V, n]
        s -= s.max(axis=-1, keepdims=True)
        p = np.exp(s)
        p /= p.sum(axis=-1, keepdims=True)
        out[:, i * V:(i + 1) * V, :] = np.matmul(p, v[:, c, :])
    return out
