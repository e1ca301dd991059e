"""Helpers for the golden fixtures in tests/golden (generated from the reference
by tests/golden/make_golden.py)."""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name: str) -> dict:
    with np.load(GOLDEN / name) as z:
        return {k: z[k] for k in z.files}


def names(prefix: str) -> list[str]:
    return sorted(p.name for p in GOLDEN.glob(prefix + "*.npz"))


def unpack_spmm_values(dev: np.ndarray, pairs: np.ndarray, csr_offsets: np.ndarray, V: int, pa: int,
                       pb: int) -> np.ndarray:
    """Invert the SpMM device value layout back to per-vector packed values
    (V lanes of pa bits each, lane v at bit v*pa; 12-bit values in 16-bit
    lanes)."""
    mma_k = 32 if (pa == 4 or pb == 4) else 16
    plane_bits = 4 if mma_k == 32 else 8
    pa = 16 if pa == 12 else pa  # 12-bit values: 16-bit lanes and layouts (top bits clear)
    planes = pa // plane_bits
    plane_bytes = V * mma_k * plane_bits // 8
    chunk_bytes = plane_bytes * planes
    m_vec = len(csr_offsets) - 1
    nnz = int(csr_offsets[-1])
    vals = np.zeros(nnz * V, dtype=np.uint32)

    def elem(buf_off: int, idx: int) -> int:
        bit = idx * plane_bits
        byte = int(dev[buf_off + bit // 8])
        return (byte >> (bit % 8)) & ((1 << plane_bits) - 1)

    for i in range(m_vec):
        start = int(pairs[2 * i])
        for j in range(int(csr_offsets[i]), int(csr_offsets[i + 1])):
            slot = start + (j - int(csr_offsets[i]))
            base = (slot // mma_k) * chunk_bytes
            jj = slot % mma_k
            for v in range(V):
                x = 0
                for p in range(planes):
                    x |= elem(base + p * plane_bytes, v * mma_k + jj) << (p * plane_bits)
                vals[j * V + v] = x
    # pack lanes little-endian
    out = np.zeros(nnz * V * pa // 8, dtype=np.uint8)
    for e, x in enumerate(vals.tolist()):
        bit = e * pa
        if pa == 4:
            out[bit // 8] |= (x & 0xF) << (bit % 8)
        elif pa == 8:
            out[e] = x & 0xFF
        else:
            out[2 * e] = x & 0xFF
            out[2 * e + 1] = (x >> 8) & 0xFF
    return out


def lane_bits(pa: int) -> int:
    """Bits per stored lane (12-bit values live in 16-bit containers)."""
    return 16 if pa == 12 else pa
