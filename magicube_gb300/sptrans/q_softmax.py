"""sptrans.q_softmax: row softmax of the SDDMM scores with requantization into
the SpMM value layout (reference: q_softmax.cpp:50-52,
q_softmax_kernel.cu:181-271,363-532)."""
from __future__ import annotations

import ctypes

import torch

from .. import _lib
from ._common import as_int32_device, check, stream_handle


def _softmax(row_indices, row_offsets, values, sqrt_dk, scale, vec_length, batch_size, bits, batched):
    if bits not in (4, 8, 16):
        raise ValueError("bits must be 4, 8 or 16")
    ri = as_int32_device(row_indices, "row_indices")
    ro = as_int32_device(row_offsets, "row_offsets")
    if values.dtype != torch.float16 or not values.is_cuda:
        raise TypeError("values must be a CUDA float16 tensor")
    values = values.contiguous()
    per = values.numel() // batch_size
    words = per * bits // 32
    out = torch.zeros((batch_size, words) if batched else (words,), dtype=torch.int32, device=values.device)
    d = _lib.McSoftmaxDesc(
        m_vec=ri.numel(), vec_length=vec_length, batch=batch_size, bits=bits, scaling=float(sqrt_dk),
        scale=float(scale), row_indices=ri.data_ptr(), row_offsets=ro.data_ptr(), scores=values.data_ptr(),
        scores_stride=per, out=out.data_ptr(), out_stride=words * 4)
    check(_lib.lib().mcQuantSoftmax(ctypes.byref(d), stream_handle()), "mcQuantSoftmax")
    return out


def q_csr_softmax(row_indices, row_offsets, values, sqrt_dk, scale, vec_length, bits):
    """Half scores [nnz*V] -> packed int32 [nnz*V*bits/32] (q_softmax.cpp:13)."""
    return _softmax(row_indices, row_offsets, values, sqrt_dk, scale, vec_length, 1, bits, False)


def q_bcsr_softmax(row_indices, row_offsets, values, sqrt_dk, scale, vec_length, batch_size, bits):
    """Half scores [B, nnz*V] -> packed int32 [B, nnz*V*bits/32] (q_softmax.cpp:37)."""
    return _softmax(row_indices, row_offsets, values, sqrt_dk, scale, vec_length, batch_size, bits, True)
