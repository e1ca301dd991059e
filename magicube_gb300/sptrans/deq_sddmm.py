"""sptrans.deq_sddmm: quantized SDDMM with half output half(acc / scale),
vector-major over the aligned slots (reference: deq_sddmm.cpp:95-99,
deq_sddmm_kernel.cu:565-700)."""
from __future__ import annotations

import ctypes

import torch

from .. import _lib
from ._common import as_int32_device, check, stream_handle


def _sddmm(row_indices, row_offsets, column_indices, lhs, rhs, vec_length, bits, scale, batched):
    if bits not in (4, 8):
        raise ValueError("bits must be 4 or 8")
    ri = as_int32_device(row_indices, "row_indices")
    ro = as_int32_device(row_offsets, "row_offsets")
    ci = as_int32_device(column_indices, "column_indices")
    lhs = as_int32_device(lhs, "lhs_matrix")
    rhs = as_int32_device(rhs, "rhs_matrix")
    k = lhs.size(-1) * (32 // bits)
    m, n = lhs.size(-2), rhs.size(-2)
    batch = rhs.size(-3) if batched else 1
    nnz = ci.numel()
    m_vec = ro.numel() // 2
    if m != m_vec * vec_length:
        raise ValueError("lhs rows must equal m_vec * vec_length")
    shape = (batch, nnz * vec_length) if batched else (nnz * vec_length,)
    out = torch.empty(shape, dtype=torch.float16, device=lhs.device)
    d = _lib.McSddmmDesc(
        m_vec=m_vec, vec_length=vec_length, n=n, k=k, lhs_bits=bits, rhs_bits=bits, is_signed=1, out_half=1,
        out_vecmajor=1, scale=float(scale), batch=batch, row_split=0,
        row_indices=ri.data_ptr(), row_offsets=ro.data_ptr(), column_indices=ci.data_ptr(),
        lhs=lhs.data_ptr(), lhs_stride=m * k * bits // 8, rhs=rhs.data_ptr(), rhs_stride=n * k * bits // 8,
        out=out.data_ptr(), out_stride=nnz * vec_length)
    check(_lib.lib().mcSddmm(ctypes.byref(d), stream_handle()), "mcSddmm")
    return out


def sddmm_4b(row_indices, row_offsets, column_indices, lhs_matrix, rhs_matrix, vec_length, bits, scale):
    return _sddmm(row_indices, row_offsets, column_indices, lhs_matrix, rhs_matrix, vec_length, bits, scale, False)


def sddmm_8b(row_indices, row_offsets, column_indices, lhs_matrix, rhs_matrix, vec_length, bits, scale):
    return _sddmm(row_indices, row_offsets, column_indices, lhs_matrix, rhs_matrix, vec_length, bits, scale, False)


def bsddmm_4b(row_indices, row_offsets, column_indices, lhs_matrix, rhs_matrix, vec_length, bits, scale):
    return _sddmm(row_indices, row_offsets, column_indices, lhs_matrix, rhs_matrix, vec_length, bits, scale, True)


def bsddmm_8b(row_indices, row_offsets, column_indices, lhs_matrix, rhs_matrix, vec_length, bits, scale):
    return _sddmm(row_indices, row_offsets, column_indices, lhs_matrix, rhs_matrix, vec_length, bits, scale, True)
