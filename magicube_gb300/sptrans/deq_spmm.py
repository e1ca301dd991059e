"""sptrans.deq_spmm: batched quantized SpMM of softmax-layout values with a
dense rhs, half output half(acc / scale) (reference: deq_spmm.cpp:142-146,
deq_spmm_kernel.cu:1057-1361)."""
from __future__ import annotations

import ctypes

import torch

from .. import _lib
from ._common import as_int32_device, check, stream_handle


def _bspmm(row_indices, row_offsets, column_indices, values, rhs, vec_length, bits_lhs, bits_rhs, scale, want):
    if (bits_lhs, bits_rhs) != want:
        raise ValueError(f"this op computes L{want[0]}-R{want[1]}, got L{bits_lhs}-R{bits_rhs}")
    ri = as_int32_device(row_indices, "row_indices")
    ro = as_int32_device(row_offsets, "row_offsets")
    ci = as_int32_device(column_indices, "column_indices")
    values = as_int32_device(values, "values")
    rhs = as_int32_device(rhs, "rhs_matrix")
    m_vec = ro.numel() // 2
    m = m_vec * vec_length
    n = rhs.size(-1) * (32 // bits_rhs)
    k = rhs.size(-2)
    batch = rhs.size(-3) if rhs.dim() >= 3 else 1
    out = torch.empty((batch, m, n), dtype=torch.float16, device=rhs.device)
    vstride = values.numel() // batch * 4 if values.dim() >= 2 else 0
    d = _lib.McSpmmDesc(
        m_vec=m_vec, vec_length=vec_length, n=n, k=k, lhs_bits=bits_lhs, rhs_bits=bits_rhs, is_signed=1, out_half=1,
        scale=float(scale), batch=batch, row_indices=ri.data_ptr(), row_offsets=ro.data_ptr(),
        column_indices=ci.data_ptr(), values=values.data_ptr(), values_stride=vstride,
        rhs=rhs.data_ptr(), rhs_stride=k * n * bits_rhs // 8, out=out.data_ptr(), out_stride=m * n,
        value_layout=_lib.VALUES_SOFTMAX)
    check(_lib.lib().mcSpmm(ctypes.byref(d), stream_handle()), "mcSpmm")
    return out


def bspmm_4b(row_indices, row_offsets, column_indices, values, rhs_matrix, vec_length, bits_lhs, bits_rhs, scale):
    return _bspmm(row_indices, row_offsets, column_indices, values, rhs_matrix, vec_length, bits_lhs, bits_rhs,
                  scale, (4, 4))


def bspmm_8b(row_indices, row_offsets, column_indices, values, rhs_matrix, vec_length, bits_lhs, bits_rhs, scale):
    return _bspmm(row_indices, row_offsets, column_indices, values, rhs_matrix, vec_length, bits_lhs, bits_rhs,
                  scale, (8, 8))


def bspmm_8b4b(row_indices, row_offsets, column_indices, values, rhs_matrix, vec_length, bits_lhs, bits_rhs, scale):
    return _bspmm(row_indices, row_offsets, column_indices, values, rhs_matrix, vec_length, bits_lhs, bits_rhs,
                  scale, (8, 4))


def bspmm_16b8b(row_indices, row_offsets, column_indices, values, rhs_matrix, vec_length, bits_lhs, bits_rhs,
                scale):
    return _bspmm(row_indices, row_offsets, column_indices, values, rhs_matrix, vec_length, bits_lhs, bits_rhs,
                  scale, (16, 8))
