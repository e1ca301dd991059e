"""The vector-sparse packer on the GPU.

Device-resident counterpart of :mod:`magicube_gb300.formats` (whose host
routines restate the reference's serial packer, SpMM/SpMM/spmm_benchmark.cpp
:177-377): plain CSR of vectors already on the device (``row_offsets`` int32
[m_vec + 1], ``col_indices`` int32 [nnz_vec], values uint8 [nnz_vec * V *
bits / 8]) becomes the aligned operand the SpMM / SDDMM kernels read, with the
library's ``mcDevice*`` entry points, on torch's current stream.  The arrays
are byte-identical to the host packer's.

``prepare_spmm`` / ``prepare_sddmm`` make one ``mcDevicePack`` call (fused
align scan, per-row column and value pass, row sort).  With ``sync=False`` no
host round trip happens: buffers are sized by the upper bound ``nnz_vec +
m_vec * (alignment - 1)`` and the exact aligned count stays on the device; the
kernels read only the slots the pairs name, so such an operand computes the
same results.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .formats import VALUES_PACKED, VALUES_SLOT_MAJOR, VALUES_SOFTMAX, lane_bits, spmm_chunk
from .ops import DeviceSddmmMask, DeviceSpmmLhs


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _i32(t: torch.Tensor, what: str) -> torch.Tensor:
    if t.dtype != torch.int32 or not t.is_cuda:
        raise TypeError(f"{what} must be an int32 CUDA tensor")
    return t.contiguous()


def _ptr(t: torch.Tensor | None) -> int | None:
    return t.data_ptr() if t is not None and t.numel() else None


def align_row_offsets(row_offsets: torch.Tensor, alignment: int) -> tuple[torch.Tensor, torch.Tensor]:
    """Aligned [start, end) pairs and the aligned count (a one-element device
    tensor; -1 for non-monotone offsets)."""
    ro = _i32(row_offsets, "row_offsets")
    m_vec = ro.numel() - 1
    pairs = torch.empty(max(2 * m_vec, 2), dtype=torch.int32, device=ro.device)
    n = torch.empty(1, dtype=torch.int32, device=ro.device)
    _lib.check(_lib.lib().mcDeviceAlignRowOffsets(m_vec, ro.data_ptr(), alignment, pairs.data_ptr(), n.data_ptr(),
                                                  _stream()), "mcDeviceAlignRowOffsets")
    return pairs[:2 * m_vec], n


def pad_column_indices(row_offsets: torch.Tensor, col_indices: torch.Tensor, pairs: torch.Tensor,
                       aligned_nnz: torch.Tensor, shuffle8: bool, capacity: int,
                       status: torch.Tensor | None = None) -> torch.Tensor:
    ro = _i32(row_offsets, "row_offsets")
    ci = _i32(col_indices, "col_indices")
    out = torch.empty(max(capacity, 1), dtype=torch.int32, device=ro.device)
    _lib.check(_lib.lib().mcDevicePadColumnIndices(ro.numel() - 1, ro.data_ptr(), _ptr(ci), _ptr(pairs),
                                                   aligned_nnz.data_ptr(), int(shuffle8), out.data_ptr(), capacity,
                                                   _ptr(status), _stream()), "mcDevicePadColumnIndices")
    return out[:capacity]


def pack_spmm_values(row_offsets: torch.Tensor, pairs: torch.Tensor, aligned_nnz: torch.Tensor,
                     values: torch.Tensor, vec_length: int, lhs_bits: int, rhs_bits: int, capacity_slots: int,
                     layout: int = VALUES_PACKED, status: torch.Tensor | None = None) -> torch.Tensor:
    ro = _i32(row_offsets, "row_offsets")
    if values.dtype != torch.uint8 or not values.is_cuda:
        raise TypeError("values must be a uint8 CUDA tensor")
    v = values.contiguous()
    nbytes = capacity_slots * vec_length * lane_bits(lhs_bits) // 8
    out = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=ro.device)
    _lib.check(_lib.lib().mcDevicePackSpmmValues(ro.numel() - 1, vec_length, lhs_bits, rhs_bits, ro.data_ptr(),
                                                 _ptr(pairs), aligned_nnz.data_ptr(), _ptr(v), out.data_ptr(), nbytes,
                                                 layout, _ptr(status), _stream()), "mcDevicePackSpmmValues")
    return out[:nbytes]


def sorted_row_swizzle(row_offsets: torch.Tensor) -> torch.Tensor:
    """Longest-first order; equal lengths in ascending row index."""
    ro = _i32(row_offsets, "row_offsets")
    m_vec = ro.numel() - 1
    out = torch.empty(max(m_vec, 1), dtype=torch.int32, device=ro.device)
    _lib.check(_lib.lib().mcDeviceSortedRowSwizzle(m_vec, ro.data_ptr(), out.data_ptr(), _stream()),
               "mcDeviceSortedRowSwizzle")
    return out[:m_vec]


class PackError(RuntimeError):
    """The device packer found inconsistent input (non-monotone offsets)."""


def _finish(n: torch.Tensor, status: torch.Tensor, sync: bool, bound: int) -> int:
    if not sync:
        return bound
    got, st = int(n.item()), int(status.item())
    if got < 0 or st:
        raise PackError("row_offsets are not monotone (or the aligned count overflows int)")
    return got


def _pack(ro: torch.Tensor, ci: torch.Tensor, values: torch.Tensor | None, vec_length: int, lhs_bits: int,
          rhs_bits: int, alignment: int, shuffle8: bool, layout: int, sort_rows: bool, bound: int):
    """One mcDevicePack call; returns (pairs, aligned count, cols, values, row order, status)."""
    m_vec = ro.numel() - 1
    dev = ro.device
    pairs = torch.empty(max(2 * m_vec, 2), dtype=torch.int32, device=dev)
    n = torch.empty(1, dtype=torch.int32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    cols = torch.empty(max(bound, 1), dtype=torch.int32, device=dev)
    nbytes = bound * vec_length * lane_bits(lhs_bits) // 8
    vals = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=dev) if lhs_bits else None
    ri = (torch.empty(max(m_vec, 1), dtype=torch.int32, device=dev) if sort_rows
          else torch.arange(max(m_vec, 1), dtype=torch.int32, device=dev))
    if values is not None and (values.dtype != torch.uint8 or not values.is_cuda):
        raise TypeError("values must be a uint8 CUDA tensor")
    v = values.contiguous() if values is not None else None
    d = _lib.McDevicePackDesc(
        m_vec=m_vec, vec_length=vec_length, lhs_bits=lhs_bits, rhs_bits=rhs_bits, alignment=alignment,
        shuffle8=int(shuffle8), value_layout=layout, sort_rows=int(sort_rows), row_offsets=ro.data_ptr(),
        col_indices=_ptr(ci), values=_ptr(v), aligned_pairs=pairs.data_ptr(), aligned_nnz=n.data_ptr(),
        out_cols=cols.data_ptr(), cols_capacity=bound, out_values=vals.data_ptr() if vals is not None else None,
        values_capacity_bytes=nbytes, row_indices=ri.data_ptr(), status=status.data_ptr())
    _lib.check(_lib.lib().mcDevicePack(ctypes.byref(d), _stream()), "mcDevicePack")
    return pairs[:2 * m_vec], n, cols[:bound], (vals[:nbytes] if vals is not None else None), ri[:m_vec], status


def prepare_spmm(row_offsets: torch.Tensor, col_indices: torch.Tensor, values: torch.Tensor, vec_length: int,
                 ncols: int, lhs_bits: int, rhs_bits: int, *, sort_rows: bool = True, layout: int = VALUES_PACKED,
                 sync: bool = True) -> DeviceSpmmLhs:
    """A device SpMM operand from device CSR (formats.prepare_spmm on the GPU)."""
    ro = _i32(row_offsets, "row_offsets")
    ci = _i32(col_indices, "col_indices")
    m_vec = ro.numel() - 1
    chunk = spmm_chunk(lhs_bits, rhs_bits)
    bound = (int(ci.numel()) + m_vec * (chunk - 1)) // chunk * chunk
    pairs, n, cols, vals, ri, status = _pack(ro, ci, values, vec_length, lhs_bits, rhs_bits, chunk,
                                             chunk == 32 and layout == VALUES_PACKED, layout, sort_rows, bound)
    aligned = _finish(n, status, sync, bound)
    if sync:
        cols, vals = cols[:aligned], vals[:aligned * vec_length * lane_bits(lhs_bits) // 8]
    if cols.numel() == 0:
        cols = torch.full((1,), -1, dtype=torch.int32, device=ro.device)
    if vals.numel() == 0:
        vals = torch.zeros(16, dtype=torch.uint8, device=ro.device)
    return DeviceSpmmLhs(m_vec, vec_length, ncols, lhs_bits, rhs_bits, ri, pairs, cols, vals)


def prepare_sddmm(row_offsets: torch.Tensor, col_indices: torch.Tensor, vec_length: int, ncols: int, *,
                  alignment: int = 8, sort_rows: bool = True, sync: bool = True) -> DeviceSddmmMask:
    """A device SDDMM mask from device CSR (formats.prepare_sddmm on the GPU)."""
    if alignment % 8:
        raise ValueError("SDDMM alignment must be a multiple of 8")
    ro = _i32(row_offsets, "row_offsets")
    ci = _i32(col_indices, "col_indices")
    m_vec = ro.numel() - 1
    bound = (int(ci.numel()) + m_vec * (alignment - 1)) // alignment * alignment
    pairs, n, cols, _, ri, status = _pack(ro, ci, None, vec_length, 0, 0, alignment, False, VALUES_PACKED,
                                          sort_rows, bound)
    aligned = _finish(n, status, sync, bound)
    if sync:
        cols = cols[:aligned]
    if cols.numel() == 0:
        cols = torch.full((1,), -1, dtype=torch.int32, device=ro.device)
    return DeviceSddmmMask(m_vec, vec_length, ncols, aligned, ri, pairs, cols)


__all__ = ["align_row_offsets", "pad_column_indices", "pack_spmm_values", "sorted_row_swizzle", "prepare_spmm",
           "prepare_sddmm", "PackError", "VALUES_PACKED", "VALUES_SOFTMAX", "VALUES_SLOT_MAJOR"]
