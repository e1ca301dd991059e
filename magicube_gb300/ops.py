"""Device-side calls of the C ABI on torch tensors (current torch stream).

torch provides device memory and streams only; all compute is the CUDA
library's.  Operands are raw packed integer payloads (uint8 / int32 tensors).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .formats import SddmmMask, SpmmLhs


def _stream_handle(stream: torch.cuda.Stream | None = None) -> ctypes.c_void_p:
    s = torch.cuda.current_stream() if stream is None else stream
    return ctypes.c_void_p(s.cuda_stream)


def _to_dev(a: np.ndarray, device) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


@dataclass
class DeviceSpmmLhs:
    """An SpMM sparse operand resident on the device."""

    m_vec: int
    vec_length: int
    k: int
    lhs_bits: int
    rhs_bits: int
    row_indices: torch.Tensor
    row_offsets: torch.Tensor
    col_indices: torch.Tensor
    values: torch.Tensor

    _chunks: torch.Tensor | None = field(default=None, repr=False, compare=False)
    _chunks_key: tuple | None = field(default=None, repr=False, compare=False)

    @classmethod
    def from_host(cls, h: SpmmLhs, device="cuda") -> "DeviceSpmmLhs":
        cols = h.col_indices if h.col_indices.size else np.full(1, -1, np.int32)
        vals = h.values if h.values.size else np.zeros(16, np.uint8)
        return cls(h.mask.m_vec, h.mask.vec_length, h.mask.ncols, h.lhs_bits, h.rhs_bits,
                   _to_dev(h.row_indices, device), _to_dev(h.row_offsets, device),
                   _to_dev(cols, device), _to_dev(vals, device))

    def chunk_starts(self, stream: torch.cuda.Stream | None = None) -> torch.Tensor:
        """The mask's k-chunk table for the dense-tile SpMM kernel, built on
        the device (mcSpmmChunkStarts) and cached until the mask's tensors
        are replaced or modified in place.  Synchronises once per build to
        read the status; raises MagicubeError if a vector-row's columns are
        not strictly increasing inside [0, k)."""
        key = (self.m_vec, self.k, self.row_offsets.data_ptr(), self.row_offsets._version,
               self.col_indices.data_ptr(), self.col_indices._version)
        if self._chunks is None or self._chunks_key != key:
            dev = self.row_offsets.device
            per = _lib.lib().mcSpmmChunkStartsCount(self.k)
            starts = torch.empty((max(1, self.m_vec), per), dtype=torch.int32, device=dev)
            status = torch.empty(1, dtype=torch.int32, device=dev)
            _lib.check(_lib.lib().mcSpmmChunkStarts(self.m_vec, self.k, self.row_offsets.data_ptr(),
                                                    self.col_indices.data_ptr(), starts.data_ptr(),
                                                    status.data_ptr(), _stream_handle(stream)), "mcSpmmChunkStarts")
            if int(status.item()) != 0:
                raise _lib.MagicubeError("mcSpmmChunkStarts: the mask's columns are not strictly increasing "
                                         "inside [0, k) per vector-row; the dense-tile SpMM cannot use it")
            self._chunks, self._chunks_key = starts, key
        return self._chunks


@dataclass
class DeviceSddmmMask:
    """An SDDMM output mask resident on the device."""

    m_vec: int
    vec_length: int
    n: int
    aligned_nnz: int
    row_indices: torch.Tensor
    row_offsets: torch.Tensor
    col_indices: torch.Tensor

    _tile: tuple | None = field(default=None, repr=False, compare=False)
    _tile_key: tuple | None = field(default=None, repr=False, compare=False)

    @classmethod
    def from_host(cls, h: SddmmMask, device="cuda") -> "DeviceSddmmMask":
        cols = h.col_indices if h.col_indices.size else np.full(1, -1, np.int32)
        return cls(h.mask.m_vec, h.mask.vec_length, h.mask.ncols, h.aligned_nnz,
                   _to_dev(h.row_indices, device), _to_dev(h.row_offsets, device), _to_dev(cols, device))

    def tile_mask(self, stream: torch.cuda.Stream | None = None) -> tuple[torch.Tensor, torch.Tensor]:
        """(bitmap, prefix) of the mask for the dense-tile SDDMM kernel, built
        on the device (mcSddmmTileMask) and cached until the mask's tensors
        are replaced or modified in place.  Synchronises once per build to
        read the status; raises MagicubeError if a vector-row's columns are
        not strictly increasing."""
        key = (self.m_vec, self.n, self.row_offsets.data_ptr(), self.row_offsets._version,
               self.col_indices.data_ptr(), self.col_indices._version)
        if self._tile is None or self._tile_key != key:
            dev = self.row_offsets.device
            words = _lib.lib().mcSddmmTileMaskWords(self.n)
            bitmap = torch.empty((max(1, self.m_vec), words), dtype=torch.int32, device=dev)
            prefix = torch.empty((max(1, self.m_vec), words), dtype=torch.int32, device=dev)
            status = torch.empty(1, dtype=torch.int32, device=dev)
            _lib.check(_lib.lib().mcSddmmTileMask(self.m_vec, self.n, self.row_offsets.data_ptr(),
                                                  self.col_indices.data_ptr(), bitmap.data_ptr(), prefix.data_ptr(),
                                                  status.data_ptr(), _stream_handle(stream)), "mcSddmmTileMask")
            if int(status.item()) != 0:
                raise _lib.MagicubeError("mcSddmmTileMask: the mask's columns are not strictly increasing per "
                                         "vector-row; the dense-tile SDDMM cannot use it")
            self._tile, self._tile_key = (bitmap, prefix), key
        return self._tile


def spmm(lhs: DeviceSpmmLhs, rhs: torch.Tensor, n: int, *, signed: bool = True, out: torch.Tensor | None = None,
         out_half: bool = False, scale: float = 1.0, batch: int = 1, values_stride: int = 0,
         rhs_stride: int | None = None, out_stride: int | None = None, mma_kind: int = 0, variant: int = 0,
         config: int = 0, stream: torch.cuda.Stream | None = None, value_layout: int | None = None) -> torch.Tensor:
    """C = A * B for a batch of `batch` entries (shared mask).

    rhs: packed B, k rows of n*rhs_bits/8 bytes per batch entry, contiguous.
    Strides are in bytes for values/rhs and elements for out; a zero stride
    shares the operand across the batch.  `config` picks the slice width and
    CTA size of variant KERNEL_RESIDENT (RESIDENT_*; 0 = automatic).
    `value_layout` names the layout of lhs.values when it is not the default
    (VALUES_SOFTMAX with half output, VALUES_PACKED otherwise):
    VALUES_SLOT_MAJOR values go to the dense-tile kernel."""
    M = lhs.m_vec * lhs.vec_length
    if rhs_stride is None:
        rhs_stride = lhs.k * n * lhs.rhs_bits // 8 if batch > 1 else 0
    if out_stride is None:
        out_stride = M * n if batch > 1 else 0
    if out is None:
        out = torch.empty((batch, M, n) if batch > 1 else (M, n),
                          dtype=torch.float16 if out_half else torch.int32, device=rhs.device)
    d = _lib.McSpmmDesc(
        m_vec=lhs.m_vec, vec_length=lhs.vec_length, n=n, k=lhs.k, lhs_bits=lhs.lhs_bits, rhs_bits=lhs.rhs_bits,
        is_signed=int(signed), out_half=int(out_half), scale=scale, batch=batch,
        row_indices=lhs.row_indices.data_ptr(), row_offsets=lhs.row_offsets.data_ptr(),
        column_indices=lhs.col_indices.data_ptr(), values=lhs.values.data_ptr(), values_stride=values_stride,
        rhs=rhs.data_ptr(), rhs_stride=rhs_stride, out=out.data_ptr(), out_stride=out_stride, mma_kind=mma_kind,
        kernel_variant=variant,
        value_layout=(value_layout if value_layout is not None
                      else _lib.VALUES_SOFTMAX if out_half else _lib.VALUES_PACKED),
        kernel_config=config)
    if variant == _lib.KERNEL_DENSE_TILE or (variant == _lib.KERNEL_AUTO and d.value_layout == _lib.VALUES_SLOT_MAJOR):
        d.chunk_starts = lhs.chunk_starts(stream).data_ptr()
    _lib.check(_lib.lib().mcSpmm(ctypes.byref(d), _stream_handle(stream)), "mcSpmm")
    return out


def sddmm(mask: DeviceSddmmMask, lhs: torch.Tensor, rhs: torch.Tensor, k: int, lhs_bits: int, rhs_bits: int, *,
          signed: bool = True, vecmajor: bool = False, out: torch.Tensor | None = None, out_half: bool = False,
          scale: float = 1.0, batch: int = 1, lhs_stride: int | None = None, rhs_stride: int | None = None,
          out_stride: int | None = None, row_split: int = 0, mma_kind: int = 0, variant: int = 0,
          stream: torch.cuda.Stream | None = None) -> torch.Tensor:
    """out = (A * B^T) on the mask's stored nonzero vectors.

    lhs: packed A (M rows of k*lhs_bits/8 bytes), rhs: packed B (n rows of
    k*rhs_bits/8 bytes), per batch entry.  Output: aligned_nnz * V values per
    batch entry, blocked (alignment 8) or vector-major layout."""
    M = mask.m_vec * mask.vec_length
    if lhs_stride is None:
        lhs_stride = M * k * lhs_bits // 8 if batch > 1 else 0
    if rhs_stride is None:
        rhs_stride = mask.n * k * rhs_bits // 8 if batch > 1 else 0
    per = mask.aligned_nnz * mask.vec_length
    if out_stride is None:
        out_stride = per if batch > 1 else 0
    if out is None:
        shape = (batch, per) if batch > 1 else (per,)
        out = torch.zeros(shape, dtype=torch.float16 if out_half else torch.int32, device=lhs.device)
    d = _lib.McSddmmDesc(
        m_vec=mask.m_vec, vec_length=mask.vec_length, n=mask.n, k=k, lhs_bits=lhs_bits, rhs_bits=rhs_bits,
        is_signed=int(signed), out_half=int(out_half), out_vecmajor=int(vecmajor), scale=scale, batch=batch,
        row_split=row_split, row_indices=mask.row_indices.data_ptr(), row_offsets=mask.row_offsets.data_ptr(),
        column_indices=mask.col_indices.data_ptr(), lhs=lhs.data_ptr(), lhs_stride=lhs_stride,
        rhs=rhs.data_ptr(), rhs_stride=rhs_stride, out=out.data_ptr(), out_stride=out_stride, mma_kind=mma_kind,
        kernel_variant=variant)
    if variant == _lib.KERNEL_DENSE_TILE:
        bitmap, prefix = mask.tile_mask(stream)
        d.tile_bitmap, d.tile_prefix = bitmap.data_ptr(), prefix.data_ptr()
    _lib.check(_lib.lib().mcSddmm(ctypes.byref(d), _stream_handle(stream)), "mcSddmm")
    return out
