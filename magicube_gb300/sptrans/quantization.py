"""sptrans.quantization: symmetric quantization of half tensors into packed
int32 words (reference: sparse_transformer_magicube/src/cuda/quantization.cpp:5-20,
quantization_kernel.cu:133-213)."""
from __future__ import annotations

import torch

from .. import _lib
from ._common import check, stream_handle


def _quantize(x: torch.Tensor, bits: int, scale: float, out_shape) -> torch.Tensor:
    if bits not in (4, 8):
        raise ValueError("bits must be 4 or 8")
    if x.dtype != torch.float16 or not x.is_cuda:
        raise TypeError("input must be a CUDA float16 tensor")
    x = x.contiguous()
    if x.size(-1) % (32 // bits):
        raise ValueError(f"the last dimension must be a multiple of {32 // bits}")
    out = torch.empty(out_shape, dtype=torch.int32, device=x.device)
    check(_lib.lib().mcQuantize(x.data_ptr(), out.data_ptr(), x.numel(), bits, float(scale), stream_handle()),
          "mcQuantize")
    return out


def quantization(input_matrix: torch.Tensor, bits: int, scale: float) -> torch.Tensor:
    """[m, n] half -> [m, n*bits/32] int32 (quantization.cpp:5)."""
    m, n = input_matrix.size(-2), input_matrix.size(-1)
    return _quantize(input_matrix, bits, scale, (m, n * bits // 32))


def bquantization(input_matrix: torch.Tensor, bits: int, scale: float) -> torch.Tensor:
    """[B, m, n] half -> [B, m, n*bits/32] int32 (quantization.cpp:12)."""
    b, m, n = input_matrix.size(-3), input_matrix.size(-2), input_matrix.size(-1)
    return _quantize(input_matrix, bits, scale, (b, m, n * bits // 32))
