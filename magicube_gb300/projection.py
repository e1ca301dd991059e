"""The attention's input projection with the quantization fused in.

``qkv_project_quantize`` replaces the reference's fp16 in-projection, the
permute to [3, H, T, d] and ``bquantization``
(end2end_eval/sparse_transformer_magicube/spattention.py:189-191,
quantization_kernel.cu:173-213) by one tcgen05 kernel (``mcQkvProjectQuantize``)
that writes the packed int8 / int4 Q, K, V operands the SDDMM and SpMM read.
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib


def qkv_project_quantize(x: torch.Tensor, weight: torch.Tensor, bias: torch.Tensor | None, heads: int, bits: int,
                         scale: float, out: torch.Tensor | None = None,
                         status: torch.Tensor | None = None) -> torch.Tensor:
    """x: [T, E] half; weight: [3E, E] half (nn.Linear layout); bias: [3E] half
    or None -> int32 [3, heads, T * (E / heads) * bits / 32]: trunc(clamp(
    half(x W^T + b) * scale)) packed little-endian, on the current stream."""
    if x.dtype != torch.float16 or weight.dtype != torch.float16:
        raise TypeError("x and weight must be float16")
    x, weight = x.contiguous(), weight.contiguous()
    T, E = x.shape
    if weight.shape != (3 * E, E):
        raise ValueError(f"weight must be [{3 * E}, {E}], got {tuple(weight.shape)}")
    d = E // heads
    words = T * d * bits // 32
    if out is None:
        out = torch.empty((3, heads, max(words, 1)), dtype=torch.int32, device=x.device)
    b = None
    if bias is not None:
        b = bias.to(torch.float16).contiguous()
    desc = _lib.McQkvProjDesc(tokens=T, hidden=E, heads=heads, head_dim=d, bits=bits, scale=float(scale),
                              x=x.data_ptr() if T else None, weight=weight.data_ptr(),
                              bias=b.data_ptr() if b is not None else None, out=out.data_ptr(),
                              status=status.data_ptr() if status is not None else None)
    _lib.check(_lib.lib().mcQkvProjectQuantize(ctypes.byref(desc),
                                               ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
               "mcQkvProjectQuantize")
    return out[:, :, :words]
