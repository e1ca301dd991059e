"""Shared helpers of the sptrans mirror."""
from __future__ import annotations

import ctypes

import torch

from .. import _lib


def stream_handle() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def as_int32_device(t: torch.Tensor, name: str) -> torch.Tensor:
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor")
    if t.dtype != torch.int32:
        raise TypeError(f"{name} must be int32, got {t.dtype}")
    return t.contiguous()


def check(rc: int, what: str) -> None:
    _lib.check(rc, what)
