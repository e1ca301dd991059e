"""Autotuner of the SpMM / SDDMM launch configuration.

For a problem signature (operation, precision pair, V, dense width, row-length
and row-count buckets, batch bucket) it times every candidate configuration on
the caller's own buffers -- tensor path (int8 or exact f16), kernel variant
(per-row, pipelined/streaming, or for SpMM the TMA-gather kernel where it
applies), for SDDMM the number of CTAs per vector-row, and for the fused
attention kernel the warps per CTA, ring stages and CTAs per SM -- and keeps
the fastest.  Results persist in a JSON cache
(``$MC_AUTOTUNE_CACHE``, default ``~/.cache/magicube_gb300/autotune.json``) so
a shape bucket is tuned once per machine.  Every candidate computes the same
integers; the choice only affects speed.
"""
from __future__ import annotations

import json
import math
import os
import threading
from pathlib import Path
from typing import Callable

import torch

from . import _lib

_lock = threading.Lock()
_cache: dict | None = None


def cache_path() -> Path:
    p = os.environ.get("MC_AUTOTUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "magicube_gb300" / "autotune.json"


def _load() -> dict:
    global _cache
    if _cache is None:
        try:
            _cache = json.loads(cache_path().read_text())
        except (OSError, ValueError):
            _cache = {}
    return _cache


def _save() -> None:
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(".tmp")
        tmp.write_text(json.dumps(_load(), indent=1, sort_keys=True))
        os.replace(tmp, p)
    except OSError:
        pass  # a read-only home only loses persistence


def _bucket(x: float) -> int:
    return int(round(math.log2(max(1.0, x))))


def signature(op: str, lhs_bits: int, rhs_bits: int, V: int, width: int, rows: int, avg_nnz: float,
              batch: int) -> str:
    dev = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    return (f"{dev}|{op}|L{lhs_bits}R{rhs_bits}|V{V}|w{width}|r{_bucket(rows)}|z{_bucket(avg_nnz)}"
            f"|b{_bucket(batch)}")


def spmm_candidates() -> list[dict]:
    out = [{"mma_kind": m, "variant": v} for m in (_lib.MMA_INT8, _lib.MMA_F16)
           for v in (_lib.KERNEL_PER_ROW, _lib.KERNEL_STREAM)]
    return out + [{"mma_kind": _lib.MMA_INT8, "variant": _lib.KERNEL_TMA}]


def sddmm_candidates(k: int, bits: int = 8) -> list[dict]:
    """Tensor path x kernel variant x row split; the dp4a path joins for 8-bit
    and 4-bit operands."""
    out = []
    for m in (_lib.MMA_INT8, _lib.MMA_F16) + ((_lib.MMA_DP4A,) if bits <= 8 else ()):
        for split in (0, 1, 2, 4):
            out.append({"mma_kind": m, "variant": _lib.KERNEL_PER_ROW, "row_split": split})
            if k == 64:
                out.append({"mma_kind": m, "variant": _lib.KERNEL_STREAM, "row_split": split})
    return out


def fused_attention_candidates() -> list[dict]:
    """Launch configurations of the fused attention kernel: warps per CTA
    (the k-split of P x V across warps), cp.async ring stages per warp, and a
    cap on resident CTAs per SM (0: as many as fit)."""
    return [{"warps": w, "stages": st, "ctas_per_sm": c} for w in (4, 8) for st in (2, 3) for c in (0, 2, 4)]


def _time(fn: Callable[[], None], reps: int) -> float:
    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    b.synchronize()
    return a.elapsed_time(b) / reps


def tune(sig: str, candidates: list[dict], run: Callable[[dict], None], reps: int = 5) -> dict:
    """Best configuration for `sig` (cached), timing `run(config)` per candidate."""
    with _lock:
        hit = _load().get(sig)
    if hit is not None:
        return hit["config"]
    best, best_ms = None, float("inf")
    for cfg in candidates:
        try:
            ms = _time(lambda: run(cfg), reps)
        except _lib.MagicubeError:
            continue  # a candidate that does not apply to these operands
        if ms < best_ms:
            best, best_ms = cfg, ms
    if best is None:
        raise RuntimeError(f"no applicable configuration for {sig}")
    with _lock:
        _load()[sig] = {"config": best, "ms": best_ms}
        _save()
    return best


def clear() -> None:
    """Forget every tuned configuration (in memory and on disk)."""
    global _cache
    with _lock:
        _cache = {}
        _save()
