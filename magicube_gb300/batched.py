"""Batched sparse attention over uneven instances in one set of launches.

Instances of different sequence lengths, each with its own vector-sparse
mask, are laid out as one block-diagonal vector-sparse problem: their
vector-rows are stacked, and each instance's column indices are offset by the
instance's first token in the stacked Q / K / V.  Heads are the batch
dimension.  One quantization, one SDDMM, one quantized softmax and one SpMM
launch then cover every (instance, head) pair -- the kernels see a single
large mask whose rows are processed longest first -- and the four launches
can be captured in a CUDA graph and replayed.  Each instance's result is the
same, bit for bit, as when it runs alone (the per-row arithmetic does not
depend on the other rows).

With ``fused=True`` the attention of every instance and head is instead one
launch of the fused kernel (mcSparseAttention) after one quantization launch;
scores and probabilities then never reach device memory.

PerInstanceSparseAttention runs the same computation with separate launches
per instance (the plain baseline).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib, autotune, formats
from .formats import VectorSparse


# (probability bits, Q/K/V bits) of the fused attention kernel
FUSED_PAIRS = ((8, 8), (16, 8), (8, 4))


@dataclass
class AttentionMaskDev:
    m_vec: int
    vec_length: int
    seq_len: int
    aligned_nnz: int
    row_indices: torch.Tensor
    row_offsets: torch.Tensor
    col_indices: torch.Tensor
    max_row_nnz: int = 0


def block_diagonal(masks: list[VectorSparse]) -> tuple[VectorSparse, np.ndarray]:
    """Stack masks into one block-diagonal mask; returns it and the token
    offset of every instance."""
    V = masks[0].vec_length
    if any(m.vec_length != V for m in masks):
        raise ValueError("all instances must use the same vector length")
    tok = np.zeros(len(masks) + 1, dtype=np.int64)
    for i, m in enumerate(masks):
        if m.ncols != m.m_vec * V:
            raise ValueError("an attention mask must be seq_len x seq_len")
        tok[i + 1] = tok[i] + m.ncols
    ro = [np.zeros(1, dtype=np.int64)]
    cols = []
    base = 0
    for i, m in enumerate(masks):
        ro.append(m.row_offsets[1:].astype(np.int64) + base)
        cols.append(m.col_indices.astype(np.int64) + tok[i])
        base += m.nnz_vec
    row_offsets = np.concatenate(ro).astype(np.int32)
    col_indices = np.concatenate(cols).astype(np.int32) if cols else np.zeros(0, np.int32)
    mega = VectorSparse(int(sum(m.m_vec for m in masks)), V, int(tok[-1]), row_offsets, col_indices)
    return mega, tok


def to_device(mask: VectorSparse, alignment: int, device) -> AttentionMaskDev:
    pairs, n = formats.align_row_offsets(mask, alignment)
    cols = formats.pad_column_indices(mask, pairs, n, shuffle8=False)
    ri = formats.sorted_row_swizzle(mask)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(device)  # noqa: E731
    lens = mask.row_lengths()
    return AttentionMaskDev(mask.m_vec, mask.vec_length, mask.ncols, n, t(ri), t(pairs),
                            t(cols if cols.size else np.full(1, -1, np.int32)), int(lens.max()) if lens.size else 0)


class _AttentionCore:
    """quantize -> SDDMM -> quantized softmax -> SpMM on one mask (heads
    batched), or quantize -> the fused attention kernel (`fused`).  requant
    "fixed" is the reference's absolute probability scale; "rowmax"
    requantizes the probabilities relative to each row's maximum (the SDDMM
    then dequantizes by scale_qkv^2 / scaling, the softmax writes per-row
    divisors and the SpMM divides by them).  Either mode gives the same bits
    fused and unfused."""

    def __init__(self, mask: AttentionMaskDev, heads: int, head_dim: int, lhs_bits: int, rhs_bits: int,
                 scale_qkv: float, scale_sfmx: float, device, tune: bool, fused: bool = False,
                 requant: str = "fixed"):
        self.fused = fused
        self.requant = _lib.REQUANT_ROWMAX if requant == "rowmax" else _lib.REQUANT_FIXED
        if fused and ((lhs_bits, rhs_bits) not in FUSED_PAIRS or head_dim != 64):
            raise ValueError("the fused attention kernel computes L8-R8, L16-R8 and L8-R4 with head_dim 64")
        if requant not in ("fixed", "rowmax"):
            raise ValueError("requant must be 'fixed' or 'rowmax'")
        if requant == "rowmax" and lhs_bits != 8:
            raise ValueError("row-max requantization writes 8-bit probabilities")
        self.status = torch.zeros(1, dtype=torch.int32, device=device)
        if head_dim % 64:
            raise ValueError("head_dim must be a multiple of 64")
        self.m, self.H, self.d = mask, heads, head_dim
        self.lb, self.rb = lhs_bits, rhs_bits
        self.scale_qkv, self.scale_sfmx = scale_qkv, scale_sfmx
        self.scaling = head_dim ** -0.5
        L, V = mask.seq_len, mask.vec_length
        self.q_words = L * head_dim * rhs_bits // 32
        self.qkv_q = torch.empty((3, heads, self.q_words), dtype=torch.int32, device=device)
        # scores and probabilities only exist in memory on the unfused path
        self.scores = None if fused else torch.empty((heads, mask.aligned_nnz * V), dtype=torch.float16,
                                                     device=device)
        self.probs = None if fused else torch.zeros((heads, mask.aligned_nnz * V * lhs_bits // 32),
                                                    dtype=torch.int32, device=device)
        self.out = torch.empty((heads, L, head_dim), dtype=torch.float16, device=device)
        # row-max mode, unfused: the softmax's per-row divisors for the SpMM
        self.row_div = (torch.empty((heads, L), dtype=torch.float32, device=device)
                        if not fused and self.requant == _lib.REQUANT_ROWMAX else None)
        # the float quotient the fused kernel computes from its two scales
        self.score_div = float(np.float32(np.float32(scale_qkv ** 2) / np.float32(self.scaling)))
        self.sddmm_cfg = {"mma_kind": _lib.MMA_INT8, "variant": _lib.KERNEL_AUTO, "row_split": 0}
        self.spmm_cfg = {"mma_kind": _lib.MMA_INT8, "variant": _lib.KERNEL_AUTO}
        self.fused_cfg: dict = {}
        self._tune = tune

    # -- the four steps -----------------------------------------------------
    def _quantize(self, qkv: torch.Tensor, stream) -> None:
        _lib.check(_lib.lib().mcQuantize(qkv.data_ptr(), self.qkv_q.data_ptr(), qkv.numel(), self.rb,
                                         float(self.scale_qkv), stream), "mcQuantize")

    def _sddmm(self, cfg: dict, stream) -> None:
        m = self.m
        bytes_per_head = self.q_words * 4
        d = _lib.McSddmmDesc(
            m_vec=m.m_vec, vec_length=m.vec_length, n=m.seq_len, k=self.d, lhs_bits=self.rb, rhs_bits=self.rb,
            is_signed=1, out_half=1, out_vecmajor=1,
            scale=self.score_div if self.row_div is not None else float(self.scale_qkv ** 2), batch=self.H,
            row_split=cfg.get("row_split", 0), row_indices=m.row_indices.data_ptr(),
            row_offsets=m.row_offsets.data_ptr(), column_indices=m.col_indices.data_ptr(),
            lhs=self.qkv_q[0].data_ptr(), lhs_stride=bytes_per_head, rhs=self.qkv_q[1].data_ptr(),
            rhs_stride=bytes_per_head, out=self.scores.data_ptr(), out_stride=self.scores.shape[1],
            mma_kind=cfg["mma_kind"], kernel_variant=cfg["variant"])
        _lib.check(_lib.lib().mcSddmm(ctypes.byref(d), stream), "mcSddmm")

    def _softmax(self, stream) -> None:
        m = self.m
        rowmax = self.row_div is not None
        d = _lib.McSoftmaxDesc(
            m_vec=m.m_vec, vec_length=m.vec_length, batch=self.H, bits=self.lb,
            scaling=1.0 if rowmax else float(self.scaling),
            scale=float(self.scale_qkv) if rowmax else float(self.scale_sfmx), row_indices=m.row_indices.data_ptr(),
            row_offsets=m.row_offsets.data_ptr(), scores=self.scores.data_ptr(), scores_stride=self.scores.shape[1],
            out=self.probs.data_ptr(), out_stride=self.probs.shape[1] * 4, requant=self.requant,
            row_div=self.row_div.data_ptr() if rowmax else None, row_div_stride=m.seq_len if rowmax else 0)
        _lib.check(_lib.lib().mcQuantSoftmax(ctypes.byref(d), stream), "mcQuantSoftmax")

    def _spmm(self, cfg: dict, stream) -> None:
        m = self.m
        d = _lib.McSpmmDesc(
            m_vec=m.m_vec, vec_length=m.vec_length, n=self.d, k=m.seq_len, lhs_bits=self.lb, rhs_bits=self.rb,
            is_signed=1, out_half=1, scale=float(self.scale_qkv * self.scale_sfmx), batch=self.H,
            row_indices=m.row_indices.data_ptr(), row_offsets=m.row_offsets.data_ptr(),
            column_indices=m.col_indices.data_ptr(), values=self.probs.data_ptr(),
            values_stride=self.probs.shape[1] * 4, rhs=self.qkv_q[2].data_ptr(), rhs_stride=self.q_words * 4,
            out=self.out.data_ptr(), out_stride=m.seq_len * self.d, mma_kind=cfg["mma_kind"],
            kernel_variant=cfg["variant"], value_layout=_lib.VALUES_SOFTMAX,
            row_div=self.row_div.data_ptr() if self.row_div is not None else None,
            row_div_stride=m.seq_len if self.row_div is not None else 0)
        _lib.check(_lib.lib().mcSpmm(ctypes.byref(d), stream), "mcSpmm")

    def tune(self, qkv: torch.Tensor) -> None:
        """Pick the SDDMM and SpMM configurations with the autotuner."""
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        m = self.m
        avg = m.aligned_nnz / max(1, m.m_vec)
        self._quantize(qkv, stream)
        sig = autotune.signature("sddmm_attn", self.rb, self.rb, m.vec_length, self.d, m.m_vec, avg, self.H)
        self.sddmm_cfg = autotune.tune(sig, autotune.sddmm_candidates(self.d, self.rb), lambda c: self._sddmm(c, stream))
        self._sddmm(self.sddmm_cfg, stream)
        self._softmax(stream)
        sig = autotune.signature("spmm_attn", self.lb, self.rb, m.vec_length, self.d, m.m_vec, avg, self.H)
        self.spmm_cfg = autotune.tune(sig, autotune.spmm_candidates(), lambda c: self._spmm(c, stream))

    def tune_fused(self, qkv: torch.Tensor) -> None:
        """Pick the fused kernel's launch configuration (warps per CTA = the
        k-split of P x V, ring stages, CTAs per SM) with the autotuner."""
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        m = self.m
        avg = m.aligned_nnz / max(1, m.m_vec)
        self._quantize(qkv, stream)
        sig = autotune.signature(f"attn_fused_{'rowmax' if self.requant else 'fixed'}", self.lb, self.rb,
                                 m.vec_length, self.d, m.m_vec, avg, self.H)
        self.fused_cfg = autotune.tune(sig, autotune.fused_attention_candidates(), lambda c: self._fused(stream, c))

    def _fused(self, stream, cfg: dict | None = None) -> None:
        m = self.m
        cfg = self.fused_cfg if cfg is None else cfg
        d = _lib.McAttnDesc(
            m_vec=m.m_vec, vec_length=m.vec_length, heads=self.H, head_dim=self.d, max_row_nnz=m.max_row_nnz,
            lhs_bits=self.lb, rhs_bits=self.rb, requant=self.requant, score_scale=float(self.scale_qkv ** 2),
            scaling=float(self.scaling), prob_scale=float(self.scale_sfmx),
            out_scale=float(self.scale_qkv if self.requant == _lib.REQUANT_ROWMAX
                            else self.scale_qkv * self.scale_sfmx),
            row_indices=m.row_indices.data_ptr(), row_offsets=m.row_offsets.data_ptr(),
            column_indices=m.col_indices.data_ptr(), q=self.qkv_q[0].data_ptr(), k=self.qkv_q[1].data_ptr(),
            v=self.qkv_q[2].data_ptr(), head_stride=self.q_words * 4, out=self.out.data_ptr(),
            out_head_stride=m.seq_len * self.d, status=self.status.data_ptr(), warps=cfg.get("warps", 0),
            stages=cfg.get("stages", 0), ctas_per_sm=cfg.get("ctas_per_sm", 0))
        _lib.check(_lib.lib().mcSparseAttention(ctypes.byref(d), stream), "mcSparseAttention")

    def run(self, qkv: torch.Tensor) -> torch.Tensor:
        """qkv: [3, H, L, d] half (contiguous) -> [H, L, d] half."""
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        if self.fused:
            if self._tune:
                self.tune_fused(qkv)
                self._tune = False
            self._quantize(qkv, stream)
            self._fused(stream)
            return self.out
        if self._tune:
            self.tune(qkv)
            self._tune = False
        self._quantize(qkv, stream)
        self._sddmm(self.sddmm_cfg, stream)
        self._softmax(stream)
        self._spmm(self.spmm_cfg, stream)
        return self.out


class BatchedSparseAttention:
    """Sparse attention of uneven instances (own length and mask each), all
    heads and instances in one quantize / SDDMM / softmax / SpMM sequence."""

    def __init__(self, masks: list[VectorSparse], heads: int, head_dim: int = 64, lhs_bits: int = 8,
                 rhs_bits: int = 8, scale_qkv: float = 36.0, scale_sfmx: float = 32.0, device="cuda",
                 tune: bool = True, fused: bool = False, requant: str = "fixed"):
        mega, self.token_offsets = block_diagonal(masks)
        align = 16 if rhs_bits == 8 else 32
        self.mask = to_device(mega, align, device)
        self.core = _AttentionCore(self.mask, heads, head_dim, lhs_bits, rhs_bits, scale_qkv, scale_sfmx, device,
                                   tune, fused=fused, requant=requant)
        self.seq_lens = [m.ncols for m in masks]
        self.total_tokens = int(self.token_offsets[-1])
        self.qkv = torch.zeros((3, heads, self.total_tokens, head_dim), dtype=torch.float16, device=device)
        self._graph = None

    def __call__(self, qkv: torch.Tensor | None = None) -> torch.Tensor:
        """qkv: [3, H, total_tokens, d] half (instances stacked along tokens);
        None runs on the internal input buffer ``self.qkv``."""
        return self.core.run(self.qkv if qkv is None else qkv.contiguous())

    def capture(self) -> "BatchedSparseAttention":
        """Capture the launch sequence (on ``self.qkv``) in a CUDA graph."""
        self.core.run(self.qkv)  # tunes and warms up outside the capture
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.core.run(self.qkv)
        torch.cuda.current_stream().wait_stream(s)
        self._graph = g
        return self

    def replay(self) -> torch.Tensor:
        self._graph.replay()
        return self.core.out

    def instance_output(self, i: int) -> torch.Tensor:
        a, b = int(self.token_offsets[i]), int(self.token_offsets[i + 1])
        return self.core.out[:, a:b]


class PerInstanceSparseAttention:
    """The plain baseline: the same steps launched separately per instance,
    either from the host (`__call__`) or replayed from one CUDA graph that
    holds every instance's launches (`capture` / `replay`: the same kernels
    without the host's per-launch cost)."""

    def __init__(self, masks: list[VectorSparse], heads: int, head_dim: int = 64, lhs_bits: int = 8,
                 rhs_bits: int = 8, scale_qkv: float = 36.0, scale_sfmx: float = 32.0, device="cuda",
                 requant: str = "fixed"):
        align = 16 if rhs_bits == 8 else 32
        self.cores = [_AttentionCore(to_device(m, align, device), heads, head_dim, lhs_bits, rhs_bits, scale_qkv,
                                     scale_sfmx, device, tune=False, requant=requant) for m in masks]
        self.seq_lens = [m.ncols for m in masks]

    def __call__(self, qkvs: list[torch.Tensor]) -> list[torch.Tensor]:
        return [c.run(x) for c, x in zip(self.cores, qkvs)]

    def capture(self, qkvs: list[torch.Tensor]) -> "PerInstanceSparseAttention":
        """Capture every instance's launches on these inputs in one CUDA graph."""
        self(qkvs)  # warm up outside the capture
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self(qkvs)
        torch.cuda.current_stream().wait_stream(s)
        self._graph = g
        return self

    def replay(self) -> list[torch.Tensor]:
        self._graph.replay()
        return [c.out for c in self.cores]


class NativeBatchedSparseAttention:
    """The same batched attention through the library's C++ engine
    (mcAttnBatch*): the block-diagonal mask is built and packed by the
    library, and every run is mcQuantize + the fused kernel, optionally
    replayed from a CUDA graph the library records -- no PyTorch on the
    path (torch only provides the device buffers here)."""

    def __init__(self, masks: list[VectorSparse], heads: int, head_dim: int = 64, lhs_bits: int = 8,
                 rhs_bits: int = 8, scale_qkv: float = 36.0, scale_sfmx: float = 32.0, device="cuda",
                 requant: str = "fixed"):
        self._ro = [np.ascontiguousarray(m.row_offsets, dtype=np.int32) for m in masks]
        self._ci = [np.ascontiguousarray(m.col_indices if m.col_indices.size else np.zeros(1, np.int32),
                                         dtype=np.int32) for m in masks]
        lens = np.array([m.ncols for m in masks], dtype=np.int32)
        ro_ptrs = (ctypes.c_void_p * len(masks))(*[a.ctypes.data for a in self._ro])
        ci_ptrs = (ctypes.c_void_p * len(masks))(*[a.ctypes.data for a in self._ci])
        d = _lib.McAttnBatchDesc(
            n_instances=len(masks), seq_lens=lens.ctypes.data, row_offsets=ctypes.addressof(ro_ptrs),
            col_indices=ctypes.addressof(ci_ptrs), vec_length=masks[0].vec_length, heads=heads, head_dim=head_dim,
            lhs_bits=lhs_bits, rhs_bits=rhs_bits,
            requant=_lib.REQUANT_ROWMAX if requant == "rowmax" else _lib.REQUANT_FIXED,
            scale_qkv=scale_qkv, scale_sfmx=scale_sfmx)
        self._h = ctypes.c_void_p()
        _lib.check(_lib.lib().mcAttnBatchCreate(ctypes.byref(d), ctypes.byref(self._h)), "mcAttnBatchCreate")
        offs = (ctypes.c_longlong * (len(masks) + 1))()
        _lib.check(_lib.lib().mcAttnBatchTokens(self._h, offs), "mcAttnBatchTokens")
        self.token_offsets = np.array(offs[:], dtype=np.int64)
        T = int(self.token_offsets[-1])
        self.qkv = torch.zeros((3, heads, T, head_dim), dtype=torch.float16, device=device)
        self.out = torch.empty((heads, T, head_dim), dtype=torch.float16, device=device)
        self.config: dict | None = None

    @staticmethod
    def _stream() -> ctypes.c_void_p:
        return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def __call__(self) -> torch.Tensor:
        _lib.check(_lib.lib().mcAttnBatchRun(self._h, self.qkv.data_ptr(), self.out.data_ptr(), self._stream()),
                   "mcAttnBatchRun")
        return self.out

    def tune(self) -> dict:
        w, st, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _lib.check(_lib.lib().mcAttnBatchTune(self._h, self.qkv.data_ptr(), self.out.data_ptr(), self._stream(),
                                              ctypes.byref(w), ctypes.byref(st), ctypes.byref(c)), "mcAttnBatchTune")
        self.config = {"warps": w.value, "stages": st.value, "ctas_per_sm": c.value}
        return self.config

    def capture(self) -> "NativeBatchedSparseAttention":
        """Record the run in a CUDA graph on a side stream (the library's
        capture needs a created stream)."""
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            _lib.check(_lib.lib().mcAttnBatchCapture(self._h, self.qkv.data_ptr(), self.out.data_ptr(),
                                                     self._stream()), "mcAttnBatchCapture")
        torch.cuda.current_stream().wait_stream(s)
        return self

    def replay(self) -> torch.Tensor:
        _lib.check(_lib.lib().mcAttnBatchReplay(self._h, self._stream()), "mcAttnBatchReplay")
        return self.out

    def status(self) -> int:
        st = ctypes.c_int()
        _lib.check(_lib.lib().mcAttnBatchStatus(self._h, ctypes.byref(st)), "mcAttnBatchStatus")
        return st.value

    def instance_output(self, i: int) -> torch.Tensor:
        a, b = int(self.token_offsets[i]), int(self.token_offsets[i + 1])
        return self.out[:, a:b]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.lib().mcAttnBatchDestroy(h)
            self._h = ctypes.c_void_p()


class NativeAttentionServer:
    """Continuous batching of sparse-attention requests in the library's C++
    request loop (mcAttnServer*): every request keeps its plain vector CSR
    mask and half Q/K/V on the device; the loop admits waiting requests as
    batches by arrival and free device memory, builds and packs each batch
    on the device and runs the fused kernel, several batches in flight on
    their own streams.  torch only provides the device buffers here."""

    def __init__(self, vec_length: int = 8, heads: int = 4, head_dim: int = 64, lhs_bits: int = 8,
                 rhs_bits: int = 8, scale_qkv: float = 36.0, scale_sfmx: float = 127.0, requant: str = "rowmax",
                 max_batch_tokens: int = 16384, max_inflight: int = 2, hbm_reserve_bytes: int = 0):
        self.desc = _lib.McAttnServerDesc(
            vec_length=vec_length, heads=heads, head_dim=head_dim, lhs_bits=lhs_bits, rhs_bits=rhs_bits,
            requant=_lib.REQUANT_ROWMAX if requant == "rowmax" else _lib.REQUANT_FIXED, scale_qkv=scale_qkv,
            scale_sfmx=scale_sfmx, max_batch_tokens=max_batch_tokens, max_inflight=max_inflight,
            hbm_reserve_bytes=hbm_reserve_bytes)
        self._h = ctypes.c_void_p()
        _lib.check(_lib.lib().mcAttnServerCreate(ctypes.byref(self.desc), ctypes.byref(self._h)),
                   "mcAttnServerCreate")

    @staticmethod
    def request(mask: VectorSparse, qkv: torch.Tensor, out: torch.Tensor, arrival_s: float = 0.0,
                device="cuda") -> tuple:
        """(ctypes request, device buffers it points at) for one sequence:
        qkv half [3][heads][L][64], out half [heads][L][64]."""
        ro = torch.from_numpy(np.ascontiguousarray(mask.row_offsets, dtype=np.int32)).to(device)
        ci = torch.from_numpy(np.ascontiguousarray(mask.col_indices if mask.col_indices.size
                                                   else np.zeros(1, np.int32), dtype=np.int32)).to(device)
        lens = np.diff(mask.row_offsets)
        r = _lib.McAttnRequest(seq_len=mask.ncols, nnz_vec=mask.nnz_vec,
                               max_row_nnz=int(lens.max()) if lens.size else 0, row_offsets=ro.data_ptr(),
                               col_indices=ci.data_ptr(), qkv=qkv.data_ptr(), out=out.data_ptr(),
                               arrival_s=float(arrival_s))
        return r, (ro, ci, qkv, out)

    def memory(self, reqs: list) -> tuple[int, int]:
        """(bytes admission charges for one batch of `reqs`, current budget)."""
        arr = (_lib.McAttnRequest * max(1, len(reqs)))(*reqs)
        need, avail = ctypes.c_longlong(), ctypes.c_longlong()
        _lib.check(_lib.lib().mcAttnServerMemory(self._h, arr, len(reqs), ctypes.byref(need), ctypes.byref(avail)),
                   "mcAttnServerMemory")
        return int(need.value), int(avail.value)

    def run(self, reqs: list) -> tuple[np.ndarray, dict]:
        """Serves the requests; returns (latency in ms per request, -1 if
        rejected) and the run's statistics."""
        arr = (_lib.McAttnRequest * max(1, len(reqs)))(*reqs)
        lat = np.zeros(max(1, len(reqs)), dtype=np.float64)
        st = _lib.McAttnServeStats()
        torch.cuda.synchronize()
        _lib.check(_lib.lib().mcAttnServerRun(self._h, arr, len(reqs),
                                              lat.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                              ctypes.byref(st)), "mcAttnServerRun")
        stats = {f: getattr(st, f) for f, _ in _lib.McAttnServeStats._fields_}
        return lat[:len(reqs)], stats

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib.lib().mcAttnServerDestroy(self._h)
            self._h = ctypes.c_void_p()
