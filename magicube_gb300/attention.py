"""Quantized vector-sparse multi-head attention (the caller of the SDDMM /
softmax / SpMM path).

Mirrors sp_multi_head_attention_forward and spMultiheadAttention of the
reference (end2end_eval/sparse_transformer_magicube/spattention.py:20-250):
in-projection, per-(batch, head) quantization of Q, K, V, quantized SDDMM with
half scores, quantized row softmax, quantized SpMM with half output,
out-projection.  The mask is one vector-sparse pattern shared by every batch
entry and head, in the attention layout: row offsets aligned to 16 (8-bit
operands) or 32 (4-bit), column indices unshuffled.
"""
from __future__ import annotations

from typing import Optional, Tuple

import torch
import torch.nn.functional as F

from .sptrans.deq_sddmm import bsddmm_4b, bsddmm_8b
from .sptrans.deq_spmm import bspmm_4b, bspmm_8b, bspmm_8b4b, bspmm_16b8b
from .sptrans.q_softmax import q_bcsr_softmax
from .sptrans.quantization import bquantization

# The reference's fixed quantization scales (spattention.py:51-53).
SCALE_QKV = 36.0
SCALE_SFMX = 32.0


def sp_multi_head_attention_forward(
    query: torch.Tensor,
    key: torch.Tensor,
    value: torch.Tensor,
    embed_dim_to_check: int,
    num_heads: int,
    in_proj_weight: torch.Tensor,
    in_proj_bias: torch.Tensor,
    bias_k: Optional[torch.Tensor],
    bias_v: Optional[torch.Tensor],
    add_zero_attn: bool,
    dropout_p: float,
    out_proj_weight: torch.Tensor,
    out_proj_bias: torch.Tensor,
    training: bool = True,
    key_padding_mask: Optional[torch.Tensor] = None,
    need_weights: bool = True,
    row_indices: Optional[torch.Tensor] = None,
    row_offsets: Optional[torch.Tensor] = None,
    column_indices: Optional[torch.Tensor] = None,
    vec_length: Optional[int] = 2,
    lhs_pre: Optional[int] = 8,
    rhs_pre: Optional[int] = 8,
    use_separate_proj_weight: bool = False,
    q_proj_weight: Optional[torch.Tensor] = None,
    k_proj_weight: Optional[torch.Tensor] = None,
    v_proj_weight: Optional[torch.Tensor] = None,
    static_k: Optional[torch.Tensor] = None,
    static_v: Optional[torch.Tensor] = None,
    scale_qkv: float = SCALE_QKV,
    scale_sfmx: float = SCALE_SFMX,
) -> Tuple[torch.Tensor, Optional[torch.Tensor]]:
    """query/key/value: (seq_len, batch, embed_dim).  Same arguments as the
    reference (spattention.py:20-46) plus the two quantization scales."""
    if key_padding_mask is not None or add_zero_attn or bias_k is not None or bias_v is not None:
        raise NotImplementedError("key_padding_mask / add_zero_attn / bias_k / bias_v are not supported "
                                  "(the reference leaves them as TODO as well)")
    tgt_len, bsz, embed_dim = query.size()
    assert embed_dim == embed_dim_to_check
    head_dim = embed_dim // num_heads
    assert head_dim * num_heads == embed_dim, "embed_dim must be divisible by num_heads"
    scaling = float(head_dim) ** -0.5

    if not use_separate_proj_weight:
        if query is key and key is value:
            q, k, v = F.linear(query, in_proj_weight, in_proj_bias).chunk(3, dim=-1)
        else:
            w_q, w_k, w_v = in_proj_weight.chunk(3, dim=0)
            b_q, b_k, b_v = (in_proj_bias.chunk(3) if in_proj_bias is not None else (None, None, None))
            q, k, v = F.linear(query, w_q, b_q), F.linear(key, w_k, b_k), F.linear(value, w_v, b_v)
    else:
        b_q, b_k, b_v = (in_proj_bias.chunk(3) if in_proj_bias is not None else (None, None, None))
        q = F.linear(query, q_proj_weight, b_q)
        k = F.linear(key, k_proj_weight, b_k)
        v = F.linear(value, v_proj_weight, b_v)

    batch = bsz * num_heads
    q = q.contiguous().view(tgt_len, batch, head_dim).transpose(0, 1).contiguous()
    k = (static_k if static_k is not None else k.contiguous().view(-1, batch, head_dim).transpose(0, 1)).contiguous()
    v = (static_v if static_v is not None else v.contiguous().view(-1, batch, head_dim).transpose(0, 1)).contiguous()
    src_len = k.size(1)

    qq = bquantization(q.half(), rhs_pre, scale_qkv)
    kq = bquantization(k.half(), rhs_pre, scale_qkv)
    vq = bquantization(v.half(), rhs_pre, scale_qkv)

    sddmm = bsddmm_8b if rhs_pre == 8 else bsddmm_4b
    scores = sddmm(row_indices, row_offsets, column_indices, qq, kq, vec_length, rhs_pre, scale_qkv * scale_qkv)
    probs = q_bcsr_softmax(row_indices, row_offsets, scores, scaling, scale_sfmx, vec_length, batch, lhs_pre)
    spmm = {(8, 8): bspmm_8b, (16, 8): bspmm_16b8b, (8, 4): bspmm_8b4b, (4, 4): bspmm_4b}[(lhs_pre, rhs_pre)]
    attn = spmm(row_indices, row_offsets, column_indices, probs, vq, vec_length, lhs_pre, rhs_pre,
                scale_qkv * scale_sfmx)

    attn = attn.transpose(0, 1).contiguous().view(tgt_len, bsz, embed_dim).to(query.dtype)
    attn = F.linear(attn, out_proj_weight, out_proj_bias)
    if need_weights:
        # The reference reshapes the packed quantized probabilities; return them as stored.
        return attn, probs
    return attn, None


class SpMultiheadAttention(torch.nn.MultiheadAttention):
    """torch.nn.MultiheadAttention whose forward runs the quantized sparse path
    (spattention.py:233-250)."""

    def forward(self, query, key, value, key_padding_mask=None, need_weights=True, row_indices=None,
                row_offsets=None, column_indices=None, vec_length: int = 2, lhs_pre: int = 8, rhs_pre: int = 8,
                scale_qkv: float = SCALE_QKV, scale_sfmx: float = SCALE_SFMX):
        return sp_multi_head_attention_forward(
            query, key, value, self.embed_dim, self.num_heads, self.in_proj_weight, self.in_proj_bias,
            self.bias_k, self.bias_v, self.add_zero_attn, self.dropout, self.out_proj.weight, self.out_proj.bias,
            training=self.training, key_padding_mask=key_padding_mask, need_weights=need_weights,
            row_indices=row_indices, row_offsets=row_offsets, column_indices=column_indices, vec_length=vec_length,
            lhs_pre=lhs_pre, rhs_pre=rhs_pre, scale_qkv=scale_qkv, scale_sfmx=scale_sfmx)


# The reference's class name (spattention.py:233).
spMultiheadAttention = SpMultiheadAttention
