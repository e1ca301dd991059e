// attn_fused.cu -- mcSparseAttention: argument checks and the dispatch to the
// fused attention kernel (mc_attn_fused.cuh; one translation unit of
// instantiations per precision pair).
#include "mc_attn_fused.cuh"

extern "C" int mcSparseAttention(const mcAttnDesc* d, cudaStream_t stream)
{
    mc::clear_error();
    if (!d) return mc::fail(1, "mcSparseAttention: null descriptor");
    if (!(d->vec_length == 2 || d->vec_length == 4 || d->vec_length == 8))
        return mc::fail(1, "mcSparseAttention: vec_length must be 2, 4 or 8");
    if (d->head_dim != 64) return mc::fail(1, "mcSparseAttention: head_dim must be 64");
    const int lb = d->lhs_bits, rb = d->rhs_bits;
    if (!((lb == 8 && rb == 8) || (lb == 16 && rb == 8) || (lb == 8 && rb == 4)))
        return mc::fail(1, "mcSparseAttention: the fused kernel computes L8-R8, L16-R8 and L8-R4 (probability bits, "
                           "Q/K/V bits)");
    if (d->requant != MC_REQUANT_FIXED && d->requant != MC_REQUANT_ROWMAX)
        return mc::fail(1, "mcSparseAttention: invalid requant mode");
    if (d->requant == MC_REQUANT_ROWMAX && lb != 8)
        return mc::fail(1, "mcSparseAttention: row-max requantization writes 8-bit probabilities");
    if (d->m_vec < 0 || d->heads < 1 || d->max_row_nnz < 0 || d->max_row_nnz > 4096)
        return mc::fail(1, "mcSparseAttention: bad m_vec / heads / max_row_nnz (at most 4096 nonzero vectors per row)");
    const int warps = d->warps ? d->warps : 4, stages = d->stages ? d->stages : 2;
    if (!(warps == 4 || warps == 8) || !(stages == 2 || stages == 3) || d->ctas_per_sm < 0)
        return mc::fail(1, "mcSparseAttention: warps must be 4 or 8, stages 2 or 3, ctas_per_sm >= 0");
    if ((long long)d->m_vec * d->heads > 0x7fffffffLL) return mc::fail(1, "mcSparseAttention: too many items");
    if (d->m_vec == 0) return 0;
    if (!d->row_indices || !d->row_offsets || !d->column_indices || !d->q || !d->k || !d->v || !d->out)
        return mc::fail(1, "mcSparseAttention: null pointer");
    auto al = [](const void* p) { return reinterpret_cast<uintptr_t>(p) % 16 == 0; };
    if (!al(d->q) || !al(d->k) || !al(d->v) || d->head_stride % 16 || !al(d->out) || d->out_head_stride % 8)
        return mc::fail(1, "mcSparseAttention: q, k, v, out must be 16-byte aligned with 16-byte strides");
    if (d->heads > 1 && (d->head_stride < 0 || d->out_head_stride < 0))
        return mc::fail(1, "mcSparseAttention: negative head stride");
    mc::AttnParams p;
    p.m_vec = d->m_vec;
    p.heads = d->heads;
    p.items = d->m_vec * d->heads;
    p.nnzp = (d->max_row_nnz + 31) & ~31;
    if (p.nnzp == 0) p.nnzp = 32;
    p.row_indices = d->row_indices;
    p.row_offsets = d->row_offsets;
    p.col_indices = d->column_indices;
    p.q = static_cast<const uint8_t*>(d->q);
    p.k = static_cast<const uint8_t*>(d->k);
    p.v = static_cast<const uint8_t*>(d->v);
    p.head_stride = d->head_stride;
    p.out = static_cast<__half*>(d->out);
    p.out_head_stride = d->out_head_stride;
    p.score_scale = d->score_scale;
    p.scaling = d->scaling;
    p.score_div = d->score_scale / d->scaling;
    p.prob_scale = d->prob_scale;
    p.out_scale = d->out_scale;
    p.status = d->status;
    if (!(p.score_scale != 0.f) || !(p.out_scale != 0.f))
        return mc::fail(1, "mcSparseAttention: score_scale and out_scale must be nonzero");
    const bool rowmax = d->requant == MC_REQUANT_ROWMAX;
    if (lb == 16) return mc::attention_dispatch_16_8(p, d->vec_length, rowmax, warps, stages, d->ctas_per_sm, stream);
    if (rb == 4) return mc::attention_dispatch_8_4(p, d->vec_length, rowmax, warps, stages, d->ctas_per_sm, stream);
    return mc::attention_dispatch_8_8(p, d->vec_length, rowmax, warps, stages, d->ctas_per_sm, stream);
}
