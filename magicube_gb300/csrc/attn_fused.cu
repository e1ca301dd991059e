// attn_fused.cu -- the quantized sparse attention in one persistent kernel.
//
// One work item = one vector-row (V query rows sharing a column pattern) of
// one head.  A CTA of 4 warps runs, per item, with everything in shared
// memory between the steps:
//   1. SDDMM: scores of the row's nonzero vectors, 16 per warp tile
//      (mma.m16n8k32 s8, K rows gathered with 128-bit loads straight into the
//      A fragment, Q rows in registers), dequantised exactly as the separate
//      SDDMM does (half(acc / scale_qkv^2)) and multiplied by the softmax
//      scaling, kept as the half [v][slot] (MC_REQUANT_ROWMAX keeps
//      half(acc / (scale_qkv^2 / scaling)), the separate SDDMM's output at
//      that scale);
//   2. softmax per vector lane: max, sum of exp, requantization to int8
//      [v][slot] -- warp w owns lanes 2w, 2w+1 and visits slots in the same
//      per-thread order and reduction tree as the separate softmax kernel,
//      so with MC_REQUANT_FIXED every probability equals its output bit for
//      bit; MC_REQUANT_ROWMAX instead stores q = round(127 exp(s - max)) and
//      dequantises the output by 127 * sum * scale_qkv per lane (probabilities
//      keep 7 bits relative to the row maximum instead of an absolute scale),
//      equal bit for bit to the separate softmax's row-max mode followed by
//      the SpMM with those per-row divisors;
//   3. SpMM: P (int8, from shared memory) times the gathered V rows, split
//      over the slots: warp w takes 32-slot steps w, w+4, ..., stages their V
//      rows through its own 2-deep cp.async ring, transposes them with
//      ldmatrix.m16n16.x2.trans.b8 and multiplies all 64 output columns; the
//      four warps' int32 partial sums are added through shared memory.
// Scores and probabilities never leave the SM: per item the kernel reads the
// Q rows, the gathered K and V rows (L2-resident per head) and writes V x 64
// half outputs.  Heads vary fastest between consecutive items.  Needs
// head_dim == 64 and rows of at most 4096 nonzero vectors (shared memory).
#include <cfloat>
#include <cstdint>

#include "mc_host.h"
#include "mc_ptx.cuh"

namespace mc {

struct AttnParams {
    int m_vec, heads, items, nnzp;
    const int* row_indices;
    const int* row_offsets;
    const int* col_indices;
    const uint8_t* q;
    const uint8_t* k;
    const uint8_t* v;
    long long head_stride;      // bytes between heads of q, k, v
    __half* out;
    long long out_head_stride;  // halves between heads of out
    float score_scale;          // fixed mode: scores = half(acc / score_scale)
    float score_div;            // row-max mode: scores = half(acc / score_div), score_div = score_scale / scaling
    float scaling;              // softmax input scaling
    float prob_scale;           // fixed requantization scale
    float out_scale;            // output divisor (fixed) or its per-lane factor (row-max)
    int* status;                // optional: set to 1 when a row exceeds nnzp
};

__device__ __forceinline__ void ldsm_x2_trans_b8_a(uint32_t (&r)[4], const void* p)
{
    asm volatile("ldmatrix.sync.aligned.m16n16.x2.trans.shared.b8 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_u32(p)));
}

// 8 CTAs per SM: every variant fits 64 registers without spills.
template <int V, bool ROWMAX>
__global__ void __launch_bounds__(128, 8) sparse_attention_kernel(const AttnParams p)
{
    constexpr int STAGES = 2;   // per-warp V-row ring depth
    constexpr int ROW = 64;     // bytes of one int8 row of d = 64
    extern __shared__ __align__(128) uint8_t smem[];
    const int SP = p.nnzp + 8;    // half score row stride (bank offset 4 words per vector lane)
    // Score row v (half) is overwritten from its start by the int8
    // probabilities of lane v: slot j's byte lies in score j / 2, already read.
    __half* S = reinterpret_cast<__half*>(smem);
    uint8_t* P = smem;
    const int PP = 2 * SP;        // probability row stride in bytes
    int* C = reinterpret_cast<int*>(smem + (size_t)V * SP * 2);
    float* DEN = reinterpret_cast<float*>(C + p.nnzp);
    float* MAXW = DEN + 8;  // [4 warps][8 lanes] partial row maxima of the scores
    uint8_t* rings = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(MAXW + 32) + 127) & ~static_cast<uintptr_t>(127));

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, t = lane & 3;
    uint8_t* ring = rings + warp * STAGES * 32 * ROW;  // this warp's private V-row ring
    const Divisor sdiv = make_divisor(ROWMAX ? p.score_div : p.score_scale);  // scores = half(acc / sdiv)

#pragma unroll 1
    for (int item = blockIdx.x; item < p.items; item += gridDim.x) {
        const int h = item % p.heads;
        const int row = __ldg(p.row_indices + item / p.heads);
        const int start = __ldg(p.row_offsets + 2 * row);
        const int nnz = __ldg(p.row_offsets + 2 * row + 1) - start;
        if (nnz > p.nnzp) {  // the caller's max_row_nnz is too small: leave the row, report it
            if (tid == 0 && p.status) atomicExch(p.status, 1);
            continue;
        }
        const uint8_t* qh = p.q + (long long)h * p.head_stride;
        const uint8_t* kh = p.k + (long long)h * p.head_stride;
        const uint8_t* vh = p.v + (long long)h * p.head_stride;

        __syncthreads();  // the previous item is done with S/P, C, DEN, MAXW and the rings
        for (int j = tid; j < nnz; j += 128) C[j] = __ldg(p.col_indices + start + j);
        int4 qf = make_int4(0, 0, 0, 0);
        if (g < V) qf = ldg_nc_v4(qh + (long long)(row * V + g) * ROW + 16 * t);
        __syncthreads();

        // The V rows of this warp's first two SpMM steps are requested now and
        // land while the scores and the softmax are computed.
        const int nround = (nnz + 31) & ~31;
        const int steps = nround >> 5;
        // Copy i moves rows 16 (i & 1) .. +15 of the step, 32-byte half
        // 2 (i >> 1) .. +1: lanes 2r and 2r + 1 take the two 16-byte chunks of
        // one sector of row r, so each copy instruction reads 16 whole 32-byte
        // sectors rather than 32 half sectors.
        auto issue = [&](int s, int slot) {
            if (s < steps) {
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int r = 16 * (i & 1) + (lane >> 1), q = 2 * (i >> 1) + (lane & 1);
                    const int j = s * 32 + r;
                    if (j < nnz)
                        cp_async16(ring + slot * 32 * ROW + r * ROW + ((q ^ ((r >> 1) & 3)) << 4),
                                   vh + (long long)C[j] * ROW + q * 16);
                }
            }
            cp_async_commit();
        };
        issue(warp, 0);
        issue(warp + 4, 1);

        // ---- 1. scores: warp w takes tiles w, w+4, ...; two tiles in flight ----
        const int ntiles = (nnz + 15) >> 4;
        float mxl[2] = {-FLT_MAX, -FLT_MAX};           // running max of lanes 2t, 2t+1
        auto store_scores = [&](int tile, const int (&acc)[4]) {
            if (2 * t >= V) return;
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int j = tile * 16 + g + 8 * hh;
                if (j >= nnz) continue;
                // Both modes keep the separate SDDMM's half output (fixed mode
                // scales it on every read, row-max mode has the scaling folded
                // into the divisor).  The maximum is taken of what the softmax
                // reads.
                const __half2 h2 = deq_half2(acc[2 * hh], acc[2 * hh + 1], sdiv, sdiv);
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const __half hs = e ? __high2half(h2) : __low2half(h2);
                    S[(2 * t + e) * SP + j] = hs;
                    mxl[e] = fmaxf(mxl[e], ROWMAX ? __half2float(hs) : __fmul_rn(__half2float(hs), p.scaling));
                }
            }
        };
#pragma unroll 1
        for (int tile = warp; tile < ntiles; tile += 8) {
            int4 r[2][2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int j0 = (tile + 4 * u) * 16 + g, j1 = j0 + 8;
                r[u][0] = j0 < nnz ? ldg_nc_v4(kh + (long long)C[j0] * ROW + 16 * t) : make_int4(0, 0, 0, 0);
                r[u][1] = j1 < nnz ? ldg_nc_v4(kh + (long long)C[j1] * ROW + 16 * t) : make_int4(0, 0, 0, 0);
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (tile + 4 * u >= ntiles) break;
                int acc[4] = {0, 0, 0, 0};
                mma_k32<true, true>(acc, r[u][0].x, r[u][1].x, r[u][0].y, r[u][1].y, qf.x, qf.y);
                mma_k32<true, true>(acc, r[u][0].z, r[u][1].z, r[u][0].w, r[u][1].w, qf.z, qf.w);
                store_scores(tile + 4 * u, acc);
            }
        }
        // lanes with the same t hold the same vector lanes: reduce over g
#pragma unroll
        for (int e = 0; e < 2; ++e) {
#pragma unroll
            for (int o = 4; o < 32; o <<= 1) mxl[e] = fmaxf(mxl[e], __shfl_xor_sync(0xffffffffu, mxl[e], o));
        }
        if (g == 0 && 2 * t < V) {
            MAXW[warp * 8 + 2 * t] = mxl[0];
            MAXW[warp * 8 + 2 * t + 1] = mxl[1];
        }
        __syncthreads();

        // ---- 2. softmax + requantization (warp w: lanes 2w, 2w+1) ------------
        // Lane l visits slot pairs (2l, 2l+1), (2l+64, 2l+65), ...: one 32-bit
        // load of two half scores, one 16-bit store of two probabilities.
        // The maximum is exact in any order; the sum keeps the per-thread
        // order and reduction tree of the separate softmax kernel.  Both
        // vector lanes of the warp and two pair iterations go through each
        // trip: their loads and exponentials are independent, only the adds
        // are chained (in each lane's order; an absent slot adds +0, which
        // leaves a sum of non-negative terms unchanged).  A __syncwarp
        // separates the scores read in a trip from the probability bytes
        // written over them: the bytes of iteration k overlay scores read in
        // iteration k / 2 or earlier.
        const int npit = (nround + 63) >> 6;
        if (2 * warp < V) {  // V is even: the warp holds lanes 2w and 2w + 1
            const int va = 2 * warp;
            const __half* sa = S + va * SP;
            const __half* sb = sa + SP;
            const float mxa = fmaxf(fmaxf(MAXW[va], MAXW[8 + va]), fmaxf(MAXW[16 + va], MAXW[24 + va]));
            const float mxb = fmaxf(fmaxf(MAXW[va + 1], MAXW[9 + va]), fmaxf(MAXW[17 + va], MAXW[25 + va]));
            uint8_t* pa = P + va * PP;
            uint8_t* pb = pa + PP;
            auto ld2 = [&](const __half* sv, int j) {
                return j < nnz ? __half22float2(*reinterpret_cast<const __half2*>(sv + j)) : make_float2(0.f, 0.f);
            };
            // exponent of score x of slot jj (0 if the slot is past the row)
            auto ex = [&](float x, float mx, int jj) {
                return jj < nnz ? exp_flush((ROWMAX ? x : __fmul_rn(x, p.scaling)) - mx) : 0.f;
            };
            float suma = 0.f, sumb = 0.f;
            if constexpr (ROWMAX) {
                for (int i = 0; i < npit; i += 2) {
                    const int j0 = 64 * i + 2 * lane, j1 = j0 + 64;
                    const float2 xa0 = ld2(sa, j0), xb0 = ld2(sb, j0), xa1 = ld2(sa, j1), xb1 = ld2(sb, j1);
                    const float ea[4] = {ex(xa0.x, mxa, j0), ex(xa0.y, mxa, j0 + 1), ex(xa1.x, mxa, j1),
                                         ex(xa1.y, mxa, j1 + 1)};
                    const float eb[4] = {ex(xb0.x, mxb, j0), ex(xb0.y, mxb, j0 + 1), ex(xb1.x, mxb, j1),
                                         ex(xb1.y, mxb, j1 + 1)};
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        suma += ea[u];
                        sumb += eb[u];
                    }
                    __syncwarp();
                    auto q2 = [](float e0, float e1) {
                        return (uint16_t)((__float2int_rn(127.f * e0) & 0xFF) | ((__float2int_rn(127.f * e1) & 0xFF) << 8));
                    };
                    if (j0 < nround) {
                        *reinterpret_cast<uint16_t*>(pa + j0) = q2(ea[0], ea[1]);
                        *reinterpret_cast<uint16_t*>(pb + j0) = q2(eb[0], eb[1]);
                    }
                    if (j1 < nround) {
                        *reinterpret_cast<uint16_t*>(pa + j1) = q2(ea[2], ea[3]);
                        *reinterpret_cast<uint16_t*>(pb + j1) = q2(eb[2], eb[3]);
                    }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    suma += __shfl_xor_sync(0xffffffffu, suma, o);
                    sumb += __shfl_xor_sync(0xffffffffu, sumb, o);
                }
            } else {
                for (int i = 0; i < npit; i += 2) {
                    const int j0 = 64 * i + 2 * lane, j1 = j0 + 64;
                    const float2 xa0 = ld2(sa, j0), xb0 = ld2(sb, j0), xa1 = ld2(sa, j1), xb1 = ld2(sb, j1);
                    const float ea[4] = {ex(xa0.x, mxa, j0), ex(xa0.y, mxa, j0 + 1), ex(xa1.x, mxa, j1),
                                         ex(xa1.y, mxa, j1 + 1)};
                    const float eb[4] = {ex(xb0.x, mxb, j0), ex(xb0.y, mxb, j0 + 1), ex(xb1.x, mxb, j1),
                                         ex(xb1.y, mxb, j1 + 1)};
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        suma += ea[u];
                        sumb += eb[u];
                    }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    suma += __shfl_xor_sync(0xffffffffu, suma, o);
                    sumb += __shfl_xor_sync(0xffffffffu, sumb, o);
                }
                const float rsa = __fdiv_rn(p.prob_scale, suma), rsb = __fdiv_rn(p.prob_scale, sumb);
                // the exponents are recomputed: same inputs, same values
                auto q = [&](float e, float rs) { return (int)fminf(fmaxf(e * rs, -128.f), 127.f); };
                auto q2 = [&](float e0, float e1, float rs) {
                    return (uint16_t)((q(e0, rs) & 0xFF) | ((q(e1, rs) & 0xFF) << 8));
                };
                for (int i = 0; i < npit; i += 2) {
                    const int j0 = 64 * i + 2 * lane, j1 = j0 + 64;
                    const float2 xa0 = ld2(sa, j0), xb0 = ld2(sb, j0), xa1 = ld2(sa, j1), xb1 = ld2(sb, j1);
                    const float ea[4] = {ex(xa0.x, mxa, j0), ex(xa0.y, mxa, j0 + 1), ex(xa1.x, mxa, j1),
                                         ex(xa1.y, mxa, j1 + 1)};
                    const float eb[4] = {ex(xb0.x, mxb, j0), ex(xb0.y, mxb, j0 + 1), ex(xb1.x, mxb, j1),
                                         ex(xb1.y, mxb, j1 + 1)};
                    __syncwarp();
                    if (j0 < nround) {
                        *reinterpret_cast<uint16_t*>(pa + j0) = q2(ea[0], ea[1], rsa);
                        *reinterpret_cast<uint16_t*>(pb + j0) = q2(eb[0], eb[1], rsb);
                    }
                    if (j1 < nround) {
                        *reinterpret_cast<uint16_t*>(pa + j1) = q2(ea[2], ea[3], rsa);
                        *reinterpret_cast<uint16_t*>(pb + j1) = q2(eb[2], eb[3], rsb);
                    }
                }
            }
            if (lane == 0) {
                DEN[va] = ROWMAX ? 127.f * suma * p.out_scale : p.out_scale;
                DEN[va + 1] = ROWMAX ? 127.f * sumb * p.out_scale : p.out_scale;
            }
        }
        __syncthreads();

        // ---- 3. out = P x V rows: warp w takes steps w, w+4, ... (k-split) ------
        // Each lane stages one gathered V row (four 16-byte copies) of the step
        // into the warp's private ring; the warp then multiplies all 64 output
        // columns (four MMAs sharing the P fragment).  No CTA barrier inside.
        int acc[4][4] = {};
        int slot = 0;
#pragma unroll 1
        for (int s = warp; s < steps; s += 4) {
            // step s sits in `slot` (requested two steps earlier, or at item start)
            cp_async_wait<1>();
            __syncwarp();
            const uint8_t* st = ring + slot * 32 * ROW;
            uint32_t b0 = 0, b1 = 0;
            if (g < V) {
                b0 = lds32(P + g * PP + s * 32 + 4 * t);
                b1 = lds32(P + g * PP + s * 32 + 16 + 4 * t);
            }
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                uint32_t a[4];
                ldsm_x2_trans_b8_a(a, st + lane * ROW + ((m ^ ((lane >> 1) & 3)) << 4));
                mma_k32<true, true>(acc[m], a[0], a[1], a[2], a[3], b0, b1);
            }
            __syncwarp();  // every lane is done with this slot before it is refilled
            issue(s + 8, slot);
            slot ^= 1;
        }
        // Cross-warp sum of the partial products (exact integer adds) through
        // the first 2 KB of each warp's own ring: its copies have landed and
        // every lane is past its last read of the ring.
        cp_async_wait<0>();
        __syncwarp();
        int* red = reinterpret_cast<int*>(ring);
#pragma unroll
        for (int m = 0; m < 4; ++m)
#pragma unroll
            for (int e = 0; e < 4; ++e) red[(m * 4 + e) * 32 + lane] = acc[m][e];
        __syncthreads();
        int tot[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            uint32_t x = 0;
#pragma unroll
            for (int w = 0; w < 4; ++w)
                x += (uint32_t)reinterpret_cast<const int*>(rings + w * STAGES * 32 * ROW)[(warp * 4 + e) * 32 + lane];
            tot[e] = (int)x;
        }
        // tot: column n = 16 warp + g (+8 for tot[2], tot[3]), lane v = 2t (+1 for odd)
        if (2 * t < V) {
            __half* o = p.out + (long long)h * p.out_head_stride + (long long)(row * V + 2 * t) * 64 + 16 * warp + g;
            const Divisor d0 = make_divisor(DEN[2 * t]), d1 = make_divisor(DEN[2 * t + 1]);
            const __half2 h01 = deq_half2(tot[0], tot[1], d0, d1), h23 = deq_half2(tot[2], tot[3], d0, d1);
            o[0] = __low2half(h01);
            o[64] = __high2half(h01);
            o[8] = __low2half(h23);
            o[72] = __high2half(h23);
        }
    }
}

inline size_t attn_smem_bytes(int V, int nnzp)
{
    // score / probability rows, column indices, DEN and MAXW
    const size_t s = (size_t)V * (nnzp + 8) * 2 + (size_t)nnzp * 4 + 8 * 4 + 32 * 4;
    return (s + 127) / 128 * 128 + 128 + 4 * 2 * 32 * 64;  // + four private 2-stage rings
}

template <int V, bool ROWMAX>
int attention_launch(const AttnParams& p, size_t smem, cudaStream_t s)
{
    auto kern = sparse_attention_kernel<V, ROWMAX>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return (int)cudaGetLastError();
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 128, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long grid = (long long)per_sm * sms;
    if (grid > p.items) grid = p.items;
    kern<<<(unsigned)(grid < 1 ? 1 : grid), 128, smem, s>>>(p);
    return (int)cudaGetLastError();
}

}  // namespace mc

extern "C" int mcSparseAttention(const mcAttnDesc* d, cudaStream_t stream)
{
    mc::clear_error();
    if (!d) return mc::fail(1, "mcSparseAttention: null descriptor");
    if (!(d->vec_length == 2 || d->vec_length == 4 || d->vec_length == 8))
        return mc::fail(1, "mcSparseAttention: vec_length must be 2, 4 or 8");
    if (d->head_dim != 64) return mc::fail(1, "mcSparseAttention: head_dim must be 64");
    if (d->lhs_bits != 8 || d->rhs_bits != 8)
        return mc::fail(1, "mcSparseAttention: the fused kernel computes L8-R8 (int8 probabilities, int8 Q/K/V)");
    if (d->requant != MC_REQUANT_FIXED && d->requant != MC_REQUANT_ROWMAX)
        return mc::fail(1, "mcSparseAttention: invalid requant mode");
    if (d->m_vec < 0 || d->heads < 1 || d->max_row_nnz < 0 || d->max_row_nnz > 4096)
        return mc::fail(1, "mcSparseAttention: bad m_vec / heads / max_row_nnz (at most 4096 nonzero vectors per row)");
    if ((long long)d->m_vec * d->heads > 0x7fffffffLL) return mc::fail(1, "mcSparseAttention: too many items");
    if (d->m_vec == 0) return 0;
    if (!d->row_indices || !d->row_offsets || !d->column_indices || !d->q || !d->k || !d->v || !d->out)
        return mc::fail(1, "mcSparseAttention: null pointer");
    auto al = [](const void* p) { return reinterpret_cast<uintptr_t>(p) % 16 == 0; };
    if (!al(d->q) || !al(d->k) || !al(d->v) || d->head_stride % 16 || !al(d->out) || d->out_head_stride % 8)
        return mc::fail(1, "mcSparseAttention: q, k, v, out must be 16-byte aligned with 16-byte strides");
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
    const size_t smem = mc::attn_smem_bytes(d->vec_length, p.nnzp);
    const bool rowmax = d->requant == MC_REQUANT_ROWMAX;
    switch (d->vec_length) {
        case 2: return rowmax ? mc::attention_launch<2, true>(p, smem, stream) : mc::attention_launch<2, false>(p, smem, stream);
        case 4: return rowmax ? mc::attention_launch<4, true>(p, smem, stream) : mc::attention_launch<4, false>(p, smem, stream);
        default: return rowmax ? mc::attention_launch<8, true>(p, smem, stream) : mc::attention_launch<8, false>(p, smem, stream);
    }
}
