// mc_attn_fused.cuh -- the quantized sparse attention in one persistent kernel.
//
// One work item = one vector-row (V query rows sharing a column pattern) of
// one head.  A CTA of WARPS warps runs, per item, with everything in shared
// memory between the steps:
//   1. SDDMM: scores of the row's nonzero vectors, 16 per warp tile
//      (mma.m16n8k32 s8, K rows gathered straight into the A fragment, Q rows
//      in registers), dequantised exactly as the separate SDDMM does
//      (half(acc / scale_qkv^2)), kept as the half [v][slot] row
//      (MC_REQUANT_ROWMAX keeps half(acc / (scale_qkv^2 / scaling)), the
//      separate SDDMM's output at that scale).  4-bit Q and K (RB = 4) enter
//      the int8 MMA as 16 x value bytes; the sums are shifted back exactly.
//   2. softmax per vector lane: max, sum of exp, requantization -- warp w
//      owns lanes 2w, 2w+1 and visits slots in the same per-thread order and
//      reduction tree as the separate softmax kernel, so with
//      MC_REQUANT_FIXED every probability equals its output bit for bit (int8
//      for LB = 8, int16 for LB = 16); MC_REQUANT_ROWMAX (LB = 8) instead
//      stores q = round(127 exp(s - max)) and dequantises the output by 127 *
//      sum * scale_qkv per lane, equal bit for bit to the separate softmax's
//      row-max mode followed by the SpMM with those per-row divisors;
//   3. SpMM: P (from shared memory) times the gathered V rows, split over the
//      slots: warp w takes 32-slot steps w, w + WARPS, ..., stages their V
//      rows through its own STAGES-deep cp.async ring, transposes them with
//      ldmatrix.m16n16.x2.trans.b8 and multiplies all 64 output columns; the
//      warps' int32 partial sums are added through shared memory.  16-bit
//      probabilities are two byte planes (signed high x V and unsigned low x
//      V, recombined by a shift); 4-bit V rows (RB = 4) give two 16-column
//      tiles per transposed 16-byte chunk (low and high nibbles as 16 x value
//      bytes; the sums are shifted back exactly).
// Scores and probabilities never leave the SM: per item the kernel reads the
// Q rows, the gathered K and V rows (L2-resident per head) and writes V x 64
// half outputs.  Heads vary fastest between consecutive items.  Needs
// head_dim == 64 and rows of at most 4096 nonzero vectors (shared memory).
#pragma once
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

// 16 k-values of one Q or K row for the SDDMM fragment: 16 bytes (8-bit) or
// 8 bytes of nibbles expanded to 16 x value bytes (4-bit; both operands get
// the same k permutation).
template <int RB>
__device__ __forceinline__ int4 load_qk16(const uint8_t* row, int t)
{
    if constexpr (RB == 8) {
        return ldg_nc_v4(row + 16 * t);
    } else {
        const int2 w = ldg_nc_v2(row + 8 * t);
        uint32_t a, b, c, d;
        unpack4_hi_u32((uint32_t)w.x, a, b);
        unpack4_hi_u32((uint32_t)w.y, c, d);
        return make_int4((int)a, (int)b, (int)c, (int)d);
    }
}

template <int WARPS, int STAGES, int RB>
constexpr size_t attn_ring_bytes()
{
    return (size_t)WARPS * STAGES * 32 * (RB == 8 ? 64 : 32);
}

// Shared memory of one CTA: score / probability rows, column indices, DEN,
// the per-warp partial row maxima, then the private V-row rings.
inline size_t attn_smem_bytes(int V, int nnzp, int warps, size_t ring_bytes)
{
    const size_t s = (size_t)V * (nnzp + 8) * 2 + (size_t)nnzp * 4 + 8 * 4 + (size_t)warps * 8 * 4;
    return (s + 127) / 128 * 128 + 128 + ring_bytes;
}

// Minimum resident CTAs per SM the register budget is compiled for: 64
// registers per thread for 8-bit probabilities, 85 for 16-bit (two
// accumulator sets in the P x V step).
template <int WARPS, int LB>
constexpr int attn_min_blocks()
{
    return (LB == 16 ? 24 : 32) / WARPS;
}

template <int V, bool ROWMAX, int LB, int RB, int WARPS, int STAGES>
__global__ void __launch_bounds__(WARPS * 32, attn_min_blocks<WARPS, LB>()) sparse_attention_kernel(const AttnParams p)
{
    static_assert(LB == 8 || LB == 16, "probabilities are 8 or 16 bits");
    static_assert(RB == 8 || RB == 4, "Q, K, V are 8 or 4 bits");
    static_assert(!ROWMAX || LB == 8, "row-max requantization writes 8-bit probabilities");
    static_assert(WARPS == 4 || WARPS == 8, "4 or 8 warps per CTA");
    static_assert(STAGES >= 2 && STAGES <= 4, "2 to 4 ring stages");
    constexpr int NT = WARPS * 32;
    constexpr int QROW = RB == 8 ? 64 : 32;  // bytes of one Q / K / V row of d = 64
    constexpr int STEP = 32 * QROW;          // bytes of one staged 32-slot step
    constexpr float LO = LB == 16 ? -32768.f : -128.f;
    constexpr float HI = LB == 16 ? 32767.f : 127.f;
    extern __shared__ __align__(128) uint8_t smem[];
    const int SP = p.nnzp + 8;    // half score row stride (bank offset 4 words per vector lane)
    // Score row v (half) is overwritten by the probabilities of lane v: for
    // 8 bits from its start (slot j's byte lies in score j / 2, already
    // read), for 16 bits in place (slot j's int16 replaces score j).
    __half* S = reinterpret_cast<__half*>(smem);
    uint8_t* P = smem;
    const int PP = 2 * SP;        // probability row stride in bytes
    int* C = reinterpret_cast<int*>(smem + (size_t)V * SP * 2);
    float* DEN = reinterpret_cast<float*>(C + p.nnzp);
    float* MAXW = DEN + 8;  // [WARPS][8] partial row maxima of the scores
    uint8_t* rings = reinterpret_cast<uint8_t*>(
        (reinterpret_cast<uintptr_t>(MAXW + WARPS * 8) + 127) & ~static_cast<uintptr_t>(127));

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, t = lane & 3;
    uint8_t* ring = rings + warp * STAGES * STEP;  // this warp's private V-row ring
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
        for (int j = tid; j < nnz; j += NT) C[j] = __ldg(p.col_indices + start + j);
        int4 qf = make_int4(0, 0, 0, 0);
        if (g < V) qf = load_qk16<RB>(qh + (long long)(row * V + g) * QROW, t);
        __syncthreads();

        // The V rows of this warp's first STAGES SpMM steps are requested now
        // and land while the scores and the softmax are computed.  Lanes 2r
        // and 2r + 1 copy the two 16-byte halves of one 32-byte sector of row
        // r, so each copy instruction reads 16 whole sectors.
        const int nround = (nnz + 31) & ~31;
        const int steps = nround >> 5;
        auto issue = [&](int s, int slot) {
            if (s < steps) {
                uint8_t* dst = ring + slot * STEP;
                if constexpr (RB == 8) {
                    // copy i: rows 16 (i & 1) .. +15, sector i >> 1 of each row
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const int r = 16 * (i & 1) + (lane >> 1), q = 2 * (i >> 1) + (lane & 1);
                        const int j = s * 32 + r;
                        if (j < nnz)
                            cp_async16(dst + r * QROW + ((q ^ ((r >> 1) & 3)) << 4),
                                       vh + (long long)C[j] * QROW + q * 16);
                    }
                } else {
                    // copy i: rows 16 i .. +15, the row's one sector
#pragma unroll
                    for (int i = 0; i < 2; ++i) {
                        const int r = 16 * i + (lane >> 1), q = lane & 1;
                        const int j = s * 32 + r;
                        if (j < nnz)
                            cp_async16(dst + r * QROW + ((q ^ ((r >> 2) & 1)) << 4),
                                       vh + (long long)C[j] * QROW + q * 16);
                    }
                }
            }
            cp_async_commit();
        };
#pragma unroll
        for (int i = 0; i < STAGES; ++i) issue(warp + i * WARPS, i);

        // ---- 1. scores: warp w takes tiles w, w + WARPS, ...; two in flight ----
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
                const int a0 = RB == 8 ? acc[2 * hh] : (acc[2 * hh] >> 8);
                const int a1 = RB == 8 ? acc[2 * hh + 1] : (acc[2 * hh + 1] >> 8);
                const __half2 h2 = deq_half2(a0, a1, sdiv, sdiv);
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const __half hs = e ? __high2half(h2) : __low2half(h2);
                    S[(2 * t + e) * SP + j] = hs;
                    mxl[e] = fmaxf(mxl[e], ROWMAX ? __half2float(hs) : __fmul_rn(__half2float(hs), p.scaling));
                }
            }
        };
#pragma unroll 1
        for (int tile = warp; tile < ntiles; tile += 2 * WARPS) {
            int4 r[2][2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int j0 = (tile + WARPS * u) * 16 + g, j1 = j0 + 8;
                r[u][0] = j0 < nnz ? load_qk16<RB>(kh + (long long)C[j0] * QROW, t) : make_int4(0, 0, 0, 0);
                r[u][1] = j1 < nnz ? load_qk16<RB>(kh + (long long)C[j1] * QROW, t) : make_int4(0, 0, 0, 0);
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                if (tile + WARPS * u >= ntiles) break;
                int acc[4] = {0, 0, 0, 0};
                mma_k32<true, true>(acc, r[u][0].x, r[u][1].x, r[u][0].y, r[u][1].y, qf.x, qf.y);
                mma_k32<true, true>(acc, r[u][0].z, r[u][1].z, r[u][0].w, r[u][1].w, qf.z, qf.w);
                store_scores(tile + WARPS * u, acc);
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

        // ---- 2. softmax + requantization (warp w < V / 2: lanes 2w, 2w+1) -----
        // Lane l visits slot pairs (2l, 2l+1), (2l+64, 2l+65), ...: one 32-bit
        // load of two half scores, one 16-bit (8-bit probabilities) or 32-bit
        // (16-bit) store of two probabilities.  The maximum is exact in any
        // order; the sum keeps the per-thread order and reduction tree of the
        // separate softmax kernel.  Both vector lanes of the warp and two pair
        // iterations go through each trip: their loads and exponentials are
        // independent, only the adds are chained (in each lane's order; an
        // absent slot adds +0, which leaves a sum of non-negative terms
        // unchanged).  A __syncwarp separates the scores read in a trip from
        // the probabilities written over them: 8-bit probabilities of
        // iteration k overlay scores read in iteration k / 2 or earlier,
        // 16-bit ones the lane's own scores of the same iteration.
        const int npit = (nround + 63) >> 6;
        if (2 * warp < V) {  // V is even: the warp holds lanes 2w and 2w + 1
            const int va = 2 * warp;
            const __half* sa = S + va * SP;
            const __half* sb = sa + SP;
            float mxa = MAXW[va], mxb = MAXW[va + 1];
#pragma unroll
            for (int w = 1; w < WARPS; ++w) {
                mxa = fmaxf(mxa, MAXW[w * 8 + va]);
                mxb = fmaxf(mxb, MAXW[w * 8 + va + 1]);
            }
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
                auto q = [&](float e, float rs) { return (int)fminf(fmaxf(e * rs, LO), HI); };
                for (int i = 0; i < npit; i += 2) {
                    const int j0 = 64 * i + 2 * lane, j1 = j0 + 64;
                    const float2 xa0 = ld2(sa, j0), xb0 = ld2(sb, j0), xa1 = ld2(sa, j1), xb1 = ld2(sb, j1);
                    const float ea[4] = {ex(xa0.x, mxa, j0), ex(xa0.y, mxa, j0 + 1), ex(xa1.x, mxa, j1),
                                         ex(xa1.y, mxa, j1 + 1)};
                    const float eb[4] = {ex(xb0.x, mxb, j0), ex(xb0.y, mxb, j0 + 1), ex(xb1.x, mxb, j1),
                                         ex(xb1.y, mxb, j1 + 1)};
                    __syncwarp();
                    if constexpr (LB == 8) {
                        auto q2 = [&](float e0, float e1, float rs) {
                            return (uint16_t)((q(e0, rs) & 0xFF) | ((q(e1, rs) & 0xFF) << 8));
                        };
                        if (j0 < nround) {
                            *reinterpret_cast<uint16_t*>(pa + j0) = q2(ea[0], ea[1], rsa);
                            *reinterpret_cast<uint16_t*>(pb + j0) = q2(eb[0], eb[1], rsb);
                        }
                        if (j1 < nround) {
                            *reinterpret_cast<uint16_t*>(pa + j1) = q2(ea[2], ea[3], rsa);
                            *reinterpret_cast<uint16_t*>(pb + j1) = q2(eb[2], eb[3], rsb);
                        }
                    } else {
                        auto q2 = [&](float e0, float e1, float rs) {
                            return (uint32_t)(q(e0, rs) & 0xFFFF) | ((uint32_t)q(e1, rs) << 16);
                        };
                        if (j0 < nround) {
                            *reinterpret_cast<uint32_t*>(pa + 2 * j0) = q2(ea[0], ea[1], rsa);
                            *reinterpret_cast<uint32_t*>(pb + 2 * j0) = q2(eb[0], eb[1], rsb);
                        }
                        if (j1 < nround) {
                            *reinterpret_cast<uint32_t*>(pa + 2 * j1) = q2(ea[2], ea[3], rsa);
                            *reinterpret_cast<uint32_t*>(pb + 2 * j1) = q2(eb[2], eb[3], rsb);
                        }
                    }
                }
            }
            if (lane == 0) {
                DEN[va] = ROWMAX ? 127.f * suma * p.out_scale : p.out_scale;
                DEN[va + 1] = ROWMAX ? 127.f * sumb * p.out_scale : p.out_scale;
            }
        }
        __syncthreads();

        // ---- 3. out = P x V rows: warp w takes steps w, w + WARPS, ... (k-split) -
        // Each step's 32 gathered V rows sit in the warp's private ring; the
        // warp multiplies all 64 output columns (four 16-column tiles sharing
        // the P fragment; a second accumulator set for the low byte plane of
        // 16-bit probabilities).  No CTA barrier inside.
        int acc[4][4] = {};
        int acc_lo[LB == 16 ? 4 : 1][4] = {};
        int slot = 0;
#pragma unroll 1
        for (int s = warp; s < steps; s += WARPS) {
            // step s sits in `slot` (requested STAGES steps earlier, or at item start)
            cp_async_wait<STAGES - 1>();
            __syncwarp();
            const uint8_t* st = ring + slot * STEP;
            uint32_t b0 = 0, b1 = 0, c0 = 0, c1 = 0;  // P fragment: high (or only) plane b, low plane c
            if (g < V) {
                if constexpr (LB == 8) {
                    b0 = lds32(P + g * PP + s * 32 + 4 * t);
                    b1 = lds32(P + g * PP + s * 32 + 16 + 4 * t);
                } else {
                    // slots 4t .. 4t+3 as int16 [lo hi] pairs: split the planes
                    const uint2 w0 = lds64(P + g * PP + 2 * (s * 32 + 4 * t));
                    const uint2 w1 = lds64(P + g * PP + 2 * (s * 32 + 16 + 4 * t));
                    c0 = prmt(w0.x, w0.y, 0x6420);
                    b0 = prmt(w0.x, w0.y, 0x7531);
                    c1 = prmt(w1.x, w1.y, 0x6420);
                    b1 = prmt(w1.x, w1.y, 0x7531);
                }
            }
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                uint32_t a[4];
                if constexpr (RB == 8) {
                    ldsm_x2_trans_b8_a(a, st + lane * QROW + ((m ^ ((lane >> 1) & 3)) << 4));
                } else {
                    // chunk m / 2 holds 32 nibble columns: low nibbles are the
                    // even columns, high nibbles the odd ones (as 16 x value)
                    uint32_t x[4];
                    ldsm_x2_trans_b8_a(x, st + lane * QROW + (((m >> 1) ^ ((lane >> 2) & 1)) << 4));
#pragma unroll
                    for (int e = 0; e < 4; ++e) a[e] = (m & 1) ? (x[e] & 0xF0F0F0F0u) : ((x[e] << 4) & 0xF0F0F0F0u);
                }
                mma_k32<true, true>(acc[m], a[0], a[1], a[2], a[3], b0, b1);
                if constexpr (LB == 16) mma_k32<true, false>(acc_lo[m], a[0], a[1], a[2], a[3], c0, c1);
            }
            __syncwarp();  // every lane is done with this slot before it is refilled
            issue(s + STAGES * WARPS, slot);
            slot = slot + 1 == STAGES ? 0 : slot + 1;
        }
        if constexpr (LB == 16) {
#pragma unroll
            for (int m = 0; m < 4; ++m)
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    acc[m][e] = (int)(((uint32_t)acc[m][e] << 8) + (uint32_t)acc_lo[m][e]);
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
        // Warp w finishes tile m = w (four warps: all four accumulators of the
        // tile) or tile w / 2, accumulators 2 (w & 1) and 2 (w & 1) + 1 (eight
        // warps).  Accumulator e of lane (g, t): tile row g + 8 (e >> 1),
        // vector lane 2t + (e & 1).
        constexpr int EPW = 16 / WARPS;  // accumulators finished per warp
        const int mt = WARPS == 4 ? warp : warp >> 1;
        const int e0 = WARPS == 4 ? 0 : 2 * (warp & 1);
        int tot[EPW];
#pragma unroll
        for (int i = 0; i < EPW; ++i) {
            uint32_t x = 0;
#pragma unroll
            for (int w = 0; w < WARPS; ++w)
                x += (uint32_t)reinterpret_cast<const int*>(rings + w * STAGES * STEP)[(mt * 4 + e0 + i) * 32 + lane];
            tot[i] = RB == 8 ? (int)x : ((int)x >> 4);
        }
        if (2 * t < V) {
            // output column of tile row r: 16 mt + r (8-bit V), or 32 (mt / 2)
            // + 2 r + (mt & 1) (4-bit V: even / odd nibble tiles)
            auto col = [&](int r) { return RB == 8 ? 16 * mt + r : 32 * (mt >> 1) + 2 * r + (mt & 1); };
            __half* o = p.out + (long long)h * p.out_head_stride + (long long)(row * V + 2 * t) * 64;
            const Divisor d0 = make_divisor(DEN[2 * t]), d1 = make_divisor(DEN[2 * t + 1]);
#pragma unroll
            for (int i = 0; i < EPW; i += 2) {
                const int r = g + 8 * ((e0 + i) >> 1);
                const __half2 hv = deq_half2(tot[i], tot[i + 1], d0, d1);
                o[col(r)] = __low2half(hv);
                o[64 + col(r)] = __high2half(hv);
            }
        }
    }
}

}  // namespace mc

namespace mc {

// Launch on as many CTAs as fit (or `ctas_per_sm` per SM when it is smaller),
// never more than there are items.
template <int V, bool ROWMAX, int LB, int RB, int WARPS, int STAGES>
int attention_launch(const AttnParams& p, int ctas_per_sm, cudaStream_t s)
{
    auto kern = sparse_attention_kernel<V, ROWMAX, LB, RB, WARPS, STAGES>;
    const size_t smem = attn_smem_bytes(V, p.nnzp, WARPS, attn_ring_bytes<WARPS, STAGES, RB>());
    if (smem > 227 * 1024) return fail(1, "mcSparseAttention: shared memory of this configuration exceeds 227 KB");
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return (int)cudaGetLastError();
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WARPS * 32, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long grid = (long long)per_sm * sms;
    if (grid > p.items) grid = p.items;
    kern<<<(unsigned)(grid < 1 ? 1 : grid), WARPS * 32, smem, s>>>(p);
    return (int)cudaGetLastError();
}

// Every (V, requantization mode, warps, stages) of one precision pair; each
// pair's instantiations live in their own translation unit.
template <int LB, int RB>
int attention_dispatch(const AttnParams& p, int V, bool rowmax, int warps, int stages, int ctas_per_sm,
                       cudaStream_t s)
{
#define MC_ATTN_CASE(VV, RM, W, ST)                                                   \
    if (V == VV && rowmax == RM && warps == W && stages == ST)                        \
        return attention_launch<VV, RM, LB, RB, W, ST>(p, ctas_per_sm, s);
#define MC_ATTN_WS(VV, RM) \
    MC_ATTN_CASE(VV, RM, 4, 2) MC_ATTN_CASE(VV, RM, 4, 3) MC_ATTN_CASE(VV, RM, 8, 2) MC_ATTN_CASE(VV, RM, 8, 3)
    MC_ATTN_WS(2, false) MC_ATTN_WS(4, false) MC_ATTN_WS(8, false)
    if constexpr (LB == 8) {
        MC_ATTN_WS(2, true) MC_ATTN_WS(4, true) MC_ATTN_WS(8, true)
    }
#undef MC_ATTN_WS
#undef MC_ATTN_CASE
    return fail(1, "mcSparseAttention: unsupported configuration (warps 4 or 8, stages 2 or 3)");
}

int attention_dispatch_8_8(const AttnParams&, int, bool, int, int, int, cudaStream_t);
int attention_dispatch_16_8(const AttnParams&, int, bool, int, int, int, cudaStream_t);
int attention_dispatch_8_4(const AttnParams&, int, bool, int, int, int, cudaStream_t);

}  // namespace mc
