// mc_sddmm_stream.cuh -- pipelined SDDMM for k == 64.
//
// Same operands and results as mc_sddmm.cuh's sddmm_kernel for k == 64 (the
// head dimension of the sparse-attention path and of the SDDMM benchmark
// configuration), with the per-tile work cut to what the data needs:
//
//  * k == 64 is one 64-element block: the V rows of A are loaded once per
//    vector-row and every tile is two mma.m16n8k32 (per byte-plane pair) with
//    no inner k loop.
//  * Each warp keeps U tiles of 16 nonzeros in flight: the gathered B rows of
//    all U are requested before any is multiplied, and the column indices of
//    the warp's next U tiles are fetched while the current ones are
//    multiplied and stored.  Latency is hidden by resident warps rather than
//    by depth within a warp (see U below).
//  * Per-row pointers are formed once; per-tile offsets are 32-bit.
// U = 1 is the measured optimum on GB300 for the 4096x4096x64 V=8 L8-R8 case:
// 32 registers per thread, 16 resident CTAs (64 warps) per SM, 124 TOP/s.
// More tiles in flight per warp cost registers and with them resident warps
// (U = 2: 56 registers, 114 TOP/s; U = 3: 108; U = 4: 78 registers, 97; U = 2
// capped at 48 registers spills: 101).
// The kernel is latency/issue bound rather than HBM bound on GB300 (the
// sm_103a int8 tensor path is the slow legacy mma.sync), so instruction count
// per tile is what sets its speed.
#pragma once
#include "mc_sddmm.cuh"

namespace mc {

template <int V, int PREA, int PREB, bool SIGNED, bool VECMAJOR, bool HALF_OUT, int WARPS, bool F16, int U = 1>
__global__ void __launch_bounds__(WARPS * 32)
sddmm_k64_kernel(const SddmmParams p)
{
    const Divisor dq = make_divisor(p.scale);  // half output: acc / scale
    constexpr int PA = BytePlanes<PREA>::N, PB = BytePlanes<PREB>::N;
    constexpr int RHS_ROW = 64 * PREB / 8, LHS_ROW = 64 * PREA / 8;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const int row = __ldg(p.row_indices + blockIdx.x);
    const int b = blockIdx.z;
    const int start = __ldg(p.row_offsets + 2 * row);
    const int nnz = __ldg(p.row_offsets + 2 * row + 1) - start;
    const int nnz8 = (nnz + 7) & ~7;
    const int ntiles = (nnz8 + 15) >> 4;
    const int stride = gridDim.y * WARPS;  // tile stride between this warp's tiles
    int ti = blockIdx.y * WARPS + warp;
    if (ti >= ntiles) return;

    const int* cols = p.col_indices + start;
    const uint8_t* rhs = p.rhs + (long long)b * p.rhs_stride;
    // L4-R4 on the int8 MMA: both operands as 16 x nibble bytes, the sums 256 x
    // the result (|result| <= 64 x 64 for k = 64: no wrap), shifted back below
    constexpr bool HI4 = PREA == 4 && PREB == 4 && !F16;

    uint32_t a[2][4] = {};
    if (g < V) {
        const uint8_t* arow = p.lhs + (long long)b * p.lhs_stride + (long long)(row * V + g) * LHS_ROW;
        if constexpr (HI4) load_kfrag_hi4(arow, 0, t, a);
        else load_kfrag<PREA, SIGNED>(arow, 0, t, a);
    }
    uint32_t ah[PA][8];
    if constexpr (F16) {
#pragma unroll
        for (int lb = 0; lb < PA; ++lb)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (SIGNED && lb == PA - 1) bytes_to_h2<true>(a[lb][q], ah[lb][2 * q], ah[lb][2 * q + 1]);
                else bytes_to_h2<false>(a[lb][q], ah[lb][2 * q], ah[lb][2 * q + 1]);
            }
    }
    // start is a multiple of 8, so both output layouts are start*V plus a
    // row-relative offset.
    const long long obase = (long long)b * p.out_stride + (long long)start * V;

    auto load_cols = [&](int tile, int (&cc)[2]) {
        const int j0 = tile * 16 + g;
        cc[0] = j0 < nnz ? __ldg(cols + j0) : -1;
        cc[1] = j0 + 8 < nnz ? __ldg(cols + j0 + 8) : -1;
    };

    int c[U][2];
#pragma unroll
    for (int u = 0; u < U; ++u) load_cols(ti + u * stride, c[u]);

#pragma unroll 1
    for (; ti < ntiles; ti += U * stride) {
        uint32_t r[U][2][2][4];  // [tile][row half][byte plane][word]
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int hf = 0; hf < 2; ++hf) {
#pragma unroll
                for (int q = 0; q < 2; ++q)
#pragma unroll
                    for (int e = 0; e < 4; ++e) r[u][hf][q][e] = 0u;
                if (c[u][hf] >= 0) {
                    if constexpr (HI4) load_kfrag_hi4(rhs + (unsigned)c[u][hf] * RHS_ROW, 0, t, r[u][hf]);
                    else load_kfrag<PREB, SIGNED>(rhs + (unsigned)c[u][hf] * RHS_ROW, 0, t, r[u][hf]);
                }
            }
        int cn[U][2];
#pragma unroll
        for (int u = 0; u < U; ++u) load_cols(ti + (U + u) * stride, cn[u]);

#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int tile = ti + u * stride;
            if (tile >= ntiles) break;
            int d[4];
            if constexpr (F16) {
                float facc[PB][PA][4] = {};
#pragma unroll
                for (int rb = 0; rb < PB; ++rb) {
                    const bool rs = SIGNED && (rb == PB - 1);
                    uint32_t h0[8], h1[8];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        if (rs) { bytes_to_h2<true>(r[u][0][rb][q], h0[2 * q], h0[2 * q + 1]); bytes_to_h2<true>(r[u][1][rb][q], h1[2 * q], h1[2 * q + 1]); }
                        else { bytes_to_h2<false>(r[u][0][rb][q], h0[2 * q], h0[2 * q + 1]); bytes_to_h2<false>(r[u][1][rb][q], h1[2 * q], h1[2 * q + 1]); }
                    }
#pragma unroll
                    for (int lb = 0; lb < PA; ++lb)
#pragma unroll
                        for (int m = 0; m < 4; ++m)
                            mma_f16(facc[rb][lb], h0[2 * m], h1[2 * m], h0[2 * m + 1], h1[2 * m + 1], ah[lb][2 * m], ah[lb][2 * m + 1]);
                }
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    uint32_t s = 0;
#pragma unroll
                    for (int rb = 0; rb < PB; ++rb)
#pragma unroll
                        for (int lb = 0; lb < PA; ++lb) s += (uint32_t)f2i_exact(facc[rb][lb][e]) << (8 * (rb + lb));
                    d[e] = (int)s;
                }
            } else {
                int acc[PB][PA][4] = {};
#pragma unroll
                for (int rb = 0; rb < PB; ++rb) {
#pragma unroll
                    for (int lb = 0; lb < PA; ++lb) {
                        const bool rs = SIGNED && (rb == PB - 1);
                        const bool ls = SIGNED && (lb == PA - 1);
#define MC_K64_MMA(RS, LS)                                                                                      \
    mma_k32<RS, LS>(acc[rb][lb], r[u][0][rb][0], r[u][1][rb][0], r[u][0][rb][1], r[u][1][rb][1], a[lb][0], a[lb][1]); \
    mma_k32<RS, LS>(acc[rb][lb], r[u][0][rb][2], r[u][1][rb][2], r[u][0][rb][3], r[u][1][rb][3], a[lb][2], a[lb][3]);
                        if (rs && ls) { MC_K64_MMA(true, true) }
                        else if (rs) { MC_K64_MMA(true, false) }
                        else if (ls) { MC_K64_MMA(false, true) }
                        else { MC_K64_MMA(false, false) }
#undef MC_K64_MMA
                    }
                }
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    uint32_t s = 0;
#pragma unroll
                    for (int rb = 0; rb < PB; ++rb)
#pragma unroll
                        for (int lb = 0; lb < PA; ++lb) s += (uint32_t)acc[rb][lb][e] << (8 * (rb + lb));
                    d[e] = HI4 ? ((int)s >> 8) : (int)s;
                }
            }
            // d[0..1]: nonzero tile*16 + g, lanes 2t, 2t+1; d[2..3]: nonzero + 8.
            if (2 * t < V) {
#pragma unroll
                for (int hh = 0; hh < 2; ++hh) {
                    const int jl = tile * 16 + g + 8 * hh;
                    if (jl >= nnz8) continue;
                    if constexpr (VECMAJOR) {
                        const long long o = obase + jl * V + 2 * t;
                        if constexpr (HALF_OUT)
                            stg_cs_s32(reinterpret_cast<__half*>(p.out) + o, (int)pack_half2(d[2 * hh], d[2 * hh + 1], dq));
                        else
                            stg_cs_v2(reinterpret_cast<int*>(p.out) + o, d[2 * hh], d[2 * hh + 1]);
                    } else {
                        const long long o = obase + (jl >> 3) * 8 * V + 16 * t + (jl & 7);
                        if constexpr (HALF_OUT) {
                            __half* out = reinterpret_cast<__half*>(p.out) + o;
                            out[0] = deq_half(d[2 * hh], dq);
                            out[8] = deq_half(d[2 * hh + 1], dq);
                        } else {
                            int* out = reinterpret_cast<int*>(p.out) + o;
                            stg_cs_s32(out, d[2 * hh]);
                            stg_cs_s32(out + 8, d[2 * hh + 1]);
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) { c[u][0] = cn[u][0]; c[u][1] = cn[u][1]; }
    }
}

}  // namespace mc
