// mc_sddmm_stream.cuh -- persistent, warp-streaming SDDMM for k == 64.
//
// Same operands and results as mc_sddmm.cuh's sddmm_kernel for k == 64 (the
// head dimension of the sparse-attention path and of the SDDMM benchmark
// configuration).  Every warp owns the tasks (batch entry, vector-row)
// w, w + W, ... (W = warps in the grid) and walks their 16-nonzero tiles as
// one stream with a three-deep software pipeline: while tile i is multiplied
// and stored, the gathered B rows of tile i+1 and the column indices of
// tile i+2 are in flight.  The V rows of A are fetched with the first tile
// of each task.  Keeping several independent loads per warp in flight is
// what the original one-tile-at-a-time loop lacked (latency-bound).
#pragma once
#include "mc_sddmm.cuh"

namespace mc {

struct SdTile {
    int task, tile, ntiles, row, b, start, nnz, nnz8;
};

template <int V, int PREA, int PREB, bool SIGNED, bool VECMAJOR, bool HALF_OUT, int WARPS, bool F16>
__global__ void __launch_bounds__(WARPS * 32)
sddmm_stream_kernel(const SddmmParams p, const int ntasks)
{
    constexpr int PA = BytePlanes<PREA>::N, PB = BytePlanes<PREB>::N;
    constexpr long long LHS_ROW = 64 * PREA / 8, RHS_ROW = 64 * PREB / 8;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const int W = gridDim.x * WARPS;

    auto load_task = [&](SdTile& c, int task) {
        for (;; task += W) {
            c.task = task;
            c.tile = 0;
            c.ntiles = 0;
            if (task >= ntasks) return;
            c.b = task / p.m_vec;
            c.row = __ldg(p.row_indices + (task - c.b * p.m_vec));
            c.start = __ldg(p.row_offsets + 2 * c.row);
            c.nnz = __ldg(p.row_offsets + 2 * c.row + 1) - c.start;
            c.nnz8 = (c.nnz + 7) & ~7;
            c.ntiles = (c.nnz8 + 15) >> 4;
            if (c.ntiles > 0) return;  // skip vector-rows without nonzeros
        }
    };
    auto advance = [&](SdTile& c) {
        if (c.task >= ntasks) return;
        if (++c.tile >= c.ntiles) load_task(c, c.task + W);
    };
    auto load_cols = [&](const SdTile& c, int& c0, int& c1) {
        c0 = c1 = -1;
        if (c.task >= ntasks) return;
        const int jl0 = c.tile * 16 + g, jl1 = jl0 + 8;
        const int* cols = p.col_indices + c.start;
        if (jl0 < c.nnz) c0 = __ldg(cols + jl0);
        if (jl1 < c.nnz) c1 = __ldg(cols + jl1);
    };
    auto load_rhs = [&](const SdTile& c, int c0, int c1, uint32_t (&r0)[2][4], uint32_t (&r1)[2][4]) {
#pragma unroll
        for (int q = 0; q < 2; ++q)
#pragma unroll
            for (int e = 0; e < 4; ++e) { r0[q][e] = 0u; r1[q][e] = 0u; }
        if (c.task >= ntasks) return;
        const uint8_t* rhs = p.rhs + (long long)c.b * p.rhs_stride;
        if (c0 >= 0) load_kfrag<PREB, SIGNED>(rhs + (long long)c0 * RHS_ROW, 0, t, r0);
        if (c1 >= 0) load_kfrag<PREB, SIGNED>(rhs + (long long)c1 * RHS_ROW, 0, t, r1);
    };
    auto load_lhs = [&](const SdTile& c, uint32_t (&a)[2][4]) {
#pragma unroll
        for (int q = 0; q < 2; ++q)
#pragma unroll
            for (int e = 0; e < 4; ++e) a[q][e] = 0u;
        if (c.task >= ntasks || g >= V) return;
        load_kfrag<PREA, SIGNED>(p.lhs + (long long)c.b * p.lhs_stride + (long long)(c.row * V + g) * LHS_ROW, 0, t, a);
    };

    // Cursors: A = tile being computed, B = its successor (B rows in flight),
    // C = the one after (column indices in flight).
    SdTile A, B, C;
    uint32_t rA0[2][4], rA1[2][4], rB0[2][4], rB1[2][4], lA[2][4], lB[2][4];
    int cB0, cB1, cC0, cC1;

    load_task(A, blockIdx.x * WARPS + warp);
    {
        int a0, a1;
        load_cols(A, a0, a1);
        load_rhs(A, a0, a1, rA0, rA1);
        load_lhs(A, lA);
    }
    B = A;
    advance(B);
    load_cols(B, cB0, cB1);
    C = B;
    advance(C);
    load_cols(C, cC0, cC1);

#pragma unroll 1
    while (A.task < ntasks) {
        // 1. gathered rows (and, on a new task, the rows of A) for tile B
        load_rhs(B, cB0, cB1, rB0, rB1);
        if (B.tile == 0) load_lhs(B, lB);

        // 2. tile A
        int acc[PB][PA][4] = {};
        float facc[PB][PA][4] = {};
#pragma unroll
        for (int rb = 0; rb < PB; ++rb) {
#pragma unroll
            for (int lb = 0; lb < PA; ++lb) {
                const bool rs = SIGNED && (rb == PB - 1);
                const bool ls = SIGNED && (lb == PA - 1);
                if constexpr (F16) {
                    uint32_t h0[8], h1[8], ah[8];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        if (rs) { bytes_to_h2<true>(rA0[rb][q], h0[2 * q], h0[2 * q + 1]); bytes_to_h2<true>(rA1[rb][q], h1[2 * q], h1[2 * q + 1]); }
                        else { bytes_to_h2<false>(rA0[rb][q], h0[2 * q], h0[2 * q + 1]); bytes_to_h2<false>(rA1[rb][q], h1[2 * q], h1[2 * q + 1]); }
                        if (ls) bytes_to_h2<true>(lA[lb][q], ah[2 * q], ah[2 * q + 1]);
                        else bytes_to_h2<false>(lA[lb][q], ah[2 * q], ah[2 * q + 1]);
                    }
#pragma unroll
                    for (int m = 0; m < 4; ++m)
                        mma_f16(facc[rb][lb], h0[2 * m], h1[2 * m], h0[2 * m + 1], h1[2 * m + 1], ah[2 * m], ah[2 * m + 1]);
                } else {
#define MC_SD_MMA(RS, LS)                                                                                  \
    mma_k32<RS, LS>(acc[rb][lb], rA0[rb][0], rA1[rb][0], rA0[rb][1], rA1[rb][1], lA[lb][0], lA[lb][1]);    \
    mma_k32<RS, LS>(acc[rb][lb], rA0[rb][2], rA1[rb][2], rA0[rb][3], rA1[rb][3], lA[lb][2], lA[lb][3]);
                    if (rs && ls) { MC_SD_MMA(true, true) }
                    else if (rs) { MC_SD_MMA(true, false) }
                    else if (ls) { MC_SD_MMA(false, true) }
                    else { MC_SD_MMA(false, false) }
#undef MC_SD_MMA
                }
            }
        }
        int d[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            uint32_t s = 0;
#pragma unroll
            for (int rb = 0; rb < PB; ++rb)
#pragma unroll
                for (int lb = 0; lb < PA; ++lb) {
                    const uint32_t x = F16 ? (uint32_t)f2i_exact(facc[rb][lb][e]) : (uint32_t)acc[rb][lb][e];
                    s += x << (8 * (rb + lb));
                }
            d[e] = (int)s;
        }
        if (2 * t < V) {
            const long long base = (long long)A.b * p.out_stride;
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int jl = A.tile * 16 + g + 8 * hh;
                if (jl >= A.nnz8) continue;
                const long long j = A.start + jl;
                if constexpr (VECMAJOR) {
                    const long long o = base + j * V + 2 * t;
                    if constexpr (HALF_OUT)
                        stg_cs_s32(reinterpret_cast<__half*>(p.out) + o, (int)pack_half2(d[2 * hh], d[2 * hh + 1], p.scale));
                    else
                        stg_cs_v2(reinterpret_cast<int*>(p.out) + o, d[2 * hh], d[2 * hh + 1]);
                } else {
                    const long long o = base + (j >> 3) * 8 * V + 8 * (2 * t) + (j & 7);
                    if constexpr (HALF_OUT) {
                        __half* out = reinterpret_cast<__half*>(p.out) + o;
                        out[0] = deq_half(d[2 * hh], p.scale);
                        out[8] = deq_half(d[2 * hh + 1], p.scale);
                    } else {
                        int* out = reinterpret_cast<int*>(p.out) + o;
                        stg_cs_s32(out, d[2 * hh]);
                        stg_cs_s32(out + 8, d[2 * hh + 1]);
                    }
                }
            }
        }

        // 3. rotate the pipeline
        const bool new_task = (B.tile == 0);
        A = B;
#pragma unroll
        for (int q = 0; q < 2; ++q)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                rA0[q][e] = rB0[q][e];
                rA1[q][e] = rB1[q][e];
                if (new_task) lA[q][e] = lB[q][e];
            }
        B = C;
        cB0 = cC0;
        cB1 = cC1;
        advance(C);
        load_cols(C, cC0, cC1);
    }
}

}  // namespace mc
