// mc_sddmm.cuh -- quantized vector-sparse SDDMM for sm_103a.
//
// out[j, v] = sum_k A[row*V + v][k] * B[col_j][k] for every stored nonzero
// vector j of every vector-row (out = (A * B^T) restricted to the mask).
// Operand and output layouts are those of the reference's
// sddmm::wmmaSddmm_* (SDDMM/SDDMM/src/wmma_sddmm.cu) and of the torch
// extension's deq_sddmm (sparse_transformer_magicube/src/cuda/deq_sddmm_kernel.cu).
//
// Design:
//  * One warp processes 16 stored nonzeros ("tile") at a time.  The MMA
//    computes D[16 nonzeros][8 vector lanes]: the A operand is the 16 gathered
//    rows of B, the B operand the V rows of A, both k-contiguous in memory, so
//    each thread fetches one 16-byte run per gathered row with a coalesced
//    128-bit load and feeds it to mma.m16n8k32 without any transposition (the
//    k order inside a 64-element block is permuted identically on both
//    operands, which leaves each dot product unchanged).
//  * The V rows of A for the first 64-element k block stay in registers for
//    the whole vector-row.
//  * 4-bit operands are unpacked to int8 in registers; 16-bit operands are
//    split into an unsigned low and a (signed) high byte plane and the partial
//    products are recombined by exact shift-add.
//  * Padding slots inside the last group of 8 are written as zero; results
//    wrap modulo 2^32.
#pragma once
#include "mc_ptx.cuh"

namespace mc {

struct SddmmParams {
    int m_vec, n, k;
    const int* row_indices;   // m_vec entries
    const int* row_offsets;   // 2*m_vec: [start, end)
    const int* col_indices;   // aligned, -1 padded
    const uint8_t* lhs;       // M x K packed
    long long lhs_stride;     // bytes between batch entries
    const uint8_t* rhs;       // N x K packed
    long long rhs_stride;     // bytes between batch entries
    void* out;                // int32 or half
    long long out_stride;     // elements between batch entries
    float scale;
};

// 16 consecutive k elements (16t .. 16t+15 of k block kb) of one packed row,
// as int8 byte planes: pl[0] = the value (8-bit / unpacked 4-bit) or the low
// byte (16-bit), pl[1] = the high byte (16-bit only).
template <int BITS, bool SIGNED>
__device__ __forceinline__ void load_kfrag(const uint8_t* row, int kb, int t, uint32_t (&pl)[2][4])
{
    if constexpr (BITS == 8) {
        int4 v = ldg_nc_v4(row + kb * 64 + 16 * t);
        pl[0][0] = v.x; pl[0][1] = v.y; pl[0][2] = v.z; pl[0][3] = v.w;
    } else if constexpr (BITS == 4) {
        int2 v = ldg_nc_v2(row + kb * 32 + 8 * t);
        unpack4_u32<SIGNED>((uint32_t)v.x, pl[0][0], pl[0][1]);
        unpack4_u32<SIGNED>((uint32_t)v.y, pl[0][2], pl[0][3]);
    } else {
        int4 v0 = ldg_nc_v4(row + kb * 128 + 32 * t);
        int4 v1 = ldg_nc_v4(row + kb * 128 + 32 * t + 16);
        const uint32_t w[8] = {(uint32_t)v0.x, (uint32_t)v0.y, (uint32_t)v0.z, (uint32_t)v0.w,
                               (uint32_t)v1.x, (uint32_t)v1.y, (uint32_t)v1.z, (uint32_t)v1.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            pl[0][q] = prmt(w[2 * q], w[2 * q + 1], 0x6420);
            pl[1][q] = prmt(w[2 * q], w[2 * q + 1], 0x7531);
        }
    }
}

// The same 16 k elements of a 4-bit row with each nibble in its byte's high
// half (16 x the value, see unpack4_hi_u32).
__device__ __forceinline__ void load_kfrag_hi4(const uint8_t* row, int kb, int t, uint32_t (&pl)[2][4])
{
    int2 v = ldg_nc_v2(row + kb * 32 + 8 * t);
    unpack4_hi_u32((uint32_t)v.x, pl[0][0], pl[0][1]);
    unpack4_hi_u32((uint32_t)v.y, pl[0][2], pl[0][3]);
}

template <int BITS>
struct BytePlanes { static constexpr int N = BITS == 16 ? 2 : 1; };

// F16: run the contraction on the f16 tensor path (mma.m16n8k16, f32
// accumulators) instead of the int8 one.  Every operand byte is converted
// exactly to f16; products are exact in f32 and the f32 partial sums are
// integers bounded by 256 * 255^2 < 2^24 between flushes into the int32
// accumulators (every 256 k elements), so no rounding ever happens and the
// result is the same integer as the int8 path's.
template <int V, int PREA, int PREB, bool SIGNED, bool VECMAJOR, bool HALF_OUT, int WARPS, bool F16>
__global__ void __launch_bounds__(WARPS * 32)
sddmm_kernel(const SddmmParams p)
{
    const Divisor dq = make_divisor(p.scale);  // half output: acc / scale
    constexpr int PA = BytePlanes<PREA>::N, PB = BytePlanes<PREB>::N;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const int row = __ldg(p.row_indices + blockIdx.x);
    const int b = blockIdx.z;
    const int start = __ldg(p.row_offsets + 2 * row);
    const int nnz = __ldg(p.row_offsets + 2 * row + 1) - start;
    const int nnz8 = (nnz + 7) & ~7;
    const int ntiles = (nnz8 + 15) >> 4;
    const int kblocks = p.k >> 6;

    const long long lhs_row_bytes = (long long)p.k * PREA / 8;
    const long long rhs_row_bytes = (long long)p.k * PREB / 8;
    const uint8_t* lhs_row = p.lhs + (long long)b * p.lhs_stride + (long long)(row * V + g) * lhs_row_bytes;
    const uint8_t* rhs = p.rhs + (long long)b * p.rhs_stride;
    const int* cols = p.col_indices + start;

    // Rows of A for k block 0 (lane g holds vector lane v = g).
    uint32_t a0[2][4] = {};
    if (g < V) load_kfrag<PREA, SIGNED>(lhs_row, 0, t, a0);
    // ... and their f16 form for the F16 path.
    uint32_t a0h[PA][8];
    if constexpr (F16) {
#pragma unroll
        for (int lb = 0; lb < PA; ++lb)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (SIGNED && lb == PA - 1) bytes_to_h2<true>(a0[lb][q], a0h[lb][2 * q], a0h[lb][2 * q + 1]);
                else bytes_to_h2<false>(a0[lb][q], a0h[lb][2 * q], a0h[lb][2 * q + 1]);
            }
    }

#pragma unroll 1
    for (int ti = blockIdx.y * WARPS + warp; ti < ntiles; ti += gridDim.y * WARPS) {
        const int jl0 = ti * 16 + g, jl1 = jl0 + 8;
        const int c0 = jl0 < nnz ? __ldg(cols + jl0) : -1;
        const int c1 = jl1 < nnz ? __ldg(cols + jl1) : -1;
        int acc[PB][PA][4] = {};
        float facc[PB][PA][4] = {};

#pragma unroll 1
        for (int kb = 0; kb < kblocks; ++kb) {
            uint32_t r0[2][4] = {}, r1[2][4] = {};
            if (c0 >= 0) load_kfrag<PREB, SIGNED>(rhs + (long long)c0 * rhs_row_bytes, kb, t, r0);
            if (c1 >= 0) load_kfrag<PREB, SIGNED>(rhs + (long long)c1 * rhs_row_bytes, kb, t, r1);
            if constexpr (F16) {
                uint32_t ah[PA][8];
                if (kb == 0) {
#pragma unroll
                    for (int lb = 0; lb < PA; ++lb)
#pragma unroll
                        for (int e = 0; e < 8; ++e) ah[lb][e] = a0h[lb][e];
                } else {
                    uint32_t av[2][4] = {};
                    if (g < V) load_kfrag<PREA, SIGNED>(lhs_row, kb, t, av);
#pragma unroll
                    for (int lb = 0; lb < PA; ++lb)
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            if (SIGNED && lb == PA - 1) bytes_to_h2<true>(av[lb][q], ah[lb][2 * q], ah[lb][2 * q + 1]);
                            else bytes_to_h2<false>(av[lb][q], ah[lb][2 * q], ah[lb][2 * q + 1]);
                        }
                }
#pragma unroll
                for (int rb = 0; rb < PB; ++rb) {
                    uint32_t h0[8], h1[8];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        if (SIGNED && rb == PB - 1) {
                            bytes_to_h2<true>(r0[rb][q], h0[2 * q], h0[2 * q + 1]);
                            bytes_to_h2<true>(r1[rb][q], h1[2 * q], h1[2 * q + 1]);
                        } else {
                            bytes_to_h2<false>(r0[rb][q], h0[2 * q], h0[2 * q + 1]);
                            bytes_to_h2<false>(r1[rb][q], h1[2 * q], h1[2 * q + 1]);
                        }
                    }
#pragma unroll
                    for (int lb = 0; lb < PA; ++lb)
#pragma unroll
                        for (int m = 0; m < 4; ++m)
                            mma_f16(facc[rb][lb], h0[2 * m], h1[2 * m], h0[2 * m + 1], h1[2 * m + 1], ah[lb][2 * m],
                                    ah[lb][2 * m + 1]);
                }
                if ((kb & 3) == 3 || kb == kblocks - 1) {
#pragma unroll
                    for (int rb = 0; rb < PB; ++rb)
#pragma unroll
                        for (int lb = 0; lb < PA; ++lb)
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                acc[rb][lb][e] = (int)((uint32_t)acc[rb][lb][e] + (uint32_t)f2i_exact(facc[rb][lb][e]));
                                facc[rb][lb][e] = 0.f;
                            }
                }
                continue;
            }
            uint32_t av[2][4];
            if (kb == 0) {
#pragma unroll
                for (int q = 0; q < 2; ++q)
#pragma unroll
                    for (int e = 0; e < 4; ++e) av[q][e] = a0[q][e];
            } else {
#pragma unroll
                for (int q = 0; q < 2; ++q)
#pragma unroll
                    for (int e = 0; e < 4; ++e) av[q][e] = 0u;
                if (g < V) load_kfrag<PREA, SIGNED>(lhs_row, kb, t, av);
            }
#pragma unroll
            for (int rb = 0; rb < PB; ++rb) {
#pragma unroll
                for (int lb = 0; lb < PA; ++lb) {
                    // Only the most significant byte plane of a signed value is signed.
                    const bool rs = SIGNED && (rb == PB - 1);
                    const bool ls = SIGNED && (lb == PA - 1);
#define MC_SDDMM_MMA(RS, LS)                                                                        \
    mma_k32<RS, LS>(acc[rb][lb], r0[rb][0], r1[rb][0], r0[rb][1], r1[rb][1], av[lb][0], av[lb][1]); \
    mma_k32<RS, LS>(acc[rb][lb], r0[rb][2], r1[rb][2], r0[rb][3], r1[rb][3], av[lb][2], av[lb][3]);
                    if (rs && ls) { MC_SDDMM_MMA(true, true) }
                    else if (rs) { MC_SDDMM_MMA(true, false) }
                    else if (ls) { MC_SDDMM_MMA(false, true) }
                    else { MC_SDDMM_MMA(false, false) }
#undef MC_SDDMM_MMA
                }
            }
        }

        // Recombine byte-plane products: plane (rb, lb) carries weight 2^(8(rb+lb)).
        int d[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            uint32_t s = 0;
#pragma unroll
            for (int rb = 0; rb < PB; ++rb)
#pragma unroll
                for (int lb = 0; lb < PA; ++lb) s += (uint32_t)acc[rb][lb][e] << (8 * (rb + lb));
            d[e] = (int)s;
        }

        // d[0..1]: nonzero jl0, lanes 2t, 2t+1; d[2..3]: nonzero jl1.
        if (2 * t < V) {
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
                const int jl = hh ? jl1 : jl0;
                if (jl >= nnz8) continue;
                const long long j = start + jl;
                const long long base = (long long)b * p.out_stride;
                if constexpr (VECMAJOR) {
                    const long long o = base + j * V + 2 * t;
                    if constexpr (HALF_OUT) {
                        stg_cs_s32(reinterpret_cast<__half*>(p.out) + o, (int)pack_half2(d[2 * hh], d[2 * hh + 1], dq));
                    } else {
                        stg_cs_v2(reinterpret_cast<int*>(p.out) + o, d[2 * hh], d[2 * hh + 1]);
                    }
                } else {
                    // Blocked layout with alignment 8: (j/8)*8V + 8v + j%8.
                    const long long o = base + (j >> 3) * 8 * V + 8 * (2 * t) + (j & 7);
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
}

}  // namespace mc
