// mc_sddmm_dp4a.cuh -- SDDMM on the CUDA cores with dp4a (8-bit and 4-bit
// operands).
//
// Same operands and results as mc_sddmm.cuh's sddmm_kernel.  An mma.m16n8k32
// always computes 8 vector lanes, so at V = 4 and V = 2 half and three
// quarters of every int8 MMA are padding; dp4a computes exactly the V lanes a
// vector-row has.  On GB300 dp4a.s32 runs at the rate of the int8 mma.sync
// path (about 159 TOP/s each, measured), so V = 2 and V = 4 gain up to 4x and
// 2x in arithmetic.
//
// Work layout (the int8 MMA kernel's, so the gathers stay coalesced):
//  * a warp takes 16 stored nonzeros per tile; lane (g, t) = (lane / 4,
//    lane % 4) loads the 16-byte k chunk t (k = 16t .. 16t+15 of the 64-element
//    block) of two gathered B rows, nonzeros g and g + 8 of the tile, and
//    holds chunk t of all V rows of A;
//  * it forms 4V dp4a partial dot products per row (one per vector lane);
//  * a transposing butterfly over the four k-chunk lanes finishes the sums:
//    exchange across t ^ 2 (each lane keeps one row), then across t ^ 1
//    (each lane keeps half of the vector lanes).  The lane-dependent row
//    order (a lane with t & 2 takes nonzero g + 8 as its own row) and vector
//    lane order (a lane with t & 1 holds the upper half of A's rows first)
//    make the kept values the first ones, so the butterfly needs no selects:
//    1.5 V shuffles and adds per 8 V dp4a.
//  * lane (g, t) ends with nonzero g + 8 (t >> 1) of the tile, vector lanes
//    (t & 1) V/2 .. (t & 1) V/2 + V/2 - 1, stored as one vector per lane.
// Both operands keep the same k order (4-bit values are unpacked the same
// way on both sides), which leaves every dot product unchanged; sums wrap
// modulo 2^32 like the MMA's int32 accumulators.
#pragma once
#include "mc_sddmm.cuh"

namespace mc {

// K64: k == 64, one k block, the A chunks stay in registers for the whole
// vector-row; otherwise they are reloaded per k block.
template <int V, int PREA, int PREB, bool SIGNED, bool VECMAJOR, bool HALF_OUT, int WARPS, bool K64>
__global__ void __launch_bounds__(WARPS * 32)
sddmm_dp4a_kernel(const SddmmParams p)
{
    static_assert(PREA != 16 && PREB != 16, "dp4a computes 8-bit and 4-bit operands");
    constexpr int H = V / 2;  // vector lanes a lane ends with
    const Divisor dq = make_divisor(p.scale);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const int tb0 = t & 1, tb1 = t >> 1;
    const int row = __ldg(p.row_indices + blockIdx.x);
    const int b = blockIdx.z;
    const int start = __ldg(p.row_offsets + 2 * row);
    const int nnz = __ldg(p.row_offsets + 2 * row + 1) - start;
    const int nnz8 = (nnz + 7) & ~7;
    const int ntiles = (nnz8 + 15) >> 4;
    const int kblocks = p.k >> 6;
    const int stride = gridDim.y * WARPS;
    int ti = blockIdx.y * WARPS + warp;
    if (ti >= ntiles) return;

    const long long lhs_row_bytes = (long long)p.k * PREA / 8;
    const long long rhs_row_bytes = (long long)p.k * PREB / 8;
    // A row of slot vv: vector lane vv ^ (tb0 ? H : 0), so this lane's kept
    // lanes come first.
    const uint8_t* lhs = p.lhs + (long long)b * p.lhs_stride + (long long)row * V * lhs_row_bytes;
    const uint8_t* rhs = p.rhs + (long long)b * p.rhs_stride;
    const int* cols = p.col_indices + start;
    auto load_a = [&](int kb, uint32_t (&a)[V][4]) {
#pragma unroll
        for (int vv = 0; vv < V; ++vv) {
            uint32_t w[2][4];
            load_kfrag<PREA, SIGNED>(lhs + (long long)(vv ^ (tb0 ? H : 0)) * lhs_row_bytes, kb, t, w);
#pragma unroll
            for (int e = 0; e < 4; ++e) a[vv][e] = w[0][e];
        }
    };
    uint32_t a0[V][4];
    if constexpr (K64) load_a(0, a0);
    const long long obase = (long long)b * p.out_stride + (long long)start * V;

#pragma unroll 1
    for (; ti < ntiles; ti += stride) {
        // own row: nonzero g + 8 tb1 of the tile; other row: g + 8 (1 - tb1)
        const int jo = ti * 16 + g + 8 * tb1, jx = ti * 16 + g + 8 * (1 - tb1);
        const int co = jo < nnz ? __ldg(cols + jo) : -1;
        const int cx = jx < nnz ? __ldg(cols + jx) : -1;
        int own[V], oth[V];
#pragma unroll
        for (int vv = 0; vv < V; ++vv) own[vv] = oth[vv] = 0;
        auto block = [&](int kb, const uint32_t (&ak)[V][4]) {
            uint32_t ro[2][4] = {}, rx[2][4] = {};
            if (co >= 0) load_kfrag<PREB, SIGNED>(rhs + (long long)co * rhs_row_bytes, kb, t, ro);
            if (cx >= 0) load_kfrag<PREB, SIGNED>(rhs + (long long)cx * rhs_row_bytes, kb, t, rx);
#pragma unroll
            for (int vv = 0; vv < V; ++vv)
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    own[vv] = dp4a<SIGNED>(ak[vv][e], ro[0][e], own[vv]);
                    oth[vv] = dp4a<SIGNED>(ak[vv][e], rx[0][e], oth[vv]);
                }
        };
        if constexpr (K64) {
            block(0, a0);
        } else {
#pragma unroll 1
            for (int kb = 0; kb < kblocks; ++kb) {
                uint32_t ak[V][4];
                load_a(kb, ak);
                block(kb, ak);
            }
        }
        // t ^ 2 holds the other row as its own: add its partials of ours.
#pragma unroll
        for (int vv = 0; vv < V; ++vv) own[vv] += __shfl_xor_sync(0xffffffffu, oth[vv], 2);
        // t ^ 1 has the opposite lane order: its second half is our first.
        int d[H];
#pragma unroll
        for (int vv = 0; vv < H; ++vv) d[vv] = own[vv] + __shfl_xor_sync(0xffffffffu, own[vv + H], 1);

        if (jo >= nnz8) continue;
        const int v0 = tb0 * H;
        if constexpr (VECMAJOR) {
            const long long o = obase + (long long)jo * V + v0;
            if constexpr (HALF_OUT) {
                __half* out = reinterpret_cast<__half*>(p.out) + o;
                if constexpr (H == 4) {  // 4-byte aligned (out_stride is only even)
                    stg_cs_s32(out, (int)pack_half2(d[0], d[1], dq));
                    stg_cs_s32(out + 2, (int)pack_half2(d[2], d[3], dq));
                } else if constexpr (H == 2) {
                    stg_cs_s32(out, (int)pack_half2(d[0], d[1], dq));
                } else {
                    *out = deq_half(d[0], dq);
                }
            } else {
                int* out = reinterpret_cast<int*>(p.out) + o;
                if constexpr (H == 4) {  // 8-byte aligned (out_stride is only even)
                    stg_cs_v2(out, d[0], d[1]);
                    stg_cs_v2(out + 2, d[2], d[3]);
                } else if constexpr (H == 2) {
                    stg_cs_v2(out, d[0], d[1]);
                } else {
                    stg_cs_s32(out, d[0]);
                }
            }
        } else {
            // Blocked layout with alignment 8: (j/8)*8V + 8v + j%8.
            const long long o = obase + (long long)(jo >> 3) * 8 * V + 8 * v0 + (jo & 7);
#pragma unroll
            for (int vv = 0; vv < H; ++vv) {
                if constexpr (HALF_OUT) reinterpret_cast<__half*>(p.out)[o + 8 * vv] = deq_half(d[vv], dq);
                else stg_cs_s32(reinterpret_cast<int*>(p.out) + o + 8 * vv, d[vv]);
            }
        }
    }
}

}  // namespace mc
