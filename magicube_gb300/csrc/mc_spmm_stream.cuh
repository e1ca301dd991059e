// mc_spmm_stream.cuh -- persistent, row-streaming SpMM for sm_103a.
//
// Same operands and results as mc_spmm.cuh's spmm_kernel (the reference's
// spmm::wmmaSpmm_* layouts), organised for short vector-rows:
//
//  * Persistent CTAs.  A "task" is one (batch entry, vector-row); CTA x of the
//    grid owns tasks x, x + gridDim.x, ... for one WARPS*32-column tile of C.
//    Its tasks' 32-slot steps form one stream that flows through a 4-stage
//    cp.async ring without draining between rows, so the pipeline fill is paid
//    once per CTA instead of once per row.
//  * Each ring stage carries everything a step needs: the 32 gathered rows of
//    B (column slice), the step's value chunk(s) and a 16-byte header
//    (row, batch entry, nonzero count, step, last/empty flags) written by the
//    producer, so the consumer reads no global metadata.
//  * ldmatrix.m16n16.x2.trans.b8 turns the staged [slot][byte] rows into the
//    k-contiguous A fragment of mma.m16n8k32 directly (rows XOR-swizzled so
//    the 16-byte row segments of each phase hit distinct banks).  8-bit B:
//    byte c is column c.  4-bit B: byte c holds columns 2c (low nibble) and
//    2c+1 (high nibble), so masking (and sign-extending) the nibbles of one
//    fragment gives the A fragments of two MMA tiles: columns 2c and 2c+1.
//  * Column indices of the next step are fetched one step ahead into
//    registers; the producer cursor runs STAGES-1 steps ahead of the consumer.
#pragma once
#include "mc_spmm.cuh"

namespace mc {

__device__ __forceinline__ void ldsm_x2_trans_b8(uint32_t (&r)[4], const void* p)
{
    asm volatile("ldmatrix.sync.aligned.m16n16.x2.trans.shared.b8 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_u32(p)));
}

// Shared-memory geometry of one stage's gathered-row slice (MT 16-column MMA
// tiles per warp).
template <int PREB, int WARPS, int MT>
struct StreamRhs {
    static constexpr int NT = WARPS * 16 * MT;
    static constexpr int RB = NT * PREB / 8;  // packed bytes per row slice
    static constexpr int CH = RB / 16;        // 16-byte chunks per row slice
    // Rows of RB packed bytes (8-bit or 4-bit B), 16-byte chunks
    // XOR-swizzled so that the eight row segments of each ldmatrix phase hit
    // distinct 16-byte bank groups: over 8 rows (RB >= 128), over 4 pairs of
    // rows (RB = 64: two rows per 128-byte line) or over 2 groups of 4 rows
    // (RB = 32: four rows per line).
    static constexpr int STRIDE = RB;
    __device__ __forceinline__ static int swz(int r, int c)
    {
        if constexpr (CH >= 8) return c ^ (r & 7);
        else if constexpr (CH == 4) return c ^ ((r >> 1) & 3);
        else return c ^ ((r >> 2) & 1);
    }
};

struct StreamTask {
    int task, step, row, b, start, nnz, steps;
};

// MT: 16-column MMA tiles per warp (2, or 4 for 8-bit B): more columns per
// warp spread each step's bookkeeping (barrier, copies, cursor, header) over
// more MMAs.
template <int V, int PREA, int PREB, bool SIGNED, int WARPS, bool HALF_OUT, bool F16, bool EXT, int MT = 2>
__global__ void __launch_bounds__(WARPS * 32)
spmm_stream_kernel(const SpmmParams p, const int ntasks)
{
    static_assert(MT == 2 || PREB == 8, "4-bit B runs with two MMA tiles per warp");
    using L = SpmmLayout<PREA, PREB, EXT>;
    using S = StreamRhs<PREB, WARPS, MT>;
    constexpr int STAGES = 4;
    constexpr int NT = WARPS * 16 * MT;
    constexpr int THREADS = WARPS * 32;
    constexpr int CPT = (32 * S::CH) / THREADS;  // rhs chunks per thread per stage
    constexpr int BP = L::BYTE_PLANES;
    constexpr int PLANE_BYTES = V * L::VCHUNK * L::PLANE_BITS / 8;
    constexpr int CHUNK_BYTES = PLANE_BYTES * L::PLANES;
    constexpr int SLOT_BYTES = V * PREA / 8;         // value bytes per vector slot
    constexpr int VALS_BYTES = 32 * SLOT_BYTES;      // value bytes per step
    constexpr int RHS_BYTES = 32 * S::STRIDE;
    constexpr int STAGE_BYTES = (RHS_BYTES + VALS_BYTES + 16 + 127) / 128 * 128;
    static_assert(VALS_BYTES / 16 <= THREADS, "value chunks exceed one per thread");

    __shared__ __align__(128) uint8_t ring[STAGES * STAGE_BYTES];

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, t = lane & 3;
    const int n0 = blockIdx.y * NT;
    const long long rhs_row_bytes = (long long)p.n * PREB / 8;

    int qrow[CPT], qch[CPT];
#pragma unroll
    for (int i = 0; i < CPT; ++i) {
        const int q = tid + i * THREADS;
        qrow[i] = q / S::CH;
        qch[i] = q % S::CH;
    }

    // ---- producer cursor ------------------------------------------------
    auto load_task = [&](StreamTask& c, int task) {
        c.task = task;
        c.step = 0;
        c.steps = 0;
        if (task < ntasks) {
            c.b = task / p.m_vec;
            c.row = __ldg(p.row_indices + (task - c.b * p.m_vec));
            c.start = __ldg(p.row_offsets + 2 * c.row);
            c.nnz = __ldg(p.row_offsets + 2 * c.row + 1) - c.start;
            c.steps = (c.nnz + 31) >> 5;
        }
    };
    // Empty tasks (no nonzeros) still occupy one stage, flagged empty, so the
    // consumer writes their zero rows.
    auto advance = [&](StreamTask& c) {
        if (c.task >= ntasks) return;
        if (++c.step >= (c.steps > 0 ? c.steps : 1)) load_task(c, c.task + gridDim.x);
    };
    auto fetch_cols = [&](const StreamTask& c, int (&col)[CPT]) {
#pragma unroll
        for (int i = 0; i < CPT; ++i) {
            const int j = c.step * 32 + qrow[i];
            col[i] = (c.task < ntasks && j < c.nnz) ? __ldg(p.col_indices + c.start + col_slot<L::SHUFFLED_COLS>(j)) : -1;
        }
    };
    auto issue = [&](const StreamTask& c, const int (&col)[CPT], int slot) {
        uint8_t* st = ring + slot * STAGE_BYTES;
        if (c.task < ntasks) {
            const uint8_t* rhs = p.rhs + (long long)c.b * p.rhs_stride + (long long)n0 * PREB / 8;
#pragma unroll
            for (int i = 0; i < CPT; ++i)
                if (col[i] >= 0)
                    cp_async16(st + qrow[i] * S::STRIDE + S::swz(qrow[i], qch[i]) * 16,
                               rhs + (long long)col[i] * rhs_row_bytes + qch[i] * 16);
            // value chunk(s) of this step: slots [32*step, min(32*step+32, aligned len))
            const int alen = (c.nnz + L::MMA_K - 1) / L::MMA_K * L::MMA_K;
            const int nslots = min(32, alen - 32 * c.step);
            if (tid * 16 < nslots * SLOT_BYTES) {
                const uint8_t* src = p.values + (long long)c.b * p.values_stride +
                                     (long long)(c.start + 32 * c.step) * SLOT_BYTES + tid * 16;
                cp_async16(st + RHS_BYTES + tid * 16, src);
            }
        }
        if (tid == 0) {
            int4 h;
            h.x = c.task < ntasks ? c.row : -1;
            h.y = c.b;
            h.z = c.nnz;
            const int last = (c.steps == 0) || (c.step == c.steps - 1);
            h.w = c.step | (last << 30) | ((c.steps == 0) << 29);
            *reinterpret_cast<int4*>(st + RHS_BYTES + VALS_BYTES) = h;
        }
    };

    StreamTask cur;
    load_task(cur, blockIdx.x);
    int cols[CPT];
    fetch_cols(cur, cols);
#pragma unroll
    for (int s = 0; s < STAGES - 1; ++s) {
        issue(cur, cols, s);
        cp_async_commit();
        advance(cur);
        fetch_cols(cur, cols);
    }

    int acc[BP][MT][4];
    float facc[BP][MT][4];
#pragma unroll
    for (int bp = 0; bp < BP; ++bp)
#pragma unroll
        for (int m = 0; m < MT; ++m)
#pragma unroll
            for (int e = 0; e < 4; ++e) { acc[bp][m][e] = 0; facc[bp][m][e] = 0.f; }

#pragma unroll 1
    for (int it = 0;; ++it) {
        cp_async_wait<STAGES - 2>();
        __syncthreads();
        const uint8_t* st = ring + (it % STAGES) * STAGE_BYTES;
        const int4 hdr = *reinterpret_cast<const int4*>(st + RHS_BYTES + VALS_BYTES);
        if (hdr.x < 0) break;  // stream exhausted (uniform across the CTA)
        // Refill the slot consumed in the previous iteration (all threads have
        // passed the barrier, so nobody reads it any more).
        issue(cur, cols, (it + STAGES - 1) % STAGES);
        cp_async_commit();
        advance(cur);
        fetch_cols(cur, cols);

        const int step = hdr.w & 0x1fffffff;
        const bool last = (hdr.w >> 30) & 1;
        const bool empty = (hdr.w >> 29) & 1;
        const int nnz = hdr.z;
        if (!empty) {
            // ---- value fragments: vals[bp][h] for vector lane v = g, slots 16h+4t..+3
            uint32_t vals[BP][2];
#pragma unroll
            for (int bp = 0; bp < BP; ++bp) { vals[bp][0] = 0u; vals[bp][1] = 0u; }
            if (g < V) {
                const uint8_t* vs = st + RHS_BYTES;
#pragma unroll
                const bool full = step * 32 + 32 <= nnz;  // no slot of this step past the row end
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const uint32_t keep = full ? 0xffffffffu : byte_mask(nnz - (step * 32 + 16 * h + 4 * t));
                    if constexpr (L::VCHUNK == 16) {
#pragma unroll
                        for (int bp = 0; bp < BP; ++bp)
                            vals[bp][h] = lds32(vs + h * CHUNK_BYTES + vword16<V, PREA, PREB, EXT>(g, t, bp)) & keep;
                    } else {
                        uint32_t nib[L::PLANES];
#pragma unroll
                        for (int pl = 0; pl < L::PLANES; ++pl)
                            nib[pl] = lds16(vs + pl * PLANE_BYTES + g * 16 + 8 * h + 2 * t);
                        if constexpr (PREA == 4) {
                            vals[0][h] = unpack4_u16<SIGNED>(nib[0]) & keep;
                        } else if constexpr (PREA == 8) {
                            vals[0][h] = merge_nibble_planes(nib[0], nib[1]) & keep;
                        } else {
                            vals[0][h] = merge_nibble_planes(nib[0], nib[1]) & keep;
                            vals[1][h] = merge_nibble_planes(nib[2], nib[3]) & keep;
                        }
                    }
                }
            }
            // ---- A fragments of this warp's 16*MT columns: af[m][0..3] for MMA m
            uint32_t af[MT][4];
            if constexpr (PREB == 8) {
                // lanes 0-15: slots 0-15, lanes 16-31: slots 16-31 of column chunk MT*warp+m
                const int r = lane;
#pragma unroll
                for (int m = 0; m < MT; ++m)
                    ldsm_x2_trans_b8(af[m], st + r * S::STRIDE + S::swz(r, MT * warp + m) * 16);
            } else {
                // this warp's 32 columns are one 16-byte chunk: one ldmatrix,
                // then MMA 0 takes the low nibbles (column 2c of byte c),
                // MMA 1 the high nibbles (column 2c + 1)
                uint32_t nb[4];
                ldsm_x2_trans_b8(nb, st + lane * S::STRIDE + S::swz(lane, warp) * 16);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const uint32_t lo = nb[q] & 0x0F0F0F0Fu, hi = (nb[q] >> 4) & 0x0F0F0F0Fu;
                    af[0][q] = SIGNED ? sext_nibble_bytes(lo) : lo;
                    af[1][q] = SIGNED ? sext_nibble_bytes(hi) : hi;
                }
            }
#pragma unroll
            for (int bp = 0; bp < BP; ++bp) {
                const bool top = (bp == BP - 1);
                if constexpr (F16) {
                    uint32_t v0l, v0h, v1l, v1h;
                    if (SIGNED && top) { bytes_to_h2<true>(vals[bp][0], v0l, v0h); bytes_to_h2<true>(vals[bp][1], v1l, v1h); }
                    else { bytes_to_h2<false>(vals[bp][0], v0l, v0h); bytes_to_h2<false>(vals[bp][1], v1l, v1h); }
#pragma unroll
                    for (int m = 0; m < MT; ++m) {
                        uint32_t a[4][2];
#pragma unroll
                        for (int q = 0; q < 4; ++q) bytes_to_h2<SIGNED>(af[m][q], a[q][0], a[q][1]);
                        mma_f16(facc[bp][m], a[0][0], a[1][0], a[0][1], a[1][1], v0l, v0h);
                        mma_f16(facc[bp][m], a[2][0], a[3][0], a[2][1], a[3][1], v1l, v1h);
                    }
                } else {
#pragma unroll
                    for (int m = 0; m < MT; ++m) {
                        if (SIGNED && top)
                            mma_k32<SIGNED, true>(acc[bp][m], af[m][0], af[m][1], af[m][2], af[m][3], vals[bp][0], vals[bp][1]);
                        else
                            mma_k32<SIGNED, false>(acc[bp][m], af[m][0], af[m][1], af[m][2], af[m][3], vals[bp][0], vals[bp][1]);
                    }
                }
            }
            if constexpr (F16) {
                if ((step & 7) == 7 || last) {
#pragma unroll
                    for (int bp = 0; bp < BP; ++bp)
#pragma unroll
                        for (int m = 0; m < MT; ++m)
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                acc[bp][m][e] = (int)((uint32_t)acc[bp][m][e] + (uint32_t)f2i_exact(facc[bp][m][e]));
                                facc[bp][m][e] = 0.f;
                            }
                }
            }
        }
        if (last) {
            // acc[.][m][e]: column c(m, e>>1), vector lane 2t + (e & 1), where
            // 8-bit B: c = 16m + 8(e>>1) + g;  4-bit B: c = 2g + m + 16(e>>1).
            const int row = hdr.x, b = hdr.y;
#pragma unroll
            for (int e2 = 0; e2 < 2; ++e2) {
                const int v = 2 * t + e2;
                if (v >= V) continue;
                int r4[2 * MT];
#pragma unroll
                for (int q = 0; q < 2 * MT; ++q) {
                    const int m = q >> 1, e = 2 * (q & 1) + e2;
                    uint32_t x = (uint32_t)acc[0][m][e];
                    if constexpr (BP == 2) x += (uint32_t)acc[1][m][e] << 8;
                    r4[q] = (int)x;
                }
                const long long obase =
                    (long long)b * p.out_stride + (long long)(row * V + v) * p.n + n0 + warp * 16 * MT;
                if constexpr (PREB == 8) {
                    // columns g, g+8, ..., g + 8 (2 MT - 1)
                    if constexpr (HALF_OUT) {
                        __half* o = reinterpret_cast<__half*>(p.out) + obase + g;
                        const Divisor dv = out_divisor(p, b, row * V + v);
#pragma unroll
                        for (int q = 0; q < 2 * MT; ++q) o[8 * q] = deq_half(r4[q], dv);
                    } else {
                        int* o = reinterpret_cast<int*>(p.out) + obase + g;
#pragma unroll
                        for (int q = 0; q < 2 * MT; ++q) stg_cs_s32(o + 8 * q, r4[q]);
                    }
                } else {
                    // r4[0], r4[2]: columns 2g, 2g+1; r4[1], r4[3]: columns 2g+16, 2g+17
                    if constexpr (HALF_OUT) {
                        __half* o = reinterpret_cast<__half*>(p.out) + obase + 2 * g;
                        const Divisor dv = out_divisor(p, b, row * V + v);
                        stg_cs_s32(o, (int)pack_half2(r4[0], r4[2], dv));
                        stg_cs_s32(o + 16, (int)pack_half2(r4[1], r4[3], dv));
                    } else {
                        int* o = reinterpret_cast<int*>(p.out) + obase + 2 * g;
                        stg_cs_v2(o, r4[0], r4[2]);
                        stg_cs_v2(o + 16, r4[1], r4[3]);
                    }
                }
            }
#pragma unroll
            for (int bp = 0; bp < BP; ++bp)
#pragma unroll
                for (int m = 0; m < MT; ++m)
#pragma unroll
                    for (int e = 0; e < 4; ++e) { acc[bp][m][e] = 0; facc[bp][m][e] = 0.f; }
        }
    }
    cp_async_wait<0>();
}

}  // namespace mc
