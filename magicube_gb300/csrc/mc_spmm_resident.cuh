// mc_spmm_resident.cuh -- SpMM with the B column slice resident in shared
// memory, for 8-bit and 4-bit B on sm_103a.
//
// Same operands and results as spmm_tma_kernel (mc_spmm_tma.cuh) on the int8
// tensor path.  A work unit is one (batch entry, column tile) pair -- its
// "slice": the K x NT block of B, 64 or 128 bytes a row -- and the grid splits the
// flat list of (slice, vector-row) units into equal contiguous ranges, one
// per CTA:
//  * for every slice its range touches, the CTA loads the whole block with
//    2-D TMA tile copies (256 rows each, swizzled at the row width) onto one
//    mbarrier, once;
//  * its warps then claim vector-rows of that slice from a shared counter
//    and run them alone: per 32-slot step, one column index per lane and the
//    value words of the step come straight from global memory into a
//    register ring PF steps ahead (row claims and row offsets two rows
//    ahead), and ldmatrix.m16n16.x2.trans.b8 gathers the 32 B rows from
//    shared memory at the lanes' own row addresses; mma.m16n8k32 with int32
//    accumulators (or, with DP4A and V <= 4, dp4a on the same fragments:
//    no padding vector lanes); finished rows of C are written from
//    registers.
// B rows are thus read from L2 once per slice rather than once per nonzero
// vector, and no copy sits between a step and its MMAs.  Rows of a slice are
// taken longest and shortest alternately (the row order array is sorted by
// length), so equal ranges carry similar work.  Slots past a row's nonzero
// count read row 0 of the slice with zeroed value bytes; a column index
// outside [0, k) reads row 0 as well, so every shared-memory access stays
// inside the slice.  The wait for a slice's copies is bounded: a wait that
// runs out increments the library's timeout counter and the CTA waits once
// more, bounded again, for its copies before it returns.
#pragma once
#include "mc_sm100.cuh"
#include "mc_spmm.cuh"
#include "mc_spmm_stream.cuh"

namespace mc {

template <int PREB, int ROWB = 64, int WARPS = 8>
struct SpmmResidentGeom {
    static constexpr int ROW_BYTES = ROWB;               // bytes of one B row in the slice (64 or 128)
    static constexpr int NT = ROW_BYTES * 8 / PREB;      // columns of C per slice
    static constexpr int MT = NT / 16;                   // 16-column MMA tiles per step
    static constexpr int BOX_ROWS = 256;                 // rows per TMA tile copy
    static constexpr int THREADS = WARPS * 32;
    // bytes of dynamic shared memory for a slice of `boxes` boxes: alignment
    // slack, the rows, the mbarrier and the row counter
    static constexpr size_t smem(int boxes) { return 1024 + (size_t)boxes * BOX_ROWS * ROW_BYTES + 64; }
};

// Byte offset of 16-byte chunk 0 of slice row r under the TMA swizzle of
// the row width: 64-byte rows, chunk bits 4-5 XOR address bits 7-8;
// 128-byte rows, chunk bits 4-6 XOR address bits 7-9.  Chunk c of the row
// is then at offset ^ (c << 4): the row's own bits 4-6 are the swizzle term.
template <int ROWB>
__device__ __forceinline__ uint32_t resident_row_offset(int r)
{
    if constexpr (ROWB == 64) return (uint32_t)r * 64u + ((uint32_t)((r >> 1) & 3) << 4);
    else return (uint32_t)r * 128u + ((uint32_t)(r & 7) << 4);
}

__device__ __forceinline__ void ldsm_x2_trans_b8_at(uint32_t (&r)[4], uint32_t saddr)
{
    asm volatile("ldmatrix.sync.aligned.m16n16.x2.trans.shared.b8 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(saddr));
}

template <int V, int PREA, int PREB, bool SIGNED, bool HALF_OUT, bool EXT, int ROWB = 64, int WARPS = 8,
          int PF = 4, bool DP4A = false>
__global__ void __launch_bounds__(WARPS * 32)
spmm_resident_kernel(const __grid_constant__ CUtensorMap tmap, const SpmmParams p, const int tiles,
                     const long long units, const int rows_per_entry, const int boxes, unsigned int* timeouts)
{
    using namespace sm100;
    using L = SpmmLayout<PREA, PREB, EXT>;
    using G = SpmmResidentGeom<PREB, ROWB, WARPS>;
    constexpr int NT = G::NT, MT = G::MT, BP = L::BYTE_PLANES;
    constexpr int SLOT_BYTES = V * PREA / 8;
    constexpr int NV = DP4A ? V : BP;  // value words a lane holds per half-step
    constexpr long long WAIT = 4000000000LL;  // about 2 s at 2 GHz
    static_assert(PREB == 8 || PREB == 4, "8-bit or 4-bit B");
    static_assert(PREB == 8 || MT % 2 == 0, "4-bit B: two MMA tiles per 16-byte chunk");
    static_assert(PREA == 4 || PREA == 8 || PREA == 16, "4-, 8- or 16-bit A");
    static_assert(!DP4A || (V <= 4 && BP == 1), "the dp4a consumer computes V = 2 and 4 with 8-bit or 4-bit A");

    extern __shared__ uint8_t smem_raw[];
    uint8_t* slice = smem_raw + ((1024u - (saddr(smem_raw) & 1023u)) & 1023u);
    const uint32_t slice_bytes = (uint32_t)boxes * G::BOX_ROWS * G::ROW_BYTES;
    uint64_t* bar = reinterpret_cast<uint64_t*>(slice + slice_bytes);
    int* counter = reinterpret_cast<int*>(bar + 1);
    const uint32_t slice_s = saddr(slice);

    const int tid = threadIdx.x, lane = tid & 31;
    const int g = lane >> 2, t = lane & 3;
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
        prefetch_tmap(&tmap);
    }
    __syncthreads();

    const long long lo = units * blockIdx.x / gridDim.x, hi = units * (blockIdx.x + 1) / gridDim.x;
    uint32_t phase = 0;

    // MMA accumulators (acc[bp][m][e]: vector lane 2t + (e & 1), columns
    // 8-bit B 16m + 8(e>>1) + g, 4-bit B 32(m>>1) + 2g + (m&1) + 16(e>>1));
    // dp4a partial sums (pacc[m][hh][v]: this lane's slots of columns g
    // (hh = 0) and g + 8 (hh = 1) of tile m, vector lane v)
    constexpr int DM = DP4A ? MT : 1, DV = DP4A ? V : 1;
    int acc[BP][MT][4];
    int pacc[DM][2][DV];
#pragma unroll
    for (int bp = 0; bp < BP; ++bp)
#pragma unroll
        for (int m = 0; m < MT; ++m)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[bp][m][e] = 0;
#pragma unroll
    for (int m = 0; m < DM; ++m)
#pragma unroll
        for (int hh = 0; hh < 2; ++hh)
#pragma unroll
            for (int v = 0; v < DV; ++v) pacc[m][hh][v] = 0;

    for (long long pos = lo; pos < hi;) {
        const long long pair = pos / p.m_vec;
        const int first = (int)(pos - pair * p.m_vec);
        const int last_slot = (int)((hi - pair * p.m_vec) < p.m_vec ? (hi - pair * p.m_vec) : p.m_vec);
        const int b = (int)(pair / tiles), n0 = (int)(pair - (long long)b * tiles) * NT;
        pos = pair * p.m_vec + last_slot;

        __syncthreads();  // every warp is done with the previous slice and counter
        if (tid == 0) {
            *counter = first;
            mbar_arrive_expect_tx(bar, slice_bytes);
            for (int x = 0; x < boxes; ++x)
                tma_load_2d(slice + x * G::BOX_ROWS * G::ROW_BYTES, &tmap, bar, n0 * PREB / 8,
                            b * rows_per_entry + x * G::BOX_ROWS);
        }
        __syncthreads();
        // the CTA goes on only if every thread saw the copies land
        if (!__syncthreads_and(mbar_wait(bar, phase, WAIT))) {
            if (tid == 0) atomicAdd(timeouts, 1u);
            mbar_wait(bar, phase, WAIT);  // the copies land before the CTA returns
            return;
        }
        phase ^= 1;

        const uint8_t* vbase = p.values + (long long)b * p.values_stride;
        // ---- rows: claimed two rows before they are produced ----
        // claim_ri: a slot from the counter and the load of its row index
        // (slot s -> sorted position: longest and shortest rows alternately)
        auto claim_ri = [&]() -> int {
            int s = 0;
            if (lane == 0) s = atomicAdd(counter, 1);
            s = __shfl_sync(0xffffffffu, s, 0);
            if (s >= last_slot) return -1;
            const int sp = (s & 1) ? p.m_vec - 1 - (s >> 1) : (s >> 1);
            return __ldg(p.row_indices + sp);
        };
        struct RowOff {
            int row, start, end;
        };
        auto fetch_off = [&](int ri) -> RowOff {
            RowOff o{ri, 0, 0};
            if (ri >= 0) {
                o.start = __ldg(p.row_offsets + 2 * ri);
                o.end = __ldg(p.row_offsets + 2 * ri + 1);
            }
            return o;
        };
        // ---- steps: a register ring PF steps deep ----
        // A slot holds the raw loads of one step (column index, value words
        // or nibble-plane halfwords); masks, clamps and unpacking are applied
        // when the step is consumed, so no load is waited on when issued.
        constexpr int RW = L::VCHUNK == 16 ? NV : L::PLANES * (DP4A ? V : 1);  // raw words per half-step
        struct Slot {
            int col, row, nnz, flags;  // flags: step | last << 30
            uint32_t raw[RW][2];
        };
        RowOff pc = fetch_off(claim_ri());
        RowOff q1 = fetch_off(pc.row >= 0 ? claim_ri() : -1);
        int ri2 = q1.row >= 0 ? claim_ri() : -1;
        int pstep = 0;
        auto produce = [&](Slot& sl) {
            sl.row = pc.row;
            if (pc.row < 0) return;  // end of this warp's stream
            const int nnz = pc.end - pc.start;
            const int steps = nnz > 0 ? (nnz + 31) >> 5 : 1;
            const bool last = pstep + 1 == steps;
            sl.nnz = nnz;
            sl.flags = pstep | ((int)last << 30);
            const int j = 32 * pstep + lane;
            sl.col = j < nnz ? __ldg(p.col_indices + pc.start + col_slot<L::SHUFFLED_COLS>(j)) : 0;
#pragma unroll
            for (int w = 0; w < RW; ++w) { sl.raw[w][0] = 0u; sl.raw[w][1] = 0u; }
            if (DP4A || g < V) {
                const int alen = (nnz + L::MMA_K - 1) / L::MMA_K * L::MMA_K;
                const uint8_t* vr = vbase + (long long)pc.start * SLOT_BYTES;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int s0 = 32 * pstep + 16 * h;  // first slot of this half-step
                    if constexpr (L::VCHUNK == 16) {
                        if (s0 < alen) {
#pragma unroll
                            for (int w = 0; w < NV; ++w)
                                sl.raw[w][h] = __ldg(reinterpret_cast<const uint32_t*>(
                                    vr + s0 * SLOT_BYTES +
                                    (DP4A ? vword16<V, PREA, PREB, EXT>(w, t, 0) : vword16<V, PREA, PREB, EXT>(g, t, w))));
                        }
                    } else if (32 * pstep < alen) {
                        // one 32-slot chunk of 4-bit planes [v][slot]
                        constexpr int PLANE_BYTES = V * 32 * L::PLANE_BITS / 8;
#pragma unroll
                        for (int w = 0; w < (DP4A ? V : 1); ++w) {
                            const uint8_t* ch = vr + 32 * pstep * SLOT_BYTES + (DP4A ? w : g) * 16 + 8 * h + 2 * t;
#pragma unroll
                            for (int pl = 0; pl < L::PLANES; ++pl)
                                sl.raw[w * L::PLANES + pl][h] =
                                    __ldg(reinterpret_cast<const unsigned short*>(ch + pl * PLANE_BYTES));
                        }
                    }
                }
            }
            if (last) {
                pc = q1;
                q1 = fetch_off(ri2);
                ri2 = q1.row >= 0 ? claim_ri() : -1;
                pstep = 0;
            } else {
                ++pstep;
            }
        };
        // the operands of a consumed step: clamped slice row, masked value words
        auto operands = [&](const Slot& sl, int& row, uint32_t (&vals)[NV][2]) {
            const int step = sl.flags & 0x3fffffff;
            row = (32 * step + lane < sl.nnz && (unsigned)sl.col < (unsigned)p.k) ? sl.col : 0;
            const bool whole = step * 32 + 32 <= sl.nnz;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint32_t keep = whole ? 0xffffffffu : byte_mask(sl.nnz - (32 * step + 16 * h + 4 * t));
                if constexpr (L::VCHUNK == 16) {
#pragma unroll
                    for (int w = 0; w < NV; ++w) vals[w][h] = sl.raw[w][h] & keep;
                } else {
#pragma unroll
                    for (int w = 0; w < (DP4A ? V : 1); ++w) {
                        if constexpr (PREA == 4) {
                            vals[w][h] = unpack4_u16<SIGNED>(sl.raw[w * L::PLANES][h]) & keep;
                        } else if constexpr (PREA == 8) {
                            vals[w][h] = merge_nibble_planes(sl.raw[w * L::PLANES][h], sl.raw[w * L::PLANES + 1][h]) &
                                         keep;
                        } else {
                            vals[0][h] = merge_nibble_planes(sl.raw[0][h], sl.raw[1][h]) & keep;
                            vals[NV - 1][h] = merge_nibble_planes(sl.raw[2][h], sl.raw[3][h]) & keep;
                        }
                    }
                }
            }
        };

        Slot ring[PF];
#pragma unroll
        for (int j = 0; j < PF; ++j) produce(ring[j]);
        bool done = false;
#pragma unroll 1
        while (!done) {
#pragma unroll
            for (int j = 0; j < PF; ++j) {
                if (ring[j].row < 0) {
                    done = true;
                    break;
                }
                const Slot cs = ring[j];
                produce(ring[j]);  // the step PF ahead of this one
                int srow;
                uint32_t vals[NV][2];
                operands(cs, srow, vals);
                // the slice is 1024-byte aligned: chunk c of the lane's row at rowa ^ (c << 4)
                const uint32_t rowa = slice_s + resident_row_offset<ROWB>(srow);
                // A fragments of the 16-column tiles from the lanes' slice rows
                if constexpr (PREB == 8) {
#pragma unroll
                    for (int m = 0; m < MT; ++m) {
                        uint32_t af[4];
                        ldsm_x2_trans_b8_at(af, rowa ^ ((uint32_t)m << 4));
                        if constexpr (DP4A) {
#pragma unroll
                            for (int v = 0; v < DV; ++v) {
                                pacc[m][0][v] = dp4a<SIGNED>(af[0], vals[v][0], pacc[m][0][v]);
                                pacc[m][0][v] = dp4a<SIGNED>(af[2], vals[v][1], pacc[m][0][v]);
                                pacc[m][1][v] = dp4a<SIGNED>(af[1], vals[v][0], pacc[m][1][v]);
                                pacc[m][1][v] = dp4a<SIGNED>(af[3], vals[v][1], pacc[m][1][v]);
                            }
                        } else {
#pragma unroll
                            for (int bp = 0; bp < BP; ++bp) {
                                if (SIGNED && bp == BP - 1)
                                    mma_k32<SIGNED, true>(acc[bp][m], af[0], af[1], af[2], af[3], vals[bp][0],
                                                          vals[bp][1]);
                                else
                                    mma_k32<SIGNED, false>(acc[bp][m], af[0], af[1], af[2], af[3], vals[bp][0],
                                                           vals[bp][1]);
                            }
                        }
                    }
                } else {
#pragma unroll
                    for (int k = 0; k < MT / 2; ++k) {
                        uint32_t nb[4], af2[2][4];
                        ldsm_x2_trans_b8_at(nb, rowa ^ ((uint32_t)k << 4));
#pragma unroll
                        for (int q = 0; q < 4; ++q) {
                            const uint32_t l = nb[q] & 0x0F0F0F0Fu, hg = (nb[q] >> 4) & 0x0F0F0F0Fu;
                            af2[0][q] = SIGNED ? sext_nibble_bytes(l) : l;
                            af2[1][q] = SIGNED ? sext_nibble_bytes(hg) : hg;
                        }
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            const int m = 2 * k + u;
                            const uint32_t(&af)[4] = af2[u];
                            if constexpr (DP4A) {
#pragma unroll
                                for (int v = 0; v < DV; ++v) {
                                    pacc[m][0][v] = dp4a<SIGNED>(af[0], vals[v][0], pacc[m][0][v]);
                                    pacc[m][0][v] = dp4a<SIGNED>(af[2], vals[v][1], pacc[m][0][v]);
                                    pacc[m][1][v] = dp4a<SIGNED>(af[1], vals[v][0], pacc[m][1][v]);
                                    pacc[m][1][v] = dp4a<SIGNED>(af[3], vals[v][1], pacc[m][1][v]);
                                }
                            } else {
#pragma unroll
                                for (int bp = 0; bp < BP; ++bp) {
                                    if (SIGNED && bp == BP - 1)
                                        mma_k32<SIGNED, true>(acc[bp][m], af[0], af[1], af[2], af[3],
                                                              vals[bp][0], vals[bp][1]);
                                    else
                                        mma_k32<SIGNED, false>(acc[bp][m], af[0], af[1], af[2], af[3],
                                                               vals[bp][0], vals[bp][1]);
                                }
                            }
                        }
                    }
                }
                if (!((cs.flags >> 30) & 1)) continue;
                if constexpr (DP4A) {
                    // sum the four t lanes' partial sums; lane t then holds
                    // vector lanes 2t, 2t + 1 in the MMA accumulator layout
#pragma unroll
                    for (int m = 0; m < MT; ++m)
#pragma unroll
                        for (int hh = 0; hh < 2; ++hh)
#pragma unroll
                            for (int v = 0; v < DV; ++v) {
                                int x = pacc[m][hh][v];
                                x += __shfl_xor_sync(0xffffffffu, x, 1);
                                x += __shfl_xor_sync(0xffffffffu, x, 2);
                                pacc[m][hh][v] = x;
                            }
#pragma unroll
                    for (int m = 0; m < MT; ++m)
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int hh = e >> 1, vo = e & 1;
                            if constexpr (DV == 4) acc[0][m][e] = t ? pacc[m][hh][2 + vo] : pacc[m][hh][vo];
                            else acc[0][m][e] = pacc[m][hh][vo < DV ? vo : 0];
                        }
#pragma unroll
                    for (int m = 0; m < MT; ++m)
#pragma unroll
                        for (int hh = 0; hh < 2; ++hh)
#pragma unroll
                            for (int v = 0; v < DV; ++v) pacc[m][hh][v] = 0;
                }
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
                    const long long obase = (long long)b * p.out_stride + (long long)(cs.row * V + v) * p.n + n0;
                    if constexpr (PREB == 8) {
                        // r4[q]: column 8q + g
                        if constexpr (HALF_OUT) {
                            __half* o = reinterpret_cast<__half*>(p.out) + obase + g;
                            const Divisor dv = out_divisor(p, b, cs.row * V + v);
#pragma unroll
                            for (int q = 0; q < 2 * MT; ++q) o[8 * q] = deq_half(r4[q], dv);
                        } else {
                            int* o = reinterpret_cast<int*>(p.out) + obase + g;
#pragma unroll
                            for (int q = 0; q < 2 * MT; ++q) stg_cs_s32(o + 8 * q, r4[q]);
                        }
                    } else {
                        // chunk k: r4[4k], r4[4k+2] -> columns 32k + 2g, +1; r4[4k+1], r4[4k+3] -> +16, +17
                        if constexpr (HALF_OUT) {
                            __half* o = reinterpret_cast<__half*>(p.out) + obase + 2 * g;
                            const Divisor dv = out_divisor(p, b, cs.row * V + v);
#pragma unroll
                            for (int k = 0; k < MT / 2; ++k) {
                                stg_cs_s32(o + 32 * k, (int)pack_half2(r4[4 * k], r4[4 * k + 2], dv));
                                stg_cs_s32(o + 32 * k + 16, (int)pack_half2(r4[4 * k + 1], r4[4 * k + 3], dv));
                            }
                        } else {
                            int* o = reinterpret_cast<int*>(p.out) + obase + 2 * g;
#pragma unroll
                            for (int k = 0; k < MT / 2; ++k) {
                                stg_cs_v2(o + 32 * k, r4[4 * k], r4[4 * k + 2]);
                                stg_cs_v2(o + 32 * k + 16, r4[4 * k + 1], r4[4 * k + 3]);
                            }
                        }
                    }
                }
#pragma unroll
                for (int bp = 0; bp < BP; ++bp)
#pragma unroll
                    for (int m = 0; m < MT; ++m)
#pragma unroll
                        for (int e = 0; e < 4; ++e) acc[bp][m][e] = 0;
            }
        }
    }
}

}  // namespace mc
