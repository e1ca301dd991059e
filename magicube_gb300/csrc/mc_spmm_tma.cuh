// mc_spmm_tma.cuh -- warp-specialised SpMM for 8-bit and 4-bit B on sm_103a:
// B rows are gathered by the tensor memory accelerator.
//
// Same operands and results as spmm_stream_kernel (mc_spmm_stream.cuh) on the
// int8 tensor path.  A task is one (batch entry, vector-row);
// CTA x of the grid owns tasks x, x + gridDim.x, ... for one NT-column tile
// of C, and their 32-slot steps flow through a STAGES-deep ring:
//  * warp CWARPS, the producer, loads a step's column indices (one per lane) and
//    issues TMA tile::gather4 copies -- four B rows x 128 bytes per copy
//    (128 columns of 8-bit B, 256 of 4-bit B), straight from the row
//    coordinates -- plus one bulk copy of the step's
//    value chunk, all completing the stage's "full" mbarrier; lane 0 writes a
//    16-byte step header (row, batch entry, nonzero count, step, last/empty
//    flags) beside them before arriving with the expected byte count;
//  * warps 0 .. CWARPS-1, the consumers (NT / (16 CWARPS) 16-column MMA
//    tiles each), wait for the stage, read the header, turn the
//    128-byte-swizzled [slot][byte] rows into mma.m16n8k32 A fragments with
//    ldmatrix.m16n16.x2.trans.b8 (4-bit B: the masked low and high nibbles of
//    one fragment are the A fragments of two MMA tiles, columns 2c and 2c+1;
//    the value chunk is the B fragment), release
//    the stage through its "empty" mbarrier and write finished rows of C from
//    registers.  No CTA barrier inside the loop.
// Slots past a row's nonzero count gather row 0 of the batch entry's B, so
// every TMA coordinate lies inside the tensor; their value bytes are zeroed
// in registers, so their products vanish.  Every mbarrier wait is bounded: a
// wait that runs out increments the library's timeout counter and the CTA
// winds down (the producer first waits, bounded again, for the copies it
// issued) instead of hanging.
#pragma once
#include "mc_sm100.cuh"
#include "mc_spmm.cuh"
#include "mc_spmm_stream.cuh"

namespace mc {

template <int V, int PREA, int PREB, int NT, int STAGES, int CWARPS = 4>
struct SpmmTmaGeom {
    static constexpr int CW = CWARPS;                 // consumer warps
    static constexpr int THREADS = (CW + 1) * 32;
    static constexpr int MT = NT / (16 * CW);         // 16-column MMA tiles per consumer warp
    static constexpr int SLOT_BYTES = V * PREA / 8;   // value bytes per vector slot
    static constexpr int RB = NT * PREB / 8;          // bytes of one gathered row slice
    static constexpr int BOXES = RB / 128;            // 128-byte TMA boxes per row slice
    static constexpr int RHS_BYTES = 32 * RB;         // one stage of gathered rows (1024-byte multiple)
    static constexpr int AUX_BYTES = (32 * SLOT_BYTES + 16 + 127) / 128 * 128;  // values + header
    static constexpr size_t SMEM = 1024 + (size_t)STAGES * (RHS_BYTES + AUX_BYTES) + 2 * STAGES * 8;
};

template <int V, int PREA, int PREB, bool SIGNED, bool HALF_OUT, bool EXT, int NT, int STAGES, int CWARPS = 4,
          bool DP4A = false>
__global__ void __launch_bounds__((CWARPS + 1) * 32)
spmm_tma_kernel(const __grid_constant__ CUtensorMap tmap, const SpmmParams p, const int ntasks,
                const int rows_per_entry, unsigned int* timeouts)
{
    using namespace sm100;
    using L = SpmmLayout<PREA, PREB, EXT>;
    using G = SpmmTmaGeom<V, PREA, PREB, NT, STAGES, CWARPS>;
    constexpr int CW = G::CW, MT = G::MT, BP = L::BYTE_PLANES;
    constexpr int SLOT_BYTES = G::SLOT_BYTES, RB = G::RB, RHS_BYTES = G::RHS_BYTES, AUX_BYTES = G::AUX_BYTES;
    constexpr int HDR = 32 * SLOT_BYTES;              // header offset inside a stage's aux block
    constexpr long long WAIT = 4000000000LL;          // about 2 s at 2 GHz
    static_assert(PREB == 8 || PREB == 4, "8-bit or 4-bit B");
    static_assert(RB == 128 || RB == 256, "one or two 128-byte TMA boxes per gathered row");
    static_assert(PREB == 8 || MT % 2 == 0, "4-bit B: two MMA tiles per 16-byte chunk");
    static_assert(HDR % 16 == 0, "header alignment");
    static_assert(!DP4A || (V <= 4 && BP == 1), "the dp4a consumer computes V = 2 and 4 with 8-bit or 4-bit A");

    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = smem_raw + ((1024u - (saddr(smem_raw) & 1023u)) & 1023u);
    uint8_t* rhs_s = smem;                                  // STAGES x [NT/128][32 rows][128 B], swizzled
    uint8_t* aux_s = smem + STAGES * RHS_BYTES;             // STAGES x (value chunk, header)
    uint64_t* full = reinterpret_cast<uint64_t*>(aux_s + STAGES * AUX_BYTES);
    uint64_t* empty = full + STAGES;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
#pragma unroll
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, CW);
        }
        fence_mbar_init();
    }
    __syncthreads();
    const int n0 = blockIdx.y * NT;

    if (warp == CW) {
        // ------------------------------- producer -------------------------------
        if (lane == 0) prefetch_tmap(&tmap);
        // The next task's metadata and the next step's column indices are
        // requested one step ahead, so their latency overlaps the ring waits.
        auto load_task = [&](StreamTask& x, int task) {
            x.task = task;
            x.step = 0;
            x.steps = 0;
            if (task < ntasks) {
                x.b = task / p.m_vec;
                x.row = __ldg(p.row_indices + (task - x.b * p.m_vec));
                x.start = __ldg(p.row_offsets + 2 * x.row);
                x.nnz = __ldg(p.row_offsets + 2 * x.row + 1) - x.start;
                x.steps = (x.nnz + 31) >> 5;
            }
        };
        auto fetch_col = [&](const StreamTask& x) {
            const int j = 32 * x.step + lane;
            return (x.task < ntasks && j < x.nnz) ? __ldg(p.col_indices + x.start + col_slot<L::SHUFFLED_COLS>(j))
                                                  : -1;
        };
        auto next_of = [&](int task) {  // task + gridDim.x without int overflow
            const long long n = (long long)task + gridDim.x;
            return n < ntasks ? (int)n : ntasks;
        };
        StreamTask c, nx;
        load_task(c, blockIdx.x);
        load_task(nx, next_of(blockIdx.x));
        int col = fetch_col(c);
        int it = 0;
        bool ok = true;
        for (;; ++it) {
            const int slot = it % STAGES;
            if (it >= STAGES && !mbar_wait(empty + slot, ((it / STAGES) - 1) & 1, WAIT)) {
                ok = false;
                break;
            }
            uint8_t* aux = aux_s + slot * AUX_BYTES;
            if (c.task >= ntasks) {  // end of the stream: an empty stage with row -1
                if (lane == 0) {
                    *reinterpret_cast<int4*>(aux + HDR) = make_int4(-1, 0, 0, 0);
                    mbar_arrive(full + slot);
                }
                break;
            }
            const int rem = c.nnz - 32 * c.step;
            const int nvalid = rem < 0 ? 0 : (rem > 32 ? 32 : rem);
            const int ngroups = (nvalid + 3) >> 2;
            const int alen = (c.nnz + L::MMA_K - 1) / L::MMA_K * L::MMA_K;
            const int vbytes = nvalid > 0 ? min(32, alen - 32 * c.step) * SLOT_BYTES : 0;
            const int ybase = c.b * rows_per_entry;
            const int y = col >= 0 ? ybase + col : ybase;
            int yq[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) yq[i] = __shfl_sync(0xffffffffu, y, 4 * (lane & 7) + i);
            if (lane == 0) {
                int4 h;
                h.x = c.row;
                h.y = c.b;
                h.z = c.nnz;
                const int last = (c.steps == 0) || (c.step == c.steps - 1);
                h.w = c.step | (last << 30) | ((c.steps == 0) << 29);
                *reinterpret_cast<int4*>(aux + HDR) = h;
                mbar_arrive_expect_tx(full + slot, (uint32_t)(ngroups * 4 * RB + vbytes));
            }
            __syncwarp();
            if (lane < ngroups) {
                uint8_t* dst = rhs_s + slot * RHS_BYTES + lane * 512;  // box rows 4 lane .. 4 lane + 3
#pragma unroll
                for (int hf = 0; hf < G::BOXES; ++hf)
                    tma_gather4(dst + hf * 4096, &tmap, full + slot, n0 * PREB / 8 + hf * 128, yq[0], yq[1], yq[2],
                                yq[3]);
            }
            if (lane == 0 && vbytes > 0)
                bulk_load(aux,
                          p.values + (long long)c.b * p.values_stride + (long long)(c.start + 32 * c.step) * SLOT_BYTES,
                          (uint32_t)vbytes, full + slot);
            if (++c.step >= (c.steps > 0 ? c.steps : 1)) {
                c = nx;
                load_task(nx, c.task < ntasks ? next_of(c.task) : ntasks);
            }
            col = fetch_col(c);
        }
        if (!ok) {
            if (lane == 0) atomicAdd(timeouts, 1u);
            // the copies of the stages issued so far land before the CTA exits
            for (int j = (it > STAGES ? it - STAGES : 0); j < it; ++j)
                mbar_wait(full + j % STAGES, (j / STAGES) & 1, WAIT);
        }
        return;
    }

    // ------------------------------- consumers ------------------------------
    const int g = lane >> 2, t = lane & 3;
    int acc[BP][MT][4];
#pragma unroll
    for (int bp = 0; bp < BP; ++bp)
#pragma unroll
        for (int m = 0; m < MT; ++m)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[bp][m][e] = 0;
    // dp4a consumer: partial sums over this lane's slots (4t..4t+3, 16+4t..)
    // of output columns g (hh = 0) and g + 8 (hh = 1) of every tile, for
    // every vector lane; summed over the four t lanes when a row ends
    constexpr int DM = DP4A ? MT : 1, DV = DP4A ? V : 1;
    int pacc[DM][2][DV];
#pragma unroll
    for (int m = 0; m < DM; ++m)
#pragma unroll
        for (int hh = 0; hh < 2; ++hh)
#pragma unroll
            for (int v = 0; v < DV; ++v) pacc[m][hh][v] = 0;

#pragma unroll 1
    for (int it = 0;; ++it) {
        const int slot = it % STAGES;
        if (!mbar_wait(full + slot, (it / STAGES) & 1, WAIT)) {
            if (lane == 0) atomicAdd(timeouts, 1u);
            break;
        }
        const uint8_t* aux = aux_s + slot * AUX_BYTES;
        const int4 hdr = *reinterpret_cast<const int4*>(aux + HDR);
        if (hdr.x < 0) break;  // stream exhausted
        const int step = hdr.w & 0x1fffffff;
        const bool last = (hdr.w >> 30) & 1;
        const bool empty_row = (hdr.w >> 29) & 1;
        const int nnz = hdr.z;
        if (!empty_row) {
            // value fragments: vals[bp][h] for vector lane v = g, slots 16h+4t..+3
            // (dp4a: vv[v][h] for every vector lane v)
            uint32_t vals[BP][2];
            uint32_t vv[DV][2];
#pragma unroll
            for (int bp = 0; bp < BP; ++bp) { vals[bp][0] = 0u; vals[bp][1] = 0u; }
            if constexpr (DP4A) {
                const bool whole = step * 32 + 32 <= nnz;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const uint32_t keep = whole ? 0xffffffffu : byte_mask(nnz - (step * 32 + 16 * h + 4 * t));
#pragma unroll
                    for (int v = 0; v < DV; ++v) {
                        if constexpr (L::VCHUNK == 16) {
                            vv[v][h] = lds32(aux + h * 16 * SLOT_BYTES + vword16<V, PREA, PREB, EXT>(v, t, 0)) & keep;
                        } else {
                            constexpr int PLANE_BYTES = V * 32 * L::PLANE_BITS / 8;
                            const int o = v * 16 + 8 * h + 2 * t;
                            if constexpr (PREA == 4)
                                vv[v][h] = unpack4_u16<SIGNED>(lds16(aux + o)) & keep;
                            else
                                vv[v][h] = merge_nibble_planes(lds16(aux + o), lds16(aux + PLANE_BYTES + o)) & keep;
                        }
                    }
                }
            } else if (g < V) {
                const bool whole = step * 32 + 32 <= nnz;  // no slot of this step past the row end
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const uint32_t keep = whole ? 0xffffffffu : byte_mask(nnz - (step * 32 + 16 * h + 4 * t));
                    if constexpr (L::VCHUNK == 16) {
#pragma unroll
                        for (int bp = 0; bp < BP; ++bp)
                            vals[bp][h] =
                                lds32(aux + h * 16 * SLOT_BYTES + vword16<V, PREA, PREB, EXT>(g, t, bp)) & keep;
                    } else {
                        // one 32-slot chunk of 4-bit planes [v][slot]
                        constexpr int PLANE_BYTES = V * 32 * L::PLANE_BITS / 8;
                        uint32_t nib[L::PLANES];
#pragma unroll
                        for (int pl = 0; pl < L::PLANES; ++pl)
                            nib[pl] = lds16(aux + pl * PLANE_BYTES + g * 16 + 8 * h + 2 * t);
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
            // A fragments of this warp's 16 MT columns: lane r addresses slot row r
            const uint8_t* st = rhs_s + slot * RHS_BYTES;
            uint32_t af[MT][4];
            if constexpr (PREB == 8) {
#pragma unroll
                for (int m = 0; m < MT; ++m) {
                    const int cc = MT * warp + m;  // 16-byte chunk = 16 columns
                    ldsm_x2_trans_b8(af[m], st + (cc >> 3) * 4096 + lane * 128 + (((cc & 7) ^ (lane & 7)) << 4));
                }
            } else {
#pragma unroll
                for (int k = 0; k < MT / 2; ++k) {
                    const int cc = (MT / 2) * warp + k;  // 16-byte chunk = 32 columns: tiles 2k (low), 2k+1 (high)
                    uint32_t nb[4];
                    ldsm_x2_trans_b8(nb, st + (cc >> 3) * 4096 + lane * 128 + (((cc & 7) ^ (lane & 7)) << 4));
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const uint32_t lo = nb[q] & 0x0F0F0F0Fu, hi = (nb[q] >> 4) & 0x0F0F0F0Fu;
                        af[2 * k][q] = SIGNED ? sext_nibble_bytes(lo) : lo;
                        af[2 * k + 1][q] = SIGNED ? sext_nibble_bytes(hi) : hi;
                    }
                }
            }
            if constexpr (DP4A) {
#pragma unroll
                for (int m = 0; m < MT; ++m)
#pragma unroll
                    for (int v = 0; v < DV; ++v) {
                        pacc[m][0][v] = dp4a<SIGNED>(af[m][0], vv[v][0], pacc[m][0][v]);
                        pacc[m][0][v] = dp4a<SIGNED>(af[m][2], vv[v][1], pacc[m][0][v]);
                        pacc[m][1][v] = dp4a<SIGNED>(af[m][1], vv[v][0], pacc[m][1][v]);
                        pacc[m][1][v] = dp4a<SIGNED>(af[m][3], vv[v][1], pacc[m][1][v]);
                    }
            }
#pragma unroll
            for (int bp = 0; bp < (DP4A ? 0 : BP); ++bp) {
                const bool top = (bp == BP - 1);
#pragma unroll
                for (int m = 0; m < MT; ++m) {
                    if (SIGNED && top)
                        mma_k32<SIGNED, true>(acc[bp][m], af[m][0], af[m][1], af[m][2], af[m][3], vals[bp][0],
                                              vals[bp][1]);
                    else
                        mma_k32<SIGNED, false>(acc[bp][m], af[m][0], af[m][1], af[m][2], af[m][3], vals[bp][0],
                                               vals[bp][1]);
                }
            }
        }
        __syncwarp();  // every lane has read the stage
        if (lane == 0) mbar_arrive(empty + slot);
        if (last) {
            if constexpr (DP4A) {
                // sum the four t lanes' partial sums; lane t then holds vector
                // lanes 2t, 2t + 1 in the MMA accumulator layout below
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
                        pacc[m][hh][vo] = 0;
                        if constexpr (DV == 4) pacc[m][hh][2 + vo] = 0;
                    }
            }
            // acc[.][m][e]: vector lane 2t + (e & 1), column of the warp's slice
            // 8-bit B: 16m + 8(e>>1) + g;  4-bit B: 32(m>>1) + 2g + (m&1) + 16(e>>1)
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
                    // r4[q]: column 8q + g
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
                    // chunk k: r4[4k], r4[4k+2] -> columns 32k + 2g, +1; r4[4k+1], r4[4k+3] -> +16, +17
                    if constexpr (HALF_OUT) {
                        __half* o = reinterpret_cast<__half*>(p.out) + obase + 2 * g;
                        const Divisor dv = out_divisor(p, b, row * V + v);
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

}  // namespace mc
