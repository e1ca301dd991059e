// mc_spmm_dense.cuh -- SpMM as dense tiles on the 5th-generation tensor
// cores (8-bit A and B, int32 output).
//
// C = A * B for a vector-sparse A (M x K, column vectors of V rows) and a
// dense B (K x N).  sm_103a has no integer tcgen05 MMA, and its int8
// mma.sync runs at 158 TOP/s while tcgen05 kind::f16 runs at about 2.4
// PFLOP/s dense.  This kernel expands each 256-row block of A into dense f16
// tiles in shared memory, 64 columns of k at a time, and multiplies the whole
// tile: at sparsity 0.9 it computes ten times the useful products, but on a
// pipe fifteen times faster, and its speed does not depend on V (the
// mma.sync kernels compute 8 vector lanes whatever V is).
//
// Exactness: every 8-bit value is an exact f16; each product is an integer
// of magnitude <= 2^14 (signed) or < 2^16 (unsigned lanes); the f32
// accumulator holds every partial sum exactly while it stays within 2^24.
// The k chunks are therefore accumulated in segments of at most 1024
// (signed) or 256 (unsigned) columns: each segment has its own TMEM
// accumulation, and the epilogue adds the segments in int32 (the first
// stores, later ones load, add and store their own earlier partial sums).
//
// Tile: 128 columns of C (the MMA's M, TMEM lanes) x 256 rows of A (the
// MMA's N, TMEM columns), k chunks of 64 (four MMAs with K = 16).  Both
// operands are MN-major with 128-byte swizzling, so neither needs a
// transpose:
//  * B chunk (64 k x 128 columns of int8): copied by TMA into a ring of raw
//    tiles; eight converter warps turn each 16-byte row piece into 16 f16
//    (prmt + sub.f16x2) and store them in [k/8][n/64][k%8][64 n] atoms;
//  * A chunk (256 rows x 64 k): the tiles start zeroed; four groups of two
//    builder warps (group g builds every fourth chunk, always into stage g)
//    write each nonzero vector whose column lies in the chunk as V
//    consecutive f16 of one k row ([k/8][r/64][k%8][64 r] atoms, one 16-byte
//    store at V = 8) and, once the MMAs have read the stage, write zeros
//    over exactly the vectors they wrote (a 64-bit mask of k offsets per
//    thread and stage), so a tile is never cleared as a whole.  The slots of
//    vector-row R in chunk c are [starts[R][c], starts[R][c+1]): the table
//    that mcSpmmChunkStarts builds, which also checks that every row's
//    columns are strictly increasing and inside [0, k);
//  * one thread issues the MMAs into one of two 256-column TMEM
//    accumulators; four epilogue warps (one per TMEM lane quadrant) read 32
//    columns at a time (tcgen05.ld 32x32b.x32), convert them to int32 and
//    store rows of 128 bytes.
// Persistent CTAs (one per SM) walk the work items (batch entry, block of
// 256 A rows, block of 128 C columns).  The roles that wait long (TMA,
// converters, epilogue) sleep between polls, leaving the issue slots to the
// builders; the MMA thread and the builders poll.  Every mbarrier wait is bounded: a
// wait that runs out increments the timeout counter and that role stops;
// the MMA thread then waits (bounded) for its MMAs, and the TMA thread for
// its copies, before the CTA frees TMEM and returns.
#pragma once
#include "mc_sm100.cuh"
#include "mc_spmm.cuh"

namespace mc {

struct SpmmDenseParams {
    SpmmParams s;
    const int* chunk_starts;  // [m_vec][kchunks + 1]
    int kchunks;              // ceil(k / 64)
    int seg;                  // k chunks per accumulation segment
    int row_blocks;           // ceil(m_vec * V / 256)
    int col_blocks;           // n / 128
    int items;                // batch * row_blocks * col_blocks
    int rows_per_entry;       // B rows between batch entries in the tensor map
};

namespace sdense {
constexpr int BN = 128;  // C columns per tile: MMA M, TMEM lanes
constexpr int AR = 256;  // A rows per tile: MMA N, TMEM columns per accumulator
constexpr int KC = 64;   // k per chunk
constexpr int STAGES = 4, RAW = 4;
constexpr int BT_BYTES = BN * KC * 2;  // f16 B chunk
constexpr int A_BYTES = AR * KC * 2;   // f16 A chunk
constexpr int RAW_BYTES = KC * BN;     // int8 B chunk as TMA writes it
constexpr int STAGE_BYTES = BT_BYTES + A_BYTES;
constexpr int RAW_OFF = STAGES * STAGE_BYTES;
constexpr int BAR_OFF = RAW_OFF + RAW * RAW_BYTES;
constexpr int NBARS = 2 * RAW + 3 * STAGES + 5;
constexpr int SMEM = 1024 + BAR_OFF + NBARS * 8 + 16;
constexpr int EPI = 4, CONV = 8, BGROUPS = 4, BUILD = 2 * BGROUPS;
constexpr int W_CONV = EPI, W_BUILD = EPI + CONV, W_TMA = EPI + CONV + BUILD, W_MMA = W_TMA + 1;
constexpr int THREADS = (W_MMA + 1) * 32;
constexpr long long WAIT = 4000000000LL;  // about 2 s at 2 GHz
// Byte strides of the MN-major atoms: between 64-element blocks along M / N
// and between groups of 8 k rows.
constexpr uint32_t BT_MN = 1024, BT_K = 2048, A_MN = 1024, A_K = 4096;
static_assert(SMEM <= 232448, "shared memory");
}  // namespace sdense

// Byte offset of element (mn, k) in an MN-major 128-byte-swizzled f16 tile
// whose 8-k groups are K_STRIDE bytes apart: [k/8][mn/64][k%8][64 mn].
template <uint32_t K_STRIDE>
__device__ __forceinline__ uint32_t mn_tile_off(int mn, int k)
{
    return (uint32_t)(k >> 3) * K_STRIDE + (uint32_t)(mn >> 6) * 1024u + (uint32_t)(k & 7) * 128u +
           ((uint32_t)(((mn & 63) >> 3) ^ (k & 7)) << 4) + (uint32_t)(mn & 7) * 2u;
}

// Shared-memory descriptor of an MN-major 128-byte-swizzled operand:
// leading-dimension offset = the stride between 64-element MN blocks,
// stride-dimension offset = the stride between 8-k groups.
__device__ __forceinline__ uint64_t desc_sw128_mn(uint32_t smem_addr, uint32_t mn_stride, uint32_t k_stride)
{
    uint64_t d = 0;
    d |= (uint64_t)((smem_addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((mn_stride >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((k_stride >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version
    d |= (uint64_t)2 << 61;  // 128-byte swizzle
    return d;
}

template <int V, bool SIGNED, bool SLOTMAJOR = false>
__global__ void __launch_bounds__(sdense::THREADS, 1)
spmm_dense_tc_kernel(const __grid_constant__ CUtensorMap tmap, const SpmmDenseParams dp, unsigned int* timeouts)
{
    using namespace sm100;
    using namespace sdense;
    static_assert(V == 2 || V == 4 || V == 8, "V");
    constexpr int NVR = AR / V;     // vector-rows per tile
    const SpmmParams& p = dp.s;
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw0 = saddr(smem_raw);
    uint8_t* smem = smem_raw + (((raw0 + 1023u) & ~1023u) - raw0);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + BAR_OFF);
    uint64_t* raw_full = bars;
    uint64_t* raw_empty = bars + RAW;
    uint64_t* bt_full = bars + 2 * RAW;
    uint64_t* a_full = bt_full + STAGES;
    uint64_t* st_empty = a_full + STAGES;
    uint64_t* t_full = st_empty + STAGES;
    uint64_t* t_empty = t_full + 2;
    uint64_t* fin = t_empty + 2;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(fin + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < STAGES * (A_BYTES / 16); i += THREADS) {
        const int s = i / (A_BYTES / 16), o = i - s * (A_BYTES / 16);
        *reinterpret_cast<uint4*>(smem + s * STAGE_BYTES + BT_BYTES + o * 16) = make_uint4(0u, 0u, 0u, 0u);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (tid == 0) {
        for (int r = 0; r < RAW; ++r) {
            mbar_init(raw_full + r, 1);
            mbar_init(raw_empty + r, CONV);
        }
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(bt_full + s, CONV);
            mbar_init(a_full + s, 2);
            mbar_init(st_empty + s, 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(t_full + i, 1);
            mbar_init(t_empty + i, EPI);
        }
        mbar_init(fin, 1);
        fence_mbar_init();
    }
    if (warp == W_MMA) {
        tmem_alloc(tmem_slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const int per_entry = dp.row_blocks * dp.col_blocks;

    if (warp == W_TMA) {
        // ------------------------------ TMA copies ------------------------------
        if (lane == 0) {
            prefetch_tmap(&tmap);
            // The vector-rows of a tile hold one contiguous range of slots: their
            // columns, values and chunk-table rows are prefetched into L2 an item
            // ahead, so the builders' loads do not wait on DRAM.
            auto prefetch_item = [&](int it) {
                if (it >= dp.items) return;
                const int b = it / per_entry, rb = (it - b * per_entry) / dp.col_blocks;
                const int R0 = rb * NVR, R1 = min(R0 + NVR, p.m_vec) - 1;
                if (R1 < R0) return;
                const int s0 = __ldg(p.row_offsets + 2 * R0), s1 = __ldg(p.row_offsets + 2 * R1 + 1);
                if (s1 > s0) {
                    const int c0 = s0 & ~3, c1 = (s1 + 3) & ~3;  // inside the aligned column array
                    bulk_prefetch_l2(p.col_indices + c0, (uint32_t)(c1 - c0) * 4u);
                    const long long v0 = (long long)(s0 >> 4) * (16 * V), v1 = (long long)((s1 + 15) >> 4) * (16 * V);
                    bulk_prefetch_l2(p.values + (long long)b * p.values_stride + v0, (uint32_t)(v1 - v0));
                }
                const uintptr_t t0 = reinterpret_cast<uintptr_t>(dp.chunk_starts + (long long)R0 * (dp.kchunks + 1));
                const uintptr_t t1 = reinterpret_cast<uintptr_t>(dp.chunk_starts + (long long)(R1 + 1) * (dp.kchunks + 1));
                const uintptr_t a0 = (t0 + 15) & ~(uintptr_t)15, a1 = t1 & ~(uintptr_t)15;
                if (a1 > a0) bulk_prefetch_l2(reinterpret_cast<const void*>(a0), (uint32_t)(a1 - a0));
            };
            prefetch_item(blockIdx.x);
            long long cc = 0;
            bool ok = true;
            for (int item = blockIdx.x; item < dp.items && ok; item += gridDim.x) {
                prefetch_item(item + gridDim.x);
                const int b = item / per_entry, cb = (item - b * per_entry) % dp.col_blocks;
                for (int kc = 0; kc < dp.kchunks; ++kc, ++cc) {
                    const int r = (int)(cc % RAW);
                    if (cc >= RAW && !mbar_wait_sleep(raw_empty + r, (uint32_t)((cc / RAW) - 1) & 1u, WAIT, 64)) {
                        ok = false;
                        break;
                    }
                    mbar_arrive_expect_tx(raw_full + r, RAW_BYTES);
                    tma_load_2d(smem + RAW_OFF + r * RAW_BYTES, &tmap, raw_full + r, cb * BN,
                                b * dp.rows_per_entry + kc * KC);
                }
            }
            if (!ok) atomicAdd(timeouts, 1u);
            // every copy issued has landed before the CTA may leave
            for (int r = 0; r < RAW; ++r) {
                const long long uses = cc > r ? (cc - 1 - r) / RAW + 1 : 0;  // copies issued into slot r
                if (uses > 0 && !mbar_wait(raw_full + r, (uint32_t)(uses - 1) & 1u, WAIT)) atomicAdd(timeouts, 1u);
            }
        }
    } else if (warp == W_MMA) {
        // --------------------------------- MMA ---------------------------------
        if (lane == 0) {
            constexpr uint32_t IDESC = idesc_f16_f32(BN, AR) | (1u << 15) | (1u << 16);  // A, B MN-major
            long long cc = 0;
            int unit = 0;
            bool ok = true;
            for (int item = blockIdx.x; item < dp.items && ok; item += gridDim.x) {
                for (int s0 = 0; s0 < dp.kchunks; s0 += dp.seg, ++unit) {
                    const int tb = unit & 1;
                    if (unit >= 2 && !mbar_wait(t_empty + tb, (uint32_t)((unit >> 1) - 1) & 1u, WAIT)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const int s1 = min(s0 + dp.seg, dp.kchunks);
                    for (int kc = s0; kc < s1; ++kc, ++cc) {
                        const int s = (int)(cc % STAGES);
                        const uint32_t ph = (uint32_t)(cc / STAGES) & 1u;
                        if (!mbar_wait(bt_full + s, ph, WAIT) || !mbar_wait(a_full + s, ph, WAIT)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t bt = saddr(smem + s * STAGE_BYTES), at = bt + BT_BYTES;
#pragma unroll
                        for (int k4 = 0; k4 < 4; ++k4)  // K = 16: two 8-k groups per MMA
                            mma_f16_ss(tmem + (uint32_t)(tb * AR), desc_sw128_mn(bt + k4 * 2 * BT_K, BT_MN, BT_K),
                                       desc_sw128_mn(at + k4 * 2 * A_K, A_MN, A_K), IDESC, (kc > s0 || k4 > 0));
                        mma_commit(st_empty + s);
                    }
                    if (!ok) break;
                    mma_commit(t_full + tb);
                }
            }
            if (!ok) atomicAdd(timeouts, 1u);
            // every MMA issued so far completes before TMEM is released
            mma_commit(fin);
            if (!mbar_wait(fin, 0, WAIT)) atomicAdd(timeouts, 1u);
        }
    } else if (warp >= W_CONV && warp < W_CONV + CONV) {
        // ------------------------------ converters ------------------------------
        const int ct = tid - 32 * W_CONV;
        long long cc = 0;
        bool ok = true;
        for (int item = blockIdx.x; item < dp.items && ok; item += gridDim.x) {
            for (int kc = 0; kc < dp.kchunks; ++kc, ++cc) {
                const int r = (int)(cc % RAW), s = (int)(cc % STAGES);
                if (!mbar_wait_sleep(raw_full + r, (uint32_t)(cc / RAW) & 1u, WAIT, 64) ||
                    (cc >= STAGES && !mbar_wait_sleep(st_empty + s, (uint32_t)((cc / STAGES) - 1) & 1u, WAIT, 64))) {
                    ok = false;
                    break;
                }
                const uint8_t* rt = smem + RAW_OFF + r * RAW_BYTES;
                uint8_t* bt = smem + s * STAGE_BYTES;
                constexpr int PIECES = RAW_BYTES / 16 / (CONV * 32);  // 16-byte row pieces per thread
                uint4 w[PIECES];
#pragma unroll
                for (int i = 0; i < PIECES; ++i)
                    w[i] = *reinterpret_cast<const uint4*>(rt + (ct + CONV * 32 * i) * 16);
                uint32_t h[PIECES][8];
#pragma unroll
                for (int i = 0; i < PIECES; ++i) {
                    bytes_to_h2<SIGNED>(w[i].x, h[i][0], h[i][1]);
                    bytes_to_h2<SIGNED>(w[i].y, h[i][2], h[i][3]);
                    bytes_to_h2<SIGNED>(w[i].z, h[i][4], h[i][5]);
                    bytes_to_h2<SIGNED>(w[i].w, h[i][6], h[i][7]);
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(raw_empty + r);
#pragma unroll
                for (int i = 0; i < PIECES; ++i) {
                    const int pc = ct + CONV * 32 * i, k = pc >> 3, n = (pc & 7) * 16;  // 16 columns of row k
                    *reinterpret_cast<uint4*>(bt + mn_tile_off<BT_K>(n, k)) =
                        make_uint4(h[i][0], h[i][1], h[i][2], h[i][3]);
                    *reinterpret_cast<uint4*>(bt + mn_tile_off<BT_K>(n + 8, k)) =
                        make_uint4(h[i][4], h[i][5], h[i][6], h[i][7]);
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(bt_full + s);
            }
        }
        if (!ok && lane == 0) atomicAdd(timeouts, 1u);
    } else if (warp >= W_BUILD && warp < W_BUILD + BUILD) {
        // ------------------------------- builders -------------------------------
        // BGROUPS groups of two warps; group g builds the chunks with
        // cc % BGROUPS == g, always into stage g, so each group has BGROUPS
        // MMA periods for the loads and stores of a chunk.  A thread owns RPT
        // vector-rows of the tile (V = 2) or shares one with G - 1 others
        // (V = 8) and takes that row's quads -- 4 aligned slots: one 16-byte
        // load of columns, one 4-byte load of values per vector lane -- with
        // index u mod G.
        constexpr int TPG = 64;                             // threads per group
        constexpr int RPT = NVR > TPG ? NVR / TPG : 1;      // vector-rows per thread
        constexpr int G = NVR < TPG ? TPG / NVR : 1;        // threads per vector-row
        constexpr int QU = V == 8 ? 2 : 3;                  // quads loaded at once
        static_assert(BGROUPS == STAGES && BUILD == 2 * BGROUPS, "one stage per two-warp group");
        const int grp = (warp - W_BUILD) >> 1;
        const int t = tid - 32 * (W_BUILD + 2 * grp);
        const int u = t % G;
        uint64_t mask[RPT];  // k offsets this thread wrote into the group's stage, per owned row
#pragma unroll
        for (int q = 0; q < RPT; ++q) mask[q] = 0;
        uint8_t* at = smem + grp * STAGE_BYTES + BT_BYTES;
        long long cc = 0;
        bool ok = true;
        for (int item = blockIdx.x; item < dp.items && ok; item += gridDim.x) {
            const int b = item / per_entry, rb = (item - b * per_entry) / dp.col_blocks;
            const uint8_t* vals = p.values + (long long)b * p.values_stride;
            // this group's first chunk of the item
            int kc = (int)((grp - cc % BGROUPS + BGROUPS) % BGROUPS);
            const long long item_cc = cc;
            for (; kc < dp.kchunks; kc += BGROUPS) {
                const long long c = item_cc + kc;
                // the chunk table entries of the owned rows (issued before the wait)
                int lo[RPT], hi[RPT];
#pragma unroll
                for (int q = 0; q < RPT; ++q) {
                    const int vi = RPT > 1 ? t + TPG * q : t / G;
                    const int R = rb * NVR + vi;
                    const bool valid = R < p.m_vec;
                    const int* cs = dp.chunk_starts + (long long)(valid ? R : 0) * (dp.kchunks + 1) + kc;
                    lo[q] = valid ? __ldg(cs) : 0;
                    hi[q] = valid ? __ldg(cs + 1) : 0;
                }
                if (c >= STAGES && !mbar_wait(st_empty + grp, (uint32_t)((c / STAGES) - 1) & 1u, WAIT)) {
                    ok = false;
                    break;
                }
                const int kbase = kc * KC;
#pragma unroll
                for (int q = 0; q < RPT; ++q) {
                    const int vi = RPT > 1 ? t + TPG * q : t / G;
                    const int r0 = vi * V;  // first A row of the vector-row in the tile
                    // zeros over the vectors written into this stage BGROUPS chunks ago
                    for (uint64_t m = mask[q]; m; m &= m - 1) {
                        uint8_t* dst = at + mn_tile_off<A_K>(r0, __ffsll((long long)m) - 1);
                        if constexpr (V == 8) *reinterpret_cast<uint4*>(dst) = make_uint4(0u, 0u, 0u, 0u);
                        else if constexpr (V == 4) *reinterpret_cast<uint2*>(dst) = make_uint2(0u, 0u);
                        else *reinterpret_cast<uint32_t*>(dst) = 0u;
                    }
                    uint64_t nm = 0;
                    const int qlo = lo[q] >> 2, qhi = (hi[q] + 3) >> 2;
                    for (int qb = qlo + u; qb < qhi; qb += G * QU) {
                        // every load of up to QU quads first, then the conversions and stores
                        int4 c4[QU];
                        uint32_t w[QU][V];
#pragma unroll
                        for (int i = 0; i < QU; ++i) {
                            const int j0 = (qb + G * i < qhi ? qb + G * i : qb) * 4;
                            c4[i] = ldg_nc_v4(p.col_indices + j0);
                            if constexpr (SLOTMAJOR) {
                                // the quad's 4 x V bytes, already slot by slot: w[s] (and
                                // w[4 + s]) as the transposes below leave them
                                const uint8_t* src = vals + (long long)j0 * V;
                                if constexpr (V == 8) {
                                    const int4 a = ldg_nc_v4(src), b = ldg_nc_v4(src + 16);
                                    w[i][0] = (uint32_t)a.x; w[i][4] = (uint32_t)a.y;
                                    w[i][1] = (uint32_t)a.z; w[i][5] = (uint32_t)a.w;
                                    w[i][2] = (uint32_t)b.x; w[i][6] = (uint32_t)b.y;
                                    w[i][3] = (uint32_t)b.z; w[i][7] = (uint32_t)b.w;
                                } else if constexpr (V == 4) {
                                    const int4 a = ldg_nc_v4(src);
                                    w[i][0] = (uint32_t)a.x; w[i][1] = (uint32_t)a.y;
                                    w[i][2] = (uint32_t)a.z; w[i][3] = (uint32_t)a.w;
                                } else {
                                    const int2 a = ldg_nc_v2(src);  // slots 0-1 in a.x, 2-3 in a.y
                                    w[i][0] = (uint32_t)a.x;
                                    w[i][1] = (uint32_t)a.y;
                                }
                            } else {
                                const uint8_t* src = vals + (long long)(j0 >> 4) * (16 * V) + (j0 & 15);
#pragma unroll
                                for (int v = 0; v < V; ++v)
                                    w[i][v] = __ldg(reinterpret_cast<const uint32_t*>(src + 16 * v));
                            }
                        }
#pragma unroll
                        for (int i = 0; i < QU; ++i) {
                            if (qb + G * i >= qhi) break;
                            const int j0 = (qb + G * i) * 4;
                            if constexpr (V >= 4 && !SLOTMAJOR) {
                                // w[v] holds lane v of the four slots; after this w[s] holds
                                // lanes 0-3 of slot s (and w[4 + s] lanes 4-7)
                                uint32_t a[4] = {w[i][0], w[i][1], w[i][2], w[i][3]};
                                transpose4x4(a);
#pragma unroll
                                for (int e = 0; e < 4; ++e) w[i][e] = a[e];
                                if constexpr (V == 8) {
                                    uint32_t c[4] = {w[i][4], w[i][5], w[i][6], w[i][7]};
                                    transpose4x4(c);
#pragma unroll
                                    for (int e = 0; e < 4; ++e) w[i][4 + e] = c[e];
                                }
                            }
                            const int cols[4] = {c4[i].x, c4[i].y, c4[i].z, c4[i].w};
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                const int j = j0 + e;
                                const int kk = cols[e] - kbase;
                                if (j < lo[q] || j >= hi[q] || (unsigned)kk >= (unsigned)KC) continue;
                                uint8_t* dst = at + mn_tile_off<A_K>(r0, kk);
                                uint32_t h0, h1;
                                if constexpr (V == 8) {
                                    uint32_t h2, h3;
                                    bytes_to_h2<SIGNED>(w[i][e], h0, h1);
                                    bytes_to_h2<SIGNED>(w[i][4 + e], h2, h3);
                                    *reinterpret_cast<uint4*>(dst) = make_uint4(h0, h1, h2, h3);
                                } else if constexpr (V == 4) {
                                    bytes_to_h2<SIGNED>(w[i][e], h0, h1);
                                    *reinterpret_cast<uint2*>(dst) = make_uint2(h0, h1);
                                } else {
                                    // slot-major: slot e's two lanes are bytes 2e, 2e + 1 of the
                                    // 8 loaded bytes; packed: byte e of lane 0's and lane 1's word
                                    const uint32_t x = SLOTMAJOR ? (w[i][e >> 1] >> (16 * (e & 1)))
                                                                 : prmt(w[i][0], w[i][1], (uint32_t)(e | ((e + 4) << 4)));
                                    bytes_to_h2<SIGNED>(x, h0, h1);
                                    *reinterpret_cast<uint32_t*>(dst) = h0;
                                }
                                nm |= 1ull << kk;
                            }
                        }
                    }
                    mask[q] = nm;
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(a_full + grp);
            }
            cc = item_cc + dp.kchunks;
        }
        if (!ok && lane == 0) atomicAdd(timeouts, 1u);
    } else {
        // ------------------------------- epilogue ------------------------------
        const int q = warp & 3;   // TMEM lanes 32q .. 32q+31: C columns; every TMEM column (A row)
        const int M = p.m_vec * V;
        int unit = 0;
        bool ok = true;
        for (int item = blockIdx.x; item < dp.items && ok; item += gridDim.x) {
            const int b = item / per_entry, rem = item - b * per_entry;
            const int rb = rem / dp.col_blocks, cb = rem - rb * dp.col_blocks;
            int* outb = reinterpret_cast<int*>(p.out) + (long long)b * p.out_stride + cb * BN + 32 * q + lane;
            for (int s0 = 0; s0 < dp.kchunks; s0 += dp.seg, ++unit) {
                const int tb = unit & 1;
                if (!mbar_wait_sleep(t_full + tb, (uint32_t)(unit >> 1) & 1u, WAIT, 256)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t tcol = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(tb * AR);
#pragma unroll 1
                for (int c = 0; c < AR; c += 32) {
                    uint32_t acc[32];
                    tmem_ld_x32(tcol + (uint32_t)c, acc);
                    tmem_ld_wait();
                    const int row0 = rb * AR + c;
                    const long long step = p.n;
                    int* o = outb + (long long)row0 * step;
                    if (s0 == 0) {
#pragma unroll
                        for (int j = 0; j < 32; ++j, o += step)
                            if (row0 + j < M) *o = __float2int_rn(__uint_as_float(acc[j]));
                    } else {
#pragma unroll
                        for (int g = 0; g < 32; g += 8) {  // earlier segments' sums, 8 rows at a time
                            int prev[8];
#pragma unroll
                            for (int j = 0; j < 8; ++j) prev[j] = row0 + g + j < M ? o[j * step] : 0;
#pragma unroll
                            for (int j = 0; j < 8; ++j)
                                if (row0 + g + j < M) o[j * step] = prev[j] + __float2int_rn(__uint_as_float(acc[g + j]));
                            o += 8 * step;
                        }
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(t_empty + tb);
            }
        }
        if (!ok && lane == 0) atomicAdd(timeouts, 1u);
    }

    tc_fence_before();
    __syncthreads();
    if (warp == W_MMA) {
        tc_fence_after();
        tmem_dealloc(tmem, 512);
    }
}

// Slot ranges of the k chunks of every vector-row, for the dense-tile SpMM:
// starts[R][c] = the first slot of vector-row R whose column is >= 64 c
// (c = 0 .. kchunks; starts[R][0] is the row's start, starts[R][kchunks]
// its end).  One warp per vector-row; status |= 1 if a row's columns are not
// strictly increasing or lie outside [0, k) -- its chunks are then all left
// empty, so a launch reads no slot of it.
__global__ void __launch_bounds__(128)
spmm_chunk_starts_kernel(int m_vec, int k, int kchunks, const int* __restrict__ row_offsets,
                         const int* __restrict__ cols, int* __restrict__ starts, int* status)
{
    const int R = blockIdx.x * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (R >= m_vec) return;
    const int start = __ldg(row_offsets + 2 * R);
    const int nnz = __ldg(row_offsets + 2 * R + 1) - start;
    const int* c = cols + start;
    bool bad = nnz < 0;
    for (int j = lane; j < nnz; j += 32) {
        const int x = __ldg(c + j);
        if (x < 0 || x >= k || (j > 0 && __ldg(c + j - 1) >= x)) bad = true;
    }
    int* out = starts + (long long)R * (kchunks + 1);
    if (__any_sync(0xffffffffu, bad)) {
        for (int ch = lane; ch <= kchunks; ch += 32) out[ch] = start;
        if (lane == 0) atomicOr(status, 1);
        return;
    }
    for (int ch = lane; ch <= kchunks; ch += 32) {
        const int key = 64 * ch;
        int lo = 0, hi = nnz;  // first j with c[j] >= key
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(c + mid) < key) lo = mid + 1;
            else hi = mid;
        }
        out[ch] = start + lo;
    }
}

}  // namespace mc
