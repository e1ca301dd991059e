// mc_sddmm_dense.cuh -- SDDMM as dense tiles on the 5th-generation tensor
// cores with a sparse epilogue (8-bit operands, k == 64).
//
// out[j, v] = A[row*V + v] . B[col_j] for every stored nonzero vector j.  At
// the sparsity of attention masks (~0.9) computing every score of a tile on
// the f16 tensor cores (2.4 PFLOP/s dense on GB300) costs less than gathering
// one 64-byte B row per nonzero for the int8 mma.sync path (158 TOP/s), and
// the B rows are read once per tile instead of once per nonzero.  Exactness:
// every int8 value is an exact f16, every product an integer below 2^15 in
// magnitude, and 64 of them sum below 2^24, so the f32 accumulator holds the
// integer dot product exactly.
//
// Tile: 128 rows of B (output columns n0 .. n0+127, the MMA's M) x 256 rows of
// A (256 / V vector-rows, the MMA's N) x k = 64; D[col][A row] lands in TMEM
// with lane = output column, column = A row.  The epilogue of vector-row r
// reads its V TMEM columns for 32 output columns per warp (one tcgen05.ld) and
// keeps the lanes whose column is stored in the mask: a bitmap of each
// vector-row's columns (one 32-bit word per 32 columns) and, per word, the
// slot of its first column (`prefix`, relative to the row start) give the
// output slot of column c as prefix + popc(word & lanes below c).  Both come
// from mcSddmmTileMask, which requires strictly increasing column indices
// within each vector-row.
//
// Warp roles (416 threads, one CTA per SM, persistent over work items =
// (batch entry, block of 256 A rows)):
//  * warps 0-7, epilogue: warps q and q + 4 read TMEM lanes 32q .. 32q+31
//    and take alternate groups of vector-rows (two warps per quadrant hide
//    the TMEM-load and store latency of each other);
//  * warps 8-11, converters: coalesced 16-byte loads of the int8 rows, exact
//    f16 conversion (prmt + sub.f16x2), stores into the 128-byte-swizzled
//    K-major layout the MMA descriptors describe; the A block once per item
//    (two buffers), the B tile once per column block (a ring of STAGES);
//  * warp 12: TMEM allocation (two 256-column accumulators) and, from one
//    thread, four tcgen05.mma (K = 16 each) per tile.
// Measured on GB300 (64 instances of 4096 x 4096 x 64, V = 8, sparsity 0.9):
// the epilogue bounds it -- about 30 instructions per (vector-row, 32-column
// chunk) whatever the number of stored columns in it, i.e. ~3,200 warp
// instructions per tile against 544 cycles of MMA -- so at sparsity 0.9 it
// is slower than the per-nonzero int8 kernel and pays off on denser masks.
// mbarriers hand the buffers over (a_full/a_empty, b_full/b_empty,
// t_full/t_empty).  Every wait is bounded: a wait that runs out bumps the
// timeout counter and that role stops; the MMA thread waits (bounded) for
// its MMAs before TMEM is released.
#pragma once
#include "mc_sddmm.cuh"
#include "mc_sm100.cuh"

namespace mc {

struct SddmmDenseParams {
    SddmmParams s;
    const uint32_t* bitmap;  // [m_vec][words]
    const int* prefix;       // [m_vec][words]
    int words;               // 4 per 128-column block
    int a_blocks;            // ceil(m_vec * V / 256)
    int c_blocks;            // ceil(n / 128)
    int items;               // batch * a_blocks
};

namespace dense {
constexpr int AR = 256, BR = 128, STAGES = 4;
constexpr int A_BYTES = AR * 128, B_BYTES = BR * 128;  // f16 tiles, 128 B per row
constexpr int B_OFF = 2 * A_BYTES;
constexpr int BAR_OFF = B_OFF + STAGES * B_BYTES;
constexpr int NBARS = 9 + 2 * STAGES;  // ..., fin (the MMAs in flight at an early stop)
constexpr int SMEM = 1024 + BAR_OFF + NBARS * 8 + 16;
constexpr int THREADS = 416;  // 8 epilogue warps, 4 converter warps, 1 MMA warp
constexpr int EPI = 8;
constexpr long long WAIT = 4000000000LL;  // ~2 s at 2 GHz
}  // namespace dense

// 8 consecutive f32 TMEM columns (or 4, 2) of this thread's lane.
template <int N>
__device__ __forceinline__ void tmem_ld_cols(uint32_t taddr, uint32_t (&r)[N])
{
    if constexpr (N == 8)
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                     : "r"(taddr));
    else if constexpr (N == 4)
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                     : "r"(taddr));
    else
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0, %1}, [%2];" : "=r"(r[0]), "=r"(r[1]) : "r"(taddr));
}

// 16 int8 values (one 16-byte k chunk q of row `row`) -> 16 f16 in the
// 128-byte-swizzled K-major tile: f16 chunks 2q and 2q + 1 of the row.
template <bool SIGNED>
__device__ __forceinline__ void store_f16_chunk(uint8_t* tile, int row, int q, int4 w)
{
    uint32_t h[8];
    bytes_to_h2<SIGNED>((uint32_t)w.x, h[0], h[1]);
    bytes_to_h2<SIGNED>((uint32_t)w.y, h[2], h[3]);
    bytes_to_h2<SIGNED>((uint32_t)w.z, h[4], h[5]);
    bytes_to_h2<SIGNED>((uint32_t)w.w, h[6], h[7]);
    uint8_t* r = tile + (row >> 3) * 1024 + (row & 7) * 128;
    const int sw = row & 7;
    *reinterpret_cast<uint4*>(r + (((2 * q) ^ sw) << 4)) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4*>(r + (((2 * q + 1) ^ sw) << 4)) = make_uint4(h[4], h[5], h[6], h[7]);
}

template <int V, bool SIGNED, bool VECMAJOR, bool HALF_OUT>
__global__ void __launch_bounds__(dense::THREADS, 1)
sddmm_dense_tc_kernel(const SddmmDenseParams dp, unsigned int* timeouts)
{
    using namespace sm100;
    using namespace dense;
    constexpr int VR = AR / V;      // vector-rows per A block
    constexpr int G = 64 / V < 16 ? 64 / V : 16;  // vector-rows per batch of TMEM loads (<= 64 registers)
    const SddmmParams& p = dp.s;
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = saddr(smem_raw);
    uint8_t* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + BAR_OFF);
    uint64_t* a_full = bars;
    uint64_t* a_empty = bars + 2;
    uint64_t* t_full = bars + 4;
    uint64_t* t_empty = bars + 6;
    uint64_t* b_full = bars + 8;
    uint64_t* b_empty = bars + 8 + STAGES;
    uint64_t* fin = bars + 8 + 2 * STAGES;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + NBARS);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(a_full + i, 128);
            mbar_init(a_empty + i, 1);
            mbar_init(t_full + i, 1);
            mbar_init(t_empty + i, EPI);
        }
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(b_full + s, 128);
            mbar_init(b_empty + s, 1);
        }
        mbar_init(fin, 1);
        fence_mbar_init();
    }
    if (warp == 12) {
        tmem_alloc(tmem_slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const long long m_rows = (long long)p.m_vec * V;

    if (warp >= EPI && warp < EPI + 4) {
        // ------------------------------ converters ------------------------------
        const int ct = tid - 32 * EPI;
        int bc = 0, ic = 0;
        bool ok = true;
        for (int item = blockIdx.x; item < dp.items && ok; item += gridDim.x, ++ic) {
            const int b = item / dp.a_blocks, ab = item - b * dp.a_blocks;
            const int abuf = ic & 1;
            if (ic >= 2 && !mbar_wait(a_empty + abuf, ((ic >> 1) - 1) & 1, WAIT)) {
                ok = false;
                break;
            }
            uint8_t* at = smem + abuf * A_BYTES;
            const uint8_t* lhs = p.lhs + (long long)b * p.lhs_stride;
            const long long r0 = (long long)ab * AR;
#pragma unroll
            for (int i = 0; i < AR * 4 / 128; ++i) {
                const int c = ct + 128 * i, row = c >> 2, q = c & 3;
                const int4 w = r0 + row < m_rows ? ldg_nc_v4(lhs + (r0 + row) * 64 + 16 * q) : make_int4(0, 0, 0, 0);
                store_f16_chunk<SIGNED>(at, row, q, w);
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(a_full + abuf);
            const uint8_t* rhs = p.rhs + (long long)b * p.rhs_stride;
            for (int cb = 0; cb < dp.c_blocks; ++cb, ++bc) {
                const int s = bc % STAGES;
                if (bc >= STAGES && !mbar_wait(b_empty + s, ((bc / STAGES) - 1) & 1, WAIT)) {
                    ok = false;
                    break;
                }
                uint8_t* bt = smem + B_OFF + s * B_BYTES;
                const int n0 = cb * BR;
#pragma unroll
                for (int i = 0; i < BR * 4 / 128; ++i) {
                    const int c = ct + 128 * i, row = c >> 2, q = c & 3;
                    const int4 w =
                        n0 + row < p.n ? ldg_nc_v4(rhs + (long long)(n0 + row) * 64 + 16 * q) : make_int4(0, 0, 0, 0);
                    store_f16_chunk<SIGNED>(bt, row, q, w);
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive(b_full + s);
            }
        }
        if (!ok && lane == 0) atomicAdd(timeouts, 1u);
    } else if (warp == 12) {
        // --------------------------------- MMA ---------------------------------
        if (lane == 0) {
            constexpr uint32_t IDESC = idesc_f16_f32(BR, AR);
            int bc = 0, ic = 0, tc = 0;
            bool ok = true;
            for (int item = blockIdx.x; item < dp.items && ok; item += gridDim.x, ++ic) {
                const int abuf = ic & 1;
                if (!mbar_wait(a_full + abuf, (ic >> 1) & 1, WAIT)) {
                    ok = false;
                    break;
                }
                const uint64_t adesc = desc_sw128_kmajor(saddr(smem + abuf * A_BYTES));
                for (int cb = 0; cb < dp.c_blocks; ++cb, ++bc, ++tc) {
                    const int s = bc % STAGES, tb = tc & 1;
                    if (!mbar_wait(b_full + s, (bc / STAGES) & 1, WAIT) ||
                        (tc >= 2 && !mbar_wait(t_empty + tb, ((tc >> 1) - 1) & 1, WAIT))) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint64_t bdesc = desc_sw128_kmajor(saddr(smem + B_OFF + s * B_BYTES));
#pragma unroll
                    for (int k = 0; k < 4; ++k)  // K = 16 per MMA: 32 bytes = 2 descriptor units
                        mma_f16_ss(tmem + tb * AR, bdesc + 2 * k, adesc + 2 * k, IDESC, k > 0);
                    mma_commit(b_empty + s);
                    mma_commit(t_full + tb);
                }
                if (ok) mma_commit(a_empty + abuf);
            }
            if (!ok) {
                atomicAdd(timeouts, 1u);
                // every MMA issued so far completes before TMEM is released
                mma_commit(fin);
                if (!mbar_wait(fin, 0, WAIT)) atomicAdd(timeouts, 1u);
            }
        }
    } else {
        // ------------------------------- epilogue ------------------------------
        const int q = warp & 3;      // TMEM lanes 32q .. 32q + 31: output columns n0 + 32q + lane
        const int half = warp >> 2;  // the two warps of a quadrant take alternate load groups
        const Divisor dq = make_divisor(p.scale);
        int tc = 0;
        bool ok = true;
        for (int item = blockIdx.x; item < dp.items && ok; item += gridDim.x) {
            const int b = item / dp.a_blocks, ab = item - b * dp.a_blocks;
            const int R0 = ab * VR;
            const long long obase = (long long)b * p.out_stride;
            int st[VR / 32];  // start of vector-row R0 + 32 i + lane
#pragma unroll
            for (int i = 0; i < VR / 32; ++i) {
                const int R = R0 + 32 * i + lane;
                st[i] = R < p.m_vec ? __ldg(p.row_offsets + 2 * R) : 0;
                // padding slots [nnz, nnz8) of the warp's share of rows are zero
                if (R < p.m_vec && ((32 * i + lane) & 7) == warp) {
                    const int nnz = __ldg(p.row_offsets + 2 * R + 1) - st[i];
                    for (int j = nnz; j < ((nnz + 7) & ~7); ++j) {
                        const int slot = st[i] + j;
#pragma unroll
                        for (int v = 0; v < V; ++v) {
                            const long long o = VECMAJOR ? obase + (long long)slot * V + v
                                                         : obase + (long long)(slot >> 3) * 8 * V + 8 * v + (slot & 7);
                            if constexpr (HALF_OUT) reinterpret_cast<__half*>(p.out)[o] = __float2half_rn(0.f);
                            else reinterpret_cast<int*>(p.out)[o] = 0;
                        }
                    }
                }
            }
            for (int cb = 0; cb < dp.c_blocks; ++cb, ++tc) {
                const int tb = tc & 1;
                const int w = cb * 4 + q;
                uint32_t word[VR / 32];
                int base[VR / 32];  // first output slot of this word's columns
#pragma unroll
                for (int i = 0; i < VR / 32; ++i) {  // issued before the wait: the loads overlap it
                    const int R = R0 + 32 * i + lane;
                    const long long e = (long long)R * dp.words + w;
                    word[i] = R < p.m_vec ? __ldg(dp.bitmap + e) : 0u;
                    base[i] = R < p.m_vec ? st[i] + __ldg(dp.prefix + e) : 0;
                }
                if (!mbar_wait(t_full + tb, (tc >> 1) & 1, WAIT)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t tcol = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(tb * AR);
                const uint32_t below = (1u << lane) - 1u;
#pragma unroll
                for (int i = 0; i < VR / 32; ++i) {
#pragma unroll 1
                    for (int l0 = half * G; l0 < 32; l0 += 2 * G) {
                        uint32_t wd[G];
                        uint32_t any = 0;
#pragma unroll
                        for (int g = 0; g < G; ++g) {
                            wd[g] = __shfl_sync(0xffffffffu, word[i], l0 + g);
                            any |= wd[g];
                        }
                        if (any == 0) continue;  // warp-uniform
                        uint32_t acc[G][V];
#pragma unroll
                        for (int g = 0; g < G; ++g) tmem_ld_cols<V>(tcol + (uint32_t)((32 * i + l0 + g) * V), acc[g]);
                        tmem_ld_wait();
#pragma unroll
                        for (int g = 0; g < G; ++g) {
                            const int bs = __shfl_sync(0xffffffffu, base[i], l0 + g);
                            if (!((wd[g] >> lane) & 1u)) continue;
                            const int slot = bs + __popc(wd[g] & below);
                            int d[V];
                            if constexpr (!HALF_OUT) {
#pragma unroll
                                // exact integers below 64 x 255^2 < 2^22 in magnitude
                                for (int v = 0; v < V; ++v) d[v] = f2i_rn_small(__uint_as_float(acc[g][v]));
                            }
                            if constexpr (VECMAJOR) {
                                const long long o = obase + (long long)slot * V;
                                if constexpr (HALF_OUT) {
                                    // the f32 accumulator is the exact integer: divide it directly
                                    // (+0 turns a -0 sum into the +0 the integer path gives)
#pragma unroll
                                    for (int v = 0; v < V; v += 2) {
                                        const __half2 h = __halves2half2(
                                            __float2half_rn(div_rn(__fadd_rn(__uint_as_float(acc[g][v]), 0.f), dq)),
                                            __float2half_rn(div_rn(__fadd_rn(__uint_as_float(acc[g][v + 1]), 0.f), dq)));
                                        stg_cs_s32(reinterpret_cast<__half*>(p.out) + o + v,
                                                   (int)*reinterpret_cast<const uint32_t*>(&h));
                                    }
                                } else {
#pragma unroll
                                    for (int v = 0; v < V; v += 2) stg_cs_v2(reinterpret_cast<int*>(p.out) + o + v, d[v], d[v + 1]);
                                }
                            } else {
                                const long long o = obase + (long long)(slot >> 3) * 8 * V + (slot & 7);
#pragma unroll
                                for (int v = 0; v < V; ++v) {
                                    if constexpr (HALF_OUT)
                                        reinterpret_cast<__half*>(p.out)[o + 8 * v] =
                                            __float2half_rn(div_rn(__fadd_rn(__uint_as_float(acc[g][v]), 0.f), dq));
                                    else stg_cs_s32(reinterpret_cast<int*>(p.out) + o + 8 * v, d[v]);
                                }
                            }
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
    if (warp == 12) {
        tc_fence_after();
        tmem_dealloc(tmem, 512);
    }
}

// Bitmap and first-slot table of a mask for the dense-tile SDDMM: one warp
// per vector-row; word w covers columns 32w .. 32w+31.  prefix[w] = number of
// the row's nonzeros with a column below 32w (binary search over the sorted
// columns); the word's bits are the columns in [prefix[w], prefix[w+1]).
// status |= 1 if a row's columns are not strictly increasing or out of
// [0, n).
__global__ void __launch_bounds__(128)
sddmm_tile_mask_kernel(int m_vec, int n, int words, const int* __restrict__ row_offsets,
                       const int* __restrict__ cols, uint32_t* __restrict__ bitmap, int* __restrict__ prefix,
                       int* status)
{
    const int R = blockIdx.x * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (R >= m_vec) return;
    const int start = __ldg(row_offsets + 2 * R);
    const int nnz = __ldg(row_offsets + 2 * R + 1) - start;
    const int* c = cols + start;
    bool bad = false;
    for (int j = lane; j < nnz; j += 32) {
        const int x = __ldg(c + j);
        if (x < 0 || x >= n || (j > 0 && __ldg(c + j - 1) >= x)) bad = true;
    }
    if (__any_sync(0xffffffffu, bad)) {
        if (lane == 0) atomicOr(status, 1);
        return;
    }
    auto lower = [&](int key) {  // first j with c[j] >= key
        int lo = 0, hi = nnz;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (__ldg(c + mid) < key) lo = mid + 1;
            else hi = mid;
        }
        return lo;
    };
    for (int w = lane; w < words; w += 32) {
        const int j0 = lower(32 * w), j1 = lower(32 * w + 32);
        uint32_t bits = 0;
        for (int j = j0; j < j1; ++j) bits |= 1u << (__ldg(c + j) & 31);
        bitmap[(long long)R * words + w] = bits;
        prefix[(long long)R * words + w] = j0;
    }
}

}  // namespace mc
