// mc_sddmm_tc.cuh -- SDDMM (8-bit x 8-bit, k = 64) on the 5th-generation
// tensor cores.
//
// sm_103a has no integer tcgen05.mma, but for k = 64 the f16 path is exact:
// every int8 operand is an exact f16, every product is an integer below 2^16
// in magnitude and the sum of 64 of them stays below 2^24 (signed: 64 x 2^14;
// unsigned: 64 x 255^2), so the f32 accumulator holds the integer result
// exactly.  Per chunk of 128 nonzero vectors of a vector-row:
//  * thread i gathers B row col[i] (64 bytes, four 16-byte loads), converts
//    it exactly to f16 (prmt + sub.f16x2) and stores it as row i of a 128 x 64
//    f16 tile in shared memory, 128-byte swizzled (the K-major layout the
//    tensor core reads);
//  * the V rows of A (this vector-row) sit in a second 16 x 64 f16 tile
//    (rows V..15 zero), converted once per vector-row;
//  * one thread issues four tcgen05.mma kind::f16 (M = 128 nonzeros, N = 16,
//    K = 16 each) into a 16-column TMEM accumulator and commits to an
//    mbarrier;
//  * thread i reads its TMEM lane (tcgen05.ld, V columns) and writes the V
//    results of nonzero i in the requested output layout.
// Persistent CTAs of 4 warps walk the (batch entry, vector-row) items; the
// overlap of gathers, MMAs and stores comes from the CTAs co-resident on an
// SM (about 19 KB of shared memory and 32 TMEM columns each).  Every mbarrier
// wait is bounded: a timeout bumps a device counter (read back with
// mcTensorCoreTimeouts) and the CTA stops instead of hanging.
#pragma once
#include "mc_sddmm.cuh"
#include "mc_sm100.cuh"

namespace mc {

static __device__ unsigned int g_tc_timeouts;

template <int V, bool SIGNED, bool VECMAJOR, bool HALF_OUT>
__global__ void __launch_bounds__(128)
sddmm_tc_kernel(const SddmmParams p, const int items)
{
    const Divisor dq = make_divisor(p.scale);  // half output: acc / scale
    using namespace sm100;
    constexpr int ROWS = 128;                 // nonzeros per chunk (MMA M)
    constexpr int N = 16;                     // MMA N (V rows of A, zero-padded)
    constexpr long long WAIT = 4000000000LL;  // ~2 s at 2 GHz
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = saddr(smem_raw);
    uint8_t* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    uint8_t* bt = smem;                        // [128 rows][128 B] gathered B rows, f16
    uint8_t* qt = smem + ROWS * 128;           // [16 rows][128 B] A rows, f16
    uint64_t* done = reinterpret_cast<uint64_t*>(qt + N * 128);
    uint32_t* tmem_s = reinterpret_cast<uint32_t*>(done + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        mbar_init(done, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_s, 32);
        tmem_relinquish();
    }
    // rows V..15 of the A tile stay zero for the whole launch
    for (int i = tid; i < (N - V) * 8; i += 128) {
        const int r = V + i / 8, c = i % 8;
        *reinterpret_cast<uint4*>(qt + r * 128 + ((c ^ (r & 7)) << 4)) = make_uint4(0, 0, 0, 0);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_s;
    const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16);  // this warp's TMEM lanes
    constexpr uint32_t idesc = idesc_f16_f32(ROWS, N);
    const uint64_t qdesc = desc_sw128_kmajor(saddr(qt));
    const uint64_t bdesc = desc_sw128_kmajor(saddr(bt));
    uint32_t phase = 0;
    bool ok = true;

    for (int item = blockIdx.x; item < items && ok; item += gridDim.x) {
        const int b = item / p.m_vec;
        const int row = __ldg(p.row_indices + item - b * p.m_vec);
        const int start = __ldg(p.row_offsets + 2 * row);
        const int nnz = __ldg(p.row_offsets + 2 * row + 1) - start;
        const int nnz8 = (nnz + 7) & ~7;
        // A rows of this vector-row -> f16 tile rows 0..V-1 (4 threads x 16
        // bytes per row).  The previous item's MMAs have completed (every
        // chunk is waited for) and the CTA passed a barrier since.
        if (tid < 4 * V) {
            const int v = tid >> 2, q = tid & 3;
            const int4 w = ldg_nc_v4(p.lhs + (long long)b * p.lhs_stride + (long long)(row * V + v) * 64 + 16 * q);
            uint32_t h[8];
            bytes_to_h2<SIGNED>((uint32_t)w.x, h[0], h[1]);
            bytes_to_h2<SIGNED>((uint32_t)w.y, h[2], h[3]);
            bytes_to_h2<SIGNED>((uint32_t)w.z, h[4], h[5]);
            bytes_to_h2<SIGNED>((uint32_t)w.w, h[6], h[7]);
            *reinterpret_cast<uint4*>(qt + v * 128 + (((2 * q) ^ (v & 7)) << 4)) = make_uint4(h[0], h[1], h[2], h[3]);
            *reinterpret_cast<uint4*>(qt + v * 128 + (((2 * q + 1) ^ (v & 7)) << 4)) = make_uint4(h[4], h[5], h[6], h[7]);
        }
        const uint8_t* rhs = p.rhs + (long long)b * p.rhs_stride;
        const long long obase = (long long)b * p.out_stride + (long long)start * V;
        for (int c0 = 0; c0 < nnz8; c0 += ROWS) {
            // ---- gather + convert: thread tid owns nonzero c0 + tid ----
            const int j = c0 + tid;
            const int col = j < nnz ? __ldg(p.col_indices + start + j) : -1;
            int4 w[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) w[q] = make_int4(0, 0, 0, 0);
            if (col >= 0) {
                const uint8_t* src = rhs + (unsigned)col * 64u;
#pragma unroll
                for (int q = 0; q < 4; ++q) w[q] = ldg_nc_v4(src + 16 * q);
            }
            uint8_t* dst = bt + tid * 128;
            const int sw = tid & 7;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                uint32_t h[8];
                bytes_to_h2<SIGNED>((uint32_t)w[q].x, h[0], h[1]);
                bytes_to_h2<SIGNED>((uint32_t)w[q].y, h[2], h[3]);
                bytes_to_h2<SIGNED>((uint32_t)w[q].z, h[4], h[5]);
                bytes_to_h2<SIGNED>((uint32_t)w[q].w, h[6], h[7]);
                *reinterpret_cast<uint4*>(dst + (((2 * q) ^ sw) << 4)) = make_uint4(h[0], h[1], h[2], h[3]);
                *reinterpret_cast<uint4*>(dst + (((2 * q + 1) ^ sw) << 4)) = make_uint4(h[4], h[5], h[6], h[7]);
            }
            // generic-proxy shared-memory writes -> visible to the tensor core
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncthreads();
            if (tid == 0) {
                tc_fence_after();
#pragma unroll
                for (int k = 0; k < 4; ++k)  // K = 16 per MMA: 32 bytes = 2 descriptor units
                    mma_f16_ss(tmem, bdesc + 2 * k, qdesc + 2 * k, idesc, k > 0);
                mma_commit(done);
            }
            const bool arrived = mbar_wait(done, phase, WAIT);
            phase ^= 1u;
            if (!__all_sync(0xffffffffu, arrived)) {
                if (lane == 0) atomicAdd(&g_tc_timeouts, 1u);
                ok = false;
            }
            if (!__syncthreads_and(ok)) {
                ok = false;
                break;
            }
            tc_fence_after();
            // ---- epilogue: TMEM lane tid = nonzero c0 + tid, columns 0..V-1 ----
            uint32_t acc[8];
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                         : "=r"(acc[0]), "=r"(acc[1]), "=r"(acc[2]), "=r"(acc[3]), "=r"(acc[4]), "=r"(acc[5]),
                           "=r"(acc[6]), "=r"(acc[7])
                         : "r"(taddr));
            tmem_ld_wait();
            // keeps every use of acc after the wait
            asm volatile("" : "+r"(acc[0]), "+r"(acc[1]), "+r"(acc[2]), "+r"(acc[3]), "+r"(acc[4]), "+r"(acc[5]),
                         "+r"(acc[6]), "+r"(acc[7])::"memory");
            if (j < nnz8) {
                int d[V];
#pragma unroll
                for (int v = 0; v < V; ++v) d[v] = j < nnz ? f2i_exact(__uint_as_float(acc[v])) : 0;
                if constexpr (VECMAJOR) {
                    const long long o = obase + (long long)j * V;
                    if constexpr (HALF_OUT) {
                        __half* out = reinterpret_cast<__half*>(p.out) + o;
#pragma unroll
                        for (int v = 0; v < V; v += 2)
                            *reinterpret_cast<uint32_t*>(out + v) = pack_half2(d[v], d[v + 1], dq);
                    } else {
                        int* out = reinterpret_cast<int*>(p.out) + o;
#pragma unroll
                        for (int v = 0; v < V; v += 2) stg_cs_v2(out + v, d[v], d[v + 1]);
                    }
                } else {
                    const long long o = obase + (long long)(j >> 3) * 8 * V + (j & 7);
#pragma unroll
                    for (int v = 0; v < V; ++v) {
                        if constexpr (HALF_OUT) reinterpret_cast<__half*>(p.out)[o + 8 * v] = deq_half(d[v], dq);
                        else stg_cs_s32(reinterpret_cast<int*>(p.out) + o + 8 * v, d[v]);
                    }
                }
            }
            tc_fence_before();
            __syncthreads();  // every lane has read TMEM and the tile before the next chunk rewrites them
        }
        __syncthreads();  // the A tile is rewritten for the next item
    }
    // An MMA issued and not waited for (a timed-out wait) completes before
    // TMEM is released.
    if (tid == 0 && !ok) {
        mma_commit(done);
        if (!mbar_wait(done, phase, WAIT)) atomicAdd(&g_tc_timeouts, 1u);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 32);
    }
}

inline size_t sddmm_tc_smem_bytes() { return 1024 + 128 * 128 + 16 * 128 + 64; }

}  // namespace mc
