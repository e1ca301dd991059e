// mc_sddmm_mixed.cuh -- SDDMM with k == 64 and 8-bit operands on two pipes:
// the int8 tensor cores (mma.sync) and the CUDA cores (dp4a) at once.
//
// Same operands and results as sddmm_k64_kernel (mc_sddmm_stream.cuh).  A
// vector-row's nonzeros are cut into units of 32; a warp takes units with
// the grid's stride.  Every R-th unit (ui % R == R - 1) runs on dp4a, the
// others on the MMA as two 16-nonzero tiles:
//  * MMA unit: the k64 kernel's tile -- each lane gathers 16 bytes of the B
//    rows of nonzeros g and g + 8 straight into the A fragment, the V rows of
//    A stay in registers as the B fragment (two m16n8k32 per tile);
//  * dp4a unit: lane l owns nonzero 32 ui + l whole: it gathers that B row
//    (64 bytes, two halves of 32) and forms all V dot products with 16 dp4a
//    each, reading the V rows of A from shared memory (broadcast loads); no
//    reduction across lanes is needed.
// The int8 MMA and dp4a issue to different pipes, so warps of the same SM in
// units of the two kinds run concurrently (one m16n8k32 plus 32 dp4a per
// step measure about 1.6x the MMA-only rate on GB300).  Both forms sum the
// same integer products modulo 2^32: the results are identical.
#pragma once
#include "mc_sddmm.cuh"

namespace mc {

// 12 resident CTAs of 4 warps per SM: at most 40 registers per thread.
template <int V, bool SIGNED, bool VECMAJOR, bool HALF_OUT, int WARPS, int R>
__global__ void __launch_bounds__(WARPS * 32, 48 / WARPS)
sddmm_k64_mixed_kernel(const SddmmParams p)
{
    static_assert(R >= 2, "every R-th unit on dp4a");
    const Divisor dq = make_divisor(p.scale);
    __shared__ __align__(16) uint8_t qs[V * 64];  // the V rows of A
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const int row = __ldg(p.row_indices + blockIdx.x);
    const int b = blockIdx.z;
    const int start = __ldg(p.row_offsets + 2 * row);
    const int nnz = __ldg(p.row_offsets + 2 * row + 1) - start;
    const int nnz8 = (nnz + 7) & ~7;
    const int nunits = (nnz8 + 31) >> 5;
    const uint8_t* lhs = p.lhs + (long long)b * p.lhs_stride + (long long)row * V * 64;
    if (threadIdx.x < V * 4)
        *reinterpret_cast<int4*>(qs + 16 * threadIdx.x) = ldg_nc_v4(lhs + 16 * threadIdx.x);
    __syncthreads();
    const int stride = gridDim.y * WARPS;
    int ui = blockIdx.y * WARPS + warp;
    if (ui >= nunits) return;

    const int* cols = p.col_indices + start;
    const uint8_t* rhs = p.rhs + (long long)b * p.rhs_stride;
    const long long obase = (long long)b * p.out_stride + (long long)start * V;
    uint32_t a[4] = {0u, 0u, 0u, 0u};  // MMA B fragment: A row g, k chunk t
    if (g < V) {
        const int4 v = *reinterpret_cast<const int4*>(qs + g * 64 + 16 * t);
        a[0] = v.x; a[1] = v.y; a[2] = v.z; a[3] = v.w;
    }

#pragma unroll 1
    for (; ui < nunits; ui += stride) {
        if (ui % R == R - 1) {
            // ---- dp4a unit: nonzero j of this lane, every vector lane ----
            const int j = ui * 32 + lane;
            const int c = j < nnz ? __ldg(cols + j) : -1;
            int acc[V];
#pragma unroll
            for (int v = 0; v < V; ++v) acc[v] = 0;
            if (c >= 0) {
                const uint8_t* brow = rhs + (unsigned)c * 64u;
#pragma unroll
                for (int hf = 0; hf < 2; ++hf) {
                    const int4 k0 = ldg_nc_v4(brow + 32 * hf), k1 = ldg_nc_v4(brow + 32 * hf + 16);
#pragma unroll
                    for (int v = 0; v < V; ++v) {
                        const int4 q0 = *reinterpret_cast<const int4*>(qs + v * 64 + 32 * hf);
                        const int4 q1 = *reinterpret_cast<const int4*>(qs + v * 64 + 32 * hf + 16);
                        int x = acc[v];
                        x = dp4a<SIGNED>(k0.x, q0.x, x);
                        x = dp4a<SIGNED>(k0.y, q0.y, x);
                        x = dp4a<SIGNED>(k0.z, q0.z, x);
                        x = dp4a<SIGNED>(k0.w, q0.w, x);
                        x = dp4a<SIGNED>(k1.x, q1.x, x);
                        x = dp4a<SIGNED>(k1.y, q1.y, x);
                        x = dp4a<SIGNED>(k1.z, q1.z, x);
                        x = dp4a<SIGNED>(k1.w, q1.w, x);
                        acc[v] = x;
                    }
                }
            }
            if (j < nnz8) {
                if constexpr (VECMAJOR) {
                    const long long o = obase + (long long)j * V;
                    if constexpr (HALF_OUT) {
#pragma unroll
                        for (int v = 0; v < V; v += 2)
                            stg_cs_s32(reinterpret_cast<__half*>(p.out) + o + v, (int)pack_half2(acc[v], acc[v + 1], dq));
                    } else {
#pragma unroll
                        for (int v = 0; v < V; v += 2) stg_cs_v2(reinterpret_cast<int*>(p.out) + o + v, acc[v], acc[v + 1]);
                    }
                } else {
                    const long long o = obase + (j >> 3) * 8 * V + (j & 7);
#pragma unroll
                    for (int v = 0; v < V; ++v) {
                        if constexpr (HALF_OUT) reinterpret_cast<__half*>(p.out)[o + 8 * v] = deq_half(acc[v], dq);
                        else stg_cs_s32(reinterpret_cast<int*>(p.out) + o + 8 * v, acc[v]);
                    }
                }
            }
            continue;
        }
        // ---- MMA unit: tiles 2 ui and 2 ui + 1 ----
#pragma unroll 1
        for (int tt = 0; tt < 2; ++tt) {
            const int tile = 2 * ui + tt;
            if (tile * 16 >= nnz8) break;
            const int j0 = tile * 16 + g;
            const int c0 = j0 < nnz ? __ldg(cols + j0) : -1;
            const int c1 = j0 + 8 < nnz ? __ldg(cols + j0 + 8) : -1;
            int4 r0 = make_int4(0, 0, 0, 0), r1 = make_int4(0, 0, 0, 0);
            if (c0 >= 0) r0 = ldg_nc_v4(rhs + (unsigned)c0 * 64u + 16 * t);
            if (c1 >= 0) r1 = ldg_nc_v4(rhs + (unsigned)c1 * 64u + 16 * t);
            int d[4] = {0, 0, 0, 0};
            mma_k32<SIGNED, SIGNED>(d, r0.x, r1.x, r0.y, r1.y, a[0], a[1]);
            mma_k32<SIGNED, SIGNED>(d, r0.z, r1.z, r0.w, r1.w, a[2], a[3]);
            // d[0..1]: nonzero tile*16 + g, lanes 2t, 2t+1; d[2..3]: nonzero + 8
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
    }
}

}  // namespace mc
