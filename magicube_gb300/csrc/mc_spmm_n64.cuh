// mc_spmm_n64.cuh -- SpMM for n == 64 with 8-bit operands, the softmax value
// layout and half output: the attention's P x V (int8 probabilities times
// gathered 64-byte V rows of head dimension 64).
//
// A 64-byte B row feeds all 64 output columns, so one warp consumes whole
// gathered rows and owns whole vector-rows: per 32-slot step each lane stages
// its slot's row (four 16-byte cp.async copies, chunk-swizzled) into the
// warp's private ring of STAGES steps, and the warp multiplies it with one
// ldmatrix.m16n16.x2.trans per 16 columns and four MMAs sharing the
// probability fragment.  Warps are persistent over the (batch entry,
// vector-row) items and never meet: no CTA barrier, no cross-warp
// reduction.  The step's probability chunks ([2][V][16] bytes, contiguous in
// the softmax layout) travel in the same cp.async group as its rows, and the
// column indices are loaded two steps before their copies are issued, so no
// global load sits on the path to the MMAs (values 16-byte aligned; the
// launcher checks).  (The per-row kernel,
// by contrast, gives each of two warps 32 of the 64 columns and transposes
// through a CTA-shared ring.)
#pragma once
#include "mc_spmm.cuh"

namespace mc {

__device__ __forceinline__ void ldsm_x2_trans_b8_n64(uint32_t (&r)[4], const void* p)
{
    asm volatile("ldmatrix.sync.aligned.m16n16.x2.trans.shared.b8 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_u32(p)));
}

namespace n64 {
constexpr int WARPS = 4, STAGES = 4, ROW = 64;  // ROW: bytes of one gathered B row
constexpr int VAL_BYTES = 2 * 8 * 16;           // a step's probability chunks (V <= 8)
constexpr int STAGE = 32 * ROW + VAL_BYTES;
}

template <int V, bool SIGNED>
__global__ void __launch_bounds__(n64::WARPS * 32) spmm_n64_kernel(const SpmmParams p, const int items)
{
    using namespace n64;
    __shared__ __align__(128) uint8_t rings[WARPS * STAGES * STAGE];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    uint8_t* ring = rings + warp * STAGES * STAGE;
    const int nwarps = gridDim.x * WARPS;

#pragma unroll 1
    for (int item = blockIdx.x * WARPS + warp; item < items; item += nwarps) {
        const int b = item / p.m_vec;
        const int row = __ldg(p.row_indices + (item - b * p.m_vec));
        const int start = __ldg(p.row_offsets + 2 * row);
        const int nnz = __ldg(p.row_offsets + 2 * row + 1) - start;
        const int steps = (nnz + 31) >> 5;
        const uint8_t* rhs = p.rhs + (long long)b * p.rhs_stride;
        const uint8_t* vals = p.values + (long long)b * p.values_stride;

        auto col_of = [&](int s) {
            const int j = s * 32 + lane;
            return (s < steps && j < nnz) ? __ldg(p.col_indices + start + j) : -1;
        };
        // step s into ring slot `slot` (one commit group per step, empty past
        // the row): lane l stages the B row of its column c, lanes 0 .. 2V-1
        // the step's probability chunks (a chunk only if it holds a stored
        // slot, so the copy stays inside the row's aligned values)
        // Copy i moves rows 16 (i & 1) .. +15, 32-byte half 2 (i >> 1) .. +1:
        // lanes 2r and 2r + 1 take the two 16-byte chunks of one sector of
        // row r, so each copy instruction reads 16 whole 32-byte sectors (not
        // 32 half sectors); the row's column comes from its lane by shuffle.
        auto issue = [&](int s, int c, int slot) {
            uint8_t* stage = ring + slot * STAGE;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = 16 * (i & 1) + (lane >> 1), q = 2 * (i >> 1) + (lane & 1);
                const int cr = __shfl_sync(0xffffffffu, c, r);
                if (cr >= 0)
                    cp_async16(stage + r * ROW + ((q ^ ((r >> 1) & 3)) << 4), rhs + (long long)cr * ROW + q * 16);
            }
            if (s < steps && lane < 2 * V && 32 * s + 16 * (lane / V) < nnz)
                cp_async16(stage + 32 * ROW + 16 * lane,
                           vals + (long long)((start + 32 * s) >> 4) * V * 16 + 16 * lane);
            cp_async_commit();
        };

        __syncwarp();  // every lane is past its reads of the previous item's ring
        {
            int c[STAGES - 1];
#pragma unroll
            for (int i = 0; i < STAGES - 1; ++i) c[i] = col_of(i);
#pragma unroll
            for (int i = 0; i < STAGES - 1; ++i) issue(i, c[i], i);
        }
        int cn = col_of(STAGES - 1), cn2 = col_of(STAGES);  // columns two steps ahead

        int acc[4][4] = {};
#pragma unroll 1
        for (int s = 0; s < steps; ++s) {
            const int cn3 = col_of(s + STAGES + 1);
            cp_async_wait<STAGES - 2>();  // step s's copies have landed
            __syncwarp();
            const uint8_t* st = ring + (s % STAGES) * STAGE;
            // probability fragment of vector lane g: slots 32s + 4t .. +3 and
            // 32s + 16 + 4t .. +3; slots past the row are masked to zero
            // (their ring rows and chunk bytes are stale)
            uint32_t b0 = 0u, b1 = 0u;
            if (g < V) {
                const int j0 = s * 32 + 4 * t, j1 = j0 + 16;
                b0 = lds32(st + 32 * ROW + g * 16 + 4 * t) & byte_mask(nnz - j0);
                b1 = lds32(st + 32 * ROW + V * 16 + g * 16 + 4 * t) & byte_mask(nnz - j1);
            }
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                uint32_t a[4];
                ldsm_x2_trans_b8_n64(a, st + lane * ROW + ((m ^ ((lane >> 1) & 3)) << 4));
                mma_k32<SIGNED, SIGNED>(acc[m], a[0], a[1], a[2], a[3], b0, b1);
            }
            // step s + STAGES - 1 goes into the slot step s - 1 used, which
            // every lane left before this step's __syncwarp
            issue(s + STAGES - 1, cn, (s + STAGES - 1) % STAGES);
            cn = cn2;
            cn2 = cn3;
        }
        cp_async_wait<0>();  // no copy of this item is left in flight

        // acc[m]: column n = 16m + g (+8 for e >= 2), lane v = 2t (+1 for odd e)
        if (2 * t < V) {
            const int orow = row * V + 2 * t;
            __half* o = reinterpret_cast<__half*>(p.out) + (long long)b * p.out_stride + (long long)orow * 64 + g;
            const Divisor d0 = out_divisor(p, b, orow), d1 = out_divisor(p, b, orow + 1);
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const __half2 h01 = deq_half2(acc[m][0], acc[m][1], d0, d1);
                const __half2 h23 = deq_half2(acc[m][2], acc[m][3], d0, d1);
                o[16 * m] = __low2half(h01);
                o[16 * m + 64] = __high2half(h01);
                o[16 * m + 8] = __low2half(h23);
                o[16 * m + 72] = __high2half(h23);
            }
        }
    }
}

}  // namespace mc
