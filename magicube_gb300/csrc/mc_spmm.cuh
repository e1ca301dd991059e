// mc_spmm.cuh -- quantized vector-sparse SpMM for sm_103a.
//
// C[M x N] = A[M x K] * B[K x N], A stored in the reference's vector-sparse
// device layout (column vectors of V rows; see mc_oracle.c / the reference
// packer SpMM/SpMM/spmm_benchmark.cpp:177-377), B dense row-major with PREB-bit
// lanes.  Same operand layouts as the reference's spmm::wmmaSpmm_* kernels
// (SpMM/SpMM/src/wmma_spmm.cu), new kernel design:
//
//  * One CTA = one vector-row (through row_indices) x WARPS*32 output columns
//    x one batch entry.  Each warp owns 32 output columns.
//  * The contraction runs "transposed": the MMA computes C^T tiles, with the
//    16-row MMA M dimension walking output columns n and the 8-wide MMA N
//    dimension holding the V rows of the vector.  The reference's
//    chunk-transposed value layout ([v][slot] per chunk) is then exactly the
//    col-major B fragment of mma.m16n8k32, loaded with one 32-bit word per
//    thread straight from global memory.
//  * 32 gathered rows of B per step are staged by cp.async 16-byte copies
//    into a 4-stage shared-memory ring (XOR-swizzled, conflict-free reads);
//    each thread byte-transposes a 4x4 block with prmt to build the A
//    fragment (4-bit B rows are unpacked to bytes on the way).
//  * 16-bit lhs values run as two byte planes (u8 low, s8/u8 high) recombined
//    by an exact shift-add; 4-bit planes are merged/unpacked to int8 in
//    registers (sm_103a's fast integer MMA path is the 8-bit one).  16-bit B
//    rows (the reference's wmmaSpmm_16b) are split into low and high byte
//    planes in registers as well: four byte-plane products per step,
//    recombined with shifts of 0, 8, 8 and 16 bits.
//  * Accumulation wraps modulo 2^32 (no .satfinite): results equal the CPU
//    oracle bit for bit for every input.
#pragma once
#include "mc_ptx.cuh"

namespace mc {

struct SpmmParams {
    int m_vec, n, k;
    const int* row_indices;   // m_vec entries: processing order of vector-rows
    const int* row_offsets;   // 2*m_vec: [start, end) of each vector-row
    const int* col_indices;   // aligned, -1 padded (shuffled by 8 when MMA_K == 32)
    const uint8_t* values;    // device value layout
    long long values_stride;  // bytes between batch entries (0 = shared)
    const uint8_t* rhs;       // K x N packed, row-major
    long long rhs_stride;     // bytes between batch entries
    void* out;                // M x N (int32 or half)
    long long out_stride;     // elements between batch entries
    float scale;              // dequantisation divisor for half output
    const float* row_div;     // optional per-output-row divisors for half output (replaces scale)
    long long row_div_stride; // floats between batch entries of row_div
};

// Divisor of output row `orow` of batch entry b for half output.
__device__ __forceinline__ Divisor out_divisor(const SpmmParams& p, int b, int orow)
{
    return make_divisor(p.row_div ? __ldg(p.row_div + (long long)b * p.row_div_stride + orow) : p.scale);
}

// Value layouts.  PACKED (EXT = false): the reference host packer's layout
// (spmm_benchmark.cpp:224-377): chunks of MMA_K slots holding PLANES bit-planes
// of PLANE_BITS each, plane-major, each plane [v][slot]; column indices of
// 4-bit-operand pairs 8-shuffled.  SOFTMAX (EXT = true): the layout the
// extension's quantized softmax writes (q_softmax_kernel.cu:133-176,258-269)
// and its batched SpMM reads: it depends on the lhs width only -- 8-bit
// [v][16 slots] per 16-slot chunk, 4-bit nibbles [v][32 slots] per 32-slot
// chunk, 16-bit [v][low 16 bytes][high 16 bytes] per 16-slot chunk; column
// indices unshuffled.
template <int PREA, int PREB, bool EXT = false>
struct SpmmLayout {
    static constexpr int MMA_K = (PREA == 4 || PREB == 4) ? 32 : 16;     // row alignment in slots
    static constexpr int VCHUNK = EXT ? (PREA == 4 ? 32 : 16) : MMA_K;   // slots per value chunk
    static constexpr int PLANE_BITS = VCHUNK == 32 ? 4 : 8;
    static constexpr int PLANES = PREA / PLANE_BITS;                     // bit-planes per chunk
    static constexpr int BYTE_PLANES = PREA == 16 ? 2 : 1;               // int8 MMA operands
    static constexpr bool INTERLEAVED = EXT && PREA == 16;               // [v][plane][16]
    static constexpr bool SHUFFLED_COLS = !EXT && MMA_K == 32;
};

// Byte offset, inside one VCHUNK == 16 value chunk, of the word holding slots
// 4t..4t+3 of vector lane g in byte plane bp.
template <int V, int PREA, int PREB, bool EXT>
__device__ __forceinline__ int vword16(int g, int t, int bp)
{
    if constexpr (SpmmLayout<PREA, PREB, EXT>::INTERLEAVED) return g * 32 + bp * 16 + 4 * t;
    else return bp * V * 16 + g * 16 + 4 * t;
}

// Shared-memory geometry of one staged gathered-row slice.  16-bit B: row
// slices of 64 bytes per warp; the 64-bit reads of a half-warp (4 rows x 32
// bytes) land in 8 distinct 16-byte bank groups through the XOR of the chunk
// index with bits 2-3 of the row.
template <int PREB, int WARPS>
struct RhsSmem {
    static constexpr int RB = WARPS * 32 * PREB / 8;  // packed bytes per row slice
    static constexpr int CH = RB / 16;                // 16-byte chunks per row slice
    static constexpr int STRIDE = (PREB == 16) ? RB : (PREB == 8) ? (CH == 8 ? 128 : 80) : (CH == 4 ? 64 : 48);
    static constexpr int STAGE_BYTES = 32 * STRIDE;
    __device__ __forceinline__ static int swz(int r, int c)
    {
        if constexpr (PREB == 16) {
            return c ^ (((r >> 2) & 3) << 1);
        } else if constexpr (PREB == 8) {
            if constexpr (CH == 8) return c ^ (((r >> 2) & 3) << 1);
            else return c ^ (((r >> 3) & 1) << 1);
        } else {
            if constexpr (CH == 4) return c ^ ((r >> 2) & 3);
            else return c ^ ((r >> 3) & 1);
        }
    }
};

// Logical slot -> stored position of its column index.  With MMA_K == 32 the
// reference stores each group of 8 as [c0 c2 c4 c6 c1 c3 c5 c7]
// (spmm_benchmark.cpp:218-222).
template <bool SHUFFLED>
__device__ __forceinline__ int col_slot(int j)
{
    if constexpr (SHUFFLED) return (j & ~7) | ((j & 1) << 2) | ((j & 7) >> 1);
    else return j;
}

// F16: contraction on the f16 tensor path (mma.m16n8k16, f32 accumulators):
// operand bytes are converted exactly to f16 and the f32 partial sums, which
// stay integers below 2^24, are flushed into int32 every 256 vector slots, so
// the result is the same integer as the int8 path's.
template <int V, int PREA, int PREB, bool SIGNED, int WARPS, bool HALF_OUT, bool F16, bool EXT>
__global__ void __launch_bounds__(WARPS * 32)
spmm_kernel(const SpmmParams p)
{
    using L = SpmmLayout<PREA, PREB, EXT>;
    using S = RhsSmem<PREB, WARPS>;
    constexpr int STAGES = 4;
    constexpr int NT = WARPS * 32;
    constexpr int THREADS = WARPS * 32;
    constexpr int CHUNKS_PER_THREAD = (32 * S::CH) / THREADS;  // 2 for 8-bit B, 1 for 4-bit B
    constexpr int BP = L::BYTE_PLANES;
    constexpr int BB = PREB == 16 ? 2 : 1;  // byte planes of B
    static_assert(!(F16 && PREB == 16), "16-bit B runs on the int8 tensor path");
    constexpr int PLANE_BYTES = V * L::VCHUNK * L::PLANE_BITS / 8;
    constexpr int CHUNK_BYTES = PLANE_BYTES * L::PLANES;

    __shared__ __align__(128) uint8_t rhs_s[STAGES * S::STAGE_BYTES];

    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, t = lane & 3;
    const int row = __ldg(p.row_indices + blockIdx.x);
    const int n0 = blockIdx.y * NT;
    const int b = blockIdx.z;

    const int start = __ldg(p.row_offsets + 2 * row);
    const int nnz = __ldg(p.row_offsets + 2 * row + 1) - start;
    const int steps = (nnz + 31) >> 5;

    const uint8_t* values = p.values + (long long)b * p.values_stride;
    const uint8_t* rhs = p.rhs + (long long)b * p.rhs_stride + (long long)n0 * PREB / 8;
    const long long rhs_row_bytes = (long long)p.n * PREB / 8;
    const int* cols = p.col_indices + start;

    // --- staging of gathered B rows -------------------------------------
    // Thread copies chunk q = tid + i*THREADS of the 32 x CH chunk grid.
    int qrow[CHUNKS_PER_THREAD], qch[CHUNKS_PER_THREAD];
#pragma unroll
    for (int i = 0; i < CHUNKS_PER_THREAD; ++i) {
        int q = tid + i * THREADS;
        qrow[i] = q / S::CH;
        qch[i] = q % S::CH;
    }
    auto fetch_cols = [&](int s, int (&c)[CHUNKS_PER_THREAD]) {
#pragma unroll
        for (int i = 0; i < CHUNKS_PER_THREAD; ++i) {
            int j = s * 32 + qrow[i];
            c[i] = (s < steps && j < nnz) ? __ldg(cols + col_slot<L::SHUFFLED_COLS>(j)) : -1;
        }
    };
    auto issue_stage = [&](int s, const int (&c)[CHUNKS_PER_THREAD]) {
        uint8_t* st = rhs_s + (s % STAGES) * S::STAGE_BYTES;
#pragma unroll
        for (int i = 0; i < CHUNKS_PER_THREAD; ++i) {
            if (c[i] >= 0) {
                const uint8_t* src = rhs + (long long)c[i] * rhs_row_bytes + qch[i] * 16;
                cp_async16(st + qrow[i] * S::STRIDE + S::swz(qrow[i], qch[i]) * 16, src);
            }
        }
    };

    // --- value fragments (MMA B operand) --------------------------------
    // vals[bp][h]: byte plane bp, half h (slots 16h + 4t .. +3) for v = g.
    auto load_vals = [&](int s, uint32_t (&vals)[BP][2]) {
#pragma unroll
        for (int bp = 0; bp < BP; ++bp) { vals[bp][0] = 0u; vals[bp][1] = 0u; }
        if (g >= V || s >= steps) return;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int jrel = s * 32 + 16 * h + 4 * t;  // first slot of this word
            const int valid = nnz - jrel;
            if (valid <= 0) continue;
            const uint32_t keep = byte_mask(valid);
            const int slot = start + jrel;
            if constexpr (L::VCHUNK == 16) {
                // 8-bit planes: element (v, j) at byte v*16 + j of its plane.
                const uint8_t* chunk = values + (long long)(slot >> 4) * CHUNK_BYTES;
#pragma unroll
                for (int bp = 0; bp < BP; ++bp)
                    vals[bp][h] = __ldg(reinterpret_cast<const uint32_t*>(chunk + vword16<V, PREA, PREB, EXT>(g, t, bp))) & keep;
            } else {
                // 4-bit planes: element (v, j) at nibble v*32 + j of its plane.
                const uint8_t* chunk = values + (long long)(slot >> 5) * CHUNK_BYTES;
                const int off = g * 16 + ((slot & 31) >> 1);
                uint32_t nib[L::PLANES];
#pragma unroll
                for (int pl = 0; pl < L::PLANES; ++pl)
                    nib[pl] = __ldg(reinterpret_cast<const unsigned short*>(chunk + pl * PLANE_BYTES + off));
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
    };

    int acc[BP * BB][2][4];   // [bp * BB + bb]: values byte plane bp x B byte plane bb
    float facc[BP][2][4];
#pragma unroll
    for (int k = 0; k < BP * BB; ++k)
#pragma unroll
        for (int m = 0; m < 2; ++m)
#pragma unroll
            for (int e = 0; e < 4; ++e) acc[k][m][e] = 0;
#pragma unroll
    for (int bp = 0; bp < BP; ++bp)
#pragma unroll
        for (int m = 0; m < 2; ++m)
#pragma unroll
            for (int e = 0; e < 4; ++e) facc[bp][m][e] = 0.f;

    // Pipeline prologue: column indices run one stage ahead of the copies.
    int cnext[CHUNKS_PER_THREAD];
    {
        int c[CHUNKS_PER_THREAD];
#pragma unroll
        for (int s = 0; s < STAGES - 1; ++s) {
            fetch_cols(s, c);
            issue_stage(s, c);
            cp_async_commit();
        }
        fetch_cols(STAGES - 1, cnext);
    }
    uint32_t vcur[BP][2], vnext[BP][2];
    load_vals(0, vcur);

    // Column byte (8-bit B) or nibble pair (4-bit B) this thread reads.
    const int ncol = warp * 32 + 4 * g;

#pragma unroll 1
    for (int s = 0; s < steps; ++s) {
        cp_async_wait<STAGES - 2>();
        __syncthreads();
        {
            const int sn = s + STAGES - 1;
            issue_stage(sn, cnext);
            cp_async_commit();
            fetch_cols(sn + 1, cnext);
        }
        load_vals(s + 1, vnext);

        const uint8_t* st = rhs_s + (s % STAGES) * S::STAGE_BYTES;
        if constexpr (PREB == 16) {
            // Columns ncol..ncol+3 of rows 16h+4t+i: 8 bytes, split into the
            // low and high bytes of the four 16-bit lanes, then byte-transposed.
            uint32_t tb[2][2][4];  // [B byte plane][h][i]
            const int byte = 2 * ncol;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int r = 16 * h + 4 * t + i;
                    const uint2 w = lds64(st + r * S::STRIDE + S::swz(r, byte >> 4) * 16 + (byte & 15));
                    tb[0][h][i] = prmt(w.x, w.y, 0x6420);
                    tb[1][h][i] = prmt(w.x, w.y, 0x7531);
                }
                transpose4x4(tb[0][h]);
                transpose4x4(tb[1][h]);
            }
#pragma unroll
            for (int bp = 0; bp < BP; ++bp) {
                const bool top = (bp == BP - 1);
#pragma unroll
                for (int bb = 0; bb < 2; ++bb) {
                    int (&a)[2][4] = acc[bp * 2 + bb];
                    const uint32_t (&T)[2][4] = tb[bb];
#define MC_MMA16(AS, VS)                                                                                  \
    mma_k32<AS, VS>(a[0], T[0][0], T[0][1], T[1][0], T[1][1], vcur[bp][0], vcur[bp][1]);                 \
    mma_k32<AS, VS>(a[1], T[0][2], T[0][3], T[1][2], T[1][3], vcur[bp][0], vcur[bp][1]);
                    // Only the high byte plane of each operand is signed.
                    if (SIGNED && bb == 1 && top) { MC_MMA16(true, true) }
                    else if (SIGNED && bb == 1) { MC_MMA16(true, false) }
                    else if (SIGNED && top) { MC_MMA16(false, true) }
                    else { MC_MMA16(false, false) }
#undef MC_MMA16
                }
            }
#pragma unroll
            for (int bp = 0; bp < BP; ++bp) { vcur[bp][0] = vnext[bp][0]; vcur[bp][1] = vnext[bp][1]; }
        } else {
        uint32_t tr[2][4];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = 16 * h + 4 * t + i;
                if constexpr (PREB == 8) {
                    const int c = ncol >> 4;
                    tr[h][i] = lds32(st + r * S::STRIDE + S::swz(r, c) * 16 + (ncol & 15));
                } else {
                    const int byte = ncol >> 1;
                    const int c = byte >> 4;
                    tr[h][i] = unpack4_u16<SIGNED>(lds16(st + r * S::STRIDE + S::swz(r, c) * 16 + (byte & 15)));
                }
            }
            if constexpr (!F16) transpose4x4(tr[h]);
        }
        if constexpr (F16) {
            // tr[h][i]: bytes of output columns ncol..ncol+3 in slot 16h+4t+i.
            // Convert each row to f16 pairs, then transpose at half granularity:
            // ah[h][c][0] = slots (16h+4t, +1), ah[h][c][1] = slots (+2, +3) of column ncol+c.
            uint32_t ah[2][4][2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                uint32_t P[4], Q[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) bytes_to_h2<SIGNED>(tr[h][i], P[i], Q[i]);
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    ah[h][0][q] = prmt(P[2 * q], P[2 * q + 1], 0x5410);
                    ah[h][1][q] = prmt(P[2 * q], P[2 * q + 1], 0x7632);
                    ah[h][2][q] = prmt(Q[2 * q], Q[2 * q + 1], 0x5410);
                    ah[h][3][q] = prmt(Q[2 * q], Q[2 * q + 1], 0x7632);
                }
            }
#pragma unroll
            for (int bp = 0; bp < BP; ++bp) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    uint32_t vlo, vhi;
                    if (SIGNED && bp == BP - 1) bytes_to_h2<true>(vcur[bp][h], vlo, vhi);
                    else bytes_to_h2<false>(vcur[bp][h], vlo, vhi);
                    mma_f16(facc[bp][0], ah[h][0][0], ah[h][1][0], ah[h][0][1], ah[h][1][1], vlo, vhi);
                    mma_f16(facc[bp][1], ah[h][2][0], ah[h][3][0], ah[h][2][1], ah[h][3][1], vlo, vhi);
                }
            }
            if ((s & 7) == 7 || s == steps - 1) {
#pragma unroll
                for (int bp = 0; bp < BP; ++bp)
#pragma unroll
                    for (int m = 0; m < 2; ++m)
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            acc[bp][m][e] = (int)((uint32_t)acc[bp][m][e] + (uint32_t)f2i_exact(facc[bp][m][e]));
                            facc[bp][m][e] = 0.f;
                        }
            }
#pragma unroll
            for (int bp = 0; bp < BP; ++bp) { vcur[bp][0] = vnext[bp][0]; vcur[bp][1] = vnext[bp][1]; }
            continue;
        }
        // tr[h][c]: slots 16h+4t..+3 of output column ncol + c.
#pragma unroll
        for (int bp = 0; bp < BP; ++bp) {
            // Only the most significant byte plane of a signed value is signed.
            const bool top = (bp == BP - 1);
            if (SIGNED && top) {
                mma_k32<SIGNED, true>(acc[bp][0], tr[0][0], tr[0][1], tr[1][0], tr[1][1], vcur[bp][0], vcur[bp][1]);
                mma_k32<SIGNED, true>(acc[bp][1], tr[0][2], tr[0][3], tr[1][2], tr[1][3], vcur[bp][0], vcur[bp][1]);
            } else {
                mma_k32<SIGNED, false>(acc[bp][0], tr[0][0], tr[0][1], tr[1][0], tr[1][1], vcur[bp][0], vcur[bp][1]);
                mma_k32<SIGNED, false>(acc[bp][1], tr[0][2], tr[0][3], tr[1][2], tr[1][3], vcur[bp][0], vcur[bp][1]);
            }
        }
#pragma unroll
        for (int bp = 0; bp < BP; ++bp) { vcur[bp][0] = vnext[bp][0]; vcur[bp][1] = vnext[bp][1]; }
        }  // PREB != 16
    }
    cp_async_wait<0>();

    // Epilogue.  acc[.][m][e]: column ncol + 2m + (e >> 1), vector lane 2t + (e & 1).
    // Byte-plane products recombine as sum acc[bp][bb] << 8 (bp + bb), mod 2^32.
    int res[2][4];
#pragma unroll
    for (int e2 = 0; e2 < 2; ++e2) {
        // vector lane v = 2t + e2, columns ncol .. ncol+3
        uint32_t c4[4] = {0u, 0u, 0u, 0u};
#pragma unroll
        for (int k = 0; k < BP * BB; ++k) {
            const int sh = 8 * (k / BB + k % BB);
            const uint32_t h4[4] = {(uint32_t)acc[k][0][e2], (uint32_t)acc[k][0][2 + e2], (uint32_t)acc[k][1][e2],
                                    (uint32_t)acc[k][1][2 + e2]};
#pragma unroll
            for (int q = 0; q < 4; ++q) c4[q] += h4[q] << sh;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) res[e2][q] = (int)c4[q];
    }
#pragma unroll
    for (int e2 = 0; e2 < 2; ++e2) {
        const int v = 2 * t + e2;
        if (v >= V) continue;
        const long long o = (long long)b * p.out_stride + (long long)(row * V + v) * p.n + n0 + ncol;
        if constexpr (HALF_OUT) {
            __half* out = reinterpret_cast<__half*>(p.out) + o;
            const Divisor dv = out_divisor(p, b, row * V + v);
            uint32_t h0 = pack_half2(res[e2][0], res[e2][1], dv);
            uint32_t h1 = pack_half2(res[e2][2], res[e2][3], dv);
            stg_cs_v2(out, (int)h0, (int)h1);
        } else {
            int* out = reinterpret_cast<int*>(p.out) + o;
            stg_cs_v4(out, res[e2][0], res[e2][1], res[e2][2], res[e2][3]);
        }
    }
}

}  // namespace mc
