// format_device.cu -- the vector-sparse packer on the GPU.
//
// Device form of the host packer in format.cpp (the reference's serial host
// code, SpMM/SpMM/spmm_benchmark.cpp:177-377 and bm_test_utils.h:222-237):
// aligned [start, end) row ranges, -1 padded / 8-shuffled column indices,
// the chunk-transposed bit-plane value layout and the longest-first row
// order.  Outputs are byte-identical to the host routines (the row order for
// rows of equal length is ascending row index; std::sort leaves it
// unspecified).  All of this is HBM-bound byte movement:
//
//  * align: three launches, no inter-CTA waits.  The first sums the aligned
//    lengths of each tile of 1024 rows into a scratch array (and writes the
//    sort keys), one CTA scans the tile sums, the third scans inside each tile
//    from its prefix and writes the pairs and the aligned count.
//  * columns and values: one warp per vector-row writes the slots from its
//    start to the next row's start (the last row up to the aligned count),
//    so every output byte is written exactly once and padding needs no
//    separate fill.  Each lane keeps several words in flight; 8-bit values in
//    16-slot chunks read whole slot vectors and transpose them in registers.
//  * row order: a stable descending radix sort of the row lengths (CUB) over
//    the key bits the slot capacity needs.
#include <cub/device/device_radix_sort.cuh>
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <mutex>
#include <type_traits>

#include "mc_host.h"

namespace mc {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanPerThread = 4;
constexpr int kScanTile = kScanThreads * kScanPerThread;  // rows per scan tile
constexpr int kUnroll = 4;                                 // words / slots in flight per lane

__device__ __forceinline__ long long round_up(long long len, int a) { return (len + a - 1) / a * a; }

__device__ __forceinline__ long long block_sum(long long v, long long* red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    long long t = 0;
#pragma unroll
    for (int w = 0; w < kScanThreads / 32; ++w) t += red[w];
    return t;
}

// Scratch of the align step: per-tile sums, then a flag word that must start
// at zero (set when some row length is negative).
struct AlignScratch {
    long long* tile_sums;
    int* bad;
};

// Also writes each row's length and index (the sort's keys and values) when
// keys is not null.
__global__ void __launch_bounds__(kScanThreads)
align_tile_sums_kernel(int m_vec, const int* __restrict__ ro, int alignment, AlignScratch sc,
                       int* __restrict__ keys, int* __restrict__ idx)
{
    __shared__ long long red[kScanThreads / 32];
    const int base = blockIdx.x * kScanTile;
    long long s = 0;
    bool neg = false;
#pragma unroll
    for (int r = 0; r < kScanPerThread; ++r) {
        const int i = base + r * kScanThreads + threadIdx.x;
        if (i < m_vec) {
            const int a = __ldg(ro + i), b = __ldg(ro + i + 1);
            const long long len = (long long)b - a;
            neg |= len < 0;
            s += round_up(len < 0 ? 0 : len, alignment);
            if (keys) {
                keys[i] = b - a;
                idx[i] = i;
            }
        }
    }
    if (neg) atomicOr(sc.bad, 1);
    s = block_sum(s, red);
    if (threadIdx.x == 0) sc.tile_sums[blockIdx.x] = s;
}

// Exclusive scan of the tile sums in place (one CTA, a carried loop over
// blocks of 256 tiles).
__global__ void __launch_bounds__(kScanThreads)
align_tile_prefix_kernel(int ntiles, AlignScratch sc)
{
    __shared__ long long wsum[kScanThreads / 32];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    long long carry = 0;
    for (int b = 0; b < ntiles; b += kScanThreads) {
        const int t = b + tid;
        const long long x = t < ntiles ? sc.tile_sums[t] : 0;
        long long inc = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) wsum[warp] = inc;
        __syncthreads();
        long long woff = 0, total = 0;
#pragma unroll
        for (int w = 0; w < kScanThreads / 32; ++w) {
            if (w < warp) woff += wsum[w];
            total += wsum[w];
        }
        if (t < ntiles) sc.tile_sums[t] = carry + woff + inc - x;
        carry += total;
        __syncthreads();
    }
}

// Shared-memory index of tile row k, padded so that thread t's consecutive
// rows fall into distinct banks across a warp.
__device__ __forceinline__ int pad_idx(int k) { return k + (k >> 5); }

__global__ void __launch_bounds__(kScanThreads)
align_scan_kernel(int m_vec, const int* __restrict__ ro, int alignment, AlignScratch sc, int ntiles,
                  int* __restrict__ pairs, int* __restrict__ aligned_nnz)
{
    __shared__ int s_ro[kScanTile + 1 + (kScanTile + 1) / 32 + 1];
    __shared__ long long wsum[kScanThreads / 32];
    const int tile = blockIdx.x, tid = threadIdx.x;
    const int base = tile * kScanTile;

    const long long pre = ntiles > 0 ? sc.tile_sums[tile] : 0;  // exclusive prefix of this tile

    for (int k = tid; k <= kScanTile; k += kScanThreads) {
        const int i = base + k;
        s_ro[pad_idx(k)] = i <= m_vec ? __ldg(ro + i) : 0;
    }
    __syncthreads();

    long long len[kScanPerThread];
    long long tsum = 0;
#pragma unroll
    for (int r = 0; r < kScanPerThread; ++r) {
        const int k = tid * kScanPerThread + r;
        const bool in = base + k < m_vec;
        const long long l = in ? (long long)s_ro[pad_idx(k + 1)] - s_ro[pad_idx(k)] : 0;
        len[r] = l < 0 ? 0 : l;
        tsum += round_up(len[r], alignment);
    }
    // Exclusive scan of the thread totals across the block.
    const int warp = tid >> 5, lane = tid & 31;
    long long inc = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    long long woff = 0, total = 0;
#pragma unroll
    for (int w = 0; w < kScanThreads / 32; ++w) {
        if (w < warp) woff += wsum[w];
        total += wsum[w];
    }
    long long start = pre + woff + inc - tsum;
#pragma unroll
    for (int r = 0; r < kScanPerThread; ++r) {
        const int i = base + tid * kScanPerThread + r;
        if (i < m_vec)
            reinterpret_cast<int2*>(pairs)[i] = make_int2((int)start, (int)(start + len[r]));
        start += round_up(len[r], alignment);
    }
    if (tile == (ntiles > 0 ? ntiles - 1 : 0) && tid == 0) {
        const long long all = pre + total;
        *aligned_nnz = (*sc.bad || all > INT_MAX) ? -1 : (int)all;
    }
}

// The slots vector-row i writes: [lo, hi) with lo = 0 for the first row and
// its start otherwise, hi = the next row's start or the aligned count; its
// nonzeros sit at [start, start + len) and come from source index src.
struct RowSpan {
    long long lo, hi, start, len, src;
};

__device__ __forceinline__ bool row_span(int i, int m_vec, const int* ro, const int* pairs, const int* total_p,
                                         int unit, long long cap, RowSpan& r)
{
    const long long total = *total_p;
    if (m_vec == 0) {
        r.start = r.lo = 0; r.len = 0; r.src = 0; r.hi = total;
    } else {
        r.start = __ldg(pairs + 2 * i);
        r.src = __ldg(ro + i);
        r.len = (long long)__ldg(ro + i + 1) - r.src;
        r.lo = i == 0 ? 0 : r.start;
        r.hi = i + 1 < m_vec ? (long long)__ldg(pairs + 2 * i + 2) : total;
    }
    return total >= 0 && r.len >= 0 && r.start >= r.lo && r.start + r.len <= r.hi && r.lo % unit == 0 &&
           r.hi % unit == 0 && r.hi <= cap;
}

__device__ __forceinline__ void pad_row_columns(const RowSpan& r, const int* __restrict__ cols, bool shuffle8,
                                                int* __restrict__ out, int lane)
{
    for (long long s0 = r.lo + lane; s0 < r.hi; s0 += 32 * kUnroll) {
        int c[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const long long jr = s0 + 32 * u - r.start;
            c[u] = (jr >= 0 && jr < r.len) ? __ldg(cols + r.src + jr) : -1;
        }
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const long long s = s0 + 32 * u;
            if (s < r.hi) out[shuffle8 ? (s & ~7LL) + (s & 1) * 4 + ((s & 7) >> 1) : s] = c[u];
        }
    }
}

// Lane `lane` (BITS bits, lane l at bit l*BITS) of a byte array.
template <int BITS>
__device__ __forceinline__ uint32_t lane_bits(const uint8_t* p, long long lane)
{
    if constexpr (BITS == 8) {
        return __ldg(p + lane);
    } else if constexpr (BITS == 16) {
        return (uint32_t)__ldg(p + 2 * lane) | ((uint32_t)__ldg(p + 2 * lane + 1) << 8);
    } else {
        return (__ldg(p + (lane >> 1)) >> ((lane & 1) * 4)) & 0xFu;
    }
}

// Value chunks: a chunk of CHUNK slots holds LHS/PLANE planes of PLANE bits;
// element (plane pl, lane v, slot jj) of the chunk is element
//   pl*V*CHUNK + v*CHUNK + jj            (plane-major), or
//   v*PLANES*CHUNK + pl*CHUNK + jj       (INTERLEAVED, the 16-bit softmax layout).
template <int V, int LHS, int CHUNK, bool INTERLEAVED>
struct ValueLayout {
    static constexpr int PLANE = CHUNK == 32 ? 4 : 8;
    static constexpr int CHUNK_BYTES = V * CHUNK * LHS / 8;
    static constexpr int WORDS = CHUNK_BYTES / 4;
};

// Output word w (counted from the row's first chunk c0) of a row's values.
template <int V, int LHS, int CHUNK, bool INTERLEAVED>
__device__ __forceinline__ uint32_t value_word(const RowSpan& r, const uint8_t* __restrict__ src, long long c0,
                                               long long w, long long nw, uint32_t vmask)
{
    using L = ValueLayout<V, LHS, CHUNK, INTERLEAVED>;
    constexpr uint32_t PMASK = (1u << L::PLANE) - 1u;
    uint32_t word = 0;
    if (w < nw) {
        const long long c = c0 + w / L::WORDS;
        const int wi = (int)(w % L::WORDS);
#pragma unroll
        for (int e = 0; e < 32 / L::PLANE; ++e) {
            const int el = wi * (32 / L::PLANE) + e;  // element index within the chunk
            int pl, v, jj;
            if constexpr (INTERLEAVED) {
                v = el / (LHS / L::PLANE * CHUNK);
                pl = (el % (LHS / L::PLANE * CHUNK)) / CHUNK;
                jj = el % CHUNK;
            } else {
                pl = el / (V * CHUNK);
                v = (el % (V * CHUNK)) / CHUNK;
                jj = el % CHUNK;
            }
            const long long jr = c * CHUNK + jj - r.start;
            if (jr >= 0 && jr < r.len) {
                const uint32_t x = lane_bits<LHS>(src, (r.src + jr) * V + v) & vmask;
                word |= ((x >> (pl * L::PLANE)) & PMASK) << (e * L::PLANE);
            }
        }
    }
    return word;
}

// 8-bit values in 16-slot chunks ([v][16] bytes per chunk): a lane takes 4
// consecutive slots of one chunk, reads their V-byte vectors whole and
// transposes them into the V output words (v, slots 4q..4q+3).
template <int V>
__device__ __forceinline__ void pack_row_values_8b16(const RowSpan& r, const uint8_t* __restrict__ src,
                                                     uint8_t* __restrict__ out, int lane)
{
    using Vec = typename std::conditional<V == 8, uint2, typename std::conditional<V == 4, uint32_t, uint16_t>::type>::type;
    const long long c0 = r.lo / 16;
    const long long ntask = (r.hi - r.lo) / 4;  // groups of 4 slots
    for (long long t0 = lane; t0 < ntask; t0 += 32 * 2) {
        uint32_t b[2][4][2];  // [task][slot][low/high 4 lanes]
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const long long jr0 = r.lo + 4 * (t0 + 32 * u) - r.start;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const long long jr = jr0 + k;
                b[u][k][0] = b[u][k][1] = 0u;
                if (t0 + 32 * u < ntask && jr >= 0 && jr < r.len) {
                    const Vec x = __ldg(reinterpret_cast<const Vec*>(src + (r.src + jr) * V));
                    if constexpr (V == 8) {
                        b[u][k][0] = x.x;
                        b[u][k][1] = x.y;
                    } else {
                        b[u][k][0] = (uint32_t)x;
                    }
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const long long t = t0 + 32 * u;
            if (t >= ntask) break;
            uint32_t* chunk = reinterpret_cast<uint32_t*>(out + (c0 + t / 4) * (16 * V));
            const int q = (int)(t % 4);
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const int h = v >> 2, sh = 8 * (v & 3);
                const uint32_t w = ((b[u][0][h] >> sh) & 0xFFu) | (((b[u][1][h] >> sh) & 0xFFu) << 8) |
                                   (((b[u][2][h] >> sh) & 0xFFu) << 16) | (((b[u][3][h] >> sh) & 0xFFu) << 24);
                chunk[v * 4 + q] = w;
            }
        }
    }
}

// FAST: the 8-bit 16-slot path (values V-byte aligned).
template <int V, int LHS, int CHUNK, bool INTERLEAVED, bool FAST>
__device__ __forceinline__ void pack_row_values(const RowSpan& r, const uint8_t* __restrict__ src,
                                                uint8_t* __restrict__ out, int lane, uint32_t vmask)
{
    using L = ValueLayout<V, LHS, CHUNK, INTERLEAVED>;
    if constexpr (FAST && LHS == 8 && CHUNK == 16 && !INTERLEAVED) {
        pack_row_values_8b16<V>(r, src, out, lane);
        return;
    }
    const long long c0 = r.lo / CHUNK;
    const long long nw = (r.hi - r.lo) / CHUNK * L::WORDS;
    for (long long w0 = lane; w0 < nw; w0 += 32 * kUnroll) {
        uint32_t word[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
            word[u] = value_word<V, LHS, CHUNK, INTERLEAVED>(r, src, c0, w0 + 32 * u, nw, vmask);
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const long long w = w0 + 32 * u;
            if (w < nw) reinterpret_cast<uint32_t*>(out + (c0 + w / L::WORDS) * L::CHUNK_BYTES)[w % L::WORDS] = word[u];
        }
    }
}

// Per-row conversion, one warp per vector-row: padded columns (cols_out not
// null) and packed values (VALUES).  unit: the multiple every row's slot range
// must be (the value chunk, 8 when shuffling, else 1); cap: slots the outputs
// hold.
template <int V, int LHS, int CHUNK, bool INTERLEAVED, bool VALUES, bool FAST = false>
__global__ void __launch_bounds__(256)
fill_rows_kernel(int m_vec, const int* __restrict__ ro, const int* __restrict__ pairs,
                 const int* __restrict__ total, int unit, long long cap, const int* __restrict__ cols,
                 int shuffle8, int* __restrict__ cols_out, const uint8_t* __restrict__ src,
                 uint8_t* __restrict__ vals_out, uint32_t vmask, int* status)
{
    const int rows = m_vec > 0 ? m_vec : 1;
    const int lane = threadIdx.x & 31;
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < rows; i += nwarps) {
        RowSpan r;
        if (!row_span(i, m_vec, ro, pairs, total, unit, cap, r)) {
            if (status && lane == 0) *status = 1;
            continue;
        }
        if (cols_out) pad_row_columns(r, cols, shuffle8 != 0, cols_out, lane);
        if constexpr (VALUES) pack_row_values<V, LHS, CHUNK, INTERLEAVED, FAST>(r, src, vals_out, lane, vmask);
    }
}

// MC_VALUES_SLOT_MAJOR, 8-bit lanes ([aligned slot][V] bytes): slot s of a
// row's aligned range takes the row's vector s - start whole, the padding
// slots zeros.  ALIGNED: the source is V-byte aligned, one load per vector.
template <int V, bool ALIGNED>
__global__ void __launch_bounds__(256)
fill_rows_slot_kernel(int m_vec, const int* __restrict__ ro, const int* __restrict__ pairs,
                      const int* __restrict__ total, int unit, long long cap, const int* __restrict__ cols,
                      int shuffle8, int* __restrict__ cols_out, const uint8_t* __restrict__ src,
                      uint8_t* __restrict__ vals_out, int* status)
{
    using Vec = typename std::conditional<V == 8, uint2, typename std::conditional<V == 4, uint32_t, uint16_t>::type>::type;
    const int rows = m_vec > 0 ? m_vec : 1;
    const int lane = threadIdx.x & 31;
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < rows; i += nwarps) {
        RowSpan r;
        if (!row_span(i, m_vec, ro, pairs, total, unit, cap, r)) {
            if (status && lane == 0) *status = 1;
            continue;
        }
        if (cols_out) pad_row_columns(r, cols, shuffle8 != 0, cols_out, lane);
        for (long long s0 = r.lo + lane; s0 < r.hi; s0 += 32 * kUnroll) {
            Vec x[kUnroll];
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                const long long jr = s0 + 32 * u - r.start;
                x[u] = Vec{};
                if (s0 + 32 * u < r.hi && jr >= 0 && jr < r.len) {
                    const uint8_t* p = src + (r.src + jr) * V;
                    if constexpr (ALIGNED) {
                        x[u] = __ldg(reinterpret_cast<const Vec*>(p));
                    } else {
                        uint8_t b[V];
#pragma unroll
                        for (int v = 0; v < V; ++v) b[v] = __ldg(p + v);
                        memcpy(&x[u], b, V);
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < kUnroll; ++u) {
                const long long s = s0 + 32 * u;
                if (s < r.hi) *reinterpret_cast<Vec*>(vals_out + s * V) = x[u];
            }
        }
    }
}

__global__ void row_keys_kernel(int m_vec, const int* __restrict__ ro, int* __restrict__ len,
                                int* __restrict__ idx)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m_vec; i += gridDim.x * blockDim.x) {
        len[i] = __ldg(ro + i + 1) - __ldg(ro + i);
        idx[i] = i;
    }
}

int grid_for_warps(long long warps)
{
    const long long ctas = (warps + 7) / 8;
    const long long cap = (long long)sm_count() * 16;
    return (int)(ctas < 1 ? 1 : (ctas > cap ? cap : ctas));
}

// Launches fill_rows_kernel for the value layout of (lhs_bits, rhs_bits,
// layout); lhs_bits == 0 converts the columns only.
struct FillArgs {
    int m_vec;
    const int* ro;
    const int* pairs;
    const int* total;
    const int* cols;
    int shuffle8;
    int* cols_out;
    long long cols_cap;
    const uint8_t* src;
    uint8_t* vals_out;
    long long vals_cap_bytes;
    int* status;
    uint32_t vmask;  // applied to every source value (12-bit values: 0xFFF)
};

template <int V, int LHS, int CHUNK, bool IL>
int fill_launch(const FillArgs& a, cudaStream_t s)
{
    const int grid = grid_for_warps(a.m_vec > 0 ? a.m_vec : 1);
    using L = ValueLayout<V, LHS, CHUNK, IL>;
    long long cap = a.vals_cap_bytes / L::CHUNK_BYTES * CHUNK;
    if (a.cols_out && a.cols_cap < cap) cap = a.cols_cap;
    if constexpr (LHS == 8 && CHUNK == 16 && !IL) {
        if (reinterpret_cast<uintptr_t>(a.src) % V == 0) {
            fill_rows_kernel<V, LHS, CHUNK, IL, true, true><<<grid, 256, 0, s>>>(
                a.m_vec, a.ro, a.pairs, a.total, CHUNK, cap, a.cols, a.shuffle8, a.cols_out, a.src, a.vals_out,
                a.vmask, a.status);
            return (int)cudaGetLastError();
        }
    }
    fill_rows_kernel<V, LHS, CHUNK, IL, true><<<grid, 256, 0, s>>>(a.m_vec, a.ro, a.pairs, a.total, CHUNK, cap,
                                                                   a.cols, a.shuffle8, a.cols_out, a.src, a.vals_out,
                                                                   a.vmask, a.status);
    return (int)cudaGetLastError();
}

// Slot-major 8-bit values: rows aligned to 16 slots, as the packed L8-R8
// layout, so one set of aligned pairs serves both.
template <int V>
int fill_slot(const FillArgs& a, cudaStream_t s)
{
    const int grid = grid_for_warps(a.m_vec > 0 ? a.m_vec : 1);
    long long cap = a.vals_cap_bytes / V;
    if (a.cols_out && a.cols_cap < cap) cap = a.cols_cap;
    if (reinterpret_cast<uintptr_t>(a.src) % V == 0)
        fill_rows_slot_kernel<V, true><<<grid, 256, 0, s>>>(a.m_vec, a.ro, a.pairs, a.total, 16, cap, a.cols,
                                                            a.shuffle8, a.cols_out, a.src, a.vals_out, a.status);
    else
        fill_rows_slot_kernel<V, false><<<grid, 256, 0, s>>>(a.m_vec, a.ro, a.pairs, a.total, 16, cap, a.cols,
                                                             a.shuffle8, a.cols_out, a.src, a.vals_out, a.status);
    return (int)cudaGetLastError();
}

template <int V>
int fill_v(int lhs_bits, int rhs_bits, int layout, const FillArgs& a, cudaStream_t s)
{
    if (layout == MC_VALUES_SLOT_MAJOR) return fill_slot<V>(a, s);
    const bool four = lhs_bits == 4 || rhs_bits == 4;
    if (layout == MC_VALUES_SOFTMAX) {
        if (lhs_bits == 4) return fill_launch<V, 4, 32, false>(a, s);
        if (lhs_bits == 8) return fill_launch<V, 8, 16, false>(a, s);
        return fill_launch<V, 16, 16, true>(a, s);
    }
    if (four) {
        if (lhs_bits == 4) return fill_launch<V, 4, 32, false>(a, s);
        if (lhs_bits == 8) return fill_launch<V, 8, 32, false>(a, s);
        return fill_launch<V, 16, 32, false>(a, s);
    }
    if (lhs_bits == 8) return fill_launch<V, 8, 16, false>(a, s);
    return fill_launch<V, 16, 16, false>(a, s);
}

int fill(int vec_length, int lhs_bits, int rhs_bits, int layout, const FillArgs& a_in, cudaStream_t s)
{
    // 12-bit values: 16-bit containers in the 16-bit layouts, top 4 bits
    // cleared (spmm_benchmark.cpp:288-358).
    FillArgs a = a_in;
    a.vmask = lhs_bits == 12 ? 0xFFFu : 0xFFFFFFFFu;
    if (lhs_bits == 12) lhs_bits = 16;
    if (lhs_bits == 0) {
        const int grid = grid_for_warps(a.m_vec > 0 ? a.m_vec : 1);
        fill_rows_kernel<2, 8, 16, false, false><<<grid, 256, 0, s>>>(
            a.m_vec, a.ro, a.pairs, a.total, a.shuffle8 ? 8 : 1, a.cols_cap, a.cols, a.shuffle8, a.cols_out,
            nullptr, nullptr, 0xFFFFFFFFu, a.status);
        return (int)cudaGetLastError();
    }
    switch (vec_length) {
        case 2: return fill_v<2>(lhs_bits, rhs_bits, layout, a, s);
        case 4: return fill_v<4>(lhs_bits, rhs_bits, layout, a, s);
        default: return fill_v<8>(lhs_bits, rhs_bits, layout, a, s);
    }
}

bool valid_pair(int lhs_bits, int rhs_bits)
{
    return (lhs_bits == 4 && rhs_bits == 4) || (lhs_bits == 8 && rhs_bits == 4) ||
           (lhs_bits == 12 && rhs_bits == 4) || (lhs_bits == 16 && rhs_bits == 4) ||
           (lhs_bits == 8 && rhs_bits == 8) || (lhs_bits == 12 && rhs_bits == 8) ||
           (lhs_bits == 16 && rhs_bits == 8) || (lhs_bits == 16 && rhs_bits == 16);
}

}  // namespace

long long align_scratch_bytes(int m_vec)
{
    const long long ntiles = ((long long)m_vec + kScanTile - 1) / kScanTile;
    return ntiles * 8 + 256;
}

// The align step with caller-provided scratch (align_scratch_bytes(m_vec)
// bytes, 8-byte aligned); keys/idx (optional, m_vec ints each) receive the
// row lengths and indices for the row sort.
int device_align_launch(int m_vec, const int* ro, int alignment, int* pairs, int* aligned_nnz, void* scratch,
                        int* keys, int* idx, cudaStream_t s)
{
    const int ntiles = (int)(((long long)m_vec + kScanTile - 1) / kScanTile);
    AlignScratch sc;
    sc.tile_sums = static_cast<long long*>(scratch);
    sc.bad = reinterpret_cast<int*>(static_cast<char*>(scratch) + (size_t)ntiles * 8);
    int rc = (int)cudaMemsetAsync(sc.bad, 0, sizeof(int), s);
    if (rc) return rc;
    if (ntiles > 0) {
        align_tile_sums_kernel<<<ntiles, kScanThreads, 0, s>>>(m_vec, ro, alignment, sc, keys, idx);
        align_tile_prefix_kernel<<<1, kScanThreads, 0, s>>>(ntiles, sc);
    }
    align_scan_kernel<<<ntiles > 0 ? ntiles : 1, kScanThreads, 0, s>>>(m_vec, ro, alignment, sc, ntiles, pairs,
                                                                         aligned_nnz);
    return (int)cudaGetLastError();
}

static int check_align_args(int m_vec, const int* ro, int alignment, const int* pairs, const int* aligned_nnz)
{
    if (m_vec < 0 || alignment <= 0 || !ro || !aligned_nnz || (m_vec > 0 && !pairs))
        return fail(1, "mcDeviceAlignRowOffsets: invalid arguments");
    if (m_vec > 0 && reinterpret_cast<uintptr_t>(pairs) % 8)
        return fail(1, "mcDeviceAlignRowOffsets: aligned_pairs must be 8-byte aligned");
    return 0;
}

// Bytes of CUB radix-sort temporary storage for m_vec rows.
static int sort_temp_bytes(int m_vec, int end_bit, size_t* bytes)
{
    *bytes = 0;
    return (int)cub::DeviceRadixSort::SortPairsDescending(nullptr, *bytes, (const int*)nullptr, (int*)nullptr,
                                                          (const int*)nullptr, (int*)nullptr, m_vec, 0, end_bit);
}

// Key bits that hold every length up to `bound` (row lengths are
// non-negative and at most the slot capacity when the input is consistent;
// inconsistent input is reported through the status word and aligned count).
static int key_bits(long long bound)
{
    int b = 1;
    while (b < 31 && (1LL << b) <= bound) ++b;
    return b;
}

static size_t round256(size_t b) { return (b + 255) / 256 * 256; }

// Scratch of mcDeviceAlignRowOffsetsNoAlloc: a file-scope device array, so
// the call allocates nothing.  Calls that overlap on the device (concurrent
// streams) share it and race.
constexpr long long kStaticAlignScratchBytes = 128 * 1024;
static __device__ __align__(256) unsigned char g_align_scratch[kStaticAlignScratchBytes];

// Device address of g_align_scratch on the current device, looked up once per
// device.
static int static_align_scratch(void** out)
{
    static std::mutex mu;
    static void* addr[64] = {};
    int dev = 0;
    int rc = (int)cudaGetDevice(&dev);
    if (rc) return rc;
    if (dev < 0 || dev >= 64) return fail(1, "mcDeviceAlignRowOffsetsNoAlloc: device index out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        rc = (int)cudaGetSymbolAddress(&p, g_align_scratch);
        if (rc) return rc;
        addr[dev] = p;
    }
    *out = addr[dev];
    return 0;
}

}  // namespace mc

extern "C" int mcDeviceAlignRowOffsetsNoAlloc(int m_vec, const int* row_offsets, int alignment, int* aligned_pairs,
                                              int* aligned_nnz, cudaStream_t stream)
{
    mc::clear_error();
    if (int rc = mc::check_align_args(m_vec, row_offsets, alignment, aligned_pairs, aligned_nnz)) return rc;
    if (mc::align_scratch_bytes(m_vec) > mc::kStaticAlignScratchBytes)
        return mc::fail(1, "mcDeviceAlignRowOffsetsNoAlloc: m_vec exceeds the static scratch (at most 16,744,448 "
                           "vector-rows)");
    void* scratch = nullptr;
    if (int rc = mc::static_align_scratch(&scratch)) return rc;
    // device_align_launch clears the flag word that must start at zero; the
    // tile sums are written before they are read.
    return mc::device_align_launch(m_vec, row_offsets, alignment, aligned_pairs, aligned_nnz, scratch, nullptr,
                                   nullptr, stream);
}

extern "C" int mcDeviceAlignRowOffsets(int m_vec, const int* row_offsets, int alignment, int* aligned_pairs,
                                       int* aligned_nnz, cudaStream_t stream)
{
    mc::clear_error();
    if (int rc = mc::check_align_args(m_vec, row_offsets, alignment, aligned_pairs, aligned_nnz)) return rc;
    void* scratch = nullptr;
    int rc = (int)cudaMallocAsync(&scratch, (size_t)mc::align_scratch_bytes(m_vec), stream);
    if (rc) return rc;
    rc = mc::device_align_launch(m_vec, row_offsets, alignment, aligned_pairs, aligned_nnz, scratch, nullptr,
                                 nullptr, stream);
    const int rf = (int)cudaFreeAsync(scratch, stream);
    return rc ? rc : rf;
}

extern "C" int mcDevicePadColumnIndices(int m_vec, const int* row_offsets, const int* col_indices,
                                        const int* aligned_pairs, const int* aligned_nnz, int shuffle8,
                                        int* out_cols, long long capacity, int* status, cudaStream_t stream)
{
    mc::clear_error();
    if (m_vec < 0 || !row_offsets || !aligned_nnz || !out_cols || capacity < 0 || (m_vec > 0 && !aligned_pairs))
        return mc::fail(1, "mcDevicePadColumnIndices: invalid arguments");
    mc::FillArgs a{m_vec, row_offsets, aligned_pairs, aligned_nnz, col_indices, shuffle8 ? 1 : 0, out_cols,
                   capacity, nullptr, nullptr, 0, status, 0xFFFFFFFFu};
    return mc::fill(0, 0, 0, MC_VALUES_PACKED, a, stream);
}

extern "C" int mcDevicePackSpmmValues(int m_vec, int vec_length, int lhs_bits, int rhs_bits, const int* row_offsets,
                                      const int* aligned_pairs, const int* aligned_nnz, const void* values,
                                      void* out, long long capacity_bytes, int value_layout, int* status,
                                      cudaStream_t stream)
{
    mc::clear_error();
    if (m_vec < 0 || !(vec_length == 2 || vec_length == 4 || vec_length == 8) || !mc::valid_pair(lhs_bits, rhs_bits) ||
        !row_offsets || !aligned_nnz || !out || capacity_bytes < 0 ||
        (value_layout != MC_VALUES_PACKED && value_layout != MC_VALUES_SOFTMAX &&
         value_layout != MC_VALUES_SLOT_MAJOR) ||
        (m_vec > 0 && !aligned_pairs) || (lhs_bits == 12 && value_layout != MC_VALUES_PACKED))
        return mc::fail(1, "mcDevicePackSpmmValues: invalid arguments");
    if (value_layout == MC_VALUES_SLOT_MAJOR && (lhs_bits != 8 || rhs_bits != 8))
        return mc::fail(1, "mcDevicePackSpmmValues: the slot-major layout holds 8-bit values of the L8-R8 pair");
    if (reinterpret_cast<uintptr_t>(out) % (value_layout == MC_VALUES_SLOT_MAJOR ? 16 : 4))
        return mc::fail(1, "mcDevicePackSpmmValues: out must be 4-byte aligned (16 for slot-major values)");
    mc::FillArgs a{m_vec, row_offsets, aligned_pairs, aligned_nnz, nullptr, 0, nullptr, 0,
                   static_cast<const uint8_t*>(values), static_cast<uint8_t*>(out), capacity_bytes, status,
                   0xFFFFFFFFu};
    return mc::fill(vec_length, lhs_bits, rhs_bits, value_layout, a, stream);
}

extern "C" int mcDeviceSortedRowSwizzle(int m_vec, const int* row_offsets, int* row_indices, cudaStream_t stream)
{
    mc::clear_error();
    if (m_vec < 0 || !row_offsets || (m_vec > 0 && !row_indices))
        return mc::fail(1, "mcDeviceSortedRowSwizzle: invalid arguments");
    if (m_vec == 0) return 0;
    size_t temp = 0;
    int rc = mc::sort_temp_bytes(m_vec, 32, &temp);
    if (rc) return rc;
    const size_t arr = mc::round256((size_t)m_vec * sizeof(int));
    char* scratch = nullptr;
    rc = (int)cudaMallocAsync(reinterpret_cast<void**>(&scratch), 3 * arr + temp, stream);
    if (rc) return rc;
    int* len = reinterpret_cast<int*>(scratch);
    int* len_sorted = reinterpret_cast<int*>(scratch + arr);
    int* idx = reinterpret_cast<int*>(scratch + 2 * arr);
    mc::row_keys_kernel<<<mc::grid_for_warps((m_vec + 31) / 32), 256, 0, stream>>>(m_vec, row_offsets, len, idx);
    rc = (int)cudaGetLastError();
    if (!rc)
        rc = (int)cub::DeviceRadixSort::SortPairsDescending(scratch + 3 * arr, temp, len, len_sorted, idx,
                                                            row_indices, m_vec, 0, 32, stream);
    const int rf = (int)cudaFreeAsync(scratch, stream);
    return rc ? rc : rf;
}

extern "C" int mcDevicePack(const mcDevicePackDesc* d, cudaStream_t stream)
{
    mc::clear_error();
    if (!d) return mc::fail(1, "mcDevicePack: null descriptor");
    const bool values = d->lhs_bits != 0;
    if (d->m_vec < 0 || !d->row_offsets || !d->aligned_nnz || !d->out_cols || d->cols_capacity < 0 ||
        (d->m_vec > 0 && (!d->aligned_pairs || (d->sort_rows && !d->row_indices))))
        return mc::fail(1, "mcDevicePack: invalid arguments");
    if (d->m_vec > 0 && reinterpret_cast<uintptr_t>(d->aligned_pairs) % 8)
        return mc::fail(1, "mcDevicePack: aligned_pairs must be 8-byte aligned");
    int alignment = d->alignment;
    if (values) {
        if (!(d->vec_length == 2 || d->vec_length == 4 || d->vec_length == 8) ||
            !mc::valid_pair(d->lhs_bits, d->rhs_bits) ||
            (d->value_layout != MC_VALUES_PACKED && d->value_layout != MC_VALUES_SOFTMAX &&
             d->value_layout != MC_VALUES_SLOT_MAJOR) ||
            !d->out_values || d->values_capacity_bytes < 0 || reinterpret_cast<uintptr_t>(d->out_values) % 4)
            return mc::fail(1, "mcDevicePack: invalid value arguments (pair, vec_length, layout, 4-byte aligned out)");
        if (d->lhs_bits == 12 && d->value_layout != MC_VALUES_PACKED)
            return mc::fail(1, "mcDevicePack: 12-bit values use the packed layout");
        if (d->value_layout == MC_VALUES_SLOT_MAJOR &&
            (d->lhs_bits != 8 || d->rhs_bits != 8 || reinterpret_cast<uintptr_t>(d->out_values) % 16))
            return mc::fail(1, "mcDevicePack: slot-major values are L8-R8 with out_values 16-byte aligned");
        const int chunk = (d->value_layout == MC_VALUES_SOFTMAX) ? (d->lhs_bits == 4 ? 32 : 16)
                                                                   : ((d->lhs_bits == 4 || d->rhs_bits == 4) ? 32 : 16);
        if (alignment == 0) alignment = (d->lhs_bits == 4 || d->rhs_bits == 4) ? 32 : 16;
        if (alignment % chunk) return mc::fail(1, "mcDevicePack: alignment must be a multiple of the value chunk");
    }
    if (alignment <= 0 || (d->shuffle8 && alignment % 8))
        return mc::fail(1, "mcDevicePack: alignment must be positive (a multiple of 8 when shuffling)");

    const int m = d->m_vec;
    size_t temp = 0;
    const int end_bit = mc::key_bits(d->cols_capacity);
    if (d->sort_rows && m > 0)
        if (int rc = mc::sort_temp_bytes(m, end_bit, &temp)) return rc;
    const size_t a0 = mc::round256((size_t)mc::align_scratch_bytes(m));
    const size_t arr = d->sort_rows && m > 0 ? mc::round256((size_t)m * sizeof(int)) : 0;
    char* scratch = nullptr;
    int rc = (int)cudaMallocAsync(reinterpret_cast<void**>(&scratch), a0 + 3 * arr + temp, stream);
    if (rc) return rc;
    int* keys = arr ? reinterpret_cast<int*>(scratch + a0) : nullptr;
    int* keys_sorted = arr ? reinterpret_cast<int*>(scratch + a0 + arr) : nullptr;
    int* idx = arr ? reinterpret_cast<int*>(scratch + a0 + 2 * arr) : nullptr;
    rc = mc::device_align_launch(m, d->row_offsets, alignment, d->aligned_pairs, d->aligned_nnz, scratch, keys, idx,
                                 stream);
    if (!rc) {
        mc::FillArgs a{m, d->row_offsets, d->aligned_pairs, d->aligned_nnz, d->col_indices, d->shuffle8 ? 1 : 0,
                       d->out_cols, d->cols_capacity, static_cast<const uint8_t*>(d->values),
                       static_cast<uint8_t*>(d->out_values), d->values_capacity_bytes, d->status, 0xFFFFFFFFu};
        rc = mc::fill(d->vec_length, values ? d->lhs_bits : 0, d->rhs_bits, d->value_layout, a, stream);
    }
    if (!rc && arr)
        rc = (int)cub::DeviceRadixSort::SortPairsDescending(scratch + a0 + 3 * arr, temp, keys, keys_sorted, idx,
                                                            d->row_indices, m, 0, end_bit, stream);
    const int rf = (int)cudaFreeAsync(scratch, stream);
    return rc ? rc : rf;
}
