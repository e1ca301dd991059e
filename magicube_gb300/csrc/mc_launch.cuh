// mc_launch.cuh -- template dispatch from a C-ABI descriptor to a kernel
// instantiation.  Included by one translation unit per precision pair so the
// instantiations compile in parallel.
#pragma once
#include "mc_host.h"
#include "mc_sddmm.cuh"
#include "mc_sddmm_dp4a.cuh"
#include "mc_spmm_n64.cuh"
#include "mc_sddmm_stream.cuh"
#include "mc_spmm.cuh"
#include "mc_spmm_stream.cuh"
#include "mc_spmm_resident.cuh"
#include "mc_spmm_tma.cuh"
#include "mc_tma_host.h"

namespace mc {

// Persistent grid: resident CTAs of `kernel` over all SMs, capped by the work.
template <typename K>
inline int persistent_ctas(K kernel, int threads, long long work_ctas)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    long long n = (long long)per_sm * sm_count();
    if (n > work_ctas) n = work_ctas;
    if (n > 0x7fffffffLL) n = 0x7fffffffLL;
    return n < 1 ? 1 : (int)n;
}

template <int V, int PA, int PB, bool S, bool H, int W, bool F, bool E, int MTILES = 2>
int spmm_launch_stream(const mcSpmmDesc& d, const SpmmParams& p, cudaStream_t s)
{
    const long long ntasks = (long long)d.m_vec * d.batch;
    if (ntasks > 0x7fffffffLL) return fail(1, "mcSpmm: m_vec * batch too large");
    constexpr int MT = MTILES;
    const int ny = d.n / (W * 16 * MT);
    auto kern = spmm_stream_kernel<V, PA, PB, S, W, H, F, E, MT>;
    // resident CTAs over all SMs, split across the ny column tiles
    const long long resident = persistent_ctas(kern, W * 32, 0x7fffffffLL);
    long long gx = (resident + ny - 1) / ny;
    if (gx > ntasks) gx = ntasks;
    dim3 grid((unsigned)(gx < 1 ? 1 : gx), (unsigned)ny, 1);
    kern<<<grid, W * 32, 0, s>>>(p, (int)ntasks);
    return (int)cudaGetLastError();
}

// The TMA SpMM (mc_spmm_tma.cuh) applies on the int8 path to 8-bit B with
// n % 128 == 0 and 4-bit B with n % 256 == 0 (rows of whole 128-byte
// boxes), with 16-byte aligned values (and values_stride) and batch entries
// of B a whole number of rows apart.
inline bool spmm_tma_eligible(const mcSpmmDesc& d)
{
    const int kind = resolve_mma_kind(d.mma_kind);
    if (kind != MC_MMA_INT8 && kind != MC_MMA_DP4A) return false;
    if (!((d.rhs_bits == 8 && d.n % 128 == 0) || (d.rhs_bits == 4 && d.n % 256 == 0))) return false;
    if (reinterpret_cast<uintptr_t>(d.values) % 16 || d.values_stride % 16) return false;
    if (reinterpret_cast<uintptr_t>(d.rhs) % 16) return false;
    const long long row_bytes = (long long)d.n * d.rhs_bits / 8;
    if (d.batch > 1 && d.rhs_stride % row_bytes) return false;
    const long long per_entry = d.batch > 1 ? d.rhs_stride / row_bytes : 0;
    return per_entry * (d.batch - 1) + d.k <= 0x7fffffffLL;
}

template <int V, int PA, int PB, bool S, bool H, int NT, int STAGES = 4, int CW = 4, bool DP4A = false>
int spmm_launch_tma_cfg(const mcSpmmDesc& d, const SpmmParams& p, cudaStream_t s)
{
    using G = SpmmTmaGeom<V, PA, PB, NT, STAGES, CW>;
    const long long ntasks = (long long)d.m_vec * d.batch;
    if (ntasks > 0x7fffffffLL) return fail(1, "mcSpmm: m_vec * batch too large");
    const long long row_bytes = (long long)d.n * PB / 8;
    const long long per_entry = d.batch > 1 ? d.rhs_stride / row_bytes : 0;
    CUtensorMap map;
    if (!encode_row_gather_u8(&map, d.rhs, per_entry * (d.batch - 1) + d.k, row_bytes, 128))
        return fail(1, "mcSpmm: TMA tensor map encoding failed");
    unsigned int* timeouts = async_timeout_counter();
    if (!timeouts) return fail(1, "mcSpmm: timeout counter unavailable");
    auto kern = spmm_tma_kernel<V, PA, PB, S, H, H, NT, STAGES, CW, DP4A>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM) != cudaSuccess)
        return (int)cudaGetLastError();
    // resident CTAs per SM from registers, shared memory and warps
    int per_sm = 1;
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, kern) == cudaSuccess) {
        const int regs = (fa.numRegs + 7) & ~7;
        const int by_regs = regs > 0 ? 65536 / (regs * G::THREADS) : 1;
        const int by_smem = (int)((228u * 1024u) / (unsigned)(G::SMEM + fa.sharedSizeBytes + 1024));
        const int by_warps = 64 / (G::THREADS / 32);
        per_sm = by_regs < by_smem ? by_regs : by_smem;
        if (per_sm > by_warps) per_sm = by_warps;
        if (per_sm < 1) per_sm = 1;
    }
    const int ny = d.n / NT;
    long long gx = ((long long)per_sm * sm_count() + ny - 1) / ny;
    if (gx > ntasks) gx = ntasks;
    kern<<<dim3((unsigned)(gx < 1 ? 1 : gx), (unsigned)ny, 1), G::THREADS, G::SMEM, s>>>(map, p, (int)ntasks,
                                                                                        (int)per_entry, timeouts);
    return (int)cudaGetLastError();
}

// Ring depth and consumer warps per column tile, measured on GB300 (8-bit
// B): a 256-column tile runs 4 consumer warps (four 16-column MMA tiles
// each) over 4 stages; a 128-column tile 2 consumer warps (four tiles each)
// over 6 stages.  Deeper rings cost resident CTAs, which matter more.  4-bit
// B: 256-column tiles (128-byte rows, half the stage of 8-bit B) over 6
// stages.
template <int V, int PA, int PB, bool S, bool H, int NT, bool DP4A = false>
int spmm_launch_tma(const mcSpmmDesc& d, const SpmmParams& p, cudaStream_t s)
{
    if constexpr (PB == 4) return spmm_launch_tma_cfg<V, PA, 4, S, H, 256, 6, 4, DP4A>(d, p, s);
    else if constexpr (NT == 256) return spmm_launch_tma_cfg<V, PA, 8, S, H, 256, 4, 4, DP4A>(d, p, s);
    else return spmm_launch_tma_cfg<V, PA, 8, S, H, 128, 6, 2, DP4A>(d, p, s);
}

// The resident-slice SpMM (mc_spmm_resident.cuh) applies on the int8 path to
// 8-bit B with n % 64 == 0 and 4-bit B with n % 128 == 0 (64-byte slice
// rows), 4-, 8- or 16-bit A (dp4a: V <= 4 with 4- or 8-bit A), k <= 3584 (a
// slice of at most 14 boxes of 256 rows in shared memory), 16-byte aligned
// values (and values_stride), column indices and rhs, and batch entries of B
// a whole number of rows apart.
constexpr int kResidentMaxBoxes = 14;

inline bool spmm_resident_eligible(const mcSpmmDesc& d)
{
    const int kind = resolve_mma_kind(d.mma_kind);
    if (kind != MC_MMA_INT8 && kind != MC_MMA_DP4A) return false;
    if (!(d.lhs_bits == 4 || d.lhs_bits == 8 || d.lhs_bits == 16)) return false;
    if (reinterpret_cast<uintptr_t>(d.column_indices) % 16) return false;
    if (!((d.rhs_bits == 8 && d.n % 64 == 0) || (d.rhs_bits == 4 && d.n % 128 == 0))) return false;
    if (d.k < 1 || (d.k + 255) / 256 > kResidentMaxBoxes) return false;
    if (reinterpret_cast<uintptr_t>(d.values) % 16 || d.values_stride % 16) return false;
    if (reinterpret_cast<uintptr_t>(d.rhs) % 16) return false;
    const long long row_bytes = (long long)d.n * d.rhs_bits / 8;
    if (d.batch > 1 && d.rhs_stride % row_bytes) return false;
    const long long per_entry = d.batch > 1 ? d.rhs_stride / row_bytes : 0;
    return per_entry * (d.batch - 1) + d.k <= 0x7fffffffLL;
}

// Configurations built per precision pair: 64-byte slices x 8 warps always;
// 64-byte x 16 warps and 128-byte x 16 warps on the MMA path with V = 8,
// where a 16-warp CTA's accumulators and step ring fit in its 128 registers
// a thread (not 16-bit A x 4-bit B; 128-byte slices with 4- or 8-bit A).
template <int V, int PA, int PB, bool DP4A>
constexpr bool resident_config_built(int cfg)
{
    if (cfg == MC_RESIDENT_S64_W8) return true;
    if (DP4A || V != 8) return false;
    if (cfg == MC_RESIDENT_S64_W16) return !(PA == 16 && PB == 4);
    if (cfg == MC_RESIDENT_S128_W16) return PA <= 8;
    return false;
}

// The configuration of a launch: the requested one, or automatic (measured
// on GB300 at V = 8, k from 1024 to 3072): 128-byte slices with 16 warps
// where they are built and fit (k <= 1792, n a multiple of their width),
// else 64-byte slices with 16 warps, else with 8.
template <int V, int PA, int PB, bool DP4A>
inline int resident_config(const mcSpmmDesc& d)
{
    if (d.kernel_config != MC_RESIDENT_AUTO) return d.kernel_config;
    const int boxes = (d.k + 255) / 256;
    const int nt128 = 128 * 8 / PB;
    if (resident_config_built<V, PA, PB, DP4A>(MC_RESIDENT_S128_W16) && d.n % nt128 == 0 && boxes <= 7)
        return MC_RESIDENT_S128_W16;
    if (resident_config_built<V, PA, PB, DP4A>(MC_RESIDENT_S64_W16)) return MC_RESIDENT_S64_W16;
    return MC_RESIDENT_S64_W8;
}

// MC_KERNEL_AUTO takes the resident-slice kernel over the TMA one where it
// applies with V = 8, or with k <= 1024 (several CTAs an SM for V = 2 and 4);
// measured on GB300, the TMA kernel wins at V <= 4 with larger k.
inline bool spmm_resident_preferred(const mcSpmmDesc& d)
{
    return spmm_resident_eligible(d) && (d.vec_length == 8 || d.k <= 1024);
}

// One wave of resident CTAs, each at least 16 vector-rows of work, over the
// flat (slice, vector-row) list; every warp runs 4 steps ahead (2 with the
// dp4a consumers, whose rings carry every vector lane's words).
template <int V, int PA, int PB, bool S, bool H, int ROWB, int WARPS, bool DP4A>
int spmm_launch_resident_cfg(const mcSpmmDesc& d, const SpmmParams& p, cudaStream_t s)
{
    constexpr int PF = DP4A ? 2 : 4;
    using G = SpmmResidentGeom<PB, ROWB, WARPS>;
    if (d.n % G::NT) return fail(1, "mcSpmm: n is not a multiple of the slice width of this configuration");
    const int boxes = (d.k + G::BOX_ROWS - 1) / G::BOX_ROWS;
    if (G::smem(boxes) > 232448) return fail(1, "mcSpmm: k too large for the slices of this configuration");
    const int tiles = d.n / G::NT;
    const long long units = (long long)d.batch * tiles * d.m_vec;
    if ((long long)d.batch * tiles > 0x7fffffffLL) return fail(1, "mcSpmm: batch * column tiles too large");
    const long long row_bytes = (long long)d.n * PB / 8;
    const long long per_entry = d.batch > 1 ? d.rhs_stride / row_bytes : 0;
    CUtensorMap map;
    if (!encode_slice_u8(&map, d.rhs, per_entry * (d.batch - 1) + d.k, row_bytes, ROWB, G::BOX_ROWS))
        return fail(1, "mcSpmm: TMA tensor map encoding failed");
    unsigned int* timeouts = async_timeout_counter();
    if (!timeouts) return fail(1, "mcSpmm: timeout counter unavailable");
    auto kern = spmm_resident_kernel<V, PA, PB, S, H, H, ROWB, WARPS, PF, DP4A>;
    const size_t smem = G::smem(boxes);
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return (int)cudaGetLastError();
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, G::THREADS, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    long long grid = (long long)per_sm * sm_count();
    const long long by_work = (units + 15) / 16;
    if (grid > by_work) grid = by_work;
    if (grid < 1) grid = 1;
    kern<<<(unsigned)grid, G::THREADS, smem, s>>>(map, p, tiles, units, (int)per_entry, boxes, timeouts);
    return (int)cudaGetLastError();
}

template <int V, int PA, int PB, bool S, bool H, bool DP4A = false>
int spmm_launch_resident(const mcSpmmDesc& d, const SpmmParams& p, cudaStream_t s)
{
    const int cfg = resident_config<V, PA, PB, DP4A>(d);
    if (!resident_config_built<V, PA, PB, DP4A>(cfg))
        return fail(1, "mcSpmm: this resident-slice configuration is not built for the precision pair / path");
    if constexpr (resident_config_built<V, PA, PB, DP4A>(MC_RESIDENT_S64_W16)) {
        if (cfg == MC_RESIDENT_S64_W16) return spmm_launch_resident_cfg<V, PA, PB, S, H, 64, 16, DP4A>(d, p, s);
    }
    if constexpr (resident_config_built<V, PA, PB, DP4A>(MC_RESIDENT_S128_W16)) {
        if (cfg == MC_RESIDENT_S128_W16) return spmm_launch_resident_cfg<V, PA, PB, S, H, 128, 16, DP4A>(d, p, s);
    }
    return spmm_launch_resident_cfg<V, PA, PB, S, H, 64, 8, DP4A>(d, p, s);
}

// n == 64, 8-bit x 8-bit, softmax value layout, half output (the attention's
// P x V): persistent CTAs, k split over four warps (mc_spmm_n64.cuh).
template <int V, bool S>
int spmm_launch_n64(const mcSpmmDesc& d, const SpmmParams& p, cudaStream_t s)
{
    const long long items = (long long)d.m_vec * d.batch;
    if (items > 0x7fffffffLL) return fail(1, "mcSpmm: m_vec * batch too large");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, spmm_n64_kernel<V, S>, 128, 0) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    long long grid = (long long)per_sm * sm_count();
    if (grid > items) grid = items;
    spmm_n64_kernel<V, S><<<(unsigned)grid, 128, 0, s>>>(p, (int)items);
    return (int)cudaGetLastError();
}

// H (half output) is compiled only with the softmax value layout (E), the
// combination the extension's batched SpMM uses; int32 output only with the
// packer layout.
template <int V, int PA, int PB, bool S, bool H>
int spmm_launch_v(const mcSpmmDesc& d, const SpmmParams& p, cudaStream_t s)
{
    constexpr bool E = H;
    if constexpr (PB == 16) {
        // 16-bit B: the per-row kernel on the int8 path (the f16 path gives the
        // same integers; it is not built for four byte-plane products).
        if (d.kernel_variant == MC_KERNEL_STREAM || d.kernel_variant == MC_KERNEL_TMA ||
            d.kernel_variant == MC_KERNEL_RESIDENT)
            return fail(1, "mcSpmm: 16-bit B runs on the per-row kernel");
        if (d.n % 128 == 0) {
            dim3 grid((unsigned)d.m_vec, (unsigned)(d.n / 128), (unsigned)d.batch);
            spmm_kernel<V, PA, PB, S, 4, H, false, E><<<grid, 128, 0, s>>>(p);
        } else {
            dim3 grid((unsigned)d.m_vec, (unsigned)(d.n / 64), (unsigned)d.batch);
            spmm_kernel<V, PA, PB, S, 2, H, false, E><<<grid, 64, 0, s>>>(p);
        }
        return (int)cudaGetLastError();
    } else {
        const bool f16 = resolve_mma_kind(d.mma_kind) == MC_MMA_F16;
        if constexpr (PA == 8 && PB == 8 && H && E) {
            if (d.n == 64 && !f16 && (d.kernel_variant == MC_KERNEL_AUTO || d.kernel_variant == MC_KERNEL_STREAM) &&
                reinterpret_cast<uintptr_t>(d.values) % 16 == 0 && d.values_stride % 16 == 0)
                return spmm_launch_n64<V, S>(d, p, s);
        }
        if (resolve_mma_kind(d.mma_kind) == MC_MMA_DP4A) {
            // CUDA-core dp4a consumers in the TMA kernel: V = 2 and 4 compute
            // no padding lanes (an int8 MMA always computes 8)
            if constexpr (V <= 4 && PA <= 8) {
                if (d.kernel_variant == MC_KERNEL_RESIDENT ||
                    (d.kernel_variant == MC_KERNEL_AUTO && spmm_resident_preferred(d))) {
                    if (!spmm_resident_eligible(d))
                        return fail(1, "mcSpmm: the resident-slice kernel needs n % 64 == 0 (8-bit B) or "
                                       "n % 128 == 0 (4-bit B), k <= 3584, 16-byte aligned values, values_stride, "
                                       "column indices and rhs, and rhs_stride a multiple of the B row bytes");
                    return spmm_launch_resident<V, PA, PB, S, H, true>(d, p, s);
                }
                if (!spmm_tma_eligible(d))
                    return fail(1, "mcSpmm: the dp4a SpMM runs on the TMA kernel: n % 128 == 0 (8-bit B) or "
                                   "n % 256 == 0 (4-bit B), 16-byte aligned values, values_stride and rhs, and "
                                   "rhs_stride a multiple of the B row bytes");
                return d.n % 256 == 0 ? spmm_launch_tma<V, PA, PB, S, H, 256, true>(d, p, s)
                                      : spmm_launch_tma<V, PA, PB, S, H, 128, true>(d, p, s);
            } else {
                return fail(1, "mcSpmm: the dp4a SpMM computes V = 2 and 4 with 8-bit or 4-bit values");
            }
        }
        if (d.kernel_variant == MC_KERNEL_RESIDENT ||
            (d.kernel_variant == MC_KERNEL_AUTO && spmm_resident_preferred(d))) {
            if constexpr (PA == 4 || PA == 8 || PA == 16) {
                if (!spmm_resident_eligible(d))
                    return fail(1, "mcSpmm: the resident-slice kernel needs the int8 path, n % 64 == 0 (8-bit B) "
                                   "or n % 128 == 0 (4-bit B), k <= 3584, 16-byte aligned values, values_stride, "
                                   "column indices and rhs, and rhs_stride a multiple of the B row bytes");
                return spmm_launch_resident<V, PA, PB, S, H>(d, p, s);
            } else {
                return fail(1, "mcSpmm: the resident-slice kernel computes 4-, 8- and 16-bit A");
            }
        }
        const bool stream_ok = (reinterpret_cast<uintptr_t>(d.values) % 16 == 0) && (d.values_stride % 16 == 0);
        if (d.kernel_variant == MC_KERNEL_STREAM && !stream_ok)
            return fail(1, "mcSpmm: the streaming kernel needs 16-byte aligned values and values_stride");
        if (d.kernel_variant == MC_KERNEL_TMA && !spmm_tma_eligible(d))
            return fail(1, "mcSpmm: the TMA kernel needs the int8 path, n % 128 == 0 (8-bit B) or n % 256 == 0 "
                           "(4-bit B), 16-byte aligned values, values_stride and rhs, and rhs_stride a multiple of "
                           "the B row bytes");
        if ((d.kernel_variant == MC_KERNEL_TMA || d.kernel_variant == MC_KERNEL_AUTO) && spmm_tma_eligible(d))
            return d.n % 256 == 0 ? spmm_launch_tma<V, PA, PB, S, H, 256>(d, p, s)
                                  : spmm_launch_tma<V, PA, PB, S, H, 128>(d, p, s);
        if (d.kernel_variant != MC_KERNEL_PER_ROW && stream_ok) {
            if constexpr (PB == 8) {
                // 8-bit B, n % 256 == 0: four 16-column MMA tiles per warp
                if (d.n % 256 == 0)
                    return f16 ? spmm_launch_stream<V, PA, PB, S, H, 4, true, E, 4>(d, p, s)
                               : spmm_launch_stream<V, PA, PB, S, H, 4, false, E, 4>(d, p, s);
            }
            if (d.n % 128 == 0)
                return f16 ? spmm_launch_stream<V, PA, PB, S, H, 4, true, E>(d, p, s)
                           : spmm_launch_stream<V, PA, PB, S, H, 4, false, E>(d, p, s);
            return f16 ? spmm_launch_stream<V, PA, PB, S, H, 2, true, E>(d, p, s)
                       : spmm_launch_stream<V, PA, PB, S, H, 2, false, E>(d, p, s);
        }
        if (d.n % 128 == 0) {
            dim3 grid((unsigned)d.m_vec, (unsigned)(d.n / 128), (unsigned)d.batch);
            if (f16) spmm_kernel<V, PA, PB, S, 4, H, true, E><<<grid, 128, 0, s>>>(p);
            else spmm_kernel<V, PA, PB, S, 4, H, false, E><<<grid, 128, 0, s>>>(p);
        } else {
            dim3 grid((unsigned)d.m_vec, (unsigned)(d.n / 64), (unsigned)d.batch);
            if (f16) spmm_kernel<V, PA, PB, S, 2, H, true, E><<<grid, 64, 0, s>>>(p);
            else spmm_kernel<V, PA, PB, S, 2, H, false, E><<<grid, 64, 0, s>>>(p);
        }
        return (int)cudaGetLastError();
    }
}

template <int PA, int PB>
int spmm_launch(const mcSpmmDesc& d, cudaStream_t s)
{
    SpmmParams p;
    p.m_vec = d.m_vec; p.n = d.n; p.k = d.k;
    p.row_indices = d.row_indices; p.row_offsets = d.row_offsets; p.col_indices = d.column_indices;
    p.values = static_cast<const uint8_t*>(d.values); p.values_stride = d.values_stride;
    p.rhs = static_cast<const uint8_t*>(d.rhs); p.rhs_stride = d.rhs_stride;
    p.out = d.out; p.out_stride = d.out_stride;
    p.scale = d.scale;
    p.row_div = static_cast<const float*>(d.row_div);
    p.row_div_stride = d.row_div_stride;
#define MC_V(V)                                                                         \
    if (d.out_half) return spmm_launch_v<V, PA, PB, true, true>(d, p, s);               \
    if (d.is_signed) return spmm_launch_v<V, PA, PB, true, false>(d, p, s);             \
    return spmm_launch_v<V, PA, PB, false, false>(d, p, s);
    switch (d.vec_length) {
        case 2: { MC_V(2) }
        case 4: { MC_V(4) }
        default: { MC_V(8) }
    }
#undef MC_V
}

template <int V, int PA, int PB, bool S, bool VM, bool H, bool F>
int sddmm_launch_k64(const mcSddmmDesc& d, const SddmmParams& p, int split, cudaStream_t s)
{
    dim3 grid((unsigned)d.m_vec, (unsigned)split, (unsigned)d.batch);
    sddmm_k64_kernel<V, PA, PB, S, VM, H, 4, F><<<grid, 128, 0, s>>>(p);
    return (int)cudaGetLastError();
}

template <int V, int PA, int PB, bool S, bool VM, bool H>
int sddmm_launch_dp4a(const mcSddmmDesc& d, const SddmmParams& p, int split, cudaStream_t s)
{
    if constexpr (PA == 16 || PB == 16) {
        return fail(1, "mcSddmm: the dp4a path computes 8-bit and 4-bit operands");
    } else {
        dim3 grid((unsigned)d.m_vec, (unsigned)split, (unsigned)d.batch);
        if (d.k == 64) sddmm_dp4a_kernel<V, PA, PB, S, VM, H, 4, true><<<grid, 128, 0, s>>>(p);
        else sddmm_dp4a_kernel<V, PA, PB, S, VM, H, 4, false><<<grid, 128, 0, s>>>(p);
        return (int)cudaGetLastError();
    }
}

// The tcgen05 SDDMM (sddmm_tc.cu).
int sddmm_tc_launch(const mcSddmmDesc& d, const SddmmParams& p, cudaStream_t s);

template <int V, int PA, int PB, bool S, bool VM, bool H>
int sddmm_launch_v(const mcSddmmDesc& d, const SddmmParams& p, int split, cudaStream_t s)
{
    if (resolve_mma_kind(d.mma_kind) == MC_MMA_TCGEN05) return sddmm_tc_launch(d, p, s);
    if (resolve_mma_kind(d.mma_kind) == MC_MMA_DP4A) return sddmm_launch_dp4a<V, PA, PB, S, VM, H>(d, p, split, s);
    // MC_MMA_DEFAULT takes the f16 path for L16-R8 on the k == 64 kernel: its
    // two byte planes double the int8 MMAs, and the f16 rate absorbs them
    // (measured 83 vs 70 TOP/s on GB300; the integers are the same)
    const bool l16_f16 = d.mma_kind == MC_MMA_DEFAULT && PA == 16 && PB == 8 && d.k == 64 &&
                         d.kernel_variant != MC_KERNEL_PER_ROW;
    const bool f16 = l16_f16 || resolve_mma_kind(d.mma_kind) == MC_MMA_F16;
    if (d.kernel_variant == MC_KERNEL_STREAM && d.k != 64)
        return fail(1, "mcSddmm: the streaming kernel needs k == 64");
    if (d.kernel_variant != MC_KERNEL_PER_ROW && d.k == 64)
        return f16 ? sddmm_launch_k64<V, PA, PB, S, VM, H, true>(d, p, split, s)
                   : sddmm_launch_k64<V, PA, PB, S, VM, H, false>(d, p, split, s);
    dim3 grid((unsigned)d.m_vec, (unsigned)split, (unsigned)d.batch);
    if (f16)
        sddmm_kernel<V, PA, PB, S, VM, H, 4, true><<<grid, 128, 0, s>>>(p);
    else
        sddmm_kernel<V, PA, PB, S, VM, H, 4, false><<<grid, 128, 0, s>>>(p);
    return (int)cudaGetLastError();
}

inline int sddmm_auto_split(const mcSddmmDesc& d)
{
    if (d.row_split > 0) return d.row_split;
    const long long ctas = (long long)d.m_vec * d.batch;
    const long long target = 152LL * 16;  // SMs x resident CTAs of 128 threads
    if (ctas >= target) return 1;
    long long split = (target + ctas - 1) / ctas;
    const long long max_split = (d.n + 63) / 64;  // at most one warp-tile of 16 per warp
    if (split > max_split) split = max_split;
    return split < 1 ? 1 : (int)split;
}

template <int PA, int PB>
int sddmm_launch(const mcSddmmDesc& d, cudaStream_t s)
{
    SddmmParams p;
    p.m_vec = d.m_vec; p.n = d.n; p.k = d.k;
    p.row_indices = d.row_indices; p.row_offsets = d.row_offsets; p.col_indices = d.column_indices;
    p.lhs = static_cast<const uint8_t*>(d.lhs); p.lhs_stride = d.lhs_stride;
    p.rhs = static_cast<const uint8_t*>(d.rhs); p.rhs_stride = d.rhs_stride;
    p.out = d.out; p.out_stride = d.out_stride;
    p.scale = d.scale;
    const int split = sddmm_auto_split(d);
#define MC_V(V)                                                                              \
    if (d.out_half) return sddmm_launch_v<V, PA, PB, true, true, true>(d, p, split, s);      \
    if (d.out_vecmajor) {                                                                    \
        if (d.is_signed) return sddmm_launch_v<V, PA, PB, true, true, false>(d, p, split, s);  \
        return sddmm_launch_v<V, PA, PB, false, true, false>(d, p, split, s);                \
    }                                                                                        \
    if (d.is_signed) return sddmm_launch_v<V, PA, PB, true, false, false>(d, p, split, s);   \
    return sddmm_launch_v<V, PA, PB, false, false, false>(d, p, split, s);
    switch (d.vec_length) {
        case 2: { MC_V(2) }
        case 4: { MC_V(4) }
        default: { MC_V(8) }
    }
#undef MC_V
}

}  // namespace mc
