// sddmm_dense.cu -- host side of the dense-tile tcgen05 SDDMM
// (mc_sddmm_dense.cuh): the mask's tile bitmap and the launch.
#include "mc_host.h"
#include "mc_sddmm_dense.cuh"
#include "mc_tma_host.h"

namespace mc {

template <int V, bool S, bool VM, bool H>
static int dense_launch_t(const SddmmDenseParams& dp, cudaStream_t s)
{
    auto kern = sddmm_dense_tc_kernel<V, S, VM, H>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, dense::SMEM) != cudaSuccess)
        return fail((int)cudaGetLastError(), "mcSddmm: cannot reserve shared memory for the dense-tile kernel");
    unsigned int* timeouts = async_timeout_counter();
    if (!timeouts) return fail(1, "mcSddmm: no timeout counter on this device");
    const int grid = dp.items < sm_count() ? dp.items : sm_count();
    kern<<<grid, dense::THREADS, dense::SMEM, s>>>(dp, timeouts);
    return (int)cudaGetLastError();
}

template <int V>
static int dense_launch_v(const mcSddmmDesc& d, const SddmmDenseParams& dp, cudaStream_t s)
{
    if (d.out_half) return dense_launch_t<V, true, true, true>(dp, s);
    if (d.out_vecmajor)
        return d.is_signed ? dense_launch_t<V, true, true, false>(dp, s) : dense_launch_t<V, false, true, false>(dp, s);
    return d.is_signed ? dense_launch_t<V, true, false, false>(dp, s) : dense_launch_t<V, false, false, false>(dp, s);
}

int sddmm_dense_launch(const mcSddmmDesc& d, cudaStream_t s)
{
    SddmmDenseParams dp;
    SddmmParams& p = dp.s;
    p.m_vec = d.m_vec; p.n = d.n; p.k = d.k;
    p.row_indices = d.row_indices; p.row_offsets = d.row_offsets; p.col_indices = d.column_indices;
    p.lhs = static_cast<const uint8_t*>(d.lhs); p.lhs_stride = d.lhs_stride;
    p.rhs = static_cast<const uint8_t*>(d.rhs); p.rhs_stride = d.rhs_stride;
    p.out = d.out; p.out_stride = d.out_stride;
    p.scale = d.scale;
    dp.bitmap = d.tile_bitmap;
    dp.prefix = d.tile_prefix;
    dp.words = mcSddmmTileMaskWords(d.n);
    dp.a_blocks = (int)(((long long)d.m_vec * d.vec_length + dense::AR - 1) / dense::AR);
    dp.c_blocks = (d.n + dense::BR - 1) / dense::BR;
    const long long items = (long long)d.batch * dp.a_blocks;
    if (items > 0x7fffffffLL) return fail(1, "mcSddmm: too many dense tiles");
    dp.items = (int)items;
    switch (d.vec_length) {
        case 2: return dense_launch_v<2>(d, dp, s);
        case 4: return dense_launch_v<4>(d, dp, s);
        default: return dense_launch_v<8>(d, dp, s);
    }
}

}  // namespace mc

extern "C" int mcSddmmTileMaskWords(int n) { return n <= 0 ? 0 : ((n + 127) / 128) * 4; }

extern "C" int mcSddmmTileMask(int m_vec, int n, const int* row_offsets, const int* column_indices, unsigned* bitmap,
                               int* prefix, int* status, cudaStream_t stream)
{
    mc::clear_error();
    if (m_vec < 0 || n <= 0) return mc::fail(1, "mcSddmmTileMask: m_vec must be >= 0 and n > 0");
    if (!status) return mc::fail(1, "mcSddmmTileMask: null status");
    if (cudaMemsetAsync(status, 0, sizeof(int), stream) != cudaSuccess) return (int)cudaGetLastError();
    if (m_vec == 0) return 0;
    if (!row_offsets || !column_indices || !bitmap || !prefix) return mc::fail(1, "mcSddmmTileMask: null pointer");
    const int words = mcSddmmTileMaskWords(n);
    mc::sddmm_tile_mask_kernel<<<(unsigned)((m_vec + 3) / 4), 128, 0, stream>>>(
        m_vec, n, words, row_offsets, column_indices, reinterpret_cast<uint32_t*>(bitmap), prefix, status);
    return (int)cudaGetLastError();
}
