// spmm_dense.cu -- host side of the dense-tile tcgen05 SpMM
// (mc_spmm_dense.cuh): the chunk-starts table and the launch.
#include "mc_host.h"
#include "mc_spmm_dense.cuh"
#include "mc_tma_host.h"

namespace mc {

template <int V, bool S, bool SM>
static int spmm_dense_launch_t(const CUtensorMap& map, const SpmmDenseParams& dp, cudaStream_t s)
{
    auto kern = spmm_dense_tc_kernel<V, S, SM>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, sdense::SMEM) != cudaSuccess)
        return fail((int)cudaGetLastError(), "mcSpmm: cannot reserve shared memory for the dense-tile kernel");
    unsigned int* timeouts = async_timeout_counter();
    if (!timeouts) return fail(1, "mcSpmm: no timeout counter on this device");
    const int grid = dp.items < sm_count() ? dp.items : sm_count();
    kern<<<grid, sdense::THREADS, sdense::SMEM, s>>>(map, dp, timeouts);
    return (int)cudaGetLastError();
}

int spmm_dense_launch(const mcSpmmDesc& d, cudaStream_t s)
{
    SpmmDenseParams dp;
    SpmmParams& p = dp.s;
    p.m_vec = d.m_vec; p.n = d.n; p.k = d.k;
    p.row_indices = d.row_indices; p.row_offsets = d.row_offsets; p.col_indices = d.column_indices;
    p.values = static_cast<const uint8_t*>(d.values); p.values_stride = d.values_stride;
    p.rhs = static_cast<const uint8_t*>(d.rhs); p.rhs_stride = d.rhs_stride;
    p.out = d.out; p.out_stride = d.out_stride;
    p.scale = d.scale;
    p.row_div = nullptr; p.row_div_stride = 0;
    dp.chunk_starts = d.chunk_starts;
    dp.kchunks = (d.k + sdense::KC - 1) / sdense::KC;
    // products of signed 8-bit lanes are at most 2^14, of unsigned ones below
    // 2^16: 1024 or 256 of them keep every partial sum within 2^24
    dp.seg = d.is_signed ? 1024 / sdense::KC : 256 / sdense::KC;
    dp.row_blocks = (int)(((long long)d.m_vec * d.vec_length + sdense::AR - 1) / sdense::AR);
    dp.col_blocks = d.n / sdense::BN;
    const long long items = (long long)d.batch * dp.row_blocks * dp.col_blocks;
    if (items > 0x7fffffffLL) return fail(1, "mcSpmm: too many dense tiles");
    dp.items = (int)items;
    const long long row_bytes = d.n;
    dp.rows_per_entry = d.batch > 1 ? (int)(d.rhs_stride / row_bytes) : 0;
    CUtensorMap map;
    if (!encode_box_u8(&map, d.rhs, (long long)dp.rows_per_entry * (d.batch - 1) + d.k, row_bytes, sdense::BN,
                       sdense::KC))
        return fail(1, "mcSpmm: TMA tensor map encoding failed");
    const bool sm = d.value_layout == MC_VALUES_SLOT_MAJOR;
#define MC_DENSE_V(VV)                                                                              \
    if (sm) return d.is_signed ? spmm_dense_launch_t<VV, true, true>(map, dp, s)                     \
                               : spmm_dense_launch_t<VV, false, true>(map, dp, s);                   \
    return d.is_signed ? spmm_dense_launch_t<VV, true, false>(map, dp, s) : spmm_dense_launch_t<VV, false, false>(map, dp, s);
    switch (d.vec_length) {
        case 2: { MC_DENSE_V(2) }
        case 4: { MC_DENSE_V(4) }
        default: { MC_DENSE_V(8) }
    }
#undef MC_DENSE_V
}

}  // namespace mc

extern "C" int mcSpmmChunkStartsCount(int k) { return k <= 0 ? 0 : (k + mc::sdense::KC - 1) / mc::sdense::KC + 1; }

extern "C" int mcSpmmChunkStarts(int m_vec, int k, const int* row_offsets, const int* column_indices, int* starts,
                                 int* status, cudaStream_t stream)
{
    mc::clear_error();
    if (m_vec < 0 || k <= 0) return mc::fail(1, "mcSpmmChunkStarts: m_vec must be >= 0 and k > 0");
    if (!status) return mc::fail(1, "mcSpmmChunkStarts: null status");
    if (cudaMemsetAsync(status, 0, sizeof(int), stream) != cudaSuccess) return (int)cudaGetLastError();
    if (m_vec == 0) return 0;
    if (!row_offsets || !column_indices || !starts) return mc::fail(1, "mcSpmmChunkStarts: null pointer");
    const int kchunks = mcSpmmChunkStartsCount(k) - 1;
    mc::spmm_chunk_starts_kernel<<<(unsigned)((m_vec + 3) / 4), 128, 0, stream>>>(m_vec, k, kchunks, row_offsets,
                                                                                  column_indices, starts, status);
    return (int)cudaGetLastError();
}
