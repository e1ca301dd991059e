// mc_launch.cuh -- template dispatch from a C-ABI descriptor to a kernel
// instantiation.  Included by one translation unit per precision pair so the
// instantiations compile in parallel.
#pragma once
#include "mc_host.h"
#include "mc_sddmm.cuh"
#include "mc_spmm.cuh"

namespace mc {

template <int V, int PA, int PB, bool S, bool H>
int spmm_launch_v(const mcSpmmDesc& d, const SpmmParams& p, cudaStream_t s)
{
    if (d.n % 128 == 0) {
        dim3 grid((unsigned)d.m_vec, (unsigned)(d.n / 128), (unsigned)d.batch);
        spmm_kernel<V, PA, PB, S, 4, H><<<grid, 128, 0, s>>>(p);
    } else {
        dim3 grid((unsigned)d.m_vec, (unsigned)(d.n / 64), (unsigned)d.batch);
        spmm_kernel<V, PA, PB, S, 2, H><<<grid, 64, 0, s>>>(p);
    }
    return (int)cudaGetLastError();
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

template <int V, int PA, int PB, bool S, bool VM, bool H>
int sddmm_launch_v(const mcSddmmDesc& d, const SddmmParams& p, int split, cudaStream_t s)
{
    dim3 grid((unsigned)d.m_vec, (unsigned)split, (unsigned)d.batch);
    sddmm_kernel<V, PA, PB, S, VM, H, 4><<<grid, 128, 0, s>>>(p);
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
