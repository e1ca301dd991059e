// SDDMM 8-bit x 8-bit, k = 64, on tcgen05 (mc_sddmm_tc.cuh): launcher and the
// reader of the kernels' timeout counter.
#include "mc_launch.cuh"
#include "mc_sddmm_tc.cuh"

namespace mc {

template <int V, bool S, bool VM, bool H>
static int tc_launch(const SddmmParams& p, int items, cudaStream_t s)
{
    auto kern = sddmm_tc_kernel<V, S, VM, H>;
    const size_t smem = sddmm_tc_smem_bytes();
    // Resident CTAs per SM from the kernel's registers and shared memory (the
    // runtime's occupancy query answers 1 for this tcgen05 kernel), at most 16
    // (32 TMEM columns per CTA, 512 per SM).
    cudaFuncAttributes fa{};
    int per_sm = 1;
    if (cudaFuncGetAttributes(&fa, kern) == cudaSuccess) {
        const int regs = (fa.numRegs + 7) & ~7;
        const int by_regs = regs > 0 ? 65536 / (regs * 128) : 16;
        const int by_smem = (int)((228u * 1024u) / (unsigned)(smem + fa.sharedSizeBytes + 1024));
        per_sm = by_regs < by_smem ? by_regs : by_smem;
        if (per_sm > 16) per_sm = 16;
        if (per_sm < 1) per_sm = 1;
    }
    long long grid = (long long)per_sm * sm_count();
    if (grid > items) grid = items;
    kern<<<(unsigned)(grid < 1 ? 1 : grid), 128, smem, s>>>(p, items);
    return (int)cudaGetLastError();
}

int sddmm_tc_launch(const mcSddmmDesc& d, const SddmmParams& p, cudaStream_t s)
{
    if (d.k != 64 || d.lhs_bits != 8 || d.rhs_bits != 8)
        return fail(1, "mcSddmm: the tcgen05 path computes L8-R8 with k == 64");
    const long long items = (long long)d.m_vec * d.batch;
    if (items > 0x7fffffffLL) return fail(1, "mcSddmm: m_vec * batch too large");
#define MC_TC(V)                                                                                     \
    if (d.out_half) return tc_launch<V, true, true, true>(p, (int)items, s);                        \
    if (d.out_vecmajor)                                                                              \
        return d.is_signed ? tc_launch<V, true, true, false>(p, (int)items, s)                       \
                           : tc_launch<V, false, true, false>(p, (int)items, s);                     \
    return d.is_signed ? tc_launch<V, true, false, false>(p, (int)items, s)                          \
                       : tc_launch<V, false, false, false>(p, (int)items, s);
    switch (d.vec_length) {
        case 2: { MC_TC(2) }
        case 4: { MC_TC(4) }
        default: { MC_TC(8) }
    }
#undef MC_TC
}

}  // namespace mc

extern "C" unsigned mcTensorCoreTimeouts(void)
{
    unsigned v = 0;
    if (cudaMemcpyFromSymbol(&v, mc::g_tc_timeouts, sizeof v) != cudaSuccess) return 0xFFFFFFFFu;
    const unsigned w = mc::async_timeouts();
    return w == 0xFFFFFFFFu ? w : v + w;
}
