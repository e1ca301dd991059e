// Instantiations of the fused attention kernel for L16-R8 (every V, mode, warps, stages).
#include "mc_attn_fused.cuh"

namespace mc {
int attention_dispatch_16_8(const AttnParams& p, int V, bool rowmax, int warps, int stages, int ctas_per_sm,
                           cudaStream_t s)
{
    return attention_dispatch<16, 8>(p, V, rowmax, warps, stages, ctas_per_sm, s);
}
}  // namespace mc
