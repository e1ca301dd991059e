// Instantiations of the fused attention kernel for L8-R4 (every V, mode, warps, stages).
#include "mc_attn_fused.cuh"

namespace mc {
int attention_dispatch_8_4(const AttnParams& p, int V, bool rowmax, int warps, int stages, int ctas_per_sm,
                           cudaStream_t s)
{
    return attention_dispatch<8, 4>(p, V, rowmax, warps, stages, ctas_per_sm, s);
}
}  // namespace mc
