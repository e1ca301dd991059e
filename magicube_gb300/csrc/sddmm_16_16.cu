// SDDMM kernels for lhs 16-bit x rhs 16-bit.
#include "mc_launch.cuh"
namespace mc {
int sddmm_launch_16_16(const mcSddmmDesc& d, cudaStream_t s) { return sddmm_launch<16, 16>(d, s); }
}  // namespace mc
