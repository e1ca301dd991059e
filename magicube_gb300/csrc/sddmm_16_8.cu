// SDDMM kernels for lhs 16-bit x rhs 8-bit.
#include "mc_launch.cuh"
namespace mc {
int sddmm_launch_16_8(const mcSddmmDesc& d, cudaStream_t s) { return sddmm_launch<16, 8>(d, s); }
}  // namespace mc
