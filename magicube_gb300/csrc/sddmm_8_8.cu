// SDDMM kernels for lhs 8-bit x rhs 8-bit.
#include "mc_launch.cuh"
namespace mc {
int sddmm_launch_8_8(const mcSddmmDesc& d, cudaStream_t s) { return sddmm_launch<8, 8>(d, s); }
}  // namespace mc
