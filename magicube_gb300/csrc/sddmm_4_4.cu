// SDDMM kernels for lhs 4-bit x rhs 4-bit.
#include "mc_launch.cuh"
namespace mc {
int sddmm_launch_4_4(const mcSddmmDesc& d, cudaStream_t s) { return sddmm_launch<4, 4>(d, s); }
}  // namespace mc
