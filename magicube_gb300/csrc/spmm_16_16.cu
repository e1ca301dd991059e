// SpMM kernels for lhs 16-bit x rhs 16-bit (the reference's wmmaSpmm_16b).
#include "mc_launch.cuh"
namespace mc {
int spmm_launch_16_16(const mcSpmmDesc& d, cudaStream_t s) { return spmm_launch<16, 16>(d, s); }
}  // namespace mc
