// SpMM kernels for lhs 16-bit x rhs 8-bit.
#include "mc_launch.cuh"
namespace mc {
int spmm_launch_16_8(const mcSpmmDesc& d, cudaStream_t s) { return spmm_launch<16, 8>(d, s); }
}  // namespace mc
