// SpMM kernels for lhs 8-bit x rhs 8-bit.
#include "mc_launch.cuh"
namespace mc {
int spmm_launch_8_8(const mcSpmmDesc& d, cudaStream_t s) { return spmm_launch<8, 8>(d, s); }
}  // namespace mc
