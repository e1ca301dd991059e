// SpMM kernels for lhs 8-bit x rhs 4-bit.
#include "mc_launch.cuh"
namespace mc {
int spmm_launch_8_4(const mcSpmmDesc& d, cudaStream_t s) { return spmm_launch<8, 4>(d, s); }
}  // namespace mc
