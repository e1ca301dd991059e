// SpMM kernels for lhs 4-bit x rhs 4-bit.
#include "mc_launch.cuh"
namespace mc {
int spmm_launch_4_4(const mcSpmmDesc& d, cudaStream_t s) { return spmm_launch<4, 4>(d, s); }
}  // namespace mc
