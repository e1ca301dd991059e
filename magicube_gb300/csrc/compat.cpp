// compat.cpp -- the reference's C++ kernel API, implemented by this library.
//
// Defines spmm::wmmaSpmm_* (SpMM/SpMM/include/wmma_spmm.cuh:15-78) and
// sddmm::wmmaSddmm_* (SDDMM/SDDMM/src/wmma_sddmm.cu:394,439,488) with the
// reference's exact signatures, so code written against the reference (its
// benchmark programs included) links against libmagicube_gb300.so in place
// of the reference's wmma_spmm.cu / wmma_sddmm.cu, unchanged.  Each function
// forwards to the matching C entry point (unsigned lanes, legacy default
// stream, the reference's device layouts), the 12-bit and 16-bit x 16-bit
// SpMM variants included.
#include <cuda_runtime_api.h>

#include "../../include/magicube_gb300_wmma.h"
#include "mc_host.h"

namespace spmm {

#define MC_SPMM_FWD(NAME, CFN)                                                                          \
    cudaError_t NAME(int m_vec, int vec_length, int n, int k, const int* __restrict__ row_indices,       \
                     const int* __restrict__ row_offsets, const int* __restrict__ column_indices,          \
                     const int* __restrict__ values, const int* __restrict__ rhs_matrix,                  \
                     int* __restrict__ output_matrix)                                                     \
    {                                                                                                    \
        return (cudaError_t)CFN(m_vec, vec_length, n, k, row_indices, row_offsets, column_indices, values, \
                                rhs_matrix, output_matrix);                                              \
    }
MC_SPMM_FWD(wmmaSpmm_4b, mcWmmaSpmm_4b)
MC_SPMM_FWD(wmmaSpmm_8b4b, mcWmmaSpmm_8b4b)
MC_SPMM_FWD(wmmaSpmm_16b4b, mcWmmaSpmm_16b4b)
MC_SPMM_FWD(wmmaSpmm_8b, mcWmmaSpmm_8b)
MC_SPMM_FWD(wmmaSpmm_16b8b, mcWmmaSpmm_16b8b)
MC_SPMM_FWD(wmmaSpmm_12b4b, mcWmmaSpmm_12b4b)
MC_SPMM_FWD(wmmaSpmm_12b8b, mcWmmaSpmm_12b8b)
MC_SPMM_FWD(wmmaSpmm_16b, mcWmmaSpmm_16b)
#undef MC_SPMM_FWD

}  // namespace spmm

namespace sddmm {

#define MC_SDDMM_FWD(NAME, CFN)                                                                      \
    cudaError_t NAME(int m_vec, int k, int n, const int* __restrict__ row_indices,                    \
                     const int* __restrict__ row_offsets, const int* __restrict__ column_indices,       \
                     const int* __restrict__ lhs_matrix, const int* __restrict__ rhs_matrix,            \
                     int* __restrict__ output_values, int vec_length)                                   \
    {                                                                                                 \
        return (cudaError_t)CFN(m_vec, k, n, row_indices, row_offsets, column_indices, lhs_matrix, rhs_matrix, \
                                output_values, vec_length);                                           \
    }
MC_SDDMM_FWD(wmmaSddmm_4b, mcWmmaSddmm_4b)
MC_SDDMM_FWD(wmmaSddmm_8b, mcWmmaSddmm_8b)
MC_SDDMM_FWD(wmmaSddmm_16b, mcWmmaSddmm_16b)
#undef MC_SDDMM_FWD

}  // namespace sddmm
