/*
 * magicube_gb300_wmma.h -- the reference's C++ kernel API as provided by
 * libmagicube_gb300.so (C++ linkage, namespaces spmm and sddmm).
 *
 * The declarations are the reference's own (SpMM/SpMM/include/wmma_spmm.cuh:15-78,
 * SDDMM/SDDMM/include/wmma_sddmm.cuh), so a program that includes the
 * reference's headers links against this library unchanged.  Semantics:
 * unsigned lanes, legacy default stream, the reference's device layouts (see
 * magicube_gb300.h), every precision variant included.
 */
#ifndef MAGICUBE_GB300_WMMA_H
#define MAGICUBE_GB300_WMMA_H

#include <cuda_runtime_api.h>

#include "magicube_gb300.h"

namespace spmm {
cudaError_t wmmaSpmm_4b(int m_vec, int vec_length, int n, int k, const int* __restrict__ row_indices,
                        const int* __restrict__ row_offsets, const int* __restrict__ column_indices,
                        const int* __restrict__ values, const int* __restrict__ rhs_matrix,
                        int* __restrict__ output_matrix);   /* wmma_spmm.cuh:14 */
cudaError_t wmmaSpmm_8b4b(int m_vec, int vec_length, int n, int k, const int* __restrict__ row_indices,
                          const int* __restrict__ row_offsets, const int* __restrict__ column_indices,
                          const int* __restrict__ values, const int* __restrict__ rhs_matrix,
                          int* __restrict__ output_matrix); /* wmma_spmm.cuh:22 */
cudaError_t wmmaSpmm_12b4b(int m_vec, int vec_length, int n, int k, const int* __restrict__ row_indices,
                           const int* __restrict__ row_offsets, const int* __restrict__ column_indices,
                           const int* __restrict__ values, const int* __restrict__ rhs_matrix,
                           int* __restrict__ output_matrix); /* wmma_spmm.cuh:30 */
cudaError_t wmmaSpmm_16b4b(int m_vec, int vec_length, int n, int k, const int* __restrict__ row_indices,
                           const int* __restrict__ row_offsets, const int* __restrict__ column_indices,
                           const int* __restrict__ values, const int* __restrict__ rhs_matrix,
                           int* __restrict__ output_matrix); /* wmma_spmm.cuh:38 */
cudaError_t wmmaSpmm_8b(int m_vec, int vec_length, int n, int k, const int* __restrict__ row_indices,
                        const int* __restrict__ row_offsets, const int* __restrict__ column_indices,
                        const int* __restrict__ values, const int* __restrict__ rhs_matrix,
                        int* __restrict__ output_matrix);    /* wmma_spmm.cuh:46 */
cudaError_t wmmaSpmm_12b8b(int m_vec, int vec_length, int n, int k, const int* __restrict__ row_indices,
                           const int* __restrict__ row_offsets, const int* __restrict__ column_indices,
                           const int* __restrict__ values, const int* __restrict__ rhs_matrix,
                           int* __restrict__ output_matrix); /* wmma_spmm.cuh:54 */
cudaError_t wmmaSpmm_16b8b(int m_vec, int vec_length, int n, int k, const int* __restrict__ row_indices,
                           const int* __restrict__ row_offsets, const int* __restrict__ column_indices,
                           const int* __restrict__ values, const int* __restrict__ rhs_matrix,
                           int* __restrict__ output_matrix); /* wmma_spmm.cuh:62 */
cudaError_t wmmaSpmm_16b(int m_vec, int vec_length, int n, int k, const int* __restrict__ row_indices,
                         const int* __restrict__ row_offsets, const int* __restrict__ column_indices,
                         const int* __restrict__ values, const int* __restrict__ rhs_matrix,
                         int* __restrict__ output_matrix);   /* wmma_spmm.cuh:70 */
}  // namespace spmm

namespace sddmm {
cudaError_t wmmaSddmm_4b(int m_vec, int k, int n, const int* __restrict__ row_indices,
                         const int* __restrict__ row_offsets, const int* __restrict__ column_indices,
                         const int* __restrict__ lhs_matrix, const int* __restrict__ rhs_matrix,
                         int* __restrict__ output_values, int vec_length);  /* wmma_sddmm.cu:394 */
cudaError_t wmmaSddmm_8b(int m_vec, int k, int n, const int* __restrict__ row_indices,
                         const int* __restrict__ row_offsets, const int* __restrict__ column_indices,
                         const int* __restrict__ lhs_matrix, const int* __restrict__ rhs_matrix,
                         int* __restrict__ output_values, int vec_length);  /* wmma_sddmm.cu:439 */
cudaError_t wmmaSddmm_16b(int m_vec, int k, int n, const int* __restrict__ row_indices,
                          const int* __restrict__ row_offsets, const int* __restrict__ column_indices,
                          const int* __restrict__ lhs_matrix, const int* __restrict__ rhs_matrix,
                          int* __restrict__ output_values, int vec_length); /* wmma_sddmm.cu:488 */
}  // namespace sddmm

#endif /* MAGICUBE_GB300_WMMA_H */
