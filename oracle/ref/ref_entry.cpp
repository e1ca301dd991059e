// ref_entry.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Compiles one of the reference's host benchmark programs from its source file
// (path given by MCREF_SRC, under the reference checkout) with `main` renamed
// (it is never called here), and exposes its host verification routine through C wrappers:
//   MCREF_SPMM:  compute_ref_integers<TypeA>   (SpMM/SpMM/spmm_benchmark.cpp:69-120)
//   MCREF_SDDMM: Host_sddmm_integers           (SDDMM/SDDMM/sddmm_benchmark.cpp:24-60)
#define main mcref_benchmark_main
#include MCREF_SRC
#undef main

#ifdef MCREF_SPMM
extern "C" double mcref_compute_ref_integers(int type_bytes, void* A, int* B, int* C, int M, int K, int N, int preA,
                                             int preA_cut, int preB, int V, int* row_offsets, int* col_indices,
                                             int m_vec, int scaleA)
{
    switch (type_bytes) {
        case 1: return compute_ref_integers<char>((char*)A, B, C, M, K, N, preA, preA_cut, preB, V, row_offsets,
                                                  col_indices, m_vec, scaleA);
        case 2: return compute_ref_integers<short>((short*)A, B, C, M, K, N, preA, preA_cut, preB, V, row_offsets,
                                                   col_indices, m_vec, scaleA);
        case 4: return compute_ref_integers<int>((int*)A, B, C, M, K, N, preA, preA_cut, preB, V, row_offsets,
                                                 col_indices, m_vec, scaleA);
        default: return compute_ref_integers<long long>((long long*)A, B, C, M, K, N, preA, preA_cut, preB, V,
                                                        row_offsets, col_indices, m_vec, scaleA);
    }
}
#endif

#ifdef MCREF_SDDMM
extern "C" double mcref_host_sddmm_integers(int* lhs, int* rhs, int* C, int M, int K, int N, int preA, int preB, int V,
                                            int* row_offsets, int* col_indices, int m_vec, int alignment)
{
    return Host_sddmm_integers(lhs, rhs, C, M, K, N, preA, preB, V, row_offsets, col_indices, m_vec, alignment);
}
#endif
