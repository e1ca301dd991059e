// sddmm_benchmark -- quantized vector-sparse SDDMM benchmark on libmagicube_gb300.
//
// Same command line and output lines as the reference's benchmark program
// (SDDMM/SDDMM/sddmm_benchmark.cpp:301-352):
//
//   sddmm_benchmark bm K V sort func sparse preA preB
//
//   bm      .smtx file of the output mask (m_vec, N, nnz_vec / offsets / columns)
//   K       inner dimension (multiple of 64);  V  vector length (2, 4, 8)
//   sort    1: longest vector-rows first;  func 1: verify on the host
//   sparse  1;  preA / preB  4-4, 8-8, 16-16 (the reference's) or 16-8
//
// Data are generated as the reference does (bm_test_utils.h:130-164), the mask
// aligned to 8 (sddmm_benchmark.cpp:82,104-127) and the output written in the
// blocked layout (j/8)*8V + 8v + j%8, unsigned lanes.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <random>
#include <string>
#include <vector>

#include "magicube_gb300.h"
#include "smtx_reader.h"

namespace {

#define CHECK_CUDA(x)                                                                      \
    do {                                                                                   \
        cudaError_t e_ = (x);                                                              \
        if (e_ != cudaSuccess) {                                                           \
            std::fprintf(stderr, "CUDA error %s at %s:%d\n", cudaGetErrorString(e_), __FILE__, __LINE__); \
            std::exit(1);                                                                  \
        }                                                                                  \
    } while (0)

void make_dense_int(long long count, int* out, std::default_random_engine gen)
{
    std::uniform_real_distribution<float> dist(0.0, 1.0);
    for (long long i = 0; i < count; ++i) {
        (void)dist(gen);
        out[i] = 0x11111111 + int(117.0 * dist(gen));
    }
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc != 9) {
        std::printf("usage: ./sddmm_benchmark [bm] [k] [v] [sort] [function] [sparse] [preA] [preB]\n");
        return argc == 2 ? 0 : 1;
    }
    const std::string bm = argv[1];
    const int K = std::atoi(argv[2]), V = std::atoi(argv[3]), sorted = std::atoi(argv[4]);
    const int func = std::atoi(argv[5]), sparse = std::atoi(argv[6]);
    const int preA = std::atoi(argv[7]), preB = std::atoi(argv[8]);
    std::printf("Sparse matrix: %s\n", bm.c_str());
    const bool pair_ok = (preA == preB && (preA == 4 || preA == 8 || preA == 16)) || (preA == 16 && preB == 8);
    if (!pair_ok || sparse != 1) {
        std::printf("Unsupported precision!\n");
        return 1;
    }
    if (!(V == 2 || V == 4 || V == 8)) {
        std::printf("Unsupported vec_length!\n");
        return 1;
    }
    Smtx s;
    std::string err;
    if (!read_smtx(bm, s, err)) {
        std::fprintf(stderr, "%s\n", err.c_str());
        return 1;
    }
    const int m_vec = s.m_vec, N = s.ncols, nnz = s.nnz;
    std::vector<int>& offsets = s.offsets;
    std::vector<int>& cols = s.cols;
    const int M = m_vec * V, alignment = 8;
    std::printf("PreA: %d, PreB: %d, vec_len: %d, M: %d, M_vec: %d, N: %d, nnz: %d, K: %d\n", preA, preB, V, M, m_vec, N,
                nnz * V, K);

    std::vector<int> pairs(2 * m_vec), ri(m_vec);
    const int aligned = mcAlignRowOffsets(m_vec, offsets.data(), alignment, pairs.data());
    std::printf(" nonzero_vec: %d aligned_ nonzero_vec: %d\n", nnz, aligned);
    std::vector<int> acols(aligned > 0 ? aligned : 1);
    if (aligned < 0 || mcPadColumnIndices(m_vec, offsets.data(), cols.data(), pairs.data(), aligned, 0, acols.data()) ||
        (sorted ? mcSortedRowSwizzle(m_vec, offsets.data(), ri.data()) : mcIdentityRowSwizzle(m_vec, ri.data()))) {
        std::fprintf(stderr, "format conversion failed: %s\n", mcGetLastErrorString());
        return 1;
    }
    std::default_random_engine generator;
    std::vector<int> A((size_t)M * K / (32 / preA)), B((size_t)N * K / (32 / preB));
    make_dense_int((long long)A.size(), A.data(), generator);
    make_dense_int((long long)B.size(), B.data(), generator);

    int *d_ri, *d_ro, *d_ci, *d_A, *d_B, *d_out;
    const size_t out_n = (size_t)aligned * V;
    CHECK_CUDA(cudaMalloc(&d_ri, sizeof(int) * ri.size()));
    CHECK_CUDA(cudaMalloc(&d_ro, sizeof(int) * pairs.size()));
    CHECK_CUDA(cudaMalloc(&d_ci, sizeof(int) * acols.size()));
    CHECK_CUDA(cudaMalloc(&d_A, sizeof(int) * A.size()));
    CHECK_CUDA(cudaMalloc(&d_B, sizeof(int) * B.size()));
    CHECK_CUDA(cudaMalloc(&d_out, sizeof(int) * (out_n ? out_n : 1)));
    CHECK_CUDA(cudaMemcpy(d_ri, ri.data(), sizeof(int) * ri.size(), cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemcpy(d_ro, pairs.data(), sizeof(int) * pairs.size(), cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemcpy(d_ci, acols.data(), sizeof(int) * acols.size(), cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemcpy(d_A, A.data(), sizeof(int) * A.size(), cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemcpy(d_B, B.data(), sizeof(int) * B.size(), cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemset(d_out, 0, sizeof(int) * (out_n ? out_n : 1)));

    mcSddmmDesc d{};
    d.m_vec = m_vec; d.vec_length = V; d.n = N; d.k = K; d.lhs_bits = preA; d.rhs_bits = preB;
    d.is_signed = 0; d.scale = 1.0f; d.batch = 1;
    d.row_indices = d_ri; d.row_offsets = d_ro; d.column_indices = d_ci; d.lhs = d_A; d.rhs = d_B; d.out = d_out;
    auto run = [&]() {
        int rc = mcSddmm(&d, 0);
        if (rc) {
            std::fprintf(stderr, "kernel launch failed (%d): %s\n", rc, mcGetLastErrorString());
            std::exit(1);
        }
    };
    for (int i = 0; i < 32; ++i) run();
    const int NUM_PROFILES = 512;
    float total = 0.f;
    cudaEvent_t e0, e1;
    CHECK_CUDA(cudaEventCreate(&e0));
    CHECK_CUDA(cudaEventCreate(&e1));
    for (int i = 0; i < NUM_PROFILES; ++i) {
        float ms = 0.f;
        cudaEventRecord(e0);
        run();
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        total += ms;
    }
    CHECK_CUDA(cudaGetLastError());
    const double avg_ms = total / NUM_PROFILES;
    std::printf("Magicube SDDMM runtime %g ms\n", avg_ms);
    if (func) {
        const double gops = 2.0 * nnz * V * (double)K / 1e9;
        std::printf("SDDMM TOPS: %g  performance TOP/s: %g\n", gops / 1000.0, gops / (avg_ms / 1000.0) / 1000.0);
        std::vector<int> got(out_n), ref(out_n, 0);
        CHECK_CUDA(cudaMemcpy(got.data(), d_out, sizeof(int) * out_n, cudaMemcpyDeviceToHost));
        // host: out[j, v] = sum_k A[i*V+v][k] * B[col_j][k], unsigned lanes
        const int pa = 32 / preA, pb = 32 / preB;
        const uint32_t ma = (1u << preA) - 1u, mb = (1u << preB) - 1u;
        const uint32_t* Au = reinterpret_cast<const uint32_t*>(A.data());
        const uint32_t* Bu = reinterpret_cast<const uint32_t*>(B.data());
        for (int i = 0; i < m_vec; ++i)
            for (int j = pairs[2 * i]; j < pairs[2 * i + 1]; ++j)
                for (int v = 0; v < V; ++v) {
                    uint32_t acc = 0;
                    const uint32_t* ar = Au + (size_t)(i * V + v) * (K / pa);
                    const uint32_t* br = Bu + (size_t)acols[j] * (K / pb);
                    for (int l = 0; l < K; ++l)
                        acc += ((ar[l / pa] >> ((l % pa) * preA)) & ma) * ((br[l / pb] >> ((l % pb) * preB)) & mb);
                    ref[(size_t)(j / alignment) * alignment * V + alignment * v + j % alignment] = (int)acc;
                }
        long long errors = 0;
        for (size_t i = 0; i < out_n; ++i) errors += got[i] != ref[i];
        if (errors) std::printf("SDDMM does not agree with SEQUENTIAL! Total %zu, %lld errors!\n", out_n, errors);
        else std::printf("SDDMM results verification: PASS\n");
    }
    cudaFree(d_ri); cudaFree(d_ro); cudaFree(d_ci); cudaFree(d_A); cudaFree(d_B); cudaFree(d_out);
    std::printf("\n");
    return 0;
}
