// spmm_benchmark -- quantized vector-sparse SpMM benchmark on libmagicube_gb300.
//
// Same command line and output lines as the reference's benchmark program
// (SpMM/SpMM/spmm_benchmark.cpp:757-836), so its sweep launchers and log
// parsers run unchanged:
//
//   spmm_benchmark bm N V kernel sort func sparse preA preB
//
//   bm      .smtx file (m_vec, K, nnz_vec / row offsets / column indices)
//   N       columns of B and C;  V  vector length (2, 4, 8)
//   kernel  0 (the library's kernels; other values are rejected)
//   sort    1: process vector-rows longest first;  func 1: verify on the host
//   sparse  1;  preA / preB  lhs / rhs bits: 4-4, 8-4, 12-4, 16-4, 8-8, 12-8,
//           16-8, 16-16 (12-bit values in 16-bit containers)
//
// Data are generated as the reference does (bm_test_utils.h:130-164: a
// default-seeded std::default_random_engine, copied into every call, and
// per-container value rules), packed with the library's host packer and run
// through the reference-compatible entry points (unsigned lanes).  With
// func = 1 the result is checked against a host computation of C = A * B.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <random>
#include <string>
#include <typeinfo>
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

// Element generator of the reference's MakeDenseMatrix for one container type.
template <typename T>
void make_dense(long long count, T* out, std::default_random_engine gen)
{
    std::uniform_real_distribution<float> dist(0.0, 1.0);
    for (long long i = 0; i < count; ++i) {
        if (typeid(T) == typeid(int)) {
            (void)dist(gen);
            out[i] = (T)(0x11111111 + int(117.0 * dist(gen)));
        } else if (typeid(T) == typeid(long long)) {
            (void)dist(gen);
            out[i] = (T)(0x1111111111111111LL + int(117.0 * dist(gen)));
        } else if (typeid(T) == typeid(short)) {
            out[i] = (T)(10240.0 * dist(gen));
        } else {
            out[i] = (T)(127.0 * dist(gen));
        }
    }
}

// Container type of one vector's values and the number of containers per
// vector, as the reference dispatches them (spmm_benchmark.cpp:805-831);
// `lane` is the bits per stored lane (16 for 12-bit values).
void container(int lane, int preB, int V, int& bytes, int& scale)
{
    scale = 1;
    if (lane == 16 && preB == 16) { bytes = 2; scale = V; }
    else if (lane == 16 && V == 8) { bytes = 8; scale = 2; }
    else bytes = V * lane / 8;
}

template <typename T>
std::vector<uint8_t> gen_values(long long nvec, int V, int preA, int scale, std::default_random_engine g)
{
    const long long count = nvec * V * (long long)scale * preA / (long long)(sizeof(T) * 8);
    std::vector<T> v((size_t)count);
    make_dense<T>(count, v.data(), g);
    std::vector<uint8_t> out(v.size() * sizeof(T));
    std::memcpy(out.data(), v.data(), out.size());
    return out;
}

// Host C = A * B over the original layout with unsigned lanes (lane: bits
// per stored lane; preA: significant bits of a value).
void host_spmm(const std::vector<uint8_t>& vals, const std::vector<int>& B, std::vector<int>& C, const Smtx& s, int V,
               int N, int lane, int preA, int preB)
{
    C.assign((size_t)s.m_vec * V * N, 0);
    const int per = 32 / preB, ipr = N / per;
    const uint32_t mb = preB == 32 ? 0xFFFFFFFFu : (1u << preB) - 1u;
    for (int i = 0; i < s.m_vec; ++i)
        for (int j = s.offsets[i]; j < s.offsets[i + 1]; ++j)
            for (int v = 0; v < V; ++v) {
                const long long bit = ((long long)j * V + v) * lane;
                uint32_t a = 0;
                for (int b = 0; b < (lane + 7) / 8 + 1 && bit / 8 + b < (long long)vals.size(); ++b)
                    a |= (uint32_t)vals[(size_t)(bit / 8 + b)] << (8 * b);
                a = (a >> (bit % 8)) & ((1u << preA) - 1u);
                uint32_t* crow = reinterpret_cast<uint32_t*>(C.data()) + (size_t)(i * V + v) * N;
                const uint32_t* brow = reinterpret_cast<const uint32_t*>(B.data()) + (size_t)s.cols[j] * ipr;
                for (int n = 0; n < ipr; ++n)
                    for (int q = 0; q < per; ++q) crow[n * per + q] += a * ((brow[n] >> (q * preB)) & mb);
            }
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc != 10) {
        std::printf("usage: spmm_benchmark [bm] [n] [v] [kernel] [sort] [function] [sparse] [preA] [preB]\n");
        return argc == 2 ? 0 : 1;
    }
    const std::string bm = argv[1];
    const int N = std::atoi(argv[2]), V = std::atoi(argv[3]), kernel = std::atoi(argv[4]);
    const int sorted = std::atoi(argv[5]), func = std::atoi(argv[6]), sparse = std::atoi(argv[7]);
    const int preA = std::atoi(argv[8]), preB = std::atoi(argv[9]);
    std::printf("Sparse matrix: %s\n", bm.c_str());
    if (kernel != 0 || sparse != 1) {
        std::printf("Unsupported Kernel \n");
        return 1;
    }
    int (*fn)(int, int, int, int, const int*, const int*, const int*, const int*, const int*, int*) = nullptr;
    if (preA == 4 && preB == 4) fn = mcWmmaSpmm_4b;
    else if (preA == 8 && preB == 4) fn = mcWmmaSpmm_8b4b;
    else if (preA == 12 && preB == 4) fn = mcWmmaSpmm_12b4b;
    else if (preA == 16 && preB == 4) fn = mcWmmaSpmm_16b4b;
    else if (preA == 8 && preB == 8) fn = mcWmmaSpmm_8b;
    else if (preA == 12 && preB == 8) fn = mcWmmaSpmm_12b8b;
    else if (preA == 16 && preB == 8) fn = mcWmmaSpmm_16b8b;
    else if (preA == 16 && preB == 16) fn = mcWmmaSpmm_16b;
    if (!fn || !(V == 2 || V == 4 || V == 8)) {
        std::printf("Unsupported precision and vec_length!\n");
        return 1;
    }
    Smtx s;
    std::string err;
    if (!read_smtx(bm, s, err)) {
        std::fprintf(stderr, "%s\n", err.c_str());
        return 1;
    }
    const int K = s.ncols, M = s.m_vec * V;
    const int mma_k = (preA == 4 || preB == 4) ? 32 : 16;
    const int lane = preA == 12 ? 16 : preA;  // bits per stored value lane
    std::printf("preA %d, preA_cut %d, preB %d, vec_length %d \n", lane, preA, preB, V);
    std::printf("m_vec %d, dimN %d, nonzeros_vec %d, dimk %d, mma_k_dim %d \n", s.m_vec, N, s.nnz, K, mma_k);

    std::default_random_engine generator;
    int bytes = 0, scale = 1;
    container(lane, preB, V, bytes, scale);
    std::vector<uint8_t> vals;
    switch (bytes) {
        case 1: vals = gen_values<char>(s.nnz, V, lane, scale, generator); break;
        case 2: vals = gen_values<short>(s.nnz, V, lane, scale, generator); break;
        case 4: vals = gen_values<int>(s.nnz, V, lane, scale, generator); break;
        default: vals = gen_values<long long>(s.nnz, V, lane, scale, generator); break;
    }
    std::vector<int> B((size_t)K * N * preB / 32);
    make_dense<int>((long long)B.size(), B.data(), generator);

    std::vector<int> pairs(2 * s.m_vec), ri(s.m_vec);
    const int aligned = mcAlignRowOffsets(s.m_vec, s.offsets.data(), mma_k, pairs.data());
    std::printf(" nonzero_vec: %d aligned_ nonzero_vec: %d\n", s.nnz, aligned);
    std::vector<int> cols(aligned > 0 ? aligned : 1);
    std::vector<uint8_t> packed((size_t)aligned * V * lane / 8 + 16);
    if (aligned < 0 || mcPadColumnIndices(s.m_vec, s.offsets.data(), s.cols.data(), pairs.data(), aligned,
                                          mma_k == 32, cols.data()) ||
        mcPackSpmmValues(s.m_vec, V, preA, preB, s.offsets.data(), pairs.data(), aligned, vals.data(),
                         packed.data()) ||
        (sorted ? mcSortedRowSwizzle(s.m_vec, s.offsets.data(), ri.data()) : mcIdentityRowSwizzle(s.m_vec, ri.data()))) {
        std::fprintf(stderr, "format conversion failed: %s\n", mcGetLastErrorString());
        return 1;
    }

    int *d_ri, *d_ro, *d_ci, *d_vals, *d_B, *d_C;
    CHECK_CUDA(cudaMalloc(&d_ri, sizeof(int) * ri.size()));
    CHECK_CUDA(cudaMalloc(&d_ro, sizeof(int) * pairs.size()));
    CHECK_CUDA(cudaMalloc(&d_ci, sizeof(int) * cols.size()));
    CHECK_CUDA(cudaMalloc(&d_vals, packed.size()));
    CHECK_CUDA(cudaMalloc(&d_B, sizeof(int) * B.size()));
    CHECK_CUDA(cudaMalloc(&d_C, sizeof(int) * (size_t)M * N));
    CHECK_CUDA(cudaMemcpy(d_ri, ri.data(), sizeof(int) * ri.size(), cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemcpy(d_ro, pairs.data(), sizeof(int) * pairs.size(), cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemcpy(d_ci, cols.data(), sizeof(int) * cols.size(), cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemcpy(d_vals, packed.data(), packed.size(), cudaMemcpyHostToDevice));
    CHECK_CUDA(cudaMemcpy(d_B, B.data(), sizeof(int) * B.size(), cudaMemcpyHostToDevice));

    auto run = [&]() {
        int rc = fn(s.m_vec, V, N, K, d_ri, d_ro, d_ci, d_vals, d_B, d_C);
        if (rc) {
            std::fprintf(stderr, "kernel launch failed (%d): %s\n", rc, mcGetLastErrorString());
            std::exit(1);
        }
    };
    for (int i = 0; i < 16; ++i) run();
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
    std::printf("Magicube SpMM runtime %g ms\n", avg_ms);
    if (func) {
        const double gops = 2.0 * s.nnz * V * (double)N / 1e9;
        std::printf("total Gflops: %g\n", gops);
        std::printf("performance TOP/s: %g\n", gops / (avg_ms / 1000.0) / 1000.0);
        std::vector<int> got((size_t)M * N), ref;
        CHECK_CUDA(cudaMemcpy(got.data(), d_C, sizeof(int) * got.size(), cudaMemcpyDeviceToHost));
        host_spmm(vals, B, ref, s, V, N, lane, preA, preB);
        long long errors = 0;
        for (size_t i = 0; i < got.size(); ++i) errors += got[i] != ref[i];
        if (errors) std::printf("SPMM does not agree with SEQUENTIAL! %lld errors!\n", errors);
        else std::printf("Results verification: PASS\n");
    }
    cudaFree(d_ri); cudaFree(d_ro); cudaFree(d_ci); cudaFree(d_vals); cudaFree(d_B); cudaFree(d_C);
    std::printf("\n");
    return 0;
}
