// probe.cu -- measured peak of the warp-level tensor paths this library uses
// (the denominator of its tensor-utilisation figures): every warp of a full
// grid issues back-to-back independent mma.sync of one kind.
#include <cstdint>

#include "mc_host.h"

namespace mc {

template <int KIND>
__global__ void __launch_bounds__(256) tensor_peak_kernel(int* out, int iters, unsigned seed)
{
    uint32_t a = seed ^ threadIdx.x, b = seed * 7u + threadIdx.x;
    int c[8][4] = {};
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            if constexpr (KIND == 0)
                asm volatile("mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3},{%4,%5,%6,%7},{%8,%9},{%0,%1,%2,%3};"
                             : "+r"(c[q][0]), "+r"(c[q][1]), "+r"(c[q][2]), "+r"(c[q][3])
                             : "r"(a), "r"(b), "r"(a), "r"(b), "r"(a), "r"(b));
            else if constexpr (KIND == 1)
                asm volatile("mma.sync.aligned.m16n8k64.row.col.s32.s4.s4.s32 {%0,%1,%2,%3},{%4,%5,%6,%7},{%8,%9},{%0,%1,%2,%3};"
                             : "+r"(c[q][0]), "+r"(c[q][1]), "+r"(c[q][2]), "+r"(c[q][3])
                             : "r"(a), "r"(b), "r"(a), "r"(b), "r"(a), "r"(b));
            else if constexpr (KIND == 3)
                asm volatile("mma.sync.aligned.m16n8k16.row.col.s32.s8.s8.s32 {%0,%1,%2,%3},{%4,%5},{%6},{%0,%1,%2,%3};"
                             : "+r"(c[q][0]), "+r"(c[q][1]), "+r"(c[q][2]), "+r"(c[q][3])
                             : "r"(a), "r"(b), "r"(a));
            else
                asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3},{%4,%5,%6,%7},{%8,%9},{%0,%1,%2,%3};"
                             : "+r"(c[q][0]), "+r"(c[q][1]), "+r"(c[q][2]), "+r"(c[q][3])
                             : "r"(a), "r"(b), "r"(a), "r"(b), "r"(a), "r"(b));
        }
    }
    int s = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) s += c[q][0] + c[q][1] + c[q][2] + c[q][3];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace mc

extern "C" int mcProbeTensorPeak(int kind, void* sink, long long sink_bytes, int iters, float* ms_out,
                                 double* ops_out, cudaStream_t stream)
{
    mc::clear_error();
    if (kind < 0 || kind > 3 || !ms_out || !ops_out || iters <= 0) return mc::fail(1, "mcProbeTensorPeak: bad arguments");
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int threads = 256, blocks = sms * 8;
    if (!sink || sink_bytes < (long long)blocks * threads * 4)
        return mc::fail(1, "mcProbeTensorPeak: sink must hold 4 bytes per thread of an 8-CTA-per-SM grid");
    int* out = static_cast<int*>(sink);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    auto launch = [&]() {
        if (kind == 0) mc::tensor_peak_kernel<0><<<blocks, threads, 0, stream>>>(out, iters, 1234u);
        else if (kind == 1) mc::tensor_peak_kernel<1><<<blocks, threads, 0, stream>>>(out, iters, 1234u);
        else if (kind == 2) mc::tensor_peak_kernel<2><<<blocks, threads, 0, stream>>>(out, iters, 1234u);
        else mc::tensor_peak_kernel<3><<<blocks, threads, 0, stream>>>(out, iters, 1234u);
    };
    launch();  // warm-up
    cudaEventRecord(e0, stream);
    launch();
    cudaEventRecord(e1, stream);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms_out, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double macs = kind == 0 ? 16.0 * 8 * 32 : (kind == 1 ? 16.0 * 8 * 64 : 16.0 * 8 * 16);  // kinds 2, 3: k = 16
    *ops_out = 2.0 * macs * (double)blocks * (threads / 32) * iters * 8;
    return (int)cudaGetLastError();
}
