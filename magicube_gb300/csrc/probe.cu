// probe.cu -- measured peak of the warp-level tensor paths this library uses
// (the denominator of its tensor-utilisation figures): every warp of a full
// grid issues back-to-back independent mma.sync of one kind.
#include <cstdint>

#include "mc_host.h"
#include "../../include/magicube_gb300_probe.h"
#include "mc_ptx.cuh"
#include "mc_sm100.cuh"

namespace mc {

// One CTA per SM; thread 0 issues `iters` x 4 back-to-back tcgen05.mma
// kind::f16 (M = 128, N, K = 16, f32 accumulator in TMEM) from zeroed
// 128-byte-swizzled shared-memory tiles, commits once and waits (bounded).
// *timeouts counts waits that ran out.
template <int N, bool LATENCY>
__global__ void __launch_bounds__(128) tc_peak_kernel(int iters, unsigned int* timeouts)
{
    using namespace sm100;
    constexpr int TCOLS = N < 32 ? 32 : N;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = smem_raw + ((1024u - (saddr(smem_raw) & 1023u)) & 1023u);
    uint8_t* at = smem;                      // 128 rows x 128 B
    uint8_t* bt = smem + 128 * 128;          // N rows x 128 B
    uint64_t* done = reinterpret_cast<uint64_t*>(bt + N * 128);
    uint32_t* tmem_s = reinterpret_cast<uint32_t*>(done + 1);
    const int tid = threadIdx.x;
    for (int i = tid; i < (128 + N) * 8; i += 128) reinterpret_cast<uint4*>(smem)[i] = make_uint4(0, 0, 0, 0);
    if (tid == 0) {
        mbar_init(done, 1);
        fence_mbar_init();
    }
    if (tid < 32) {
        tmem_alloc(tmem_s, TCOLS);
        tmem_relinquish();
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_s;
    if (tid == 0) {
        const uint64_t ad = desc_sw128_kmajor(saddr(at)), bd = desc_sw128_kmajor(saddr(bt));
        constexpr uint32_t idesc = idesc_f16_f32(128, N);
        uint32_t phase = 0;
        for (int it = 0; it < iters; ++it) {
#pragma unroll
            for (int k = 0; k < 4; ++k) mma_f16_ss(tmem, ad + 2 * k, bd + 2 * k, idesc, (it | k) != 0);
            if (LATENCY) {  // each group of four waited for before the next is issued
                mma_commit(done);
                if (!mbar_wait(done, phase, 4000000000LL)) {
                    atomicAdd(timeouts, 1u);
                    break;
                }
                phase ^= 1u;
            }
        }
        if (!LATENCY) {
            mma_commit(done);
            if (!mbar_wait(done, 0, 4000000000LL)) atomicAdd(timeouts, 1u);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (tid < 32) {
        tc_fence_after();
        tmem_dealloc(tmem, TCOLS);
    }
}

// Compares div_rn (the kernels' quotient from a prepared divisor) with the
// IEEE division __fdiv_rn for every integer numerator in [lo, hi), bit for
// bit, in the scalar form and in both lanes of the packed form (the second
// lane on the numerator a ^ 0x55555555); counters[0] += mismatches,
// counters[1] = min(first mismatching numerator).
__global__ void __launch_bounds__(256) quotient_check_kernel(float d, long long lo, long long hi,
                                                             unsigned long long* counters)
{
    const Divisor v = make_divisor(d);
    unsigned long long bad = 0;
    long long first = hi;
    const long long step = (long long)gridDim.x * blockDim.x;
    for (long long a = lo + blockIdx.x * (long long)blockDim.x + threadIdx.x; a < hi; a += step) {
        const float x = __int2float_rn((int)a);
        // the packed form, its second lane on another numerator
        const float x2 = __int2float_rn((int)((uint32_t)a ^ 0x55555555u));
        const float2 q2 = div_rn2(x, x2, v, v);
        const uint32_t ref = __float_as_uint(__fdiv_rn(x, d));
        if (__float_as_uint(div_rn(x, v)) != ref || __float_as_uint(q2.x) != ref ||
            __float_as_uint(q2.y) != __float_as_uint(__fdiv_rn(x2, d))) {
            ++bad;
            if (a < first) first = a;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
        const long long f = __shfl_xor_sync(0xffffffffu, first, o);
        first = f < first ? f : first;
    }
    if ((threadIdx.x & 31) == 0 && bad) {
        atomicAdd(counters, bad);
        atomicMin(reinterpret_cast<long long*>(counters + 1), first);
    }
}

// f2i_rn_small / f2i_rz_small against __float2int_rn / __float2int_rz for
// every float whose bit pattern (sign included) is in [lo, hi); counters[0]
// += mismatches, counters[1] = min(first mismatching pattern).
__global__ void __launch_bounds__(256) small_int_check_kernel(unsigned long long lo, unsigned long long hi,
                                                              unsigned long long* counters)
{
    unsigned long long bad = 0, first = hi;
    const unsigned long long step = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long u = lo + blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; u < hi; u += step) {
        const float f = __uint_as_float((uint32_t)u);
        if (f2i_rn_small(f) != __float2int_rn(f) || f2i_rz_small(f) != __float2int_rz(f)) {
            ++bad;
            if (u < first) first = u;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
        const unsigned long long f = __shfl_xor_sync(0xffffffffu, first, o);
        first = f < first ? f : first;
    }
    if ((threadIdx.x & 31) == 0 && bad) {
        atomicAdd(counters, bad);
        atomicMin(counters + 1, first);
    }
}

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
            else if constexpr (KIND == 4) {  // CUDA-core dp4a: four independent chains per slot
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    asm volatile("dp4a.s32.s32 %0, %1, %2, %0;" : "+r"(c[q][e]) : "r"(a), "r"(b));
            } else if constexpr (KIND == 3)
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

// Kind 5: per step one mma.sync m16n8k32 s8 and 32 dp4a (about equal pipe
// time if the two run on separate units): the combined rate shows whether
// the int8 MMA and dp4a overlap.
__global__ void __launch_bounds__(256) mixed_peak_kernel(int* out, int iters, unsigned seed)
{
    uint32_t a = seed ^ threadIdx.x, b = seed * 7u + threadIdx.x;
    int c[8][4] = {};
    int d[32] = {};
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            asm volatile("mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3},{%4,%5,%6,%7},{%8,%9},{%0,%1,%2,%3};"
                         : "+r"(c[q][0]), "+r"(c[q][1]), "+r"(c[q][2]), "+r"(c[q][3])
                         : "r"(a), "r"(b), "r"(a), "r"(b), "r"(a), "r"(b));
#pragma unroll
            for (int e = 0; e < 32; ++e) asm volatile("dp4a.s32.s32 %0, %1, %2, %0;" : "+r"(d[e]) : "r"(a), "r"(b));
        }
    }
    int s = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) s += c[q][0] + c[q][1] + c[q][2] + c[q][3];
#pragma unroll
    for (int e = 0; e < 32; ++e) s += d[e];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace mc

extern "C" int mcProbeTensorPeak(int kind, void* sink, long long sink_bytes, int iters, float* ms_out,
                                 double* ops_out, cudaStream_t stream)
{
    mc::clear_error();
    if (kind < 0 || kind > 5 || !ms_out || !ops_out || iters <= 0) return mc::fail(1, "mcProbeTensorPeak: bad arguments");
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
        else if (kind == 3) mc::tensor_peak_kernel<3><<<blocks, threads, 0, stream>>>(out, iters, 1234u);
        else if (kind == 4) mc::tensor_peak_kernel<4><<<blocks, threads, 0, stream>>>(out, iters, 1234u);
        else mc::mixed_peak_kernel<<<blocks, threads, 0, stream>>>(out, iters, 1234u);
    };
    launch();  // warm-up
    cudaEventRecord(e0, stream);
    launch();
    cudaEventRecord(e1, stream);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms_out, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    // MACs per warp per slot q: an MMA's m x n x k; kind 4: 4 dp4a x 32 lanes
    // x 4; kind 5: one m16n8k32 and 32 dp4a
    const double macs = kind == 0   ? 16.0 * 8 * 32
                        : kind == 1 ? 16.0 * 8 * 64
                        : kind == 4 ? 4.0 * 32 * 4
                        : kind == 5 ? 16.0 * 8 * 32 + 32.0 * 32 * 4
                                    : 16.0 * 8 * 16;  // kinds 2, 3: k = 16
    *ops_out = 2.0 * macs * (double)blocks * (threads / 32) * iters * 8;
    return (int)cudaGetLastError();
}

extern "C" int mcProbeTensorCorePeak(int n, int iters, float* ms_out, double* ops_out, unsigned int* timeouts,
                                     cudaStream_t stream)
{
    mc::clear_error();
    const bool latency = n < 0;  // -n: each group of four MMAs committed and waited for in turn
    if (latency) n = -n;
    if (!(n == 16 || n == 64 || n == 256) || iters <= 0 || !ms_out || !ops_out || !timeouts)
        return mc::fail(1, "mcProbeTensorCorePeak: |n| must be 16, 64 or 256; iters > 0; non-null outputs");
    const int sms = mc::sm_count();
    const size_t smem = 1024 + (size_t)(128 + n) * 128 + 64;
    auto launch = [&]() {
        if (n == 16) {
            if (latency) mc::tc_peak_kernel<16, true><<<sms, 128, smem, stream>>>(iters, timeouts);
            else mc::tc_peak_kernel<16, false><<<sms, 128, smem, stream>>>(iters, timeouts);
        } else if (n == 64) {
            if (latency) mc::tc_peak_kernel<64, true><<<sms, 128, smem, stream>>>(iters, timeouts);
            else mc::tc_peak_kernel<64, false><<<sms, 128, smem, stream>>>(iters, timeouts);
        } else {
            if (latency) mc::tc_peak_kernel<256, true><<<sms, 128, smem, stream>>>(iters, timeouts);
            else mc::tc_peak_kernel<256, false><<<sms, 128, smem, stream>>>(iters, timeouts);
        }
    };
    if (n == 256 && (cudaFuncSetAttribute(mc::tc_peak_kernel<256, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem) != cudaSuccess ||
                     cudaFuncSetAttribute(mc::tc_peak_kernel<256, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem) != cudaSuccess))
        return (int)cudaGetLastError();
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    launch();  // warm-up
    cudaEventRecord(e0, stream);
    launch();
    cudaEventRecord(e1, stream);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms_out, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ops_out = 2.0 * 128.0 * n * 16.0 * 4.0 * (double)iters * sms;
    return (int)cudaGetLastError();
}

extern "C" int mcCheckQuotients(float divisor, long long lo, long long hi, void* counters, cudaStream_t stream)
{
    mc::clear_error();
    if (!counters || reinterpret_cast<uintptr_t>(counters) % 8 || lo < -2147483648LL || hi > 2147483648LL || lo > hi)
        return mc::fail(1, "mcCheckQuotients: counters must be 8-byte aligned; [lo, hi) must lie in the int32 range");
    if (lo == hi) return 0;
    const int blocks = mc::sm_count() * 8;
    mc::quotient_check_kernel<<<blocks, 256, 0, stream>>>(divisor, lo, hi, static_cast<unsigned long long*>(counters));
    return (int)cudaGetLastError();
}

extern "C" int mcCheckSmallIntConversions(unsigned long long lo, unsigned long long hi, void* counters,
                                          cudaStream_t stream)
{
    mc::clear_error();
    if (!counters || reinterpret_cast<uintptr_t>(counters) % 8 || hi > 0x100000000ULL || lo > hi)
        return mc::fail(1, "mcCheckSmallIntConversions: counters must be 8-byte aligned; [lo, hi) must lie in "
                           "the 32-bit pattern range");
    if (lo == hi) return 0;
    const int blocks = mc::sm_count() * 8;
    mc::small_int_check_kernel<<<blocks, 256, 0, stream>>>(lo, hi, static_cast<unsigned long long*>(counters));
    return (int)cudaGetLastError();
}
