/* magicube_gb300_probe.h -- diagnostics of the GB300 build, in their own
 * library (libmagicube_gb300_probe.so, linked against libmagicube_gb300.so):
 * the measured peaks of the tensor paths the kernels use (the denominators of
 * the benchmark's utilisation figures) and exhaustive checks of two
 * arithmetic building blocks of the kernels.  No counterpart in the
 * reference; nothing in the product path calls them. */
#ifndef MAGICUBE_GB300_PROBE_H
#define MAGICUBE_GB300_PROBE_H

#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

/* mcProbeTensorPeak: times one full-grid launch of back-to-back independent
 * mma.sync of `kind` (0: m16n8k32 s8, 1: m16n8k64 s4, 2: m16n8k16 f16 with f32
 * accumulators, 3: m16n8k16 s8; 4: the CUDA-core dp4a.s32.s32, four MACs per
 * thread instruction; 5: one m16n8k32 s8 and 32 dp4a per step, which shows
 * whether the two overlap) and returns its duration and operation count (2 per MAC), the
 * measured tensor peak its kernels are compared with.  sink: device buffer of
 * at least 4 bytes x 256 threads x 8 CTAs x SMs that receives each thread's
 * (meaningless) accumulator sum, so the MMAs are not optimised away. */
int mcProbeTensorPeak(int kind, void* sink, long long sink_bytes, int iters, float* ms_out,
                      double* ops_out, cudaStream_t stream);

/* mcProbeTensorCorePeak: times one launch of one CTA per SM whose single
 * issuing thread runs iters x 4 back-to-back tcgen05.mma kind::f16 of
 * M = 128, N = n (16, 64 or 256), K = 16 into TMEM; returns the duration and
 * the operation count (2 per MAC, padding included).  n < 0 (N = -n)
 * commits each group of four and waits for it before the next: the
 * duration / iters is then the issue-to-completion latency of a group.
 * timeouts: device counter of completion waits that ran out (0 unless the
 * device stalled). */
int mcProbeTensorCorePeak(int n, int iters, float* ms_out, double* ops_out, unsigned int* timeouts,
                          cudaStream_t stream);

/* mcCheckQuotients: compares, bit for bit, the dequantisation quotient the
 * kernels compute from a prepared divisor (RN(1/d) and two FMA correction
 * steps) with the IEEE division a / d for every integer numerator a in
 * [lo, hi) (within the int32 range).  counters: device buffer of two 8-byte
 * words; word 0 accumulates the mismatches, word 1 (signed) is lowered to the
 * first mismatching numerator -- initialise them to 0 and hi. */
int mcCheckQuotients(float divisor, long long lo, long long hi, void* counters, cudaStream_t stream);
/* mcCheckSmallIntConversions: compares the kernels' float-to-int conversion
 * for |f| < 2^22 (one add of 1.5 * 2^23, then the bit pattern) with the
 * hardware conversions, round-to-nearest-even and toward zero, for every
 * float whose 32-bit pattern is in [lo, hi).  counters: two device uint64,
 * zeroed and UINT64_MAX by the caller; receives the number of mismatches and
 * the smallest mismatching pattern.  Asynchronous. */
int mcCheckSmallIntConversions(unsigned long long lo, unsigned long long hi, void* counters, cudaStream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* MAGICUBE_GB300_PROBE_H */
