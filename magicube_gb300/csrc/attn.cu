// attn.cu -- the element-wise steps around the integer SDDMM / SpMM of the
// quantized sparse attention: symmetric quantization of half activations and
// the quantized row softmax.
//
//  * mcQuantize: q = trunc(clamp(float(x) * scale, lo, hi)), packed
//    little-endian, 8 or 4 bits per lane -- the reference's
//    quantizationKernel_{8b,4b} (sparse_transformer_magicube/src/cuda/
//    quantization_kernel.cu:14-131), for any element count divisible by 8.
//  * mcQuantSoftmax: per vector-row and vector lane, over the row's stored
//    nonzeros, q = trunc(clamp(exp(x * scaling - max) * (scale / sum))) (the
//    reference divides each p by the sum, then scales; here one division per
//    row and lane gives scale / sum),
//    written in the value layout the SpMM reads (MC_VALUES_SOFTMAX) -- the
//    reference's csrSoftmaxKernel_ (q_softmax_kernel.cu:181-271).  One warp per
//    vector-row; three passes over the row (max, sum, write) read the scores
//    from L1/L2.  The maximum starts from -inf for every lane (the reference
//    starts lanes 1..V-1 from 0, which only shifts the exponent's argument).
#include <cfloat>
#include <cstdint>
#include <type_traits>

#include "mc_host.h"
#include "mc_ptx.cuh"

namespace mc {

template <int BITS>
__global__ void __launch_bounds__(256) quantize_kernel(const __half* __restrict__ in, uint8_t* __restrict__ out,
                                                        long long groups, float scale)
{
    constexpr float LO = BITS == 8 ? -128.f : -8.f, HI = BITS == 8 ? 127.f : 7.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < groups;
         i += (long long)gridDim.x * blockDim.x) {
        const int4 raw = ldg_nc_v4(in + 8 * i);
        const __half* h = reinterpret_cast<const __half*>(&raw);
        uint32_t q[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            float f = __half2float(h[e]) * scale;
            f = fminf(fmaxf(f, LO), HI);
            q[e] = (uint32_t)(int)f;  // truncation toward zero, as a C cast
        }
        if constexpr (BITS == 8) {
            uint32_t w0 = (q[0] & 0xff) | (q[1] & 0xff) << 8 | (q[2] & 0xff) << 16 | (q[3] & 0xff) << 24;
            uint32_t w1 = (q[4] & 0xff) | (q[5] & 0xff) << 8 | (q[6] & 0xff) << 16 | (q[7] & 0xff) << 24;
            *reinterpret_cast<uint2*>(out + 8 * i) = make_uint2(w0, w1);
        } else {
            uint32_t w = 0;
#pragma unroll
            for (int e = 0; e < 8; ++e) w |= (q[e] & 0xf) << (4 * e);
            *reinterpret_cast<uint32_t*>(out + 4 * i) = w;
        }
    }
}

struct SoftmaxParams {
    int m_vec, batch;
    const int* row_indices;
    const int* row_offsets;
    const __half* scores;     // per batch entry: aligned_nnz * V halves, vector-major
    long long scores_stride;  // halves
    uint8_t* out;             // per batch entry: aligned_nnz * V * BITS / 8 bytes
    long long out_stride;     // bytes
    float scaling, scale;
    float* row_div;           // MC_REQUANT_ROWMAX: per batch entry, m_vec * V divisors
    long long row_div_stride; // floats
};

// V raw halves of one slot (one 16-, 8- or 4-byte load) and their scaled
// floats.
template <int V>
struct RawVec {
    using T = typename std::conditional<V == 8, int4, typename std::conditional<V == 4, int2, int>::type>::type;
};
template <int V>
__device__ __forceinline__ typename RawVec<V>::T ld_raw(const __half* p)
{
    return *reinterpret_cast<const typename RawVec<V>::T*>(p);
}
template <int V>
__device__ __forceinline__ void cvt_vec(const typename RawVec<V>::T& r, float (&x)[V], float s)
{
    const __half* h = reinterpret_cast<const __half*>(&r);
#pragma unroll
    for (int v = 0; v < V; ++v) x[v] = __fmul_rn(__half2float(h[v]), s);
}

// Running maximum and minimum of raw half scores, V lanes as V/2 half2.
template <int V>
struct HalfRange {
    __half2 hi[V / 2], lo[V / 2];
    __device__ __forceinline__ HalfRange()
    {
#pragma unroll
        for (int i = 0; i < V / 2; ++i) {
            hi[i] = __half2half2(__ushort_as_half((unsigned short)0xFC00u));  // -inf
            lo[i] = __half2half2(__ushort_as_half((unsigned short)0x7C00u));  // +inf
        }
    }
    __device__ __forceinline__ void add(const typename RawVec<V>::T& r)
    {
        __half2 h[V / 2];
        *reinterpret_cast<typename RawVec<V>::T*>(h) = r;
#pragma unroll
        for (int i = 0; i < V / 2; ++i) {
            hi[i] = __hmax2(hi[i], h[i]);  // a NaN input yields the other operand
            lo[i] = __hmin2(lo[i], h[i]);
        }
    }
    // max over the slots of x = float(h) * s, with -FLT_MAX for none: the
    // scaling is monotone in h (non-decreasing for s >= 0, non-increasing for
    // s < 0), so the maximum is the scaled maximum or the scaled minimum; a
    // NaN product (s = 0 or infinite against an infinite or zero h) is
    // ignored by fmaxf as it is when every slot is scaled first.  A lane that
    // saw no slot, or only NaN, still has min > max (the initial +inf and
    // -inf) and keeps -FLT_MAX.
    __device__ __forceinline__ void scaled_max(float s, float (&mx)[V]) const
    {
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const __half a = (v & 1) ? __high2half(hi[v / 2]) : __low2half(hi[v / 2]);
            const __half b = (v & 1) ? __high2half(lo[v / 2]) : __low2half(lo[v / 2]);
            mx[v] = __hgt(b, a) ? -FLT_MAX
                                : fmaxf(-FLT_MAX, fmaxf(__fmul_rn(__half2float(a), s), __fmul_rn(__half2float(b), s)));
        }
    }
};

// Stores the probabilities of slots j (even) and j + 1 of lane v.  `two`:
// slot j + 1 is in the row (otherwise q1 is 0 and, for 8 and 16 bits, only
// slot j is written).  Layouts (relative to the row start): 8 bits
// [j/16][V][16] bytes; 16 bits [j/16][V][low 16 | high 16] bytes; 4 bits
// [j/32][V][16] bytes, slot j in the low and j + 1 in the high nibble.
template <int V, int BITS>
__device__ __forceinline__ void store_pair(uint8_t* out, int j, int v, int q0, int q1, bool two)
{
    if constexpr (BITS == 8) {
        uint8_t* o = out + (j >> 4) * V * 16 + v * 16 + (j & 15);
        if (two) *reinterpret_cast<uint16_t*>(o) = (uint16_t)((q0 & 0xff) | ((q1 & 0xff) << 8));
        else *o = (uint8_t)q0;
    } else if constexpr (BITS == 16) {
        uint8_t* o = out + (j >> 4) * V * 32 + v * 32 + (j & 15);
        if (two) {
            *reinterpret_cast<uint16_t*>(o) = (uint16_t)((q0 & 0xff) | ((q1 & 0xff) << 8));
            *reinterpret_cast<uint16_t*>(o + 16) = (uint16_t)(((q0 >> 8) & 0xff) | (q1 & 0xff00));
        } else {
            o[0] = (uint8_t)(q0 & 0xff);
            o[16] = (uint8_t)((q0 >> 8) & 0xff);
        }
    } else {
        out[(j >> 5) * V * 16 + v * 16 + ((j & 31) >> 1)] = (uint8_t)((q0 & 0xf) | ((q1 & 0xf) << 4));
    }
}

// One warp per vector-row.  The maximum comes from the raw halves (one pass
// of half2 max/min), the sum and the probabilities walk the slots in pairs:
// lane l takes slots 2l, 2l+1, 2l+64, 2l+65, ... in that order, the order of
// the fused attention kernel, which reads two slots per load.
// ROWMAX (8 bits): q = round(127 exp(x - max)) needs no sum, so the sum and
// the probabilities come from one pass, and lane 0 writes the row divisors
// 127 * sum * scale -- the separate-launch form of the fused kernel's row-max
// mode (same expressions, same summation order).
template <int V, int BITS, bool ROWMAX = false>
__global__ void __launch_bounds__(128) quant_softmax_kernel(const SoftmaxParams p)
{
    static_assert(!ROWMAX || BITS == 8, "row-max requantization writes 8-bit probabilities");
    constexpr float LO = BITS == 16 ? -32768.f : (BITS == 8 ? -128.f : -8.f);
    constexpr float HI = BITS == 16 ? 32767.f : (BITS == 8 ? 127.f : 7.f);
    const int lane = threadIdx.x & 31;
    const int r = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (r >= p.m_vec) return;
    const int b = blockIdx.y;
    const int row = __ldg(p.row_indices + r);
    const int start = __ldg(p.row_offsets + 2 * row);
    const int nnz = __ldg(p.row_offsets + 2 * row + 1) - start;
    const __half* sc = p.scores + (long long)b * p.scores_stride + (long long)start * V;
    uint8_t* out = p.out + (long long)b * p.out_stride + (long long)start * V * BITS / 8;

    float mx[V], sum[V], x[V];
    {
        // four independent loads per lane in flight: the scores come from
        // DRAM on this pass, and the maximum does not depend on the order
        HalfRange<V> range;
        for (int j0 = lane; j0 < nnz; j0 += 128) {
            typename RawVec<V>::T r[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (j0 + 32 * u < nnz) r[u] = ld_raw<V>(sc + (long long)(j0 + 32 * u) * V);
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (j0 + 32 * u < nnz) range.add(r[u]);
        }
        range.scaled_max(p.scaling, mx);
    }
#pragma unroll
    for (int v = 0; v < V; ++v) {
        sum[v] = 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx[v] = fmaxf(mx[v], __shfl_xor_sync(0xffffffffu, mx[v], o));
    }

    if constexpr (ROWMAX) {
        // two slot pairs per iteration (j, j+1, j+64, j+65: the lane's order),
        // their four loads issued first
        for (int jj = 2 * lane; jj < nnz; jj += 128) {
            typename RawVec<V>::T r[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int j = jj + 64 * (u >> 1) + (u & 1);
                if (j < nnz) r[u] = ld_raw<V>(sc + (long long)j * V);
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int j = jj + 64 * h;
                if (j >= nnz) break;
                const bool two = j + 1 < nnz;
                int q0[V], q1[V];
                cvt_vec<V>(r[2 * h], x, p.scaling);
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    const float e = exp_flush(x[v] - mx[v]);
                    sum[v] += e;
                    q0[v] = __float2int_rn(127.f * e);
                    q1[v] = 0;
                }
                if (two) {
                    cvt_vec<V>(r[2 * h + 1], x, p.scaling);
#pragma unroll
                    for (int v = 0; v < V; ++v) {
                        const float e = exp_flush(x[v] - mx[v]);
                        sum[v] += e;
                        q1[v] = __float2int_rn(127.f * e);
                    }
                }
#pragma unroll
                for (int v = 0; v < V; ++v) store_pair<V, 8>(out, j, v, q0[v], q1[v], two);
            }
        }
#pragma unroll
        for (int v = 0; v < V; ++v)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sum[v] += __shfl_xor_sync(0xffffffffu, sum[v], o);
        if (lane == 0) {
            float* dv = p.row_div + (long long)b * p.row_div_stride + (long long)row * V;
#pragma unroll
            for (int v = 0; v < V; ++v) dv[v] = 127.f * sum[v] * p.scale;
        }
        return;
    }

    for (int jj = 2 * lane; jj < nnz; jj += 128) {  // slots jj, jj+1, jj+64, jj+65 in this order
        typename RawVec<V>::T r[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int j = jj + 64 * (u >> 1) + (u & 1);
            if (j < nnz) r[u] = ld_raw<V>(sc + (long long)j * V);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (jj + 64 * (u >> 1) + (u & 1) >= nnz) continue;
            cvt_vec<V>(r[u], x, p.scaling);
#pragma unroll
            for (int v = 0; v < V; ++v) sum[v] += exp_flush(x[v] - mx[v]);
        }
    }
    float rs[V];  // scale / sum: one division per vector lane
#pragma unroll
    for (int v = 0; v < V; ++v) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) sum[v] += __shfl_xor_sync(0xffffffffu, sum[v], o);
        rs[v] = __fdiv_rn(p.scale, sum[v]);
    }
    for (int jj = 2 * lane; jj < nnz; jj += 128) {
        typename RawVec<V>::T r[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int j = jj + 64 * (u >> 1) + (u & 1);
            if (j < nnz) r[u] = ld_raw<V>(sc + (long long)j * V);
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int j = jj + 64 * h;
            if (j >= nnz) break;
            const bool two = j + 1 < nnz;
            int q0[V], q1[V];
            cvt_vec<V>(r[2 * h], x, p.scaling);
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const float f = fminf(fmaxf(exp_flush(x[v] - mx[v]) * rs[v], LO), HI);
                q0[v] = (int)f;
                q1[v] = 0;
            }
            if (two) {
                cvt_vec<V>(r[2 * h + 1], x, p.scaling);
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    const float f = fminf(fmaxf(exp_flush(x[v] - mx[v]) * rs[v], LO), HI);
                    q1[v] = (int)f;
                }
            }
#pragma unroll
            for (int v = 0; v < V; ++v) store_pair<V, BITS>(out, j, v, q0[v], q1[v], two);
        }
    }
}

}  // namespace mc

extern "C" int mcQuantize(const void* in, void* out, long long count, int bits, float scale, cudaStream_t stream)
{
    mc::clear_error();
    if (bits != 8 && bits != 4) return mc::fail(1, "mcQuantize: bits must be 4 or 8");
    if (count < 0 || count % 8) return mc::fail(1, "mcQuantize: count must be a non-negative multiple of 8");
    if (count == 0) return 0;
    if (!in || !out || reinterpret_cast<uintptr_t>(in) % 16 || reinterpret_cast<uintptr_t>(out) % 8)
        return mc::fail(1, "mcQuantize: input must be 16-byte and output 8-byte aligned");
    const long long groups = count / 8;
    long long blocks = (groups + 255) / 256;
    if (blocks > 152LL * 32) blocks = 152LL * 32;
    if (bits == 8)
        mc::quantize_kernel<8><<<(unsigned)blocks, 256, 0, stream>>>(static_cast<const __half*>(in),
                                                                      static_cast<uint8_t*>(out), groups, scale);
    else
        mc::quantize_kernel<4><<<(unsigned)blocks, 256, 0, stream>>>(static_cast<const __half*>(in),
                                                                      static_cast<uint8_t*>(out), groups, scale);
    return (int)cudaGetLastError();
}

extern "C" int mcQuantSoftmax(const mcSoftmaxDesc* d, cudaStream_t stream)
{
    mc::clear_error();
    if (!d) return mc::fail(1, "mcQuantSoftmax: null descriptor");
    if (!(d->vec_length == 2 || d->vec_length == 4 || d->vec_length == 8))
        return mc::fail(1, "mcQuantSoftmax: vec_length must be 2, 4 or 8");
    if (!(d->bits == 4 || d->bits == 8 || d->bits == 16)) return mc::fail(1, "mcQuantSoftmax: bits must be 4, 8 or 16");
    if (d->m_vec < 0 || d->batch < 1 || d->batch > 65535) return mc::fail(1, "mcQuantSoftmax: bad m_vec or batch");
    if (d->m_vec == 0) return 0;
    if (!d->row_indices || !d->row_offsets || !d->scores || !d->out) return mc::fail(1, "mcQuantSoftmax: null pointer");
    if (reinterpret_cast<uintptr_t>(d->scores) % 16 || d->scores_stride % 8)
        return mc::fail(1, "mcQuantSoftmax: scores must be 16-byte aligned, stride a multiple of 8 halves");
    if (reinterpret_cast<uintptr_t>(d->out) % 2 || d->out_stride % 2)  // slot pairs are stored as 16-bit words
        return mc::fail(1, "mcQuantSoftmax: out must be 2-byte aligned, stride a multiple of 2 bytes");
    if (d->batch > 1 && (d->scores_stride < 0 || d->out_stride < 0))
        return mc::fail(1, "mcQuantSoftmax: negative stride");
    if (d->requant != MC_REQUANT_FIXED && d->requant != MC_REQUANT_ROWMAX)
        return mc::fail(1, "mcQuantSoftmax: requant must be MC_REQUANT_FIXED or MC_REQUANT_ROWMAX");
    if (d->requant == MC_REQUANT_ROWMAX &&
        (d->bits != 8 || !d->row_div || reinterpret_cast<uintptr_t>(d->row_div) % 4 || d->row_div_stride < 0))
        return mc::fail(1, "mcQuantSoftmax: row-max requantization needs bits 8 and a 4-byte aligned row_div");
    mc::SoftmaxParams p;
    p.m_vec = d->m_vec; p.batch = d->batch;
    p.row_indices = d->row_indices; p.row_offsets = d->row_offsets;
    p.scores = static_cast<const __half*>(d->scores); p.scores_stride = d->scores_stride;
    p.out = static_cast<uint8_t*>(d->out); p.out_stride = d->out_stride;
    p.scaling = d->scaling; p.scale = d->scale;
    p.row_div = static_cast<float*>(d->row_div); p.row_div_stride = d->row_div_stride;
    dim3 grid((unsigned)((d->m_vec + 3) / 4), (unsigned)d->batch);
    if (d->requant == MC_REQUANT_ROWMAX) {
        switch (d->vec_length) {
            case 2: mc::quant_softmax_kernel<2, 8, true><<<grid, 128, 0, stream>>>(p); break;
            case 4: mc::quant_softmax_kernel<4, 8, true><<<grid, 128, 0, stream>>>(p); break;
            default: mc::quant_softmax_kernel<8, 8, true><<<grid, 128, 0, stream>>>(p); break;
        }
        return (int)cudaGetLastError();
    }
#define MC_SM(V, B) mc::quant_softmax_kernel<V, B><<<grid, 128, 0, stream>>>(p)
#define MC_SMV(B)                                           \
    switch (d->vec_length) {                                \
        case 2: MC_SM(2, B); break;                         \
        case 4: MC_SM(4, B); break;                         \
        default: MC_SM(8, B); break;                        \
    }
    if (d->bits == 4) { MC_SMV(4) }
    else if (d->bits == 8) { MC_SMV(8) }
    else { MC_SMV(16) }
#undef MC_SMV
#undef MC_SM
    return (int)cudaGetLastError();
}
