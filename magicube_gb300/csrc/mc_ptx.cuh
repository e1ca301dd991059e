// mc_ptx.cuh -- inline-PTX building blocks for the sm_103a integer kernels.
//
// sm_103a has no tcgen05 integer MMA (ptxas rejects tcgen05.mma kind::i8 for
// this target), so the integer contraction runs on the warp-level
// mma.sync.m16n8k32 s8/u8 forms, accumulating in int32 without saturation
// (results wrap modulo 2^32, like the CPU oracle).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_fp16.h>

namespace mc {

// D += A * B with A 16x32 (row), B 32x8 (col), int32 accumulators.
// ASIGNED / BSIGNED pick .s8 or .u8 for each operand.
template <bool ASIGNED, bool BSIGNED>
__device__ __forceinline__ void mma_k32(int (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                        uint32_t a3, uint32_t b0, uint32_t b1)
{
    if constexpr (ASIGNED && BSIGNED) {
        asm volatile(
            "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
            : "+r"(d[0]), "+r"(d[1]), "+r"(d[2]), "+r"(d[3])
            : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    } else if constexpr (ASIGNED && !BSIGNED) {
        asm volatile(
            "mma.sync.aligned.m16n8k32.row.col.s32.s8.u8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
            : "+r"(d[0]), "+r"(d[1]), "+r"(d[2]), "+r"(d[3])
            : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    } else if constexpr (!ASIGNED && BSIGNED) {
        asm volatile(
            "mma.sync.aligned.m16n8k32.row.col.s32.u8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
            : "+r"(d[0]), "+r"(d[1]), "+r"(d[2]), "+r"(d[3])
            : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    } else {
        asm volatile(
            "mma.sync.aligned.m16n8k32.row.col.s32.u8.u8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
            : "+r"(d[0]), "+r"(d[1]), "+r"(d[2]), "+r"(d[3])
            : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
    }
}

// c + the dot product of the four bytes of a and b (both signed or both
// unsigned), modulo 2^32.
template <bool SIGNED>
__device__ __forceinline__ int dp4a(uint32_t a, uint32_t b, int c)
{
    int d;
    if constexpr (SIGNED) asm("dp4a.s32.s32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    else asm("dp4a.u32.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

// D += A * B with A 16x16 (row), B 16x8 (col), f16 operands, f32 accumulators.
__device__ __forceinline__ void mma_f16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                        uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel)
{
    uint32_t r;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(a), "r"(b), "r"(sel));
    return r;
}

// 4x4 byte transpose: w[i] holds bytes (i,0..3); on return w[c] holds bytes (0..3,c).
__device__ __forceinline__ void transpose4x4(uint32_t (&w)[4])
{
    uint32_t x0 = prmt(w[0], w[1], 0x5140), x1 = prmt(w[0], w[1], 0x7362);
    uint32_t y0 = prmt(w[2], w[3], 0x5140), y1 = prmt(w[2], w[3], 0x7362);
    w[0] = prmt(x0, y0, 0x5410);
    w[1] = prmt(x0, y0, 0x7632);
    w[2] = prmt(x1, y1, 0x5410);
    w[3] = prmt(x1, y1, 0x7632);
}

// Four zero-extended nibbles in bytes -> sign-extended int4 values in bytes.
__device__ __forceinline__ uint32_t sext_nibble_bytes(uint32_t z)
{
    return z | ((z & 0x08080808u) * 0x1Eu);
}

// 16 packed nibbles (n0 in bits 0..3) of a 16-bit value -> 4 bytes [n0 n1 n2 n3].
template <bool SIGNED>
__device__ __forceinline__ uint32_t unpack4_u16(uint32_t x)
{
    uint32_t lo = x & 0x0F0Fu, hi = (x >> 4) & 0x0F0Fu;
    uint32_t r = prmt(lo, hi, 0x5140);
    return SIGNED ? sext_nibble_bytes(r) : r;
}

// 8 packed nibbles of a 32-bit word -> two words of bytes (nibbles 0..3, 4..7).
template <bool SIGNED>
__device__ __forceinline__ void unpack4_u32(uint32_t x, uint32_t& out0, uint32_t& out1)
{
    uint32_t even = x & 0x0F0F0F0Fu, odd = (x >> 4) & 0x0F0F0F0Fu;
    out0 = prmt(even, odd, 0x5140);
    out1 = prmt(even, odd, 0x7362);
    if (SIGNED) { out0 = sext_nibble_bytes(out0); out1 = sext_nibble_bytes(out1); }
}

// 8 packed nibbles -> two words of bytes holding each nibble in the byte's
// high half (nibbles 0..3, 4..7): the byte is 16 x the nibble, as a signed
// byte exactly 16 x its sign extension.  A product of two such bytes is 256 x
// the nibbles' product, so an int32 sum of them is 256 x the nibble sum
// (exact while |sum| < 2^23) and an arithmetic shift by 8 recovers it; five
// integer operations per word instead of the unpack and sign extension.
__device__ __forceinline__ void unpack4_hi_u32(uint32_t x, uint32_t& out0, uint32_t& out1)
{
    const uint32_t even = (x << 4) & 0xF0F0F0F0u, odd = x & 0xF0F0F0F0u;
    out0 = prmt(even, odd, 0x5140);
    out1 = prmt(even, odd, 0x7362);
}

// Combine a low-nibble plane word and a high-nibble plane word (each four
// nibbles in the low 16 bits) into four bytes (hi << 4 | lo).
__device__ __forceinline__ uint32_t merge_nibble_planes(uint32_t lo16, uint32_t hi16)
{
    uint32_t lo = prmt(lo16 & 0x0F0Fu, (lo16 >> 4) & 0x0F0Fu, 0x5140);
    uint32_t hi = prmt(hi16 & 0x0F0Fu, (hi16 >> 4) & 0x0F0Fu, 0x5140);
    return lo | (hi << 4);
}

// Exact int8 / uint8 -> f16 conversion of the four bytes of a word into two
// f16x2 registers (bytes 0,1 and bytes 2,3).  A byte u placed under the f16
// pattern 0x64 is the half 1024 + u (exact: f16 has an 11-bit significand);
// signed bytes are first biased by 128 (xor 0x80).  Subtracting the bias is
// exact because every intermediate is an integer below 2048.
__device__ __forceinline__ uint32_t hsub2(uint32_t a, uint32_t b)
{
    uint32_t r;
    asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
}
template <bool SIGNED>
__device__ __forceinline__ void bytes_to_h2(uint32_t w, uint32_t& lo, uint32_t& hi)
{
    const uint32_t x = SIGNED ? (w ^ 0x80808080u) : w;
    const uint32_t bias = SIGNED ? 0x64806480u : 0x64006400u;  // f16x2 (1152, 1152) or (1024, 1024)
    lo = hsub2(prmt(x, 0x64646464u, 0x5140), bias);
    hi = hsub2(prmt(x, 0x64646464u, 0x5342), bias);
}

// f32 accumulator holding an exact integer -> int32.
__device__ __forceinline__ int f2i_exact(float f) { return __float2int_rn(f); }

// e^y for the softmax: 2^(y log2 e) on the MUFU unit (ex2.approx, relative
// error about 2^-22), results below 2^-126 flushed to zero.  A flushed term
// cannot change a row sum that contains e^0 = 1, and it quantizes to 0 for
// any probability scale below 2^126, so the flush changes no output there;
// without it the non-flushing ex2 needs extra instructions around the MUFU
// operation in this (non-ftz) build.  The separate and the fused softmax both
// use it, which keeps them bit-identical.
__device__ __forceinline__ float exp_flush(float y)
{
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(__fmul_rn(y, 1.4426950408889634f)));
    return r;
}

// float -> int for |f| < 2^22 on the FMA and integer pipes instead of the
// quarter-rate conversion unit: f + 1.5 * 2^23 lies in [2^23, 2^24), where
// the f32 spacing is 1, so rounding the sum rounds f to an integer, and the
// sum's bit pattern is 0x4B400000 plus that integer.
// f2i_rn_small(f) == __float2int_rn(f) (nearest, ties to even);
// f2i_rz_small(f) == (int)f (toward zero).  Both are checked against the
// conversion instructions for every float with |f| < 2^22
// (mcCheckSmallIntConversions).  Worth it where the conversion unit is the
// bottleneck (the dense-tile SDDMM epilogue); elsewhere the extra issue slots
// cost more than they save (measured slower in the softmax).
__device__ __forceinline__ int f2i_rn_small(float f)
{
    return __float_as_int(__fadd_rn(f, 12582912.0f)) - 0x4B400000;
}
__device__ __forceinline__ int f2i_rz_small(float f)
{
    const int m = __float_as_int(__fadd_rz(fabsf(f), 12582912.0f)) - 0x4B400000;
    return f < 0.f ? -m : m;
}

// Byte mask keeping the first `valid` (clamped to 0..4) bytes of a word.
__device__ __forceinline__ uint32_t byte_mask(int valid)
{
    return valid >= 4 ? 0xffffffffu : (valid <= 0 ? 0u : ((1u << (8 * valid)) - 1u));
}

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(smem)), "l"(gmem));
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_u32(smem)), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ uint32_t lds32(const void* p)
{
    uint32_t v;
    asm volatile("ld.shared.b32 %0, [%1];" : "=r"(v) : "r"(smem_u32(p)));
    return v;
}
__device__ __forceinline__ uint2 lds64(const void* p)
{
    uint2 v;
    asm volatile("ld.shared.v2.b32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(smem_u32(p)));
    return v;
}
__device__ __forceinline__ uint32_t lds16(const void* p)
{
    unsigned short v;
    asm volatile("ld.shared.u16 %0, [%1];" : "=h"(v) : "r"(smem_u32(p)));
    return v;
}

__device__ __forceinline__ int4 ldg_nc_v4(const void* p)
{
    int4 v;
    asm volatile("ld.global.nc.v4.s32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
    return v;
}
__device__ __forceinline__ int2 ldg_nc_v2(const void* p)
{
    int2 v;
    asm volatile("ld.global.nc.v2.s32 {%0,%1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}

// Streaming stores: outputs are written once and not re-read by this kernel.
__device__ __forceinline__ void stg_cs_v4(void* p, int a, int b, int c, int d)
{
    asm volatile("st.global.cs.v4.s32 [%0], {%1,%2,%3,%4};" ::"l"(p), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}
__device__ __forceinline__ void stg_cs_v2(void* p, int a, int b)
{
    asm volatile("st.global.cs.v2.s32 [%0], {%1,%2};" ::"l"(p), "r"(a), "r"(b) : "memory");
}
__device__ __forceinline__ void stg_cs_s32(void* p, int a)
{
    asm volatile("st.global.cs.s32 [%0], %1;" ::"l"(p), "r"(a) : "memory");
}

// A divisor prepared once for many correctly rounded quotients a / d.
// r = RN(1/d) where the fast quotient below applies (|d| in [2^-60, 2^60]),
// else 0 (the quotient then uses the IEEE division).
struct Divisor {
    float d, r;
};
__device__ __forceinline__ Divisor make_divisor(float d)
{
    const float ad = fabsf(d);
    return {d, (ad >= 0x1p-60f && ad <= 0x1p60f) ? __frcp_rn(d) : 0.f};
}

// RN(a / d) by Markstein's correction step (P. Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Develop. 34(1), 1990): with y = RN(1/d) and a quotient q within one ulp of
// a/d, the remainder a - q d is exact in one FMA and RN(q + (a - q d) y) is
// the correctly rounded quotient.  q0 = RN(a y) can be up to 1.5 ulps off,
// so a first correction makes it faithful and a second one rounds it
// correctly.  Valid for |a| < 2^32 (integer accumulators) with |d| in
// [2^-60, 2^60]: no step overflows or leaves the normal range.  Checked bit
// for bit against __fdiv_rn over every int32 numerator (mcCheckQuotients).
__device__ __forceinline__ float div_rn(float a, Divisor v)
{
    if (v.r == 0.f) return __fdiv_rn(a, v.d);
    float q = __fmul_rn(a, v.r);
    float r = __fmaf_rn(-q, v.d, a);
    q = __fmaf_rn(r, v.r, q);
    r = __fmaf_rn(-q, v.d, a);
    return __fmaf_rn(r, v.r, q);
}

// Dequantised half output: half(float(acc) / scale), both steps rounded to
// nearest -- the epilogue of the reference's extension kernels
// (sparse_transformer_magicube/src/cuda/spmm_utils/output_tile.h:119).
__device__ __forceinline__ __half deq_half(int acc, Divisor v)
{
    return __float2half_rn(div_rn(__int2float_rn(acc), v));
}
// Two quotients at once, a0 / v0.d and a1 / v1.d: the steps of div_rn on
// packed f32x2 operations (Blackwell).  Each lane rounds as the scalar
// instruction does, and the residual is formed as q * (-d) + a, the same
// product as (-q) * d, so both results equal div_rn's bit for bit.
__device__ __forceinline__ float2 div_rn2(float a0, float a1, Divisor v0, Divisor v1)
{
    if (v0.r == 0.f || v1.r == 0.f) return make_float2(div_rn(a0, v0), div_rn(a1, v1));
    unsigned long long A, R, ND, q, e;
    asm("mov.b64 %0, {%1, %2};" : "=l"(A) : "f"(a0), "f"(a1));
    asm("mov.b64 %0, {%1, %2};" : "=l"(R) : "f"(v0.r), "f"(v1.r));
    asm("mov.b64 %0, {%1, %2};" : "=l"(ND) : "f"(-v0.d), "f"(-v1.d));
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(q) : "l"(A), "l"(R));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(e) : "l"(q), "l"(ND), "l"(A));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(q) : "l"(e), "l"(R), "l"(q));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(e) : "l"(q), "l"(ND), "l"(A));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(q) : "l"(e), "l"(R), "l"(q));
    float lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(q));
    return make_float2(lo, hi);
}

// half(a / v.d) and half(b / v.d) packed (a in the low half), as deq_half.
__device__ __forceinline__ uint32_t pack_half2(int a, int b, Divisor v)
{
    const float2 q = div_rn2(__int2float_rn(a), __int2float_rn(b), v, v);
    __half2 h = __floats2half2_rn(q.x, q.y);
    return *reinterpret_cast<uint32_t*>(&h);
}
// Two integers with their own divisors -> two halves.
__device__ __forceinline__ __half2 deq_half2(int a, int b, Divisor va, Divisor vb)
{
    const float2 q = div_rn2(__int2float_rn(a), __int2float_rn(b), va, vb);
    return __floats2half2_rn(q.x, q.y);
}

}  // namespace mc
