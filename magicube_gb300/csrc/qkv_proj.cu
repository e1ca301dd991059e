// qkv_proj.cu -- the attention's input projection with the quantization fused
// into its epilogue, on the 5th-generation tensor cores.
//
// out[which][h][t][c] = trunc(clamp(float(half(x[t] . W[n] + b[n])) * scale))
// with n = which*E + h*d + c: the reference computes the projection in fp16
// (F.linear, end2end_eval/sparse_transformer_magicube/spattention.py:189-191),
// permutes it to [3][H][T][d] and quantizes it with bquantization
// (quantization_kernel.cu:173-213).  Here one kernel reads x and W once and
// writes the packed int8 (or int4) operands of the SDDMM / SpMM directly.
//
// Persistent CTAs of 12 warps, each owning one BN-column tile of W for the
// whole launch and a stride of 128-token tiles:
//  * warp 0 (one thread): TMA producer -- the W tile once (resident in shared
//    memory), then 128 x 64 f16 boxes of x through a 6-stage ring;
//  * warp 1: allocates 2 x BN TMEM columns (two accumulators); one thread
//    issues tcgen05.mma kind::f16 (M = 128, N = BN, K = 16) from the swizzled
//    shared-memory tiles and commits to the ring's "empty" barriers and to
//    the accumulator's "full" barrier;
//  * warps 4-11: epilogue -- warps 4+q and 8+q read TMEM lanes 32q..32q+31
//    (one token each), half of the columns each: bias, rounding to half,
//    scaling, truncation, packing, 16-byte stores of whole (token, head)
//    rows; then they release the accumulator, so the epilogue of one tile
//    overlaps the MMAs of the next.
// Every mbarrier wait is bounded; a timeout sets *status = 1 and the CTA
// winds down (waiting, bounded again, for its own copies and MMAs) instead
// of hanging.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstdint>

#include "mc_host.h"
#include "mc_sm100.cuh"
#include "mc_tma_host.h"

namespace mc {
namespace {

using namespace sm100;

constexpr int BM = 128;                        // tokens per tile (MMA M, TMEM lanes)
constexpr int BK = 64;                         // f16 per 128-byte swizzled row
constexpr int STAGES = 6;                      // x ring depth (6 x 16 KB beside a 128 KB W tile)
constexpr int X_STAGE_BYTES = BM * BK * 2;     // 16 KB
constexpr long long WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz

struct ProjParams {
    int tokens, hidden, heads, head_dim, n_total, bits;
    float scale;
    const __half* bias;  // may be null
    uint8_t* out;
    int* status;
};

// CH consecutive f32 columns of this thread's TMEM lane (CH = 32 or 64).
template <int CH>
__device__ __forceinline__ void tmem_ld_chunk(uint32_t taddr, uint32_t (&r)[CH])
{
    tmem_ld_x32(taddr, *reinterpret_cast<uint32_t(*)[32]>(&r[0]));
    if constexpr (CH == 64) tmem_ld_x32(taddr + 32, *reinterpret_cast<uint32_t(*)[32]>(&r[32]));
}

// Orders every use of r after the preceding tcgen05.wait::ld: the registers
// are redefined by an (empty) volatile asm that the compiler cannot move
// above the wait.
template <int CH>
__device__ __forceinline__ void tmem_reg_fence(uint32_t (&r)[CH])
{
#pragma unroll
    for (int i = 0; i < CH; i += 8)
        asm volatile("" : "+r"(r[i]), "+r"(r[i + 1]), "+r"(r[i + 2]), "+r"(r[i + 3]), "+r"(r[i + 4]),
                     "+r"(r[i + 5]), "+r"(r[i + 6]), "+r"(r[i + 7])::"memory");
}

// q = trunc(clamp(float(half(acc + bias)) * scale)) for CH columns, packed
// little-endian (8-bit: 4 per word; 4-bit: 8 per word, low nibble first).
// fmaxf maps NaN to the lower bound as the reference's clamp does; for 8 bits
// the saturating conversion then does the upper clamp and the truncation.
template <int CH, int BITS>
__device__ __forceinline__ void quantize_chunk(const uint32_t (&r)[CH], const float* bias, float scale,
                                               uint32_t (&packed)[CH * BITS / 32])
{
#pragma unroll
    for (int e = 0; e < CH; e += 4) {
        int qv[4];
#pragma unroll
        for (int k = 0; k < 4; k += 2) {
            const __half2 h = __floats2half2_rn(__uint_as_float(r[e + k]) + bias[e + k],
                                                __uint_as_float(r[e + k + 1]) + bias[e + k + 1]);
            const float2 f = __half22float2(h);
            const float fx = f.x * scale, fy = f.y * scale;
            if constexpr (BITS == 8) {
                asm("cvt.rzi.sat.s8.f32 %0, %1;" : "=r"(qv[k]) : "f"(fmaxf(fx, -128.f)));
                asm("cvt.rzi.sat.s8.f32 %0, %1;" : "=r"(qv[k + 1]) : "f"(fmaxf(fy, -128.f)));
            } else {
                qv[k] = (int)fminf(fmaxf(fx, -8.f), 7.f);
                qv[k + 1] = (int)fminf(fmaxf(fy, -8.f), 7.f);
            }
        }
        if constexpr (BITS == 8) {
            packed[e / 4] = __byte_perm(__byte_perm(qv[0], qv[1], 0x0040), __byte_perm(qv[2], qv[3], 0x0040), 0x5410);
        } else {
            const uint32_t w = (qv[0] & 0xF) | (qv[1] & 0xF) << 4 | (qv[2] & 0xF) << 8 | (qv[3] & 0xF) << 12;
            if ((e & 4) == 0) packed[e / 8] = w;
            else packed[e / 8] |= w << 16;
        }
    }
}

template <int BN, int BITS>
__global__ void __launch_bounds__(384, 1)
qkv_proj_quant_kernel(const __grid_constant__ CUtensorMap tmap_x, const __grid_constant__ CUtensorMap tmap_w,
                      const ProjParams p)
{
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = saddr(smem_raw);
    uint8_t* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);  // 1024-byte aligned (swizzle atoms)
    const int K = p.hidden, KB = K / BK;
    uint8_t* w_s = smem;                                         // KB x [BN rows x 128 B]
    uint8_t* x_s = w_s + (size_t)KB * BN * 128;                  // STAGES x [128 rows x 128 B]
    uint64_t* bars = reinterpret_cast<uint64_t*>(x_s + STAGES * X_STAGE_BYTES);
    uint64_t* full = bars;                  // [STAGES]
    uint64_t* empty = bars + STAGES;        // [STAGES]
    uint64_t* w_full = bars + 2 * STAGES;   // [1]
    uint64_t* acc_full = w_full + 1;        // [2]
    uint64_t* acc_empty = acc_full + 2;     // [2]
    uint64_t* drain = acc_empty + 2;        // [1]
    uint32_t* tmem_base_s = reinterpret_cast<uint32_t*>(drain + 1);
    volatile int* abort_s = reinterpret_cast<volatile int*>(tmem_base_s + 1);
    float* bias_s = reinterpret_cast<float*>(tmem_base_s + 4);   // [BN]

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n_tiles = p.n_total / BN;
    const int n_tile = blockIdx.x % n_tiles;
    const int n0 = n_tile * BN;
    const int m_tiles = (p.tokens + BM - 1) / BM;
    const int m_first = blockIdx.x / n_tiles, m_stride = gridDim.x / n_tiles;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(w_full, 1);
        for (int a = 0; a < 2; ++a) {
            mbar_init(&acc_full[a], 1);
            mbar_init(&acc_empty[a], 256);
        }
        mbar_init(drain, 1);
        *abort_s = 0;
        fence_mbar_init();
    }
    if (warp == 1) {
        tmem_alloc(tmem_base_s, 2 * BN);
        tmem_relinquish();
    }
    if (threadIdx.x >= 128) {
        for (int i = threadIdx.x - 128; i < BN; i += 256)
            bias_s[i] = p.bias ? __half2float(p.bias[n0 + i]) : 0.f;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_base_s;

    auto fail = [&]() {
        *abort_s = 1;
        if (p.status) atomicExch(p.status, 1);
    };

    if (warp == 0 && lane == 0) {
        // ---- TMA producer ----
        prefetch_tmap(&tmap_x);
        prefetch_tmap(&tmap_w);
        mbar_arrive_expect_tx(w_full, (uint32_t)(KB * BN * 128));
        for (int kb = 0; kb < KB; ++kb) tma_load_2d(w_s + (size_t)kb * BN * 128, &tmap_w, w_full, kb * BK, n0);
        int it = 0;
        for (int m = m_first; m < m_tiles && !*abort_s; m += m_stride) {
            for (int kb = 0; kb < KB; ++kb, ++it) {
                const int s = it % STAGES;
                const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
                if (!mbar_wait(&empty[s], ph ^ 1u, WAIT_CYCLES)) { fail(); break; }
                mbar_arrive_expect_tx(&full[s], X_STAGE_BYTES);
                tma_load_2d(x_s + s * X_STAGE_BYTES, &tmap_x, &full[s], kb * BK, m * BM);
            }
        }
        // Every copy this thread issued has landed before the CTA exits: the
        // newest fill of each stage (older fills were consumed) and W.
        for (int j = it - 1; j >= 0 && j >= it - STAGES; --j)
            if (!mbar_wait(&full[j % STAGES], (uint32_t)(j / STAGES) & 1u, WAIT_CYCLES)) fail();
        if (!mbar_wait(w_full, 0, WAIT_CYCLES)) fail();
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer ----
        constexpr uint32_t idesc = idesc_f16_f32(BM, BN);
        const uint32_t w_addr = saddr(w_s), x_addr = saddr(x_s);
        bool ok = mbar_wait(w_full, 0, WAIT_CYCLES);
        if (!ok) fail();
        int it = 0, u = 0;
        for (int m = m_first; ok && m < m_tiles && !*abort_s; m += m_stride, ++u) {
            const int a = u & 1;
            if (!mbar_wait(&acc_empty[a], ((uint32_t)(u >> 1) & 1u) ^ 1u, WAIT_CYCLES)) { fail(); break; }
            tc_fence_after();
            const uint32_t d_tmem = tmem + (uint32_t)(a * BN);
            for (int kb = 0; kb < KB; ++kb, ++it) {
                const int s = it % STAGES;
                if (!mbar_wait(&full[s], (uint32_t)(it / STAGES) & 1u, WAIT_CYCLES)) { fail(); ok = false; break; }
                tc_fence_after();
                const uint64_t ad = desc_sw128_kmajor(x_addr + s * X_STAGE_BYTES);
                const uint64_t bd = desc_sw128_kmajor(w_addr + kb * BN * 128);
#pragma unroll
                for (int k = 0; k < BK / 16; ++k)  // 16 f16 = 32 bytes = 2 descriptor units per step
                    mma_f16_ss(d_tmem, ad + 2 * k, bd + 2 * k, idesc, (kb | k) != 0);
                mma_commit(&empty[s]);  // frees the x stage once these MMAs are done
            }
            if (!ok) break;
            mma_commit(&acc_full[a]);
        }
        // All MMAs complete before TMEM is released.
        mma_commit(drain);
        if (!mbar_wait(drain, 0, WAIT_CYCLES)) fail();
    } else if (warp >= 4) {
        // ---- epilogue: warps 4+q and 8+q own TMEM lanes 32q..32q+31 (one
        // token each) and split the tile's columns in halves ----
        constexpr int CW = BN / 2;             // columns per epilogue warp
        constexpr int CH = CW < 64 ? CW : 64;  // columns per chunk (within one head: d % 64 == 0)
        constexpr int NCH = CW / CH;
        const int q = warp & 3, part = (warp - 4) >> 2;
        const int row = 32 * q + lane;
        const int E = p.hidden, d = p.head_dim;
        const long long T = p.tokens;
        const float scale = p.scale;
        int u = 0;
        for (int m = m_first; m < m_tiles; m += m_stride, ++u) {
            // warp-uniform control flow around the .sync.aligned TMEM loads
            if (__any_sync(0xffffffffu, *abort_s != 0)) break;
            const int a = u & 1;
            const bool ok = mbar_wait(&acc_full[a], (uint32_t)(u >> 1) & 1u, WAIT_CYCLES);
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) fail();
                break;
            }
            tc_fence_after();
            const long long t = (long long)m * BM + row;
            const uint32_t tbase = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(a * BN + part * CW);
            // The loads of chunk i+1 are in flight while chunk i is converted.
            uint32_t r[2][CH];
            tmem_ld_chunk<CH>(tbase, r[0]);
            tmem_ld_wait();
            tmem_reg_fence<CH>(r[0]);
#pragma unroll
            for (int i = 0; i < NCH; ++i) {
                if (i + 1 < NCH) tmem_ld_chunk<CH>(tbase + (uint32_t)((i + 1) * CH), r[(i + 1) & 1]);
                const int c = part * CW + i * CH;  // tile column of the chunk
                uint32_t packed[CH * BITS / 32];
                quantize_chunk<CH, BITS>(r[i & 1], bias_s + c, scale, packed);
                if (t < T) {
                    const int n = n0 + c;
                    const int which = n / E, h = (n % E) / d, cc = n % d;
                    const long long elem = (((long long)which * p.heads + h) * T + t) * d + cc;
                    uint4* dst = reinterpret_cast<uint4*>(p.out + elem * BITS / 8);
#pragma unroll
                    for (int v = 0; v < CH * BITS / 128; ++v)
                        dst[v] = make_uint4(packed[4 * v], packed[4 * v + 1], packed[4 * v + 2], packed[4 * v + 3]);
                }
                if (i + 1 < NCH) {
                    tmem_ld_wait();
                    tmem_reg_fence<CH>(r[(i + 1) & 1]);
                }
            }
            tc_fence_before();
            mbar_arrive(&acc_empty[a]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, 2 * BN);
    }
}

size_t proj_smem_bytes(int BN, int K)
{
    // alignment slack + W tile + x ring + (2 STAGES + 6) mbarriers + TMEM address / abort flag + bias
    return 1024 + (size_t)(K / BK) * BN * 128 + (size_t)STAGES * X_STAGE_BYTES + (2 * STAGES + 6) * 8 + 16 +
           (size_t)BN * 4;
}

// Row-major [rows][K] f16 matrix, boxes of box_rows x 64, 128-byte swizzle.
bool encode_kmajor(CUtensorMap* map, const void* base, long long rows, int K, int box_rows)
{
    auto fn = tensor_map_encoder();
    if (!fn) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
    const cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN, int BITS>
int proj_launch(const mcQkvProjDesc& d, const ProjParams& p, cudaStream_t s)
{
    CUtensorMap mx, mw;
    if (!encode_kmajor(&mx, d.x, d.tokens, d.hidden, BM) || !encode_kmajor(&mw, d.weight, p.n_total, d.hidden, BN))
        return fail(1, "mcQkvProjectQuantize: tensor map encoding failed");
    const size_t smem = proj_smem_bytes(BN, d.hidden);
    auto kern = qkv_proj_quant_kernel<BN, BITS>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return (int)cudaGetLastError();
    const int n_tiles = p.n_total / BN;
    const int m_tiles = (d.tokens + BM - 1) / BM;
    int per_n = sm_count() / n_tiles;
    if (per_n < 1) per_n = 1;
    if (per_n > m_tiles) per_n = m_tiles;
    kern<<<per_n * n_tiles, 384, smem, s>>>(mx, mw, p);
    return (int)cudaGetLastError();
}

}  // namespace
}  // namespace mc

extern "C" int mcQkvProjectQuantize(const mcQkvProjDesc* d, cudaStream_t stream)
{
    mc::clear_error();
    if (!d) return mc::fail(1, "mcQkvProjectQuantize: null descriptor");
    if (d->tokens < 0 || d->hidden < 64 || d->hidden > 256 || d->hidden % 64 || d->head_dim < 64 ||
        d->head_dim % 64 || d->heads < 1 || d->heads * d->head_dim != d->hidden)
        return mc::fail(1, "mcQkvProjectQuantize: need 64 <= hidden <= 256, hidden % 64 == 0, head_dim % 64 == 0, "
                           "heads * head_dim == hidden");
    if (d->bits != 8 && d->bits != 4) return mc::fail(1, "mcQkvProjectQuantize: bits must be 8 or 4");
    if (!std::isfinite(d->scale) || d->scale == 0.f) return mc::fail(1, "mcQkvProjectQuantize: bad scale");
    if (d->tokens == 0) return 0;
    auto al = [](const void* p, uintptr_t a) { return reinterpret_cast<uintptr_t>(p) % a == 0; };
    if (!d->x || !d->weight || !d->out || !al(d->x, 16) || !al(d->weight, 16) || !al(d->out, 16) ||
        (d->bias && !al(d->bias, 2)))
        return mc::fail(1, "mcQkvProjectQuantize: x, weight, out must be non-null and 16-byte aligned");
    mc::ProjParams p;
    p.tokens = d->tokens;
    p.hidden = d->hidden;
    p.heads = d->heads;
    p.head_dim = d->head_dim;
    p.n_total = 3 * d->hidden;
    p.bits = d->bits;
    p.scale = d->scale;
    p.bias = static_cast<const __half*>(d->bias);
    p.out = static_cast<uint8_t*>(d->out);
    p.status = d->status;
    const int n = p.n_total;
    if (n % 256 == 0)
        return d->bits == 8 ? mc::proj_launch<256, 8>(*d, p, stream) : mc::proj_launch<256, 4>(*d, p, stream);
    if (n % 128 == 0)
        return d->bits == 8 ? mc::proj_launch<128, 8>(*d, p, stream) : mc::proj_launch<128, 4>(*d, p, stream);
    return d->bits == 8 ? mc::proj_launch<64, 8>(*d, p, stream) : mc::proj_launch<64, 4>(*d, p, stream);
}
