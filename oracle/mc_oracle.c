/*
 * mc_oracle.c -- CPU oracle for the quantized vector-sparse SpMM / SDDMM path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests, the smoke entry
 * point and the CPU-baseline leg of the benchmark call it to verify or time the
 * CUDA library.  The product path never links, loads or calls it.
 *
 * It restates, in plain C, the reference's host verification routines:
 *   - compute_ref_integers   SpMM/SpMM/spmm_benchmark.cpp:69-120
 *   - Host_sddmm_integers    SDDMM/SDDMM/sddmm_benchmark.cpp:24-60
 * following their loop order, plus a decoder of the device-side operand layout
 * produced by the reference's host packer (spmm_benchmark.cpp:177-377), which
 * specifies what the GPU kernels consume.
 *
 * Lane semantics ("mode"):
 *   MCO_LITERAL  exactly the reference routines: every SpMM lhs lane is
 *                unsigned (masked with maskA_cut, spmm_benchmark.cpp:101); the
 *                top lane of each packed rhs int is sign-extended by the signed
 *                ">>" (spmm_benchmark.cpp:106); in SDDMM the top lane of both
 *                operands is sign-extended (sddmm_benchmark.cpp:48-49).
 *   MCO_UNSIGNED every lane unsigned: the semantics of the reference's GPU
 *                kernels (mma .u8.u8 / .u4.u4, wmma_spmm.cu, wmma_sddmm.cu).
 *   MCO_SIGNED   every lane two's-complement (int4 / int8 / int16).
 * Accumulation wraps modulo 2^32 (uint32 arithmetic), as the reference's int
 * accumulators do in practice.
 */
#include <stdint.h>
#include <string.h>

enum { MCO_LITERAL = 0, MCO_UNSIGNED = 1, MCO_SIGNED = 2 };
enum { MCO_OUT_BLOCKED = 0, MCO_OUT_VECMAJOR = 1 };

/* Lane `lane` of `bits` bits of a little-endian bit stream (reads only the
 * bytes that hold it). */
static inline uint32_t lane_u(const uint8_t* p, int64_t lane, int bits)
{
    int64_t bit = lane * bits;
    uint32_t w = 0;
    int nbytes = (bits + (int)(bit % 8) + 7) / 8;
    for (int b = 0; b < nbytes; ++b) w |= (uint32_t)p[bit / 8 + b] << (8 * b);
    w >>= (bit % 8);
    return w & ((bits >= 32) ? 0xffffffffu : ((1u << bits) - 1u));
}

static inline int32_t sext(uint32_t v, int bits)
{
    uint32_t m = 1u << (bits - 1);
    return (int32_t)((v ^ m) - m);
}

/* Value of lane `lane` (0-based within its packed 32-bit word) of width `bits`
 * under `mode`; `top` marks the most significant lane of the word. */
static inline int32_t lane_val(uint32_t raw, int bits, int mode, int top)
{
    if (mode == MCO_SIGNED) return sext(raw, bits);
    if (mode == MCO_LITERAL && top) return sext(raw, bits);
    return (int32_t)raw;
}

/*
 * SpMM on the original (unpacked) operand layout.
 * Restates compute_ref_integers (SpMM/SpMM/spmm_benchmark.cpp:69-120).
 *
 * values       one packed vector per nonzero: V lanes of preA bits, lane v at
 *              bit v*preA (this is the TypeA/scaleA container of the reference,
 *              read as bytes: spmm_benchmark.cpp:89-99).
 * rhs          K x N, preB-bit lanes packed little-endian into int32,
 *              N*preB/32 ints per row.
 * out          M x N int32 row-major, M = m_vec*V; overwritten.
 * row_offsets  plain CSR offsets, m_vec+1 entries; col_indices unpadded.
 * preA_cut     number of valid low bits of each lhs lane (12 for the 12-bit
 *              variants stored in 16-bit containers, else preA).
 */
void mco_spmm_host(const uint8_t* values, const int32_t* rhs, int32_t* out,
                   int m_vec, int V, int K, int N, int preA, int preA_cut, int preB,
                   const int32_t* row_offsets, const int32_t* col_indices, int mode)
{
    (void)K;
    const int M = m_vec * V;
    uint32_t* acc = (uint32_t*)out;
    memset(out, 0, sizeof(int32_t) * (size_t)M * (size_t)N);
    const int b_tile = 32 / preB;
    const int ints_per_row = N / b_tile;
    const uint32_t cut_mask = (preA_cut >= 32) ? 0xffffffffu : ((1u << preA_cut) - 1u);
    const int vec_bytes = (V * preA + 7) / 8;
    for (int i = 0; i < m_vec; ++i) {
        for (int j = row_offsets[i]; j < row_offsets[i + 1]; ++j) {
            const int col = col_indices[j];
            const uint8_t* vec = values + (size_t)j * vec_bytes;
            for (int av = 0; av < V; ++av) {
                const int row = i * V + av;
                uint32_t raw = lane_u(vec, av, preA) & cut_mask;
                /* MCO_LITERAL, L16-R16: the reference keeps those values in
                 * `short` containers (spmm_benchmark.cpp:829-831), where
                 * maskA and maskA_cut are (short)0xFFFF == -1 (:77-79), so
                 * the lane is used sign-extended (:96). */
                int32_t a = (mode == MCO_SIGNED || (mode == MCO_LITERAL && preA == 16 && preB == 16))
                                ? sext(raw, preA_cut)
                                : (int32_t)raw;
                const uint32_t* brow = (const uint32_t*)rhs + (size_t)col * ints_per_row;
                uint32_t* crow = acc + (size_t)row * N;
                for (int n = 0; n < ints_per_row; ++n) {
                    uint32_t w = brow[n];
                    for (int bv = 0; bv < b_tile; ++bv) {
                        uint32_t braw = (w >> (bv * preB)) & ((preB == 32) ? 0xffffffffu : ((1u << preB) - 1u));
                        int32_t b = lane_val(braw, preB, mode, bv == b_tile - 1);
                        crow[n * b_tile + bv] += (uint32_t)a * (uint32_t)b;
                    }
                }
            }
        }
    }
}

/*
 * SDDMM.  Restates Host_sddmm_integers (SDDMM/SDDMM/sddmm_benchmark.cpp:24-60)
 * and generalises it to preA != preB (the reference asserts a_tiles==b_tiles,
 * :42): element l of a row is lane l % (32/pre) of int l / (32/pre), and the
 * top-lane rule of MCO_LITERAL is applied per operand.
 *
 * lhs  M x K packed (K*preA/32 ints per row); rhs  N x K packed.
 * row_offsets  aligned [start, end) pairs (2*m_vec ints); col_indices aligned
 *              and padded with -1 (only [start, end) is read).
 * out_layout   MCO_OUT_BLOCKED: out[(j/align)*align*V + align*v + j%align]
 *              (sddmm_benchmark.cpp:55); MCO_OUT_VECMAJOR: out[j*V + v] (the
 *              layout of the torch extension's SDDMM, deq_sddmm_kernel.cu).
 * Positions of padding slots are not written.
 */
void mco_sddmm_host(const int32_t* lhs, const int32_t* rhs, int32_t* out,
                    int m_vec, int V, int K, int N, int preA, int preB,
                    const int32_t* row_offsets, const int32_t* col_indices,
                    int alignment, int out_layout, int mode)
{
    (void)N;
    const int a_tiles = 32 / preA, b_tiles = 32 / preB;
    const uint32_t ma = (1u << preA) - 1u, mb = (1u << preB) - 1u;
    const uint32_t* A = (const uint32_t*)lhs;
    const uint32_t* B = (const uint32_t*)rhs;
    for (int i = 0; i < m_vec; ++i) {
        for (int j = row_offsets[2 * i]; j < row_offsets[2 * i + 1]; ++j) {
            const int idx_n = col_indices[j];
            for (int v = 0; v < V; ++v) {
                const int idx_m = i * V + v;
                uint32_t accu = 0;
                const uint32_t* arow = A + (size_t)idx_m * (K / a_tiles);
                const uint32_t* brow = B + (size_t)idx_n * (K / b_tiles);
                for (int l = 0; l < K; ++l) {
                    int la = l % a_tiles, lb = l % b_tiles;
                    uint32_t araw = (arow[l / a_tiles] >> (la * preA)) & ma;
                    uint32_t braw = (brow[l / b_tiles] >> (lb * preB)) & mb;
                    int32_t a = lane_val(araw, preA, mode, la == a_tiles - 1);
                    int32_t b = lane_val(braw, preB, mode, lb == b_tiles - 1);
                    accu += (uint32_t)a * (uint32_t)b;
                }
                size_t pos = (out_layout == MCO_OUT_BLOCKED)
                    ? (size_t)(j / alignment) * alignment * V + (size_t)alignment * v + (j % alignment)
                    : (size_t)j * V + v;
                out[pos] = (int32_t)accu;
            }
        }
    }
}

/*
 * Decoder of the SpMM device operand layout, i.e. the arrays the reference's
 * host packer hands to spmm::wmmaSpmm_* (spmm_benchmark.cpp:177-377,421-431):
 *   row_offsets  2*m_vec ints, [start, end) per vector-row, start aligned to
 *                mma_k (32 when preA_cut == 4 or preB == 4, else 16);
 *   col_indices  aligned, -1 padded; when mma_k == 32 each group of 8 is
 *                stored as [c0 c2 c4 c6 c1 c3 c5 c7] (:218-222);
 *   values       per chunk of mma_k vector slots, `planes` bit-planes, each a
 *                [V][mma_k] array of plane_bits-bit elements (element (v, j) at
 *                element index v*mma_k + j); planes are the low..high slices
 *                of the lhs value: L8-R8 one 8-bit plane; L4-R4 one 4-bit plane;
 *                L8-R4 two 4-bit planes (:253-270); L16-R8 two 8-bit planes
 *                (lo, hi byte, :337-344); L16-R4 four 4-bit planes (:288-335).
 * Computes out (M x N int32, overwritten) = A * B with the lane semantics of
 * `mode` (MCO_UNSIGNED or MCO_SIGNED; in MCO_SIGNED the top plane is signed).
 */
void mco_spmm_device(const int32_t* row_offsets, const int32_t* col_indices,
                     const uint8_t* values, const int32_t* rhs, int32_t* out,
                     int m_vec, int V, int K, int N, int preA, int preB, int mode, int layout)
{
    (void)K;
    const int mma_k = (preA == 4 || preB == 4) ? 32 : 16;
    /* layout 0: the packer's (above).  layout 1: the layout the extension's
     * quantized softmax writes (q_softmax_kernel.cu:133-176,258-269): chunks of
     * 16 slots ([v][16] bytes for 8-bit, [v][low 16][high 16] for 16-bit) or
     * of 32 slots for 4-bit ([v][32] nibbles); column indices unshuffled. */
    const int softmax = layout == 1;
    const int chunk = softmax ? (preA == 4 ? 32 : 16) : mma_k;
    const int plane_bits = chunk == 32 ? 4 : 8;
    const int planes = preA / plane_bits;
    const int interleaved = softmax && preA == 16;
    const int chunk_bytes = V * chunk * preA / 8;
    const int plane_elems = interleaved ? chunk : V * chunk;
    const int vstride = interleaved ? planes * chunk : chunk;
    const int b_tile = 32 / preB;
    const int ints_per_row = N / b_tile;
    const uint32_t mb = (1u << preB) - 1u;
    const int M = m_vec * V;
    uint32_t* acc = (uint32_t*)out;
    memset(out, 0, sizeof(int32_t) * (size_t)M * (size_t)N);
    for (int i = 0; i < m_vec; ++i) {
        const int start = row_offsets[2 * i], end = row_offsets[2 * i + 1];
        for (int j = start; j < end; ++j) {
            int stored = j;
            if (mma_k == 32 && !softmax) {
                int p = j % 8;  /* logical position p lives at shuffled slot */
                stored = (j / 8) * 8 + (p % 2) * 4 + p / 2;
            }
            const int col = col_indices[stored];
            const int ci = j / chunk, jj = j % chunk;
            const uint8_t* cbase = values + (size_t)ci * chunk_bytes;
            for (int v = 0; v < V; ++v) {
                uint32_t raw = 0;
                for (int p = 0; p < planes; ++p)
                    raw |= lane_u(cbase, (int64_t)p * plane_elems + (int64_t)v * vstride + jj, plane_bits) << (p * plane_bits);
                int32_t a = (mode == MCO_SIGNED) ? sext(raw, planes * plane_bits) : (int32_t)raw;
                const uint32_t* brow = (const uint32_t*)rhs + (size_t)col * ints_per_row;
                uint32_t* crow = acc + (size_t)(i * V + v) * N;
                for (int n = 0; n < ints_per_row; ++n) {
                    uint32_t w = brow[n];
                    for (int bv = 0; bv < b_tile; ++bv) {
                        uint32_t braw = (w >> (bv * preB)) & mb;
                        int32_t b = (mode == MCO_SIGNED) ? sext(braw, preB) : (int32_t)braw;
                        crow[n * b_tile + bv] += (uint32_t)a * (uint32_t)b;
                    }
                }
            }
        }
    }
}

/* Sequential multiply-accumulate count of one SpMM / SDDMM call, for timing. */
double mco_spmm_ops(const int32_t* row_offsets, int m_vec, int V, int N)
{
    return 2.0 * (double)(row_offsets[m_vec] - row_offsets[0]) * V * N;
}
