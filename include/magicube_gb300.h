/*
 * magicube_gb300.h -- C ABI of the GB300 (sm_103a) quantized vector-sparse
 * SpMM / SDDMM library (libmagicube_gb300.so).
 *
 * All functions return a cudaError_t value as int: 0 on success,
 * cudaErrorInvalidValue (1) for rejected arguments (mcGetLastErrorString()
 * says why), or the CUDA error of the launch.  All pointers passed to compute
 * entry points are device pointers unless stated otherwise; buffers are owned
 * by the caller.  Nothing here allocates device memory except the
 * device-side format conversion entry points, which take their scratch from
 * the stream-ordered allocator (cudaMallocAsync / cudaFreeAsync on the
 * caller's stream).
 *
 * Storage format (identical to the reference's): a sparse M x K matrix is
 * stored as m_vec = M / V vector-rows of column vectors of V = 2, 4 or 8
 * rows.  row_offsets holds 2*m_vec ints, the [start, end) range of each
 * vector-row in the aligned slot arrays; each start is a multiple of the
 * alignment (SpMM: 16, or 32 when either operand is 4-bit; SDDMM: 8);
 * column_indices is aligned the same way and padded with -1.
 */
#ifndef MAGICUBE_GB300_H
#define MAGICUBE_GB300_H

#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Text of the last argument error on the calling thread ("" if none). */
const char* mcGetLastErrorString(void);
/* Library version, e.g. "0.1.0". */
const char* mcVersion(void);

/* ---- Reference-compatible SpMM entry points --------------------------------
 * Same arguments, layouts and unsigned-lane semantics as the reference's
 * spmm::wmmaSpmm_<P> (SpMM/SpMM/include/wmma_spmm.cuh:15-78), launched on the
 * legacy default stream.  output_matrix is M x N int32 row-major.
 * Requires n % 64 == 0.  values is the packer's device layout. */
int mcWmmaSpmm_4b(int m_vec, int vec_length, int n, int k, const int* row_indices,
                  const int* row_offsets, const int* column_indices, const int* values,
                  const int* rhs_matrix, int* output_matrix);    /* wmma_spmm.cuh:15 */
int mcWmmaSpmm_8b4b(int m_vec, int vec_length, int n, int k, const int* row_indices,
                    const int* row_offsets, const int* column_indices, const int* values,
                    const int* rhs_matrix, int* output_matrix);  /* wmma_spmm.cuh:23 */
int mcWmmaSpmm_16b4b(int m_vec, int vec_length, int n, int k, const int* row_indices,
                     const int* row_offsets, const int* column_indices, const int* values,
                     const int* rhs_matrix, int* output_matrix); /* wmma_spmm.cuh:39 */
int mcWmmaSpmm_8b(int m_vec, int vec_length, int n, int k, const int* row_indices,
                  const int* row_offsets, const int* column_indices, const int* values,
                  const int* rhs_matrix, int* output_matrix);    /* wmma_spmm.cuh:47 */
int mcWmmaSpmm_16b8b(int m_vec, int vec_length, int n, int k, const int* row_indices,
                     const int* row_offsets, const int* column_indices, const int* values,
                     const int* rhs_matrix, int* output_matrix); /* wmma_spmm.cuh:63 */
/* 12-bit values in the reference's 12-bit layouts (the 16-bit ones with the
 * top 4 bits clear) and 16-bit x 16-bit. */
int mcWmmaSpmm_12b4b(int m_vec, int vec_length, int n, int k, const int* row_indices,
                     const int* row_offsets, const int* column_indices, const int* values,
                     const int* rhs_matrix, int* output_matrix); /* wmma_spmm.cuh:31 */
int mcWmmaSpmm_12b8b(int m_vec, int vec_length, int n, int k, const int* row_indices,
                     const int* row_offsets, const int* column_indices, const int* values,
                     const int* rhs_matrix, int* output_matrix); /* wmma_spmm.cuh:55 */
int mcWmmaSpmm_16b(int m_vec, int vec_length, int n, int k, const int* row_indices,
                   const int* row_offsets, const int* column_indices, const int* values,
                   const int* rhs_matrix, int* output_matrix);   /* wmma_spmm.cuh:71 */

/* ---- Reference-compatible SDDMM entry points -------------------------------
 * Same arguments, layouts and unsigned-lane semantics as the reference's
 * sddmm::wmmaSddmm_<P> (SDDMM/SDDMM/src/wmma_sddmm.cu:394,439,488), legacy
 * default stream.  output_values uses the blocked layout
 * (j/8)*8*V + 8*v + j%8 over the aligned slots (alignment 8); padding slots of
 * each vector-row's last group of 8 are written as 0.  Requires k % 64 == 0. */
int mcWmmaSddmm_4b(int m_vec, int k, int n, const int* row_indices, const int* row_offsets,
                   const int* column_indices, const int* lhs_matrix, const int* rhs_matrix,
                   int* output_values, int vec_length);         /* wmma_sddmm.cu:394 */
int mcWmmaSddmm_8b(int m_vec, int k, int n, const int* row_indices, const int* row_offsets,
                   const int* column_indices, const int* lhs_matrix, const int* rhs_matrix,
                   int* output_values, int vec_length);         /* wmma_sddmm.cu:439 */
int mcWmmaSddmm_16b(int m_vec, int k, int n, const int* row_indices, const int* row_offsets,
                    const int* column_indices, const int* lhs_matrix, const int* rhs_matrix,
                    int* output_values, int vec_length);        /* wmma_sddmm.cu:488 */

/* ---- Tensor path ------------------------------------------------------------
 * Both tensor paths give bit-identical integer results.
 * MC_MMA_INT8: mma.sync m16n8k32 s8/u8 with int32 accumulation.
 * MC_MMA_F16:  operand bytes converted exactly to f16, mma.sync m16n8k16 with
 *              f32 accumulation flushed into int32 every 256 products (every
 *              partial sum is an integer below 2^24, so nothing rounds); on
 *              sm_103a the f16 tensor rate is several times the int8 one.
 * MC_MMA_DEFAULT selects the library default (mcSetDefaultMmaKind), except
 *              for the SDDMM L16-R8 at k == 64, which it runs on the f16 path
 *              (faster there on GB300: the 16-bit operand's two byte planes
 *              double the int8 MMAs). */
/* MC_MMA_TCGEN05 (SDDMM L8-R8 with k == 64 only): operands converted exactly
 *              to f16 in shared memory, tcgen05.mma kind::f16 (M = 128
 *              nonzeros, N = 16, K = 64) with the f32 accumulator in TMEM;
 *              exact because 64 products of 8-bit integers stay below 2^24. */
/* MC_MMA_DP4A (SDDMM with 8-bit or 4-bit operands): no tensor core; each
 *              vector lane is a chain of CUDA-core dp4a, so V = 2 and V = 4
 *              compute no padding lanes (an int8 MMA always computes 8). */
enum { MC_MMA_DEFAULT = 0, MC_MMA_INT8 = 1, MC_MMA_F16 = 2, MC_MMA_TCGEN05 = 3, MC_MMA_DP4A = 4 };
/* Number of bounded mbarrier waits that ran out in the tcgen05 SDDMM and the
 * TMA SpMM (0 unless the device stalled; an affected launch's results are
 * incomplete).  Synchronous. */
unsigned mcTensorCoreTimeouts(void);
/* Sets the default tensor path; returns the previous one (or -1 if invalid). */
int mcSetDefaultMmaKind(int kind);

/* ---- Kernel variant ---------------------------------------------------------
 * MC_KERNEL_PER_ROW: one CTA per (vector-row, column tile / row split, batch
 *                    entry); any k.
 * MC_KERNEL_STREAM:  the pipelined kernels: SpMM -- persistent CTAs that
 *                    stream many vector-rows through one cp.async ring (needs
 *                    16-byte aligned values); for n == 64 with 8-bit operands,
 *                    the softmax value layout and half output (the attention's
 *                    P x V) one warp per vector-row with a private ring that
 *                    carries the gathered rows and the probability chunks;
 *                    SDDMM -- the k == 64 kernel with a warp per 16-nonzero
 *                    tile at full occupancy (needs k == 64).
 * MC_KERNEL_TMA:     SpMM only, on the int8 path: persistent warp-specialised
 *                    CTAs -- one producer warp gathers B rows with TMA
 *                    (tile::gather4) into an mbarrier ring, consumer warps
 *                    multiply (needs 8-bit B with n % 128 == 0 or 4-bit B
 *                    with n % 256 == 0, 16-byte aligned values,
 *                    values_stride and rhs, rhs_stride a multiple of the B
 *                    row bytes).
 * MC_KERNEL_DENSE_TILE: SDDMM, 8-bit operands with k == 64: every score
 *                    of 128-column x 256-row tiles on the tcgen05 f16 tensor
 *                    cores (exact: 64 products of int8 values sum below 2^24),
 *                    accumulators in TMEM, and an epilogue that stores the
 *                    masked ones, located through the mask's tile bitmap
 *                    (mcSddmmTileMask; needs strictly increasing columns per
 *                    vector-row).  Computes every vector-row (row_indices is
 *                    not read).  Wins where the mask is dense enough that a
 *                    dense tile costs less than per-nonzero gathers (about
 *                    sparsity <= 0.95 on GB300).
 *                    SpMM, L8-R8 with int32 output and n % 128 == 0: each
 *                    256-row block of A is expanded into dense f16 tiles in
 *                    shared memory, 64 columns of k at a time, and multiplied
 *                    whole with B on the tcgen05 f16 tensor cores (exact:
 *                    k is accumulated in segments of at most 1024 columns,
 *                    256 with unsigned lanes, whose f32 sums stay within 2^24,
 *                    and the segments are added in int32).  Needs the chunk
 *                    table of mcSpmmChunkStarts (strictly increasing columns
 *                    per vector-row) in chunk_starts and 16-byte aligned
 *                    column indices; it reads MC_VALUES_PACKED or
 *                    MC_VALUES_SLOT_MAJOR values (the latter 16-byte aligned
 *                    with values_stride a multiple of 16); row_indices is not
 *                    read.
 *                    Its time does not depend on V or on the sparsity.
 * MC_KERNEL_RESIDENT: SpMM only, on the int8 path: each CTA holds a K x 64-byte
 *                    column slice of B in shared memory (loaded once by TMA)
 *                    and its warps gather the rows of their vector-rows'
 *                    nonzeros from there with ldmatrix (needs 8-bit B with
 *                    n % 64 == 0 or 4-bit B with n % 128 == 0, 4-, 8- or
 *                    16-bit A, k <= 3584, 16-byte aligned values,
 *                    values_stride and rhs, rhs_stride a multiple of the B
 *                    row bytes).
 * MC_KERNEL_AUTO:    SpMM: the TMA kernel where it applies, else the
 *                    streaming kernel (the warp-per-row one for the n == 64
 *                    attention shape), else per-row; SDDMM: the pipelined
 *                    kernel where it applies, else per-row. */
enum {
    MC_KERNEL_AUTO = 0, MC_KERNEL_PER_ROW = 1, MC_KERNEL_STREAM = 2, MC_KERNEL_TMA = 3, MC_KERNEL_DENSE_TILE = 4,
    MC_KERNEL_RESIDENT = 5
};

/* ---- Value layouts of the SpMM sparse operand --------------------------------
 * MC_VALUES_PACKED:  the reference host packer's layout (what
 *                    mcPackSpmmValues writes; column indices 8-shuffled when
 *                    either operand is 4-bit).
 * MC_VALUES_SOFTMAX: the layout the quantized softmax writes (mcQuantSoftmax;
 *                    the reference extension's q_softmax): chunks of 16 slots
 *                    [v][16] for 8-bit values, 32-slot nibble chunks for
 *                    4-bit, [v][low 16 bytes][high 16 bytes] for 16-bit;
 *                    column indices unshuffled.
 * int32 output is provided with MC_VALUES_PACKED, half output with
 * MC_VALUES_SOFTMAX (the combinations the reference uses). */
/* MC_VALUES_SLOT_MAJOR: 8-bit values as [aligned slot][V] bytes (the V lanes
 *                    of a slot contiguous; column indices unshuffled), what
 *                    mcPackSpmmValuesEx / mcDevicePack write for that
 *                    layout; read only by MC_KERNEL_DENSE_TILE (which
 *                    MC_KERNEL_AUTO then picks), whose builders load whole
 *                    slots instead of one byte per lane and chunk row.  No
 *                    reference counterpart. */
enum { MC_VALUES_PACKED = 0, MC_VALUES_SOFTMAX = 1, MC_VALUES_SLOT_MAJOR = 2 };

/* ---- Extended entry points: batch, stream, signedness, dequantised output --
 * These generalise the reference's batched extension kernels
 * (batched_wmmaSpmm_* in sparse_transformer_magicube/src/cuda/deq_spmm_kernel.cu,
 * batched_wmmaSddmm_* in deq_sddmm_kernel.cu): batch entries share one mask and
 * advance each operand by its stride (a zero stride shares the operand;
 * negative strides are rejected).
 * is_signed = 1 reads every lane as two's complement (16-bit values: signed
 * high byte, unsigned low byte); 0 reads lanes unsigned, as the reference's
 * GPU kernels do.  out_half = 1 writes half(float(acc) / scale). */
typedef struct mcSpmmDesc {
    int m_vec, vec_length, n, k;
    int lhs_bits, rhs_bits;     /* (4,4) (8,4) (12,4) (16,4) (8,8) (12,8) (16,8) (16,16);
                                   12-bit: unsigned lanes, int32 output */
    int is_signed;
    int out_half;
    float scale;
    int batch;                  /* >= 1 */
    const int* row_indices;
    const int* row_offsets;
    const int* column_indices;
    const void* values;   long long values_stride;  /* bytes */
    const void* rhs;      long long rhs_stride;     /* bytes */
    void* out;            long long out_stride;     /* elements */
    int mma_kind;               /* MC_MMA_DEFAULT / MC_MMA_INT8 / MC_MMA_F16 */
    int kernel_variant;         /* MC_KERNEL_AUTO / _PER_ROW / _STREAM / _TMA / _RESIDENT */
    int value_layout;           /* MC_VALUES_PACKED / _SOFTMAX / _SLOT_MAJOR */
    /* Optional, half output only: out[row][c] = half(acc / row_div[row]) per
     * output row (M = m_vec * vec_length floats per batch entry, e.g. the
     * divisors mcQuantSoftmax writes with MC_REQUANT_ROWMAX) instead of / scale. */
    const void* row_div;  long long row_div_stride;  /* floats between batch entries */
    /* MC_KERNEL_RESIDENT only: slice width and CTA size (MC_RESIDENT_*);
     * 0 = automatic.  Other variants ignore it. */
    int kernel_config;
    /* MC_KERNEL_DENSE_TILE only: the mask's chunk table (mcSpmmChunkStarts),
     * m_vec x mcSpmmChunkStartsCount(k) ints.  Other variants ignore it. */
    const int* chunk_starts;
} mcSpmmDesc;
/* Configurations of MC_KERNEL_RESIDENT: 64-byte slice rows (64 columns of
 * 8-bit B, 128 of 4-bit B) with 8 or 16 warps a CTA, 128-byte slice rows
 * (k <= 1792, n a multiple of 128 / 256 columns) with 16 warps.  The
 * 16-warp ones run V = 8 on the int8 tensor path, not with 16-bit A and
 * 4-bit B; 128-byte slices with 4- or 8-bit A. */
enum { MC_RESIDENT_AUTO = 0, MC_RESIDENT_S64_W8 = 1, MC_RESIDENT_S64_W16 = 2, MC_RESIDENT_S128_W16 = 3 };
int mcSpmm(const mcSpmmDesc* desc, cudaStream_t stream);

/* Chunk table of an SpMM mask for MC_KERNEL_DENSE_TILE: starts[R][c] is the
 * first slot of vector-row R (an index into column_indices) whose column is
 * >= 64 c, for c = 0 .. ceil(k / 64), so the slots of k chunk c are
 * [starts[R][c], starts[R][c+1]).  Built on the device on `stream`; *status
 * (device int) is set to 0, or to 1 if a vector-row's columns are not
 * strictly increasing or lie outside [0, k) (that row's chunks are then left
 * empty).  No reference counterpart: the reference's kernels walk the slots
 * in order and need no table. */
int mcSpmmChunkStartsCount(int k);  /* entries per vector-row: ceil(k / 64) + 1 */
int mcSpmmChunkStarts(int m_vec, int k, const int* row_offsets, const int* column_indices, int* starts,
                      int* status, cudaStream_t stream);

typedef struct mcSddmmDesc {
    int m_vec, vec_length, n, k;
    int lhs_bits, rhs_bits;     /* (4,4) (8,8) (16,8) (16,16) */
    int is_signed;
    int out_half;
    int out_vecmajor;           /* 0: blocked (j/8)*8V+8v+j%8; 1: j*V+v */
    float scale;
    int batch;
    int row_split;              /* CTAs per vector-row (0 = automatic) */
    const int* row_indices;
    const int* row_offsets;
    const int* column_indices;
    const void* lhs;      long long lhs_stride;     /* bytes */
    const void* rhs;      long long rhs_stride;     /* bytes */
    void* out;            long long out_stride;     /* elements */
    int mma_kind;               /* MC_MMA_DEFAULT / MC_MMA_INT8 / MC_MMA_F16 */
    int kernel_variant;         /* MC_KERNEL_AUTO / _PER_ROW / _STREAM / _DENSE_TILE */
    /* MC_KERNEL_DENSE_TILE only: the mask's tile bitmap and first-slot table
     * (mcSddmmTileMask), m_vec x mcSddmmTileMaskWords(n) entries each. */
    const unsigned* tile_bitmap;
    const int* tile_prefix;
} mcSddmmDesc;
int mcSddmm(const mcSddmmDesc* desc, cudaStream_t stream);
/* Tile bitmap of an SDDMM mask for MC_KERNEL_DENSE_TILE: per vector-row,
 * bitmap word w has bit c set if column 32w + c is stored, and prefix[w] is
 * the number of the row's stored columns below 32w.  bitmap and prefix hold
 * m_vec x mcSddmmTileMaskWords(n) entries (device memory, caller-owned).
 * *status (device int) is set to 0, or to 1 if some vector-row's columns are
 * not strictly increasing within [0, n) (the dense-tile kernel must not be
 * used with that mask).  Asynchronous on `stream`. */
int mcSddmmTileMaskWords(int n);
int mcSddmmTileMask(int m_vec, int n, const int* row_offsets, const int* column_indices, unsigned* bitmap,
                    int* prefix, int* status, cudaStream_t stream);

/* ---- Quantized attention steps ----------------------------------------------
 * mcQuantize: out = packed trunc(clamp(float(in) * scale)) for `count` half
 * inputs (count % 8 == 0), 8 bits ([-128, 127]) or 4 bits ([-8, 7]) per lane,
 * little-endian -- sparse_transformer_magicube/src/cuda/quantization_kernel.cu:14-131. */
int mcQuantize(const void* in, void* out, long long count, int bits, float scale, cudaStream_t stream);

/* mcQuantSoftmax: row softmax of SDDMM scores over each vector-row's stored
 * nonzeros, per vector lane: q = trunc(clamp(exp(score * scaling - max) *
 * (scale / sum))) -- the reference's trunc(clamp(exp(..) / sum * scale)) with
 * one division per row and lane -- in `bits` (4, 8, 16) bits, written in the
 * MC_VALUES_SOFTMAX layout at the aligned slots [start, end) of each row
 * (padding slots are not written) -- q_softmax_kernel.cu:181-271.  scores are
 * half, vector-major (j*V + v), as mcSddmm writes with out_half.
 * requant = MC_REQUANT_ROWMAX (bits 8) instead writes q = round(127 *
 * exp(score * scaling - max)) and, per vector-row and lane, the divisor
 * row_div[row * V + v] = 127 * sum * scale for mcSpmm's row_div -- the
 * separate-launch form of mcSparseAttention's row-max mode. */
enum { MC_REQUANT_FIXED = 0, MC_REQUANT_ROWMAX = 1 };
typedef struct mcSoftmaxDesc {
    int m_vec, vec_length, batch, bits;
    float scaling;              /* applied to each score (1/sqrt(head_dim)) */
    float scale;                /* quantization scale of the probabilities */
    const int* row_indices;
    const int* row_offsets;
    const void* scores;   long long scores_stride;  /* halves between batch entries */
    void* out;            long long out_stride;     /* bytes between batch entries */
    int requant;                /* MC_REQUANT_FIXED (0) or MC_REQUANT_ROWMAX */
    void* row_div;        long long row_div_stride; /* ROWMAX: float divisors, floats between batch entries */
} mcSoftmaxDesc;
int mcQuantSoftmax(const mcSoftmaxDesc* desc, cudaStream_t stream);

/* mcSparseAttention: the quantized sparse attention of every vector-row and
 * head in one persistent kernel (SDDMM, softmax + requantization, SpMM with
 * scores and probabilities kept on chip); the reference composes it from
 * batched_deq_sddmm, csrSoftmaxKernel_ and batched_deq_spmm launches
 * (spattention.py:189-216).  Precision pairs (lhs_bits = probabilities,
 * rhs_bits = Q / K / V): L8-R8, L16-R8 (fixed requantization only) and L8-R4.
 * q, k, v: [heads][tokens][64] packed int8 or int4 (mcQuantize output), out:
 * half [heads][tokens][64]; the mask in the attention layout (columns
 * unshuffled).
 *   MC_REQUANT_FIXED:  s = half(acc / score_scale) * scaling,
 *                      q = trunc(clamp(exp(s - max) * (prob_scale / sum))),
 *                      out = half(acc / out_scale) -- bit-identical to
 *                      mcSddmm + mcQuantSoftmax + mcSpmm with the same scales;
 *   MC_REQUANT_ROWMAX: s = half(acc / (score_scale / scaling)) (float
 *                      quotient of the two scales), q = round(127 * exp(s -
 *                      max)), out = half(acc / (127 * sum * out_scale)) --
 *                      bit-identical to mcSddmm (scale = score_scale /
 *                      scaling) + mcQuantSoftmax (ROWMAX, scaling 1, scale =
 *                      out_scale) + mcSpmm (row_div).
 * max_row_nnz must be at least every row's nonzero count (at most 4096); a
 * longer row is skipped and *status (if given) set to 1. */
typedef struct mcAttnDesc {
    int m_vec, vec_length, heads, head_dim, max_row_nnz;
    int lhs_bits, rhs_bits;     /* probabilities, Q/K/V: 8, 8 */
    int requant;
    float score_scale, scaling, prob_scale, out_scale;
    const int* row_indices;
    const int* row_offsets;
    const int* column_indices;
    const void* q;
    const void* k;
    const void* v;
    long long head_stride;      /* bytes between heads of q, k, v */
    void* out;
    long long out_head_stride;  /* halves between heads of out */
    int* status;                /* optional device int */
    /* launch configuration (0 = default; every choice gives the same bits):
     * warps per CTA 4 or 8 (the k-split of P x V), cp.async ring stages per
     * warp 2 or 3, at most ctas_per_sm resident CTAs per SM */
    int warps, stages, ctas_per_sm;
} mcAttnDesc;
int mcSparseAttention(const mcAttnDesc* desc, cudaStream_t stream);

/* ---- Input projection with fused quantization ------------------------------
 * out[which][h][t][c] = trunc(clamp(float(half(x[t] . W[n] + b[n])) * scale))
 * for n = which*hidden + h*head_dim + c (which = q, k, v): the reference's
 * fp16 F.linear + permute + bquantization (spattention.py:189-191,
 * quantization_kernel.cu:173-213) in one tcgen05 (5th-generation tensor core)
 * kernel.  x: [tokens][hidden] half, weight: [3*hidden][hidden] half (the
 * nn.Linear layout), bias: [3*hidden] half or NULL, all 16-byte aligned; out:
 * [3][heads][tokens][head_dim] packed int8 (bits 8) or int4 (bits 4, two per
 * byte, low nibble first).  Needs 64 <= hidden <= 256, hidden % 64 == 0,
 * head_dim % 64 == 0, heads * head_dim == hidden.  The f32 accumulation order
 * differs from cuBLAS's, so an element whose half rounding or truncation sits
 * on a boundary can differ by one step from the unfused path.  *status
 * (optional) is set to 1 if an internal wait timed out. */
typedef struct mcQkvProjDesc {
    int tokens, hidden, heads, head_dim;
    int bits;
    float scale;
    const void* x;
    const void* weight;
    const void* bias;
    void* out;
    int* status;
} mcQkvProjDesc;
int mcQkvProjectQuantize(const mcQkvProjDesc* desc, cudaStream_t stream);

/* ---- Batched attention engine (host C++, no PyTorch) -------------------------
 * The reference runs its sparse attention one sequence at a time, four
 * launches each, from Python (spattention.py:189-216).  mcAttnBatch holds the
 * attention of `n_instances` sequences of different lengths and masks, all
 * heads, as one problem: mcAttnBatchCreate stacks the instances' masks into
 * one block-diagonal vector-sparse mask (rows stacked, each instance's
 * columns offset by its first token), packs it (aligned pairs, padded
 * columns, longest-first row order) and keeps it and the quantized operands
 * on the device; mcAttnBatchRun is then two launches (mcQuantize, then the
 * fused mcSparseAttention) for every instance and head.  Results equal the
 * separate launches of the same pair and requantization mode, bit for bit.
 *   qkv: device half [3][heads][T][head_dim], the instances' tokens back to
 *        back (T = total tokens, instance i from token_offsets[i]);
 *   out: device half [heads][T][head_dim].
 * mcAttnBatchTune times the fused kernel's launch configurations (warps per
 * CTA 4 / 8, ring stages 2 / 3, CTAs per SM unlimited / 2 / 4) on these
 * buffers and keeps the fastest (the same bits for every choice).
 * mcAttnBatchCapture records Run on `stream` (not the legacy default stream)
 * into a CUDA graph; mcAttnBatchReplay launches that graph. */
typedef struct mcAttnBatch mcAttnBatch;
typedef struct mcAttnBatchDesc {
    int n_instances;
    const int* seq_lens;            /* tokens per instance, multiples of vec_length */
    const int* const* row_offsets;  /* per instance, host: plain vector CSR, seq_len / vec_length + 1 entries */
    const int* const* col_indices;  /* per instance, host: column vectors in [0, seq_len) */
    int vec_length, heads, head_dim; /* V = 2, 4, 8; head_dim 64 */
    int lhs_bits, rhs_bits;         /* probabilities, Q/K/V: (8, 8), (16, 8) or (8, 4) */
    int requant;                    /* MC_REQUANT_FIXED or MC_REQUANT_ROWMAX (8-bit probabilities) */
    float scale_qkv, scale_sfmx;    /* quantization scale of Q/K/V; fixed requantization scale.  Scores
                                       are dequantized by scale_qkv * scale_qkv rounded once to float
                                       (the square of the float scale) */
} mcAttnBatchDesc;
int mcAttnBatchCreate(const mcAttnBatchDesc* desc, mcAttnBatch** batch);
/* token_offsets: host array of n_instances + 1 entries. */
int mcAttnBatchTokens(const mcAttnBatch* batch, long long* token_offsets);
int mcAttnBatchRun(mcAttnBatch* batch, const void* qkv, void* out, cudaStream_t stream);
int mcAttnBatchTune(mcAttnBatch* batch, const void* qkv, void* out, cudaStream_t stream, int* warps, int* stages,
                    int* ctas_per_sm);
int mcAttnBatchCapture(mcAttnBatch* batch, const void* qkv, void* out, cudaStream_t stream);
int mcAttnBatchReplay(mcAttnBatch* batch, cudaStream_t stream);
/* Synchronous: 0, or 1 if a row exceeded the fused kernel's limit. */
int mcAttnBatchStatus(mcAttnBatch* batch, int* status);
void mcAttnBatchDestroy(mcAttnBatch* batch);

/* ---- Attention request server (host C++, no PyTorch) ------------------------
 * A continuous-batching request loop for sparse attention, the serving path
 * that the reference does not have (its end-to-end script runs one sequence
 * at a time, end_to_end.py:47-85).  Each request is one sequence: its plain
 * vector CSR mask and half Q/K/V stay resident in device memory, owned by the
 * caller, and the server writes its half output.  mcAttnServerRun plays the
 * requests at their arrival times on the host clock and, while requests are
 * waiting and fewer than max_inflight batches are on the device, admits the
 * waiting ones in arrival order (up to max_batch_tokens tokens, at least one
 * request) as one batch, provided the batch's device memory fits the free
 * memory (cudaMemGetInfo, plus what the default stream-ordered pool holds
 * unused) less hbm_reserve_bytes and less the batches already in flight,
 * each charged at its full footprint; a request that does not
 * fit even with nothing in flight is rejected (latency -1) and never
 * launched.  A batch is built on the device on its own stream with
 * stream-ordered allocations: the requests' masks stacked block-diagonally
 * (one kernel), packed by mcDevicePack (aligned pairs, padded columns,
 * longest-first rows), Q/K/V staged with one 2-D copy per request, then
 * mcQuantize and the fused mcSparseAttention, and the outputs copied back
 * into each request's buffer.  Each request's output equals its output when
 * served alone, bit for bit.  Latency = host-observed completion of the
 * request's batch minus its arrival.  No reference counterpart. */
typedef struct mcAttnServer mcAttnServer;
typedef struct mcAttnServerDesc {
    int vec_length, heads, head_dim;  /* V = 2, 4, 8; head_dim 64 */
    int lhs_bits, rhs_bits;           /* (8, 8), (16, 8) or (8, 4) */
    int requant;                      /* MC_REQUANT_FIXED or MC_REQUANT_ROWMAX */
    float scale_qkv, scale_sfmx;
    long long max_batch_tokens;       /* tokens per batch (a longer single request is admitted alone) */
    int max_inflight;                 /* batches on the device at once, 1 .. 8 */
    long long hbm_reserve_bytes;      /* free device memory admission leaves untouched */
} mcAttnServerDesc;
typedef struct mcAttnRequest {
    int seq_len;                      /* tokens, a positive multiple of vec_length */
    int nnz_vec, max_row_nnz;         /* the mask's nonzero vectors and longest vector-row (<= 4096) */
    const int* row_offsets;           /* device: seq_len / V + 1 plain CSR offsets, starting at 0 */
    const int* col_indices;           /* device: nnz_vec column indices in [0, seq_len), increasing per row */
    const void* qkv;                  /* device half [3][heads][seq_len][head_dim] */
    void* out;                        /* device half [heads][seq_len][head_dim] */
    double arrival_s;                 /* arrival time, seconds after the run starts */
} mcAttnRequest;
typedef struct mcAttnServeStats {
    double makespan_s, req_per_s, p50_ms, p99_ms, mean_ms;
    int served, rejected, batches, max_inflight_seen, held_back;
} mcAttnServeStats;
int mcAttnServerCreate(const mcAttnServerDesc* desc, mcAttnServer** server);
/* Serves `n` requests; latency_ms (host, n entries) receives each request's
 * latency or -1 if rejected.  Returns when every request is done. */
int mcAttnServerRun(mcAttnServer* server, const mcAttnRequest* requests, int n, double* latency_ms,
                    mcAttnServeStats* stats);
/* The device bytes admission charges for one batch of the n requests
 * (batch_bytes) and the current admission budget: free device memory plus
 * what the default stream-ordered pool holds unused, less the reserve
 * (available_bytes).  Either output may be null. */
int mcAttnServerMemory(const mcAttnServer* server, const mcAttnRequest* requests, int n, long long* batch_bytes,
                       long long* available_bytes);
void mcAttnServerDestroy(mcAttnServer* server);

/* ---- Host-side format conversion (host pointers) ---------------------------
 * The reference's host packer (SpMM/SpMM/spmm_benchmark.cpp:177-377,
 * SDDMM/SDDMM/sddmm_benchmark.cpp:104-127) as library routines. */

/* Aligned [start, end) pairs from plain CSR offsets (m_vec+1 entries); returns
 * the aligned slot count (spmm_benchmark.cpp:177-201), or -1 on error. */
int mcAlignRowOffsets(int m_vec, const int* row_offsets, int alignment, int* aligned_pairs);
/* Scatter column indices into the aligned slots, padding with -1; shuffle8 = 1
 * applies the 4-bit-operand order [c0 c2 c4 c6 c1 c3 c5 c7] per group of 8
 * (spmm_benchmark.cpp:204-222). */
int mcPadColumnIndices(int m_vec, const int* row_offsets, const int* col_indices,
                       const int* aligned_pairs, int aligned_nnz, int shuffle8, int* out_cols);
/* Pack original per-vector values (V lanes of lhs_bits, lane v at bit
 * v*lhs_bits; 12-bit values in 16-bit lanes) into the SpMM device value layout
 * for the (lhs_bits, rhs_bits) pair: chunk transpose and bit-plane
 * decomposition (spmm_benchmark.cpp:224-377).  out holds
 * aligned_nnz*V*lhs_bits/8 bytes (16 bits per lane for 12-bit values). */
int mcPackSpmmValues(int m_vec, int vec_length, int lhs_bits, int rhs_bits, const int* row_offsets,
                     const int* aligned_pairs, int aligned_nnz, const void* values, void* out);
/* Same, for any value layout (MC_VALUES_PACKED, MC_VALUES_SOFTMAX, or
 * MC_VALUES_SLOT_MAJOR for 8-bit values of the L8-R8 pair). */
int mcPackSpmmValuesEx(int m_vec, int vec_length, int lhs_bits, int rhs_bits, const int* row_offsets,
                       const int* aligned_pairs, int aligned_nnz, const void* values, void* out,
                       int value_layout);
/* Vector-row processing order: longest first (bm_test_utils.h:222-237), or identity. */
int mcSortedRowSwizzle(int m_vec, const int* row_offsets, int* row_indices);
int mcIdentityRowSwizzle(int m_vec, int* row_indices);

/* ---- Device-side format conversion (device pointers, stream-ordered) -------
 * The host packer above run on the GPU (the reference has it only as serial
 * host code: spmm_benchmark.cpp:177-377, bm_test_utils.h:222-237).  Outputs
 * are byte-identical to the host routines.  The aligned slot count stays in
 * device memory, so a caller that sizes its buffers by the upper bound
 * nnz_vec + m_vec * (alignment - 1) packs without a host round trip. */

/* Aligned pairs (8-byte aligned device array of 2*m_vec ints) and the aligned
 * slot count (*aligned_nnz, a device int; -1 when the offsets are not
 * monotone or the count overflows int).  Scratch of 8 * ceil(m_vec / 1024) +
 * 256 bytes (one 8-byte sum per 1,024-row scan tile, then the flag word) comes
 * from the stream-ordered allocator and is released on the stream. */
int mcDeviceAlignRowOffsets(int m_vec, const int* row_offsets, int alignment, int* aligned_pairs,
                            int* aligned_nnz, cudaStream_t stream);
/* mcDeviceAlignRowOffsets without any allocation (no counterpart in the
 * reference).  For callers that may not allocate device memory at all: a
 * serving process that reserved its whole HBM budget up front, or a host
 * framework whose own allocator owns the device and forbids cudaMalloc and
 * the stream-ordered pool.  The caller still passes row_offsets,
 * aligned_pairs and aligned_nnz.  The scratch is a 128 KB file-scope device
 * array that every GPU loading the library holds until exit, so at most
 * 16,744,448 vector-rows (larger m_vec is rejected with status 1 before any
 * launch).  The first call on each device looks up that array's device
 * address (cudaGetSymbolAddress) with the device current; make that first
 * call before any stream capture.  Every call shares the array and the flag
 * word is cleared on each call; calls that overlap on the device (concurrent
 * streams) race. */
int mcDeviceAlignRowOffsetsNoAlloc(int m_vec, const int* row_offsets, int alignment, int* aligned_pairs,
                                   int* aligned_nnz, cudaStream_t stream);
/* Column indices into the aligned slots, -1 padded, 8-shuffled if shuffle8
 * (col_indices and, below, values may be NULL when no row has nonzeros).
 * Vector-row i fills the slots from its start to the next row's start (the
 * first row from slot 0, the last up to *aligned_nnz); capacity = elements of
 * out_cols.  A row whose slots are inconsistent (overlap, past capacity, not
 * multiples of 8 when shuffling) is skipped and *status (optional device
 * int) set to 1. */
int mcDevicePadColumnIndices(int m_vec, const int* row_offsets, const int* col_indices,
                             const int* aligned_pairs, const int* aligned_nnz, int shuffle8, int* out_cols,
                             long long capacity, int* status, cudaStream_t stream);
/* Values into the SpMM device layout (as mcPackSpmmValuesEx); out 4-byte
 * aligned (16-byte for MC_VALUES_SLOT_MAJOR), capacity_bytes its size.  Row
 * slots must be whole value chunks (16 slots for the slot-major layout). */
int mcDevicePackSpmmValues(int m_vec, int vec_length, int lhs_bits, int rhs_bits, const int* row_offsets,
                           const int* aligned_pairs, const int* aligned_nnz, const void* values, void* out,
                           long long capacity_bytes, int value_layout, int* status, cudaStream_t stream);
/* Longest-first vector-row order; rows of equal length in ascending index
 * order (a stable sort).  Scratch from the stream-ordered allocator. */
int mcDeviceSortedRowSwizzle(int m_vec, const int* row_offsets, int* row_indices, cudaStream_t stream);

/* All of the above in one call (fused: one align scan, one per-row pass
 * writing columns and values, one row sort).  lhs_bits = 0 converts a mask
 * without values (SDDMM; alignment must then be given).  alignment = 0 with
 * values: the SpMM alignment of the pair (16, or 32 with a 4-bit operand). */
typedef struct mcDevicePackDesc {
    int m_vec, vec_length;
    int lhs_bits, rhs_bits;       /* the SpMM pair, or lhs_bits = 0 */
    int alignment;
    int shuffle8;                 /* 8-shuffle the columns (packed layout with a 4-bit operand) */
    int value_layout;             /* MC_VALUES_PACKED / _SOFTMAX / _SLOT_MAJOR (L8-R8) */
    int sort_rows;                /* 1: longest-first row_indices; 0: row_indices untouched */
    const int* row_offsets;       /* m_vec + 1 */
    const int* col_indices;
    const void* values;           /* nnz_vec * V * lhs_bits / 8 bytes */
    int* aligned_pairs;           /* 2 * m_vec, 8-byte aligned */
    int* aligned_nnz;             /* one device int */
    int* out_cols;       long long cols_capacity;         /* elements */
    void* out_values;    long long values_capacity_bytes; /* 4-byte aligned (slot-major: 16) */
    int* row_indices;             /* m_vec */
    int* status;                  /* optional device int, set to 1 on inconsistent rows */
} mcDevicePackDesc;
int mcDevicePack(const mcDevicePackDesc* desc, cudaStream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* MAGICUBE_GB300_H */
