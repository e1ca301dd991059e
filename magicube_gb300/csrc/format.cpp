// format.cpp -- host-side conversion into the vector-sparse device layout.
//
// Library form of the reference's host packer (SpMM/SpMM/spmm_benchmark.cpp
// :177-377, SDDMM/SDDMM/sddmm_benchmark.cpp:104-127): aligned [start, end)
// row ranges, -1 padded (and, for 4-bit operands, 8-shuffled) column indices,
// and the chunk-transposed, bit-plane-decomposed value layout.  The reference
// spells each precision pair out as its own loop nest; here one formulation
// covers all of them: a chunk of MMA_K vector slots holds PLANES bit-planes,
// each a [V][MMA_K] array of PLANE_BITS-bit elements, plane p carrying bits
// [p*PLANE_BITS, (p+1)*PLANE_BITS) of every value.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#include "../../include/magicube_gb300.h"
#include "mc_host.h"

namespace {

inline uint32_t get_bits(const uint8_t* p, long long lane, int bits)
{
    long long bit = lane * bits;
    uint32_t w = 0;
    int nbytes = (bits + (int)(bit % 8) + 7) / 8;
    for (int b = 0; b < nbytes; ++b) w |= (uint32_t)p[bit / 8 + b] << (8 * b);
    w >>= (bit % 8);
    return w & ((1u << bits) - 1u);
}

inline void or_bits(uint8_t* p, long long lane, int bits, uint32_t v)
{
    long long bit = lane * bits;
    int nbytes = (bits + (int)(bit % 8) + 7) / 8;
    uint32_t w = v << (bit % 8);
    for (int b = 0; b < nbytes; ++b) p[bit / 8 + b] |= (uint8_t)(w >> (8 * b));
}

bool valid_pair(int lhs_bits, int rhs_bits)
{
    return (lhs_bits == 4 && rhs_bits == 4) || (lhs_bits == 8 && rhs_bits == 4) ||
           (lhs_bits == 12 && rhs_bits == 4) || (lhs_bits == 16 && rhs_bits == 4) ||
           (lhs_bits == 8 && rhs_bits == 8) || (lhs_bits == 12 && rhs_bits == 8) ||
           (lhs_bits == 16 && rhs_bits == 8) || (lhs_bits == 16 && rhs_bits == 16);
}

}  // namespace

extern "C" int mcAlignRowOffsets(int m_vec, const int* row_offsets, int alignment, int* aligned_pairs)
{
    if (m_vec < 0 || alignment <= 0 || !row_offsets || (m_vec > 0 && !aligned_pairs))
        return mc::fail(-1, "mcAlignRowOffsets: invalid arguments");
    long long aligned = 0;
    for (int i = 0; i < m_vec; ++i) {
        const long long len = (long long)row_offsets[i + 1] - row_offsets[i];
        if (len < 0) return mc::fail(-1, "mcAlignRowOffsets: row_offsets not monotone");
        if (aligned + len > 0x7fffffffLL) return mc::fail(-1, "mcAlignRowOffsets: aligned size overflows int");
        aligned_pairs[2 * i] = (int)aligned;
        aligned_pairs[2 * i + 1] = (int)(aligned + len);
        aligned += (len + alignment - 1) / alignment * alignment;
        if (aligned > 0x7fffffffLL) return mc::fail(-1, "mcAlignRowOffsets: aligned size overflows int");
    }
    return (int)aligned;
}

extern "C" int mcPadColumnIndices(int m_vec, const int* row_offsets, const int* col_indices,
                                  const int* aligned_pairs, int aligned_nnz, int shuffle8, int* out_cols)
{
    if (m_vec < 0 || aligned_nnz < 0 || !row_offsets || !aligned_pairs || !out_cols)
        return mc::fail(1, "mcPadColumnIndices: invalid arguments");
    if (shuffle8 && aligned_nnz % 8)
        return mc::fail(1, "mcPadColumnIndices: shuffled layout needs aligned_nnz % 8 == 0");
    std::vector<int> plain((size_t)aligned_nnz, -1);
    for (int i = 0; i < m_vec; ++i) {
        const int b = row_offsets[i], e = row_offsets[i + 1];
        const long long dst = aligned_pairs[2 * i];
        if (e > b && !col_indices) return mc::fail(1, "mcPadColumnIndices: null col_indices");
        if (dst < 0) return mc::fail(1, "mcPadColumnIndices: negative aligned start");
        if (e > b && dst + ((long long)e - b) > aligned_nnz)
            return mc::fail(1, "mcPadColumnIndices: aligned_nnz too small");
        for (int j = b; j < e; ++j) plain[(size_t)(dst + (j - b))] = col_indices[j];
    }
    if (!shuffle8) {
        std::memcpy(out_cols, plain.data(), sizeof(int) * (size_t)aligned_nnz);
    } else {
        for (int g = 0; g < aligned_nnz / 8; ++g)
            for (int j = 0; j < 8; ++j) out_cols[g * 8 + (j % 2) * 4 + j / 2] = plain[(size_t)g * 8 + j];
    }
    return 0;
}

extern "C" int mcPackSpmmValues(int m_vec, int vec_length, int lhs_bits, int rhs_bits, const int* row_offsets,
                                const int* aligned_pairs, int aligned_nnz, const void* values, void* out)
{
    return mcPackSpmmValuesEx(m_vec, vec_length, lhs_bits, rhs_bits, row_offsets, aligned_pairs, aligned_nnz,
                              values, out, MC_VALUES_PACKED);
}

extern "C" int mcPackSpmmValuesEx(int m_vec, int vec_length, int lhs_bits, int rhs_bits, const int* row_offsets,
                                  const int* aligned_pairs, int aligned_nnz, const void* values, void* out,
                                  int value_layout)
{
    const int V = vec_length;
    if (m_vec < 0 || !(V == 2 || V == 4 || V == 8) || !valid_pair(lhs_bits, rhs_bits) || !row_offsets ||
        !aligned_pairs || !out || aligned_nnz < 0 ||
        (value_layout != MC_VALUES_PACKED && value_layout != MC_VALUES_SOFTMAX &&
         value_layout != MC_VALUES_SLOT_MAJOR) ||
        (lhs_bits == 12 && value_layout != MC_VALUES_PACKED) ||
        (value_layout == MC_VALUES_SLOT_MAJOR && (lhs_bits != 8 || rhs_bits != 8)))
        return mc::fail(1, "mcPackSpmmValues: invalid arguments");
    if (value_layout == MC_VALUES_SLOT_MAJOR) {
        // [aligned slot][V] bytes: the lanes of a slot side by side
        const uint8_t* src = static_cast<const uint8_t*>(values);
        uint8_t* dst = static_cast<uint8_t*>(out);
        std::memset(dst, 0, (size_t)aligned_nnz * V);
        for (int i = 0; i < m_vec; ++i) {
            const int b = row_offsets[i], e = row_offsets[i + 1];
            if (e > b && (!src || aligned_pairs[2 * i] < 0))
                return mc::fail(1, "mcPackSpmmValues: null values or negative aligned start");
            for (int j = b; j < e; ++j) {
                const long long slot = (long long)aligned_pairs[2 * i] + (j - b);
                if (slot >= aligned_nnz) return mc::fail(1, "mcPackSpmmValues: aligned_nnz too small");
                std::memcpy(dst + slot * V, src + (long long)j * V, (size_t)V);
            }
        }
        return 0;
    }
    // 12-bit values sit in 16-bit containers and use the 16-bit layouts with
    // the top 4 bits cleared (spmm_benchmark.cpp:288-358).
    const uint32_t vmask = lhs_bits == 12 ? 0xFFFu : 0xFFFFFFFFu;
    if (lhs_bits == 12) lhs_bits = 16;
    const int mma_k = (lhs_bits == 4 || rhs_bits == 4) ? 32 : 16;
    if (aligned_nnz % mma_k) return mc::fail(1, "mcPackSpmmValues: aligned_nnz not a multiple of the chunk size");
    // Chunk of `chunk` slots holding `planes` planes of `plane_bits`; element
    // (v, jj) of plane pl sits at element index pl*plane_elems + v*vstride + jj.
    const bool softmax = value_layout == MC_VALUES_SOFTMAX;
    const int chunk = softmax ? (lhs_bits == 4 ? 32 : 16) : mma_k;
    const int plane_bits = chunk == 32 ? 4 : 8;
    const int planes = lhs_bits / plane_bits;
    const bool interleaved = softmax && lhs_bits == 16;  // [v][plane][16]
    const long long chunk_bytes = (long long)V * chunk * lhs_bits / 8;
    const long long plane_elems = interleaved ? chunk : (long long)V * chunk;
    const long long vstride = interleaved ? (long long)planes * chunk : chunk;
    const uint8_t* src = static_cast<const uint8_t*>(values);
    uint8_t* dst = static_cast<uint8_t*>(out);
    std::memset(dst, 0, (size_t)(aligned_nnz / chunk) * (size_t)chunk_bytes);
    const uint32_t pmask = (1u << plane_bits) - 1u;
    for (int i = 0; i < m_vec; ++i) {
        const int b = row_offsets[i], e = row_offsets[i + 1];
        if (e > b && (!src || aligned_pairs[2 * i] < 0))
            return mc::fail(1, "mcPackSpmmValues: null values or negative aligned start");
        for (int j = b; j < e; ++j) {
            const long long slot = (long long)aligned_pairs[2 * i] + (j - b);
            if (slot >= aligned_nnz) return mc::fail(1, "mcPackSpmmValues: aligned_nnz too small");
            uint8_t* cbase = dst + (slot / chunk) * chunk_bytes;
            const int jj = (int)(slot % chunk);
            for (int v = 0; v < V; ++v) {
                const uint32_t x = get_bits(src, (long long)j * V + v, lhs_bits) & vmask;
                for (int pl = 0; pl < planes; ++pl)
                    or_bits(cbase, pl * plane_elems + v * vstride + jj, plane_bits, (x >> (pl * plane_bits)) & pmask);
            }
        }
    }
    return 0;
}

extern "C" int mcSortedRowSwizzle(int m_vec, const int* row_offsets, int* row_indices)
{
    if (m_vec < 0 || !row_offsets || (m_vec > 0 && !row_indices))
        return mc::fail(1, "mcSortedRowSwizzle: invalid arguments");
    std::vector<int> idx((size_t)m_vec);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [row_offsets](int a, int b) {
        return ((long long)row_offsets[a + 1] - row_offsets[a]) > ((long long)row_offsets[b + 1] - row_offsets[b]);
    });
    std::memcpy(row_indices, idx.data(), sizeof(int) * (size_t)m_vec);
    return 0;
}

extern "C" int mcIdentityRowSwizzle(int m_vec, int* row_indices)
{
    if (m_vec < 0 || (m_vec > 0 && !row_indices)) return mc::fail(1, "mcIdentityRowSwizzle: invalid arguments");
    std::iota(row_indices, row_indices + m_vec, 0);
    return 0;
}
