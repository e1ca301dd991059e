// capi.cpp -- argument checking and the exported C entry points.
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <string>

#include "mc_host.h"

namespace mc {

static thread_local std::string g_last_error;
static std::atomic<int> g_default_mma{MC_MMA_INT8};

int default_mma_kind() { return g_default_mma.load(std::memory_order_relaxed); }

int fail(int code, const char* msg)
{
    g_last_error = msg;
    return code;
}
void clear_error() { g_last_error.clear(); }

static bool aligned(const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

static int check_spmm(const mcSpmmDesc& d)
{
    char buf[256];
    if (d.m_vec < 0 || d.n <= 0 || d.k <= 0) return fail(1, "mcSpmm: m_vec must be >= 0 and n, k > 0");
    if (!(d.vec_length == 2 || d.vec_length == 4 || d.vec_length == 8))
        return fail(1, "mcSpmm: vec_length must be 2, 4 or 8");
    const bool pair_ok = (d.lhs_bits == 4 && d.rhs_bits == 4) || (d.lhs_bits == 8 && d.rhs_bits == 4) ||
                         (d.lhs_bits == 12 && d.rhs_bits == 4) || (d.lhs_bits == 16 && d.rhs_bits == 4) ||
                         (d.lhs_bits == 8 && d.rhs_bits == 8) || (d.lhs_bits == 12 && d.rhs_bits == 8) ||
                         (d.lhs_bits == 16 && d.rhs_bits == 8) || (d.lhs_bits == 16 && d.rhs_bits == 16);
    if (!pair_ok) {
        std::snprintf(buf, sizeof buf, "mcSpmm: unsupported precision pair L%d-R%d", d.lhs_bits, d.rhs_bits);
        return fail(1, buf);
    }
    if (d.lhs_bits == 12 && (d.is_signed || d.out_half))
        return fail(1, "mcSpmm: 12-bit values are unsigned lanes with int32 output (the reference's 12-bit "
                       "kernels); signed 12-bit data runs as lhs_bits = 16 with sign-extended values");
    if (d.n % 64) return fail(1, "mcSpmm: n must be a multiple of 64");
    if (d.n / 64 > 65535) return fail(1, "mcSpmm: n too large");
    if (d.batch < 1 || d.batch > 65535) return fail(1, "mcSpmm: batch must be in [1, 65535]");
    if (d.out_half && !d.is_signed) return fail(1, "mcSpmm: half output requires is_signed = 1");
    const bool slot_major = d.value_layout == MC_VALUES_SLOT_MAJOR && d.kernel_variant == MC_KERNEL_DENSE_TILE;
    if (d.value_layout != (d.out_half ? MC_VALUES_SOFTMAX : MC_VALUES_PACKED) && !slot_major)
        return fail(1, "mcSpmm: half output is built for the softmax value layout and int32 output for the "
                       "packer layout (or, for the dense-tile kernel, the slot-major layout)");
    if (d.out_half && !d.row_div && !(d.scale != 0.0f))
        return fail(1, "mcSpmm: half output requires a nonzero scale or row divisors");
    if (d.row_div && !d.out_half) return fail(1, "mcSpmm: row divisors apply to half output only");
    if (d.row_div && (reinterpret_cast<uintptr_t>(d.row_div) % 4 || (d.batch > 1 && d.row_div_stride < 0)))
        return fail(1, "mcSpmm: row_div must be 4-byte aligned with a non-negative stride");
    if (d.mma_kind < MC_MMA_DEFAULT || d.mma_kind > MC_MMA_DP4A || d.mma_kind == MC_MMA_TCGEN05)
        return fail(1, "mcSpmm: invalid mma_kind (the SpMM runs on MC_MMA_INT8, MC_MMA_F16 or MC_MMA_DP4A)");
    if (d.mma_kind == MC_MMA_DP4A && (d.lhs_bits > 8 || d.rhs_bits > 8 || d.vec_length > 4))
        return fail(1, "mcSpmm: the dp4a SpMM computes V = 2 and 4 with 8-bit or 4-bit operands");
    if (d.kernel_variant < MC_KERNEL_AUTO || d.kernel_variant > MC_KERNEL_RESIDENT)
        return fail(1, "mcSpmm: invalid kernel_variant");
    if (d.kernel_variant == MC_KERNEL_DENSE_TILE) {
        if (d.lhs_bits != 8 || d.rhs_bits != 8 || d.out_half)
            return fail(1, "mcSpmm: the dense-tile kernel computes L8-R8 with int32 output");
        if (d.n % 128) return fail(1, "mcSpmm: the dense-tile kernel needs n % 128 == 0");
        if (d.mma_kind != MC_MMA_DEFAULT)
            return fail(1, "mcSpmm: the dense-tile kernel runs on the tcgen05 f16 path (mma_kind must be "
                           "MC_MMA_DEFAULT)");
        if (d.m_vec > 0 && (!d.chunk_starts || !aligned(d.chunk_starts, 4)))
            return fail(1, "mcSpmm: the dense-tile kernel needs the mask's chunk table (mcSpmmChunkStarts)");
        if (d.batch > 1 && d.rhs_stride % d.n)
            return fail(1, "mcSpmm: the dense-tile kernel needs rhs_stride a multiple of the B row bytes");
        if (!aligned(d.column_indices, 16))
            return fail(1, "mcSpmm: the dense-tile kernel needs 16-byte aligned column indices");
        if (slot_major && (!aligned(d.values, 16) || d.values_stride % 16))
            return fail(1, "mcSpmm: slot-major values must be 16-byte aligned with values_stride % 16 == 0");
    }
    if (d.kernel_config < MC_RESIDENT_AUTO || d.kernel_config > MC_RESIDENT_S128_W16)
        return fail(1, "mcSpmm: invalid kernel_config");
    if (d.m_vec == 0) return 0;
    if (!d.row_indices || !d.row_offsets || !d.column_indices || !d.values || !d.rhs || !d.out)
        return fail(1, "mcSpmm: null pointer");
    if (!aligned(d.values, 4) || d.values_stride % 4) return fail(1, "mcSpmm: values must be 4-byte aligned");
    if (!aligned(d.rhs, 16) || d.rhs_stride % 16) return fail(1, "mcSpmm: rhs must be 16-byte aligned");
    if (!aligned(d.out, d.out_half ? 8 : 16) || d.out_stride % 4)
        return fail(1, "mcSpmm: output must be 16-byte aligned (8 for half) with stride % 4 == 0");
    if (d.batch > 1 && (d.values_stride < 0 || d.rhs_stride < 0 || d.out_stride < 0))
        return fail(1, "mcSpmm: negative stride");
    return 0;
}

static int check_sddmm(const mcSddmmDesc& d)
{
    char buf[256];
    if (d.m_vec < 0 || d.n <= 0 || d.k <= 0) return fail(1, "mcSddmm: m_vec must be >= 0 and n, k > 0");
    if (!(d.vec_length == 2 || d.vec_length == 4 || d.vec_length == 8))
        return fail(1, "mcSddmm: vec_length must be 2, 4 or 8");
    const bool pair_ok = (d.lhs_bits == 4 && d.rhs_bits == 4) || (d.lhs_bits == 8 && d.rhs_bits == 8) ||
                         (d.lhs_bits == 16 && d.rhs_bits == 8) || (d.lhs_bits == 16 && d.rhs_bits == 16);
    if (!pair_ok) {
        std::snprintf(buf, sizeof buf, "mcSddmm: unsupported precision pair L%d-R%d", d.lhs_bits, d.rhs_bits);
        return fail(1, buf);
    }
    if (d.k % 64) return fail(1, "mcSddmm: k must be a multiple of 64");
    if (d.batch < 1 || d.batch > 65535) return fail(1, "mcSddmm: batch must be in [1, 65535]");
    if (d.row_split < 0 || d.row_split > 65535) return fail(1, "mcSddmm: row_split must be in [0, 65535]");
    if (d.out_half && (!d.is_signed || !d.out_vecmajor))
        return fail(1, "mcSddmm: half output requires is_signed = 1 and out_vecmajor = 1");
    if (d.out_half && !(d.scale != 0.0f)) return fail(1, "mcSddmm: half output requires a nonzero scale");
    if (d.mma_kind < MC_MMA_DEFAULT || d.mma_kind > MC_MMA_DP4A) return fail(1, "mcSddmm: invalid mma_kind");
    if (d.mma_kind == MC_MMA_DP4A && (d.lhs_bits > 8 || d.rhs_bits > 8))
        return fail(1, "mcSddmm: the dp4a path computes 8-bit and 4-bit operands");
    if (d.mma_kind == MC_MMA_TCGEN05 && (d.lhs_bits != 8 || d.rhs_bits != 8 || d.k != 64))
        return fail(1, "mcSddmm: the tcgen05 path computes L8-R8 with k == 64");
    if (d.kernel_variant < MC_KERNEL_AUTO || d.kernel_variant > MC_KERNEL_DENSE_TILE ||
        d.kernel_variant == MC_KERNEL_TMA)
        return fail(1, "mcSddmm: invalid kernel_variant");
    if (d.kernel_variant == MC_KERNEL_DENSE_TILE) {
        if (d.lhs_bits != 8 || d.rhs_bits != 8 || d.k != 64)
            return fail(1, "mcSddmm: the dense-tile kernel computes L8-R8 with k == 64");
        if (d.m_vec > 0 && (!d.tile_bitmap || !d.tile_prefix || !aligned(d.tile_bitmap, 4) || !aligned(d.tile_prefix, 4)))
            return fail(1, "mcSddmm: the dense-tile kernel needs the mask's tile bitmap and prefix (mcSddmmTileMask)");
    }
    if (d.m_vec == 0) return 0;
    if (!d.row_indices || !d.row_offsets || !d.column_indices || !d.lhs || !d.rhs || !d.out)
        return fail(1, "mcSddmm: null pointer");
    if (!aligned(d.lhs, 16) || d.lhs_stride % 16) return fail(1, "mcSddmm: lhs must be 16-byte aligned");
    if (!aligned(d.rhs, 16) || d.rhs_stride % 16) return fail(1, "mcSddmm: rhs must be 16-byte aligned");
    if (!aligned(d.out, 8) || d.out_stride % 2) return fail(1, "mcSddmm: output must be 8-byte aligned");
    if (d.batch > 1 && (d.lhs_stride < 0 || d.rhs_stride < 0 || d.out_stride < 0))
        return fail(1, "mcSddmm: negative stride");
    return 0;
}

}  // namespace mc

extern "C" {

const char* mcGetLastErrorString(void) { return mc::g_last_error.c_str(); }
const char* mcVersion(void) { return "0.1.0"; }

int mcSetDefaultMmaKind(int kind)
{
    if (kind != MC_MMA_INT8 && kind != MC_MMA_F16) return -1;
    return mc::g_default_mma.exchange(kind);
}

int mcSpmm(const mcSpmmDesc* desc, cudaStream_t stream)
{
    mc::clear_error();
    if (!desc) return mc::fail(1, "mcSpmm: null descriptor");
    mcSpmmDesc d = *desc;
    // slot-major values are read by the dense-tile kernel alone
    if (d.kernel_variant == MC_KERNEL_AUTO && d.value_layout == MC_VALUES_SLOT_MAJOR)
        d.kernel_variant = MC_KERNEL_DENSE_TILE;
    if (int rc = mc::check_spmm(d)) return rc;
    if (d.m_vec == 0) return 0;
    if (d.kernel_variant == MC_KERNEL_DENSE_TILE) return mc::spmm_dense_launch(d, stream);
    if (d.lhs_bits == 12) {
        // 12-bit values use the 16-bit layouts with the top 4 bits clear
        // (spmm_benchmark.cpp:288-358): the 16-bit kernels compute them.
        mcSpmmDesc e = d;
        e.lhs_bits = 16;
        return d.rhs_bits == 4 ? mc::spmm_launch_16_4(e, stream) : mc::spmm_launch_16_8(e, stream);
    }
    if (d.rhs_bits == 4) {
        if (d.lhs_bits == 4) return mc::spmm_launch_4_4(d, stream);
        if (d.lhs_bits == 8) return mc::spmm_launch_8_4(d, stream);
        return mc::spmm_launch_16_4(d, stream);
    }
    if (d.rhs_bits == 16) return mc::spmm_launch_16_16(d, stream);
    if (d.lhs_bits == 8) return mc::spmm_launch_8_8(d, stream);
    return mc::spmm_launch_16_8(d, stream);
}

int mcSddmm(const mcSddmmDesc* desc, cudaStream_t stream)
{
    mc::clear_error();
    if (!desc) return mc::fail(1, "mcSddmm: null descriptor");
    const mcSddmmDesc& d = *desc;
    if (int rc = mc::check_sddmm(d)) return rc;
    if (d.m_vec == 0) return 0;
    if (d.kernel_variant == MC_KERNEL_DENSE_TILE) return mc::sddmm_dense_launch(d, stream);
    if (d.lhs_bits == 4) return mc::sddmm_launch_4_4(d, stream);
    if (d.lhs_bits == 8) return mc::sddmm_launch_8_8(d, stream);
    if (d.rhs_bits == 8) return mc::sddmm_launch_16_8(d, stream);
    return mc::sddmm_launch_16_16(d, stream);
}

static int legacy_spmm(int lhs_bits, int rhs_bits, int m_vec, int vec_length, int n, int k,
                       const int* row_indices, const int* row_offsets, const int* column_indices,
                       const int* values, const int* rhs_matrix, int* output_matrix)
{
    mcSpmmDesc d{};
    d.m_vec = m_vec; d.vec_length = vec_length; d.n = n; d.k = k;
    d.lhs_bits = lhs_bits; d.rhs_bits = rhs_bits;
    d.is_signed = 0; d.out_half = 0; d.scale = 1.0f; d.batch = 1;
    d.row_indices = row_indices; d.row_offsets = row_offsets; d.column_indices = column_indices;
    d.values = values; d.rhs = rhs_matrix; d.out = output_matrix;
    return mcSpmm(&d, 0);
}

int mcWmmaSpmm_4b(int m_vec, int vec_length, int n, int k, const int* ri, const int* ro, const int* ci,
                  const int* values, const int* rhs, int* out)
{ return legacy_spmm(4, 4, m_vec, vec_length, n, k, ri, ro, ci, values, rhs, out); }
int mcWmmaSpmm_8b4b(int m_vec, int vec_length, int n, int k, const int* ri, const int* ro, const int* ci,
                    const int* values, const int* rhs, int* out)
{ return legacy_spmm(8, 4, m_vec, vec_length, n, k, ri, ro, ci, values, rhs, out); }
int mcWmmaSpmm_16b4b(int m_vec, int vec_length, int n, int k, const int* ri, const int* ro, const int* ci,
                     const int* values, const int* rhs, int* out)
{ return legacy_spmm(16, 4, m_vec, vec_length, n, k, ri, ro, ci, values, rhs, out); }
int mcWmmaSpmm_8b(int m_vec, int vec_length, int n, int k, const int* ri, const int* ro, const int* ci,
                  const int* values, const int* rhs, int* out)
{ return legacy_spmm(8, 8, m_vec, vec_length, n, k, ri, ro, ci, values, rhs, out); }
int mcWmmaSpmm_16b8b(int m_vec, int vec_length, int n, int k, const int* ri, const int* ro, const int* ci,
                     const int* values, const int* rhs, int* out)
{ return legacy_spmm(16, 8, m_vec, vec_length, n, k, ri, ro, ci, values, rhs, out); }
int mcWmmaSpmm_12b4b(int m_vec, int vec_length, int n, int k, const int* ri, const int* ro, const int* ci,
                     const int* values, const int* rhs, int* out)
{ return legacy_spmm(12, 4, m_vec, vec_length, n, k, ri, ro, ci, values, rhs, out); }
int mcWmmaSpmm_12b8b(int m_vec, int vec_length, int n, int k, const int* ri, const int* ro, const int* ci,
                     const int* values, const int* rhs, int* out)
{ return legacy_spmm(12, 8, m_vec, vec_length, n, k, ri, ro, ci, values, rhs, out); }
int mcWmmaSpmm_16b(int m_vec, int vec_length, int n, int k, const int* ri, const int* ro, const int* ci,
                   const int* values, const int* rhs, int* out)
{ return legacy_spmm(16, 16, m_vec, vec_length, n, k, ri, ro, ci, values, rhs, out); }

static int legacy_sddmm(int bits, int m_vec, int k, int n, const int* row_indices, const int* row_offsets,
                        const int* column_indices, const int* lhs, const int* rhs, int* out, int vec_length)
{
    mcSddmmDesc d{};
    d.m_vec = m_vec; d.vec_length = vec_length; d.n = n; d.k = k;
    d.lhs_bits = bits; d.rhs_bits = bits;
    d.is_signed = 0; d.out_half = 0; d.out_vecmajor = 0; d.scale = 1.0f; d.batch = 1; d.row_split = 0;
    d.row_indices = row_indices; d.row_offsets = row_offsets; d.column_indices = column_indices;
    d.lhs = lhs; d.rhs = rhs; d.out = out;
    return mcSddmm(&d, 0);
}

int mcWmmaSddmm_4b(int m_vec, int k, int n, const int* ri, const int* ro, const int* ci, const int* lhs,
                   const int* rhs, int* out, int vec_length)
{ return legacy_sddmm(4, m_vec, k, n, ri, ro, ci, lhs, rhs, out, vec_length); }
int mcWmmaSddmm_8b(int m_vec, int k, int n, const int* ri, const int* ro, const int* ci, const int* lhs,
                   const int* rhs, int* out, int vec_length)
{ return legacy_sddmm(8, m_vec, k, n, ri, ro, ci, lhs, rhs, out, vec_length); }
int mcWmmaSddmm_16b(int m_vec, int k, int n, const int* ri, const int* ro, const int* ci, const int* lhs,
                    const int* rhs, int* out, int vec_length)
{ return legacy_sddmm(16, m_vec, k, n, ri, ro, ci, lhs, rhs, out, vec_length); }

}  // extern "C"
