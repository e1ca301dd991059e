// tma_host.cu -- host side of the TMA kernels: tensor-map encoding through the
// driver entry point, and the device counter of bounded waits that ran out.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "mc_host.h"
#include "mc_tma_host.h"

namespace mc {

// Incremented by a kernel whose bounded mbarrier wait gave up (TMA SpMM).
__device__ unsigned int g_async_timeouts;

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
    });
    return fn;
}

bool encode_row_gather_u8(CUtensorMap* map, const void* base, long long rows, long long row_bytes, int box_bytes)
{
    auto fn = tensor_map_encoder();
    if (!fn || rows <= 0 || row_bytes <= 0 || row_bytes % 16 || box_bytes > 128 || box_bytes % 16) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)row_bytes, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)row_bytes};
    const cuuint32_t box[2] = {(cuuint32_t)box_bytes, 1};  // gather4: boxes one row high
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool encode_slice_u8(CUtensorMap* map, const void* base, long long rows, long long row_bytes, int box_bytes,
                     int box_rows)
{
    auto fn = tensor_map_encoder();
    if (!fn || rows <= 0 || !(box_bytes == 64 || box_bytes == 128) || row_bytes < box_bytes || row_bytes % 16 ||
        box_rows < 1 || box_rows > 256)
        return false;
    const cuuint64_t dims[2] = {(cuuint64_t)row_bytes, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)row_bytes};
    const cuuint32_t box[2] = {(cuuint32_t)box_bytes, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, box_bytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool encode_box_u8(CUtensorMap* map, const void* base, long long rows, long long row_bytes, int box_bytes,
                   int box_rows)
{
    auto fn = tensor_map_encoder();
    if (!fn || rows <= 0 || row_bytes < box_bytes || row_bytes % 16 || box_bytes % 16 || box_bytes > 256 ||
        box_rows < 1 || box_rows > 256)
        return false;
    const cuuint64_t dims[2] = {(cuuint64_t)row_bytes, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)row_bytes};
    const cuuint32_t box[2] = {(cuuint32_t)box_bytes, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void*>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Device address of g_async_timeouts on the current device, looked up once
// per device under a lock (the library assumes the primary context of a
// device is never reset while it is loaded).
unsigned int* async_timeout_counter()
{
    static std::mutex mu;
    static unsigned int* cache[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!cache[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_async_timeouts) != cudaSuccess) return nullptr;
        cache[dev] = static_cast<unsigned int*>(p);
    }
    return cache[dev];
}

unsigned int async_timeouts()
{
    unsigned int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_async_timeouts, sizeof v) != cudaSuccess) return 0xFFFFFFFFu;
    return v;
}

}  // namespace mc
