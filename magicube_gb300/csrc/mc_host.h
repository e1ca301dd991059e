// mc_host.h -- host-side helpers shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime_api.h>

#include "../../include/magicube_gb300.h"

namespace mc {

// Tensor path used by a call whose descriptor asks for MC_MMA_DEFAULT.
int default_mma_kind();
inline int resolve_mma_kind(int k) { return k == MC_MMA_DEFAULT ? default_mma_kind() : k; }

// Number of SMs of the current device (cached per device).
inline int sm_count()
{
    static int cache[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (!cache[dev]) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
        cache[dev] = n;
    }
    return cache[dev];
}

// Records `msg` as the calling thread's last argument error and returns `code`.
int fail(int code, const char* msg);
// Clears the calling thread's last argument error.
void clear_error();

// Per-precision-pair launchers (one translation unit each).
int spmm_launch_4_4(const mcSpmmDesc& d, cudaStream_t s);
int spmm_launch_8_4(const mcSpmmDesc& d, cudaStream_t s);
int spmm_launch_16_4(const mcSpmmDesc& d, cudaStream_t s);
int spmm_launch_8_8(const mcSpmmDesc& d, cudaStream_t s);
int spmm_launch_16_8(const mcSpmmDesc& d, cudaStream_t s);
int spmm_launch_16_16(const mcSpmmDesc& d, cudaStream_t s);
int sddmm_launch_4_4(const mcSddmmDesc& d, cudaStream_t s);
int sddmm_launch_8_8(const mcSddmmDesc& d, cudaStream_t s);
int sddmm_launch_16_8(const mcSddmmDesc& d, cudaStream_t s);
int sddmm_launch_16_16(const mcSddmmDesc& d, cudaStream_t s);
int sddmm_dense_launch(const mcSddmmDesc& d, cudaStream_t s);
int spmm_dense_launch(const mcSpmmDesc& d, cudaStream_t s);

}  // namespace mc
