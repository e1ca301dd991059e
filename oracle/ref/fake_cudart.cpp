// fake_cudart.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A host-memory stand-in for the few CUDA runtime calls the reference's host
// benchmark programs make (SpMM/SpMM/spmm_benchmark.cpp,
// SDDMM/SDDMM/sddmm_benchmark.cpp), so that those programs -- their data
// generator, format conversion and host verification -- run unmodified on a
// machine without a GPU.  "Device" buffers are host allocations; copies are
// memcpy; events measure nothing.
#include <cuda_profiler_api.h>
#include <cuda_runtime_api.h>

#include <cstdlib>
#include <cstring>
#include <map>

static std::map<const void*, size_t>& allocations()
{
    static std::map<const void*, size_t> m;
    return m;
}

// Size of a buffer returned by the fake cudaMalloc (0 if unknown).
extern "C" size_t mcref_alloc_size(const void* p)
{
    auto it = allocations().find(p);
    return it == allocations().end() ? 0 : it->second;
}

extern "C" {

cudaError_t CUDARTAPI cudaMalloc(void** devPtr, size_t size)
{
    *devPtr = std::calloc(size ? size : 1, 1);
    allocations()[*devPtr] = size;
    return *devPtr ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t CUDARTAPI cudaFree(void* devPtr)
{
    allocations().erase(devPtr);
    std::free(devPtr);
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaMemcpy(void* dst, const void* src, size_t count, enum cudaMemcpyKind)
{
    std::memcpy(dst, src, count);
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaGetDevice(int* device)
{
    *device = 0;
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaGetDeviceProperties(struct cudaDeviceProp* prop, int)
{
    std::memset(prop, 0, sizeof(*prop));
    prop->multiProcessorCount = 1;
    return cudaSuccess;
}
const char* CUDARTAPI cudaGetErrorString(cudaError_t e) { return e == cudaSuccess ? "no error" : "fake runtime error"; }
cudaError_t CUDARTAPI cudaEventCreate(cudaEvent_t* event)
{
    static int token;
    *event = reinterpret_cast<cudaEvent_t>(&token);
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaEventDestroy(cudaEvent_t) { return cudaSuccess; }
cudaError_t CUDARTAPI cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
cudaError_t CUDARTAPI cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
cudaError_t CUDARTAPI cudaEventElapsedTime(float* ms, cudaEvent_t, cudaEvent_t)
{
    *ms = 1.0f;
    return cudaSuccess;
}
cudaError_t CUDARTAPI cudaProfilerStart(void) { return cudaSuccess; }
cudaError_t CUDARTAPI cudaProfilerStop(void) { return cudaSuccess; }
cudaError_t CUDARTAPI cudaGetLastError(void) { return cudaSuccess; }

}  // extern "C"
