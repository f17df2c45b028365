// th_gaussian_blur_noalloc: the Gaussian blur with no device allocation.
//
// Who needs it: callers that cannot or must not call cudaMalloc.  Examples are
// a process where another framework has already reserved nearly all device
// memory up front (a fresh cudaMalloc there fails or fragments its pool), a
// per-frame loop with a latency budget (cudaMalloc/cudaFree can synchronize the
// whole device and stall other streams), and a caller that has to account for
// every byte of device memory before it starts.  th_gaussian_blur takes its
// scratch (tile flags and the weight table) from a context pool that grows
// with cudaMalloc; this variant takes it from one fixed array instead.
//
// The scratch is a file-scope __device__ array of kNoAllocScratchBytes
// (16 MiB).  Every GPU that loads this library holds it until the process
// exits, whether or not the entry point is called.  A request needs
// B * (H / (k/2) + 1) * (W / (k/2) + 1) bytes of tile flags plus
// 8 * (k*k + 1) + 16 bytes of weights; larger requests are rejected with
// TH_ERR_INVALID_ARGUMENT.  All calls share the array: the tile flags are
// cleared at the start of each call, and two calls whose work overlaps on the
// GPU (different streams, no ordering between them) race on it and give
// undefined results.
//
// Host code must not use the array's name as a device address (in host code
// it names a host-side stand-in).  The first call on each device looks up the
// real device address with cudaGetSymbolAddress, with that device current,
// and caches it; make that first call before any stream capture begins.

#include <mutex>

#include "th_internal.h"

namespace
{

constexpr int64_t kNoAllocScratchBytes = int64_t{ 16 } << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_lock;
uint8_t* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device, or nullptr.
uint8_t* scratch_on_current_device(cudaError_t* err)
{
    int dev = 0;
    *err = cudaGetDevice(&dev);
    if (*err != cudaSuccess)
        return nullptr;
    if (dev < 0 || dev >= kMaxDevices)
    {
        *err = cudaErrorInvalidDevice;
        return nullptr;
    }
    std::lock_guard<std::mutex> g(g_setup_lock);
    if (!g_scratch_ptr[dev])
    {
        void* p = nullptr;
        *err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (*err != cudaSuccess)
            return nullptr;
        g_scratch_ptr[dev] = static_cast<uint8_t*>(p);
    }
    return g_scratch_ptr[dev];
}

} // namespace

extern "C" th_status th_gaussian_blur_noalloc(const void* images,
                                              int32_t images_dtype,
                                              int64_t batch,
                                              int64_t height,
                                              int64_t width,
                                              int32_t kernel_size,
                                              float sigma,
                                              int32_t sparse,
                                              void* out,
                                              int32_t out_dtype,
                                              void* stream)
{
    if (kernel_size <= 0 || kernel_size % 2 != 1 || !(sigma > 0.f))
        return TH_ERR_INVALID_ARGUMENT;
    if (!(out_dtype == TH_FLOAT16 || out_dtype == TH_FLOAT32 || out_dtype == TH_FLOAT64))
        return out_dtype == TH_BFLOAT16 ? TH_ERR_UNSUPPORTED_DTYPE : TH_ERR_INVALID_ARGUMENT;
    if (images_dtype < TH_UINT8 || images_dtype > TH_FLOAT64)
        return TH_ERR_UNSUPPORTED_DTYPE;
    if (batch < 0 || height < 0 || width < 0)
        return TH_ERR_INVALID_ARGUMENT;
    if (batch * height * width == 0)
        return TH_OK;
    if (!images || !out)
        return TH_ERR_INVALID_ARGUMENT;
    if (th::blur_tile_bytes(batch, height, width, kernel_size) > kNoAllocScratchBytes)
        return TH_ERR_INVALID_ARGUMENT;
    cudaError_t err = cudaSuccess;
    uint8_t* scratch = scratch_on_current_device(&err);
    if (!scratch)
        return TH_ERR_CUDA;
    try
    {
        th::launch_gaussian_blur(images, images_dtype, batch, height, width, kernel_size, sigma, sparse != 0, out,
                                 out_dtype, scratch, static_cast<cudaStream_t>(stream));
    }
    catch (const th::CudaError&)
    {
        return TH_ERR_CUDA;
    }
    return TH_OK;
}
