// Host-side declarations shared by the CUDA translation units of the library.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>

#include <cuda_runtime.h>

#include "../../include/torchhull_gb300.h"

namespace th
{

struct CudaError
{
    cudaError_t code;
    std::string where;
};

#define TH_CUDA(expr)                                                                                                  \
    do                                                                                                                 \
    {                                                                                                                  \
        cudaError_t th_err_ = (expr);                                                                                  \
        if (th_err_ != cudaSuccess)                                                                                    \
            throw ::th::CudaError{ th_err_, std::string(#expr) + " at " + __FILE__ + ":" + std::to_string(__LINE__) }; \
    } while (0)

// Counts kernels launched by this library (th_launch_count).
void note_launches(int n);
// Throws CudaError if the last launch failed.
void check_launch(const char* what);

// After one kernel launch: check it and count it.
#define TH_LAUNCH_CHECK()                                                                                              \
    do                                                                                                                 \
    {                                                                                                                  \
        TH_CUDA(cudaGetLastError());                                                                                   \
        ::th::note_launches(1);                                                                                        \
    } while (0)

// Number of SMs of the current device (cached per device).
int sm_count();

// Grid size for a grid-stride kernel over work_items items: enough blocks to
// cover the work, at most 8 resident blocks per SM.
int grid_for(int64_t work_items, int threads);

// Zeroes `bytes` of device memory with a kernel (capi.cu): the per-request
// clears of the pipeline must not wait behind a caller's bulk copies, which a
// copy-engine memset could.
void launch_zero(void* p, size_t bytes, cudaStream_t s);

// Scratch of the single-pass integral image (sat.cu): device memory of at
// least sat_scratch_bytes(B, H, W, dtype) bytes (each launch clears what it needs).
struct SatScratch
{
    void* p = nullptr;
};

// Bytes of scratch the single pass needs, 0 when it does not apply.
int64_t sat_scratch_bytes(int64_t B, int64_t H, int64_t W, int dtype);

// Integral image (sat.cu).  masks [B,H,W] of dtype, out [B,H,W] float32.
// nonbinary (optional, zeroed by the caller) is set non-zero if any mask value
// is neither 0 nor 1.  With scratch and nonbinary, 0/1 masks take the single
// pass; otherwise (and after it, gated on the device) the exact two passes.
void launch_integral_image(const void* masks,
                           int dtype,
                           int64_t B,
                           int64_t H,
                           int64_t W,
                           float* out,
                           cudaStream_t s,
                           unsigned int* nonbinary = nullptr,
                           SatScratch scratch = {});

// Transform conversion to float32 row-major [B,16] (sat.cu).
void launch_convert_transforms(const void* tf, int dtype, int64_t B, float* out, cudaStream_t s);

// Gaussian blur (blur.cu).  edge_tiles: scratch of tiles_bytes(B,H,W,k) bytes.
int64_t blur_tile_bytes(int64_t B, int64_t H, int64_t W, int kernel_size);
void launch_gaussian_blur(const void* images,
                          int idt,
                          int64_t B,
                          int64_t H,
                          int64_t W,
                          int kernel_size,
                          float sigma,
                          bool sparse,
                          void* out,
                          int odt,
                          uint8_t* edge_tiles,
                          cudaStream_t s);

// Candidate wireframe of one level (wire.cu): verts [8n,3], edges [12n,2].
void launch_wireframe(const int64_t* cand, int64_t n, int shift, const float corner[3], float length, float* verts, int64_t* edges, cudaStream_t s);
// OBJ/PLY writer (wire.cu); false for an unsupported extension.
std::string file_extension(const std::string& filename);
bool store_curve_network(const std::string& filename, const float* verts, int64_t nv, const int64_t* edges, int64_t ne, bool verbose);

} // namespace th
