// Test-only probe (built by tests/probe/build_probe.py, never shipped):
// evaluates, on the device, the two arithmetic rules the CPU oracle has to
// emulate and that cannot be read off the reference's source:
//  * the float -> int64 conversion of out-of-range and NaN values (glm's
//    i64vec2 constructor, visual_hull_cuda.cu:239-240), and
//  * whether nvcc fuses the reference's world-coordinate expression
//    `c + float(v) / float(r) * L` (visual_hull_cuda.cu:206-213) into one fma.
// The second kernel deliberately spells the expression the way the reference
// does and is compiled with the reference's default flags (-fmad=true).

#include <cstdint>

#include <cuda_runtime.h>

namespace
{

__global__ void probe_kernel(const float* __restrict__ in,
                             int64_t* __restrict__ out_i64,
                             int64_t n,
                             const int64_t* __restrict__ v,
                             float r,
                             float c,
                             float L,
                             float* __restrict__ out_f32)
{
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    out_i64[i] = static_cast<int64_t>(in[i]);
    out_f32[i] = c + static_cast<float>(v[i]) / r * L;
}

} // namespace

// 0 on success, 1 for invalid arguments, 2 for a failed launch.
extern "C" int probe_arithmetic(const float* in,
                                int64_t* out_i64,
                                int64_t n,
                                const int64_t* v,
                                float r,
                                float c,
                                float L,
                                float* out_f32,
                                void* stream)
{
    if (n <= 0)
        return 0;
    if (!in || !out_i64 || !v || !out_f32)
        return 1;
    const unsigned grid = static_cast<unsigned>((n + 255) / 256);
    probe_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(in, out_i64, n, v, r, c, L, out_f32);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}
