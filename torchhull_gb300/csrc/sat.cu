// Integral images (summed-area tables) of the masks, one per view.
//
// The reference builds them with torch::cumsum over H and then over W in
// float32 (visual_hull_cuda.cu:76-90).  torch scans a non-innermost dimension
// one element at a time from 0, so every SAT value is the float result of that
// fixed sequence of additions.  The two kernels below perform exactly the same
// additions in the same order, which makes the table bit-identical for any
// mask values: exact integer sums for binary masks (totals < 2^24) and the
// same rounded sums for blurred, non-binary masks.
//
// Column pass: one thread per (view, column) walks down the column; a warp
// covers 32 adjacent columns, so each step is one coalesced 128-byte row read.
// Row pass: one warp per 32 rows walks across them through 32x33 shared
// tiles (coalesced loads and stores, one lane per row scanning its 32 values).
// HBM traffic: read masks + write columns + read columns + write SAT.

#include "th_common.cuh"
#include "th_internal.h"

namespace th
{

namespace
{

constexpr int kColUnroll = 16;

// Column pass.  Also flags (nonbinary != nullptr) whether any mask value,
// as float, is neither 0 nor 1: binary masks make every SAT value an exact
// integer, which the carve's view skipping relies on.
template <int DT>
__global__ void __launch_bounds__(256) sat_columns_kernel(const void* __restrict__ masks,
                                                          float* __restrict__ out,
                                                          int64_t B,
                                                          int64_t H,
                                                          int64_t W,
                                                          unsigned int* __restrict__ nonbinary)
{
    const int64_t col = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (col >= B * W)
        return;
    const int64_t b = col / W, x = col - b * W;
    const int64_t base = b * H * W + x;
    float acc = 0.f;
    bool nb = false;
    int64_t y = 0;
    // two chunks of rows in flight: the next chunk's loads are issued before
    // the current one is summed (a thread walks its column sequentially)
    const int64_t full = H - H % kColUnroll;
    float v[kColUnroll];
    if (full > 0)
    {
#pragma unroll
        for (int k = 0; k < kColUnroll; ++k)
            v[k] = load_f32<DT>(masks, base + k * W);
    }
    for (; y < full; y += kColUnroll)
    {
        float nx[kColUnroll];
        if (y + kColUnroll < full)
        {
#pragma unroll
            for (int k = 0; k < kColUnroll; ++k)
                nx[k] = load_f32<DT>(masks, base + (y + kColUnroll + k) * W);
        }
#pragma unroll
        for (int k = 0; k < kColUnroll; ++k)
        {
            nb |= (v[k] != 0.f) & (v[k] != 1.f);
            acc = __fadd_rn(acc, v[k]);
            out[base + (y + k) * W] = acc;
        }
#pragma unroll
        for (int k = 0; k < kColUnroll; ++k)
            v[k] = nx[k];
    }
    for (; y < H; ++y)
    {
        const float v = load_f32<DT>(masks, base + y * W);
        nb |= (v != 0.f) & (v != 1.f);
        acc = __fadd_rn(acc, v);
        out[base + y * W] = acc;
    }
    if (nb && nonbinary)
        atomicOr(nonbinary, 1u);
}

constexpr int kRowWarps = 4;

// Row pass: a warp owns 32 rows and walks across them in 32-column tiles
// through shared memory; the next tile is loaded while the current one is
// scanned (double buffer).
__global__ void __launch_bounds__(32 * kRowWarps) sat_rows_kernel(float* __restrict__ data, int64_t rows, int64_t W)
{
    __shared__ float tile[kRowWarps][2][32][33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t row0 = (static_cast<int64_t>(blockIdx.x) * kRowWarps + warp) * 32;
    if (row0 >= rows)
        return;
    const int nrows = static_cast<int>(rows - row0 < 32 ? rows - row0 : 32);
    float(*t)[32][33] = tile[warp];
    auto load = [&](int buf, int64_t x0) {
        const int64_t x = x0 + lane;
        const bool xin = x < W;
        for (int r = 0; r < nrows; ++r)
            t[buf][r][lane] = xin ? data[(row0 + r) * W + x] : 0.f;
    };
    load(0, 0);
    float carry = 0.f;
    int buf = 0;
    for (int64_t x0 = 0; x0 < W; x0 += 32)
    {
        if (x0 + 32 < W)
            load(buf ^ 1, x0 + 32);
        __syncwarp();
        if (lane < nrows)
        {
            const int cnt = static_cast<int>(W - x0 < 32 ? W - x0 : 32);
            for (int c = 0; c < cnt; ++c)
            {
                carry = __fadd_rn(carry, t[buf][lane][c]);
                t[buf][lane][c] = carry;
            }
        }
        __syncwarp();
        const int64_t x = x0 + lane;
        for (int r = 0; r < nrows; ++r)
            if (x < W)
                data[(row0 + r) * W + x] = t[buf][r][lane];
        __syncwarp();
        buf ^= 1;
    }
}

template <int DT>
__global__ void convert_transforms_kernel(const void* __restrict__ tf, int64_t n, float* __restrict__ out)
{
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = load_f32<DT>(tf, i);
}

} // namespace

void launch_integral_image(const void* masks,
                           int dtype,
                           int64_t B,
                           int64_t H,
                           int64_t W,
                           float* out,
                           cudaStream_t s,
                           unsigned int* nonbinary)
{
    if (B * H * W == 0)
        return;
    const int64_t cols = B * W;
    const unsigned grid = static_cast<unsigned>((cols + 255) / 256);
    bool ok = dispatch_image_dtype(dtype, [&]<int DT>() {
        sat_columns_kernel<DT><<<grid, 256, 0, s>>>(masks, out, B, H, W, nonbinary);
    });
    if (!ok)
        throw CudaError{ cudaErrorInvalidValue, "integral image: unsupported mask dtype" };
    TH_LAUNCH_CHECK();
    const int64_t rows = B * H;
    const unsigned grid_rows = static_cast<unsigned>((rows + 32 * kRowWarps - 1) / (32 * kRowWarps));
    sat_rows_kernel<<<grid_rows, 32 * kRowWarps, 0, s>>>(out, rows, W);
    TH_LAUNCH_CHECK();
}

void launch_convert_transforms(const void* tf, int dtype, int64_t B, float* out, cudaStream_t s)
{
    const int64_t n = B * 16;
    if (n == 0)
        return;
    const unsigned grid = static_cast<unsigned>((n + 255) / 256);
    switch (dtype)
    {
    case TH_FLOAT16:
        convert_transforms_kernel<TH_FLOAT16><<<grid, 256, 0, s>>>(tf, n, out);
        break;
    case TH_FLOAT32:
        convert_transforms_kernel<TH_FLOAT32><<<grid, 256, 0, s>>>(tf, n, out);
        break;
    case TH_FLOAT64:
        convert_transforms_kernel<TH_FLOAT64><<<grid, 256, 0, s>>>(tf, n, out);
        break;
    default:
        throw CudaError{ cudaErrorInvalidValue, "transforms: unsupported dtype" };
    }
    TH_LAUNCH_CHECK();
}

} // namespace th
