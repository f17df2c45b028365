// Gaussian blur of masks, sparse (boundary tiles only) and dense.
//
// Sparse (reference: gaussian_blur_cuda.cu:288-507).  The reference flags edge
// pixels, compacts them with cub, expands each to the 3x3 window of tiles
// (tile side kernel_size/2) around its tile, sorts and uniques those tile ids,
// and convolves only the pixels of the listed tiles; every other pixel keeps
// its input value.  Here pass 1 sets one byte per tile that holds an edge
// pixel; pass 2 writes every output pixel once: a pixel whose tile has an edge
// tile within one tile in x and y (the reference's clamped 3x3 window) gets the
// convolution, any other pixel the converted input.  No compaction, no sort,
// and the output is written in the same pass as the copy the reference makes
// with images.clone().
//
// The convolution keeps the reference's arithmetic: 2-D taps with the x
// offset outer and the y offset inner, weights expf(-(i^2+j^2)/(2 sigma^2))
// rounded to the output type, acc += w * v fused for float and double (nvcc
// contracts the reference's expression), c10::Half rounding after every
// operation for half, and division by the sum of the weights in the same
// order.  The weight table and its sum are computed once per call on the
// device with the same expression, so results are bit-identical per pixel.
//
// Dense (reference: :20-114, reflect pad + torch conv2d with the normalised
// kernel).  Same halo reads; the weights are normalised first as the
// reference does, and the sum is accumulated in float (double for double
// output).  The reference's conv2d order belongs to cuDNN, so dense output
// agrees within rounding, as the reference's own dense/sparse test allows.

#include "th_common.cuh"
#include "th_internal.h"

namespace th
{

namespace
{

constexpr int kMaxTaps = 63 * 63;

template <int DT>
__device__ __forceinline__ double load_f64(const void* p, int64_t i)
{
    using T = typename Elem<DT>::T;
    if constexpr (DT == TH_FLOAT16)
        return static_cast<double>(__half2float(static_cast<const __half*>(p)[i]));
    else
        return static_cast<double>(static_cast<const T*>(p)[i]);
}

__device__ __forceinline__ float round_half(float v)
{
    return __half2float(__float2half_rn(v));
}

// Input element as the output type (static_cast<BlurredImageT>(ImageT)),
// returned widened to double; for half through float like c10::Half does.
template <int DT, int OT>
__device__ __forceinline__ double as_out(const void* p, int64_t i)
{
    if constexpr (OT == TH_FLOAT64)
        return load_f64<DT>(p, i);
    else if constexpr (OT == TH_FLOAT32)
        return static_cast<double>(load_f32<DT>(p, i));
    else
        return static_cast<double>(round_half(load_f32<DT>(p, i)));
}

template <int OT>
__device__ __forceinline__ void store_out(void* p, int64_t i, double v)
{
    if constexpr (OT == TH_FLOAT64)
        static_cast<double*>(p)[i] = v;
    else if constexpr (OT == TH_FLOAT32)
        static_cast<float*>(p)[i] = static_cast<float>(v);
    else
        static_cast<__half*>(p)[i] = __float2half_rn(static_cast<float>(v));
}

// image_utils.h:129-160
__device__ __forceinline__ int64_t reflect(int64_t y, int64_t n)
{
    if (n == 1)
        return 0;
    const int64_t m = n - 1;
    const int64_t flips = y / m + (y < 0 ? 1 : 0);
    int64_t rem = y % m;
    if (rem < 0)
        rem += m;
    return (flips % 2 == 0) ? rem : m - rem;
}

template <int DT>
__device__ __forceinline__ bool differs(const void* p, int64_t a, int64_t b)
{
    using T = typename Elem<DT>::T;
    if constexpr (DT == TH_FLOAT16)
        return __half2float(static_cast<const __half*>(p)[a]) != __half2float(static_cast<const __half*>(p)[b]);
    else
        return static_cast<const T*>(p)[a] != static_cast<const T*>(p)[b];
}

// edge_kernel (gaussian_blur_cuda.cu:116-142) folded into tile flags.
template <int DT>
__global__ void __launch_bounds__(256) edge_tiles_kernel(const void* __restrict__ img,
                                                         int64_t B,
                                                         int64_t H,
                                                         int64_t W,
                                                         int64_t ts,
                                                         int64_t TH,
                                                         int64_t TW,
                                                         uint8_t* __restrict__ tiles)
{
    const int64_t n = B * H * W;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        const int64_t x = i % W, y = i / W % H, b = i / (W * H);
        const bool edge = (x + 1 < W && differs<DT>(img, i, i + 1)) || (y + 1 < H && differs<DT>(img, i, i + W));
        if (edge)
        {
            uint8_t* t = tiles + (b * TH + y / ts) * TW + x / ts;
            if (*t == 0)
                *t = 1;
        }
    }
}

// Weight table (k*k, x offset major) and its sum, in the output type's arithmetic.
template <int OT>
__global__ void weights_kernel(int k, float sigma, bool normalise, double* __restrict__ w, double* __restrict__ norm)
{
    if (threadIdx.x != 0 || blockIdx.x != 0)
        return;
    const int r = k / 2;
    const float den = __fmul_rn(__fmul_rn(2.f, sigma), sigma);
    if (!normalise)
    {
        // tile_convolution_kernel (:268-283): kernel_val per tap, normalization += kernel_val
        double s = 0.0;
        float sh = 0.f, sf = 0.f;
        for (int i = -r; i <= r; ++i)
            for (int j = -r; j <= r; ++j)
            {
                const float e = expf(__fdiv_rn(-static_cast<float>(i * i + j * j), den));
                double v;
                if constexpr (OT == TH_FLOAT64)
                {
                    v = static_cast<double>(e);
                    s = __dadd_rn(s, v);
                }
                else if constexpr (OT == TH_FLOAT32)
                {
                    v = static_cast<double>(e);
                    sf = __fadd_rn(sf, e);
                }
                else
                {
                    const float eh = round_half(e);
                    v = static_cast<double>(eh);
                    sh = round_half(__fadd_rn(sh, eh));
                }
                w[(i + r) * k + (j + r)] = v;
            }
        *norm = (OT == TH_FLOAT64) ? s : (OT == TH_FLOAT32 ? static_cast<double>(sf) : static_cast<double>(sh));
    }
    else
    {
        // create_gaussian_kernel (:20-71): kernel[y][x] in the output type,
        // divided by its float32 sum.  Stored here x offset major like above.
        float sum = 0.f;
        for (int y = 0; y < k; ++y)
            for (int x = 0; x < k; ++x)
            {
                const int dy = y - r, dx = x - r;
                const float e = expf(__fdiv_rn(-static_cast<float>(dy * dy + dx * dx), den));
                const float ev = (OT == TH_FLOAT16) ? round_half(e) : e;
                sum = __fadd_rn(sum, ev);
            }
        for (int y = 0; y < k; ++y)
            for (int x = 0; x < k; ++x)
            {
                const int dy = y - r, dx = x - r;
                const float e = expf(__fdiv_rn(-static_cast<float>(dy * dy + dx * dx), den));
                double v;
                if constexpr (OT == TH_FLOAT64)
                    v = __ddiv_rn(static_cast<double>(e), static_cast<double>(sum));
                else if constexpr (OT == TH_FLOAT32)
                    v = static_cast<double>(__fdiv_rn(e, sum));
                else
                    v = static_cast<double>(round_half(__fdiv_rn(round_half(e), sum)));
                w[x * k + y] = v;
            }
        *norm = 1.0;
    }
}

struct BlurGeom
{
    int64_t B, H, W, ts, TH, TW;
    int k;
};

__device__ __forceinline__ bool tile_active(const uint8_t* tiles, const BlurGeom& g, int64_t b, int64_t y, int64_t x)
{
    const int64_t tx = x / g.ts, ty = y / g.ts;
    for (int64_t dy = -1; dy <= 1; ++dy)
    {
        const int64_t yy = ty + dy;
        if (yy < 0 || yy >= g.TH)
            continue;
        for (int64_t dx = -1; dx <= 1; ++dx)
        {
            const int64_t xx = tx + dx;
            if (xx < 0 || xx >= g.TW)
                continue;
            if (tiles[(b * g.TH + yy) * g.TW + xx])
                return true;
        }
    }
    return false;
}

// One output pixel per thread.  SPARSE: only pixels of active tiles are
// convolved (reference arithmetic); DENSE: all pixels, normalised weights.
template <int DT, int OT, bool SPARSE>
__global__ void __launch_bounds__(256) blur_kernel(const void* __restrict__ img,
                                                   void* __restrict__ out,
                                                   BlurGeom g,
                                                   const uint8_t* __restrict__ tiles,
                                                   const double* __restrict__ wtab,
                                                   const double* __restrict__ norm_ptr)
{
    __shared__ double w[kMaxTaps > 1024 ? 1024 : kMaxTaps];
    const int taps = g.k * g.k;
    const bool smem_w = taps <= 1024;
    if (smem_w)
    {
        for (int i = threadIdx.x; i < taps; i += blockDim.x)
            w[i] = wtab[i];
        __syncthreads();
    }
    const double norm = *norm_ptr;
    const int r = g.k / 2;
    const int64_t n = g.B * g.H * g.W;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        const int64_t x = i % g.W, y = i / g.W % g.H, b = i / (g.W * g.H);
        if (SPARSE && !tile_active(tiles, g, b, y, x))
        {
            store_out<OT>(out, i, as_out<DT, OT>(img, i));
            continue;
        }
        const int64_t img_base = b * g.H * g.W;
        if constexpr (OT == TH_FLOAT64)
        {
            double acc = 0.0;
            for (int dx = -r; dx <= r; ++dx)
            {
                const int64_t xx = reflect(x + dx, g.W);
                for (int dy = -r; dy <= r; ++dy)
                {
                    const int64_t yy = reflect(y + dy, g.H);
                    const int t = (dx + r) * g.k + (dy + r);
                    const double kv = smem_w ? w[t] : wtab[t];
                    acc = __fma_rn(kv, load_f64<DT>(img, img_base + yy * g.W + xx), acc);
                }
            }
            store_out<OT>(out, i, SPARSE ? __ddiv_rn(acc, norm) : acc);
        }
        else if constexpr (OT == TH_FLOAT32)
        {
            float acc = 0.f;
            for (int dx = -r; dx <= r; ++dx)
            {
                const int64_t xx = reflect(x + dx, g.W);
                for (int dy = -r; dy <= r; ++dy)
                {
                    const int64_t yy = reflect(y + dy, g.H);
                    const int t = (dx + r) * g.k + (dy + r);
                    const float kv = static_cast<float>(smem_w ? w[t] : wtab[t]);
                    acc = __fmaf_rn(kv, load_f32<DT>(img, img_base + yy * g.W + xx), acc);
                }
            }
            store_out<OT>(out, i, SPARSE ? static_cast<double>(__fdiv_rn(acc, static_cast<float>(norm))) : acc);
        }
        else
        {
            float acc = 0.f;
            for (int dx = -r; dx <= r; ++dx)
            {
                const int64_t xx = reflect(x + dx, g.W);
                for (int dy = -r; dy <= r; ++dy)
                {
                    const int64_t yy = reflect(y + dy, g.H);
                    const int t = (dx + r) * g.k + (dy + r);
                    const float kv = static_cast<float>(smem_w ? w[t] : wtab[t]);
                    const float iv = round_half(load_f32<DT>(img, img_base + yy * g.W + xx));
                    if (SPARSE)
                        acc = round_half(__fadd_rn(acc, round_half(__fmul_rn(kv, iv))));
                    else
                        acc = __fmaf_rn(kv, iv, acc);
                }
            }
            const float res = SPARSE ? round_half(__fdiv_rn(acc, static_cast<float>(norm))) : acc;
            store_out<OT>(out, i, static_cast<double>(res));
        }
    }
}

template <int DT, int OT>
__global__ void __launch_bounds__(256) convert_kernel(const void* __restrict__ img, void* __restrict__ out, int64_t n)
{
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        store_out<OT>(out, i, as_out<DT, OT>(img, i));
}

template <class F>
void dispatch_out(int odt, F&& f)
{
    switch (odt)
    {
    case TH_FLOAT16:
        f.template operator()<TH_FLOAT16>();
        break;
    case TH_FLOAT32:
        f.template operator()<TH_FLOAT32>();
        break;
    default:
        f.template operator()<TH_FLOAT64>();
        break;
    }
}

} // namespace

int64_t blur_tile_bytes(int64_t B, int64_t H, int64_t W, int kernel_size)
{
    const int64_t ts = kernel_size / 2;
    if (ts < 1)
        return 0;
    // tile table plus the weight table (k*k doubles) and its sum
    return B * (H / ts + 1) * (W / ts + 1) + 16 + 8 * (static_cast<int64_t>(kernel_size) * kernel_size + 1);
}

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
                          uint8_t* scratch,
                          cudaStream_t s)
{
    const int64_t n = B * H * W;
    if (n == 0)
        return;
    const int grid = grid_for(n, 256);
    if (kernel_size == 1)
    {
        dispatch_image_dtype(idt, [&]<int DT>() {
            dispatch_out(odt, [&]<int OT>() { convert_kernel<DT, OT><<<grid, 256, 0, s>>>(images, out, n); });
        });
        TH_LAUNCH_CHECK();
        return;
    }
    BlurGeom g;
    g.B = B;
    g.H = H;
    g.W = W;
    g.k = kernel_size;
    g.ts = kernel_size / 2;
    g.TH = H / g.ts + 1;
    g.TW = W / g.ts + 1;
    const int64_t tile_bytes = B * g.TH * g.TW;
    uint8_t* tiles = scratch;
    const int64_t woff = (tile_bytes + 15) / 16 * 16;
    double* wtab = reinterpret_cast<double*>(scratch + woff);
    double* norm = wtab + static_cast<int64_t>(kernel_size) * kernel_size;
    dispatch_out(odt, [&]<int OT>() { weights_kernel<OT><<<1, 32, 0, s>>>(kernel_size, sigma, !sparse, wtab, norm); });
    TH_LAUNCH_CHECK();
    if (sparse)
    {
        TH_CUDA(cudaMemsetAsync(tiles, 0, tile_bytes, s));
        dispatch_image_dtype(idt, [&]<int DT>() {
            edge_tiles_kernel<DT><<<grid, 256, 0, s>>>(images, B, H, W, g.ts, g.TH, g.TW, tiles);
        });
        TH_LAUNCH_CHECK();
    }
    dispatch_image_dtype(idt, [&]<int DT>() {
        dispatch_out(odt, [&]<int OT>() {
            if (sparse)
                blur_kernel<DT, OT, true><<<grid, 256, 0, s>>>(images, out, g, tiles, wtab, norm);
            else
                blur_kernel<DT, OT, false><<<grid, 256, 0, s>>>(images, out, g, tiles, wtab, norm);
        });
    });
    TH_LAUNCH_CHECK();
}

} // namespace th
