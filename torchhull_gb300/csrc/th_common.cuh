// Shared device helpers: element loads, the reference's float arithmetic
// (operation for operation, so results match bit for bit), index helpers and
// a device-wide scan built from two grid-stride kernels.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/torchhull_gb300.h"

namespace th
{

constexpr int kMaxLevel = 12;

// ---------------------------------------------------------------------------
// element loads: value of element i converted the way static_cast<float>(T)
// converts it (round to nearest for wide integers and double).

template <int DT>
struct Elem;
template <>
struct Elem<TH_UINT8>
{
    using T = uint8_t;
};
template <>
struct Elem<TH_INT8>
{
    using T = int8_t;
};
template <>
struct Elem<TH_INT16>
{
    using T = int16_t;
};
template <>
struct Elem<TH_INT32>
{
    using T = int32_t;
};
template <>
struct Elem<TH_INT64>
{
    using T = int64_t;
};
template <>
struct Elem<TH_FLOAT16>
{
    using T = __half;
};
template <>
struct Elem<TH_FLOAT32>
{
    using T = float;
};
template <>
struct Elem<TH_FLOAT64>
{
    using T = double;
};

template <int DT>
__device__ __forceinline__ float load_f32(const void* p, int64_t i)
{
    using T = typename Elem<DT>::T;
    if constexpr (DT == TH_FLOAT16)
        return __half2float(static_cast<const __half*>(p)[i]);
    else
        return static_cast<float>(static_cast<const T*>(p)[i]);
}

// Calls f.template operator()<DT>() for a mask/image dtype code; returns false
// for dtypes the reference's dispatch does not cover (bool, bfloat16).
template <class F>
bool dispatch_image_dtype(int dt, F&& f)
{
    switch (dt)
    {
    case TH_UINT8:
        f.template operator()<TH_UINT8>();
        return true;
    case TH_INT8:
        f.template operator()<TH_INT8>();
        return true;
    case TH_INT16:
        f.template operator()<TH_INT16>();
        return true;
    case TH_INT32:
        f.template operator()<TH_INT32>();
        return true;
    case TH_INT64:
        f.template operator()<TH_INT64>();
        return true;
    case TH_FLOAT16:
        f.template operator()<TH_FLOAT16>();
        return true;
    case TH_FLOAT32:
        f.template operator()<TH_FLOAT32>();
        return true;
    case TH_FLOAT64:
        f.template operator()<TH_FLOAT64>();
        return true;
    default:
        return false;
    }
}

// ---------------------------------------------------------------------------
// reference arithmetic (torchhull image_utils.h, math.h, visual_hull_cuda.cu)

__device__ __forceinline__ bool in_image(int64_t y, int64_t x, int64_t h, int64_t w, int64_t margin = 0)
{
    return margin <= y && y < h - margin && margin <= x && x < w - margin;
}

__device__ __forceinline__ float lerp(float v0, float v1, float t)
{
    return __fmaf_rn(t, v1, __fmaf_rn(-t, v0, v0));
}

__device__ __forceinline__ float bilerp(float v00, float v10, float v01, float v11, float ty, float tx)
{
    float v0 = lerp(v00, v10, ty);
    float v1 = lerp(v01, v11, ty);
    return lerp(v0, v1, tx);
}

// c + v/r * L with the product fused, as nvcc contracts the reference's
// expression (visual_hull_cuda.cu:206-213); v/r is exact (r a power of two).
__device__ __forceinline__ float world_coordinate(int64_t v, float r, float corner, float length)
{
    return __fmaf_rn(__fdiv_rn(static_cast<float>(v), r), length, corner);
}

// float -> int64 truncation; the hardware conversion saturates and maps NaN to 0.
__device__ __forceinline__ int64_t f2i64(float f)
{
    return __float2ll_rz(f);
}

// Exact conversions between small non-negative integers and floats with
// adds and bit moves only: the conversion instructions run on narrow pipes
// (the 64-bit ones on the FP64 pipe) and bound the carve otherwise.  Floats
// in [2^23, 2^24) are spaced 1 apart, so 2^23 + n carries the integer n in
// its low mantissa bits.
constexpr float kTwo23 = 8388608.f;
constexpr int32_t kTwo23Bits = 0x4B000000;

// float(n) for n in [0, 2^23).
__device__ __forceinline__ float small_i2f(int32_t n)
{
    return __fsub_rn(__int_as_float(kTwo23Bits | n), kTwo23);
}

struct Snapped
{
    int32_t i; // the integer
    float f;   // the same integer as a float
};

// roundf(v) (half away from zero) clamped to [0, hi], hi an integer below
// 2^23.  Rounding commutes with clamping to integer bounds; for y >= 0,
// round(y) = floor(y + 0.5), and y + 0.5 rounded toward zero keeps that floor
// because every integer below 2^24 is a float; the second add toward zero then
// leaves 2^23 + floor.  NaN clamps to 0, as a saturating conversion and the
// clamp do.
__device__ __forceinline__ Snapped round_clamp(float v, float hi)
{
    const float y = fminf(fmaxf(v, 0.f), hi);
    const float t = __fadd_rz(__fadd_rz(y, 0.5f), kTwo23);
    return Snapped{ __float_as_int(t) - kTwo23Bits, __fsub_rn(t, kTwo23) };
}

// roundf(v) for |v| < 2^22 (round_clamp's adds on |v|, then the sign); false
// (and nothing written) otherwise, NaN included.
__device__ __forceinline__ bool round_small(float v, Snapped& out)
{
    const float a = fabsf(v);
    if (!(a < 4194304.f))
        return false;
    const float t = __fadd_rz(__fadd_rz(a, 0.5f), kTwo23);
    const int32_t n = __float_as_int(t) - kTwo23Bits;
    const float nf = __fsub_rn(t, kTwo23);
    out = Snapped{ v < 0.f ? -n : n, copysignf(nf, v) }; // roundf(-0.f) is -0.f
    return true;
}

// Unsigned 32-bit division by a run-time invariant divisor with one high
// multiply (Granlund & Montgomery, "Division by invariant integers using
// multiplication", 1994, Fig. 4.1): l = ceil(log2 d),
// m = floor(2^32 (2^l - d) / d) + 1, q = (t + ((n - t) >> min(l,1))) >> max(l-1,0)
// with t = mulhi(m, n); exact for every 32-bit n and d >= 1.
struct FastDiv
{
    uint32_t d, m, s1, s2;
};

inline FastDiv make_fastdiv(uint32_t d)
{
    uint32_t l = 0;
    while (l < 32 && (uint64_t{ 1 } << l) < d)
        ++l;
    FastDiv f;
    f.d = d;
    f.m = static_cast<uint32_t>(((uint64_t{ 1 } << 32) * ((uint64_t{ 1 } << l) - d)) / d + 1);
    f.s1 = l < 1 ? l : 1;
    f.s2 = l > 1 ? l - 1 : 0;
    return f;
}

__device__ __forceinline__ uint32_t fast_div(const FastDiv& f, uint32_t n)
{
    const uint32_t t = __umulhi(f.m, n);
    return (t + ((n - t) >> f.s1)) >> f.s2;
}

// Pixel position of a camera-space point (image_utils.h:62-82) from the
// view's rows x, y and divisor (w for OpenGL, z for OpenCV) of its row-major
// 4x4 matrix: K*T*[x,y,z,1] with nested fmaf (visual_hull_cuda.cu:142-156),
// then the division and, for OpenGL, (n + 1) * size / 2 - 0.5 (x / 2 ==
// x * 0.5 exactly).
__device__ __forceinline__ void to_pixel_rows(const float4& rx, const float4& ry, const float4& rd, float x, float y, float z, bool opengl, float H, float W, float& px, float& py)
{
    const float cx = __fmaf_rn(rx.x, x, __fmaf_rn(rx.y, y, __fmaf_rn(rx.z, z, rx.w)));
    const float cy = __fmaf_rn(ry.x, x, __fmaf_rn(ry.y, y, __fmaf_rn(ry.z, z, ry.w)));
    const float cd = __fmaf_rn(rd.x, x, __fmaf_rn(rd.y, y, __fmaf_rn(rd.z, z, rd.w)));
    if (opengl)
    {
        const float nx = __fdiv_rn(cx, cd);
        const float ny = __fdiv_rn(cy, cd);
        px = __fsub_rn(__fmul_rn(__fmul_rn(__fadd_rn(nx, 1.f), W), 0.5f), 0.5f);
        py = __fsub_rn(__fmul_rn(__fmul_rn(__fadd_rn(ny, 1.f), H), 0.5f), 0.5f);
    }
    else
    {
        px = __fsub_rn(__fdiv_rn(cx, cd), 0.5f);
        py = __fsub_rn(__fdiv_rn(cy, cd), 0.5f);
    }
}

// ---------------------------------------------------------------------------
// device-wide scan over n items (n read from device memory) whose counts come
// from a functor.  Pass 1 writes one sum per tile and the block that finishes
// last turns them into exclusive tile offsets (no inter-block waiting); pass 2
// rescans each tile and hands every item its exclusive offset.

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

// Work items dealt out to a warp's lanes: lane s owns the items [excl_s,
// excl_s + count_s) (excl a non-decreasing exclusive prefix sum over the
// lanes).  Slot owning item k: the last lane whose exclusive offset is <= k.
__device__ __forceinline__ int item_slot(int excl, int k)
{
    int s = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1)
    {
        const int e = __shfl_sync(0xffffffffu, excl, s + step);
        if (s + step < 32 && e <= k)
            s += step;
    }
    return s;
}

// Position of the set bit of m with j set bits below it (j < popc(m)).
__device__ __forceinline__ int nth_set_bit(uint32_t m, int j)
{
    int pos = 0;
#pragma unroll
    for (int w = 16; w > 0; w >>= 1)
    {
        const uint32_t low = m & ((1u << w) - 1u);
        const int c = __popc(low);
        if (j >= c)
        {
            j -= c;
            pos += w;
            m >>= w;
        }
        else
            m = low;
    }
    return pos;
}

template <typename T>
__device__ __forceinline__ T warp_inclusive_scan(T v)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1)
    {
        T u = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d)
            v += u;
    }
    return v;
}

// Exclusive scan across the block; returns the thread's exclusive prefix and
// writes the block total to *total (all threads).
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* total)
{
    __shared__ T warp_sums[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    T inc = warp_inclusive_scan(v);
    if (lane == 31)
        warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0)
    {
        T s = lane < nwarps ? warp_sums[lane] : T(0);
        T si = warp_inclusive_scan(s);
        if (lane < nwarps)
            warp_sums[lane] = si - s;
        if (lane == nwarps - 1)
            warp_sums[31] = si;
    }
    __syncthreads();
    T out = warp_sums[warp] + inc - v;
    *total = warp_sums[31];
    __syncthreads();
    return out;
}

struct ScanState
{
    unsigned int blocks_done;
    unsigned int pad;
    unsigned long long total;
};

// Item count of a scan: read from device memory when ptr is set, else val.
struct Count
{
    const int64_t* ptr;
    int64_t val;
    int64_t mul = 1; // items per counted unit (with ptr)
    __device__ __forceinline__ int64_t get() const
    {
        return ptr ? *ptr * mul : val;
    }
};

struct NoEpilogue
{
    __device__ void operator()(unsigned long long) const {}
};

// Called by every block of a tile-sum kernel after its last tile sum is
// written: the block that finishes last turns tile_sums[0, ntiles) into
// exclusive offsets (no inter-block waiting) and runs epi(total) once.
template <class EpiF>
__device__ __forceinline__ void finish_tile_sums(int64_t ntiles,
                                                 unsigned long long* __restrict__ tile_sums,
                                                 ScanState* __restrict__ state,
                                                 EpiF epi)
{
    __threadfence();
    __shared__ bool is_last;
    if (threadIdx.x == 0)
        is_last = (atomicAdd(&state->blocks_done, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!is_last)
        return;
    __threadfence();
    // exclusive scan of the tile sums, in place
    unsigned long long carry = 0;
    for (int64_t b = 0; b < ntiles; b += kScanThreads)
    {
        int64_t t = b + threadIdx.x;
        unsigned long long v = t < ntiles ? *((volatile unsigned long long*)&tile_sums[t]) : 0ull;
        unsigned long long tot;
        unsigned long long ex = block_exclusive_scan(v, &tot);
        if (t < ntiles)
            tile_sums[t] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0)
    {
        state->total = carry;
        state->blocks_done = 0;
        epi(carry);
    }
}

// epi(total) runs once, on one thread, after all tile offsets are final.
template <class CountF, class EpiF>
__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(CountF count,
                                                                   Count n_src,
                                                                   unsigned long long* __restrict__ tile_sums,
                                                                   ScanState* __restrict__ state,
                                                                   EpiF epi)
{
    const int64_t n = n_src.get();
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
    {
        unsigned long long s = 0;
        const int64_t base = tile * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k)
            if (base + k < n)
                s += count(base + k);
        unsigned long long tot;
        block_exclusive_scan(s, &tot);
        if (threadIdx.x == 0)
            tile_sums[tile] = tot;
    }
    finish_tile_sums(ntiles, tile_sums, state, epi);
}

// emit(i, exclusive_offset, count) is called for every item (count may be 0).
// A warp takes kScanItems chunks of 32 consecutive items, one item per lane,
// so that the counts' loads and the emits' stores of a chunk are coalesced;
// a warp scan per chunk and the warps' totals give the offsets.
template <class CountF, class EmitF>
__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(CountF count,
                                                                  EmitF emit,
                                                                  Count n_src,
                                                                  const unsigned long long* __restrict__ tile_offsets)
{
    __shared__ unsigned long long warp_tot[kScanThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t n = n_src.get();
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
    {
        const int64_t first = tile * kScanTile + static_cast<int64_t>(w) * (32 * kScanItems);
        unsigned long long c[kScanItems];
        unsigned long long s = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k)
        {
            const int64_t i = first + k * 32 + lane;
            c[k] = (i < n) ? count(i) : 0ull;
            s += c[k];
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1)
            s += __shfl_xor_sync(0xffffffffu, s, d);
        if (lane == 0)
            warp_tot[w] = s;
        __syncthreads();
        unsigned long long off = tile_offsets[tile];
        for (int v = 0; v < w; ++v)
            off += warp_tot[v];
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kScanItems; ++k)
        {
            const unsigned long long incl = warp_inclusive_scan(c[k]);
            const int64_t i = first + k * 32 + lane;
            if (i < n)
                emit(i, off + incl - c[k], c[k]);
            off += __shfl_sync(0xffffffffu, incl, 31);
        }
    }
}

int sm_count();
void note_launches(int n);
void check_launch(const char* what);

inline int scan_grid(int64_t n_max)
{
    const int64_t tiles = (n_max + kScanTile - 1) / kScanTile;
    const int64_t cap = 4LL * sm_count();
    return static_cast<int>(tiles < 1 ? 1 : (tiles < cap ? tiles : cap));
}

// Pass 1 on stream s: tile sums, then exclusive tile offsets in tile_sums and
// epi(total).  n_max bounds the item count on the host side (it sizes the
// grid; tile_sums must hold ceil(n_max / kScanTile) entries).
template <class CountF, class EpiF>
inline void run_scan_reduce(CountF count,
                            EpiF epi,
                            Count n,
                            int64_t n_max,
                            unsigned long long* tile_sums,
                            ScanState* state,
                            cudaStream_t s)
{
    scan_reduce_kernel<<<scan_grid(n_max), kScanThreads, 0, s>>>(count, n, tile_sums, state, epi);
    check_launch("device-wide scan (reduce)");
    note_launches(1);
}

// Pass 2 on stream s, after run_scan_reduce over the same items: emit(i,
// offset, count) for every item.
template <class CountF, class EmitF>
inline void run_scan_apply(CountF count, EmitF emit, Count n, int64_t n_max, const unsigned long long* tile_sums, cudaStream_t s)
{
    scan_apply_kernel<<<scan_grid(n_max), kScanThreads, 0, s>>>(count, emit, n, tile_sums);
    check_launch("device-wide scan (apply)");
    note_launches(1);
}

// Both scan passes on stream s.
template <class CountF, class EmitF, class EpiF>
inline void run_scan(CountF count,
                     EmitF emit,
                     EpiF epi,
                     Count n,
                     int64_t n_max,
                     unsigned long long* tile_sums,
                     ScanState* state,
                     cudaStream_t s)
{
    run_scan_reduce(count, epi, n, n_max, tile_sums, state, s);
    run_scan_apply(count, emit, n, n_max, tile_sums, s);
}

} // namespace th
