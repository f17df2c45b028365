// Integral images (summed-area tables) of the masks, one per view.
//
// The reference builds them with torch::cumsum over H and then over W in
// float32 (visual_hull_cuda.cu:76-90).  torch scans a non-innermost dimension
// one element at a time from 0, so every SAT value is the float result of that
// fixed sequence of additions.
//
// Two implementations give that exact table:
//
// * 0/1 masks (the usual case) with H*W <= 2^24: every partial sum is an
//   integer below 2^24, so float32 addition is exact in any order and the
//   table can be built in one pass.  sat_bands_kernel: a block takes a band
//   of rows of one view (a ticket from an atomic counter, so bands start in
//   order; the counter and the bands' status words are zeroed before each
//   launch), stages it in shared memory with one TMA bulk copy (an mbarrier
//   tracks the bytes), computes the band's local 2-D prefix sums in int32
//   (column sums per thread, row prefix per warp slice, slice offsets per row
//   through shared memory), publishes the band's last local row (its
//   aggregate), then looks back over the preceding bands of the same view,
//   32 at a time (decoupled look-back: a band that already knows its
//   inclusive prefix ends the walk), for the column carries, publishes its
//   own inclusive prefix, and writes its rows once.  DRAM traffic: the masks
//   read once and the table written once, plus two int32 row vectors per band.
// * anything else (blurred masks, very large images): the two sequential
//   passes below, which perform exactly torch's additions in torch's order,
//   so the table is bit-identical for any mask values.  They also run, gated
//   on the device, after the single pass when it found a value other than 0
//   or 1 (or when one of its bounded waits gave up): they recompute the whole
//   table then.
//
// Column pass: one thread per (view, column) walks down the column; a warp
// covers 32 adjacent columns, so each step is one coalesced 128-byte row read.
// Row pass: one warp per 32 rows walks across them through 32x33 shared
// tiles (coalesced loads and stores, one lane per row scanning its 32 values).
// HBM traffic: read masks + write columns + read columns + write SAT.

#include <algorithm>
#include <atomic>
#include <cstring>
#include <type_traits>

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
                                                          unsigned int* __restrict__ nonbinary,
                                                          const unsigned int* __restrict__ gate)
{
    // gate: run only when the single pass could not be used (see the file comment)
    if (gate && *gate == 0u)
        return;
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
__global__ void __launch_bounds__(32 * kRowWarps) sat_rows_kernel(float* __restrict__ data, int64_t rows, int64_t W,
                                                                  const unsigned int* __restrict__ gate)
{
    if (gate && *gate == 0u)
        return;
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

// ---- single pass for 0/1 masks -------------------------------------------

constexpr int kBandThreads = 256;
constexpr int kBandWarps = kBandThreads / 32;
constexpr int kMaxBandRows = 32;
constexpr uint32_t kSpinLimit = 1u << 20; // bounded waits (about a second at most)

struct SatBandPlan
{
    const void* masks;
    float* out;
    unsigned int* flags; // bit 0: a value other than 0/1; bit 1: a wait gave up
    uint32_t* sched;     // [0] next band ticket (zeroed before the launch)
    uint32_t* status;    // per band: 0, 1 (aggregate published) or 2 (inclusive prefix published); zeroed before the launch
    int32_t* agg;        // per band: its last local row (W values)
    int32_t* incl;       // per band: the table's row at its last row (W values)
    int64_t H, W;
    int32_t rows;        // rows per band (<= kMaxBandRows)
    int32_t bands_per_view;
    int64_t nbands;      // grid size: one block per band
    int32_t vec_out;     // out is 16-byte aligned and W % 4 == 0: rows stored as float4
    int32_t vec_in;      // staged rows start on multiples of min(C * element size, 16) bytes: vector shared loads
};

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_gpu(uint32_t* p, uint32_t v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Arrives on the barrier and expects `bytes` of transactions; returns the phase token.
__device__ __forceinline__ uint64_t mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    uint64_t state;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
                 : "=l"(state)
                 : "r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
    return state;
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t done;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(smem_addr(bar)), "r"(parity)
                 : "memory");
    return done != 0;
}

// One TMA bulk copy global -> shared (16-byte aligned addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ int32_t warp_sum_i32(int32_t v)
{
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, d);
    return v;
}

__device__ __forceinline__ int32_t warp_exclusive_i32(int32_t v, int lane)
{
    int32_t inc = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1)
    {
        const int32_t o = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d)
            inc += o;
    }
    return inc - v;
}

template <int DT>
__device__ __forceinline__ float elem_f32(typename Elem<DT>::T v)
{
    if constexpr (DT == TH_FLOAT16)
        return __half2float(v);
    else
        return static_cast<float>(v);
}

// The C values of a thread's columns in one staged row, as floats.  vec: the
// row's start and the thread's run are aligned for vector loads (the run is
// read with 4-, 8- or 16-byte shared loads, which keeps the warp's reads free
// of bank conflicts); otherwise element by element, zero beyond the image.
template <int DT, int C>
__device__ __forceinline__ void load_run(const void* tile, int64_t row0, int64_t x0, int64_t W, bool vec, float v[C])
{
    using T = typename Elem<DT>::T;
    constexpr int kBytes = C * static_cast<int>(sizeof(T));
    if constexpr (kBytes == 4 || kBytes == 8 || kBytes % 16 == 0)
    {
        if (vec && x0 + C <= W)
        {
            using V = std::conditional_t<kBytes == 4, uint32_t, std::conditional_t<kBytes == 8, uint2, uint4>>;
            constexpr int kPer = static_cast<int>(sizeof(V) / sizeof(T));
            const V* src = reinterpret_cast<const V*>(static_cast<const T*>(tile) + row0 + x0);
#pragma unroll
            for (int q = 0; q < C / kPer; ++q)
            {
                const V u = src[q];
                T e[kPer];
                memcpy(e, &u, sizeof(V));
#pragma unroll
                for (int i = 0; i < kPer; ++i)
                    v[q * kPer + i] = elem_f32<DT>(e[i]);
            }
            return;
        }
    }
#pragma unroll
    for (int c = 0; c < C; ++c)
        v[c] = x0 + c < W ? load_f32<DT>(tile, row0 + x0 + c) : 0.f;
}

// C columns per thread (thread t owns columns [t*C, t*C + C)); TMA: the band
// is staged with one bulk copy (else by plain loads).
template <int DT, int C, bool TMA>
__global__ void __launch_bounds__(kBandThreads) sat_bands_kernel(SatBandPlan p)
{
    using T = typename Elem<DT>::T;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ int32_t wsum[kMaxBandRows][kBandWarps];
    __shared__ int32_t woff[kMaxBandRows][kBandWarps];
    __shared__ uint32_t s_band, s_state;
    __shared__ unsigned int s_flag;
    T* tile = reinterpret_cast<T*>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t W = p.W;

    if (tid == 0)
    {
        s_band = atomicAdd(&p.sched[0], 1u);
        s_flag = 0;
        if (TMA)
            mbar_init(&bar, 1);
    }
    __syncthreads();
    const int64_t band = s_band;
    if (band >= p.nbands)
    {
        // cannot happen with the counter zeroed before the launch; if it does,
        // the exact passes recompute the table
        if (tid == 0)
            atomicOr(p.flags, 2u);
        return;
    }
    const int64_t view = band / p.bands_per_view;
    const int k = static_cast<int>(band - view * p.bands_per_view);
    const int64_t y0 = static_cast<int64_t>(k) * p.rows;
    const int rows = static_cast<int>(p.H - y0 < p.rows ? p.H - y0 : p.rows);
    const int64_t n = rows * W;
    const T* src = static_cast<const T*>(p.masks) + (view * p.H + y0) * W;

    if (TMA)
    {
        if (tid == 0)
        {
            const uint32_t bytes = static_cast<uint32_t>(n * static_cast<int64_t>(sizeof(T)));
            mbar_expect_tx(&bar, bytes);
            bulk_load(tile, src, bytes, &bar);
        }
        bool ok = false;
        for (uint32_t it = 0; it < kSpinLimit && !ok; ++it)
            ok = mbar_try_wait(&bar, 0);
        if (!ok)
        {
            atomicOr(&s_flag, 2u); // results unusable: the exact passes recompute the table
            for (uint32_t it = 0; it < kSpinLimit && !ok; ++it)
                ok = mbar_try_wait(&bar, 0); // the copy must land before the block leaves
        }
    }
    else
    {
        for (int64_t i = tid; i < n; i += kBandThreads)
            tile[i] = src[i];
    }
    __syncthreads();

    const int64_t x0 = static_cast<int64_t>(tid) * C;
    // sweep 1: column sums over the band, per row the sum of each warp's slice
    int32_t col[C];
#pragma unroll
    for (int c = 0; c < C; ++c)
        col[c] = 0;
    bool nb = false;
    for (int r = 0; r < rows; ++r)
    {
        int32_t tsum = 0;
        float v[C];
        load_run<DT, C>(tile, r * W, x0, W, p.vec_in != 0, v);
#pragma unroll
        for (int c = 0; c < C; ++c)
        {
            nb |= (v[c] != 0.f) & (v[c] != 1.f);
            col[c] += v[c] == 1.f ? 1 : 0;
            tsum += col[c];
        }
        tsum = warp_sum_i32(tsum);
        if (lane == 0)
            wsum[r][warp] = tsum;
    }
    if (nb)
        atomicOr(&s_flag, 1u);
    __syncthreads();
    if (tid < rows * kBandWarps)
    {
        const int r = tid / kBandWarps, w = tid % kBandWarps;
        int32_t acc = 0;
        for (int j = 0; j < w; ++j)
            acc += wsum[r][j];
        woff[r][w] = acc;
    }
    if (tid == 0 && s_flag)
        atomicOr(p.flags, s_flag);
    __syncthreads();

    // the band's aggregate: its last local row
    int32_t lp[C], agg[C], carry[C];
    {
        int32_t run = 0;
#pragma unroll
        for (int c = 0; c < C; ++c)
        {
            run += col[c];
            lp[c] = run;
        }
        const int32_t ex = warp_exclusive_i32(run, lane) + woff[rows - 1][warp];
#pragma unroll
        for (int c = 0; c < C; ++c)
        {
            agg[c] = ex + lp[c];
            carry[c] = 0;
        }
    }
    int32_t* aggv = p.agg + band * W;
    int32_t* inclv = p.incl + band * W;
#pragma unroll
    for (int c = 0; c < C; ++c)
        if (x0 + c < W)
        {
            aggv[x0 + c] = agg[c];
            if (k == 0)
                inclv[x0 + c] = agg[c];
        }
    __syncthreads();
    if (tid == 0)
    {
        __threadfence();
        st_release_gpu(&p.status[band], k == 0 ? 2u : 1u);
    }
    if (k > 0)
    {
        // Look back over the preceding bands of this view, 32 at a time: warp 0
        // reads their status words; the window folds in the aggregates up to
        // the nearest band whose inclusive prefix is published (the view's
        // first band always publishes one), or all 32 aggregates and moves on.
        const int64_t first = view * p.bands_per_view;
        int64_t j = band - 1;
        for (;;)
        {
            if (warp == 0)
            {
                const int64_t jj = j - lane;
                const bool in = jj >= first;
                int cut = 0;
                bool ready = false, incl_found = false;
                for (uint32_t it = 0; it < kSpinLimit && !ready; ++it)
                {
                    const uint32_t v = in ? ld_acquire_gpu(&p.status[jj]) : 0u;
                    const uint32_t m2 = __ballot_sync(0xffffffffu, in && v == 2u);
                    const uint32_t m0 = __ballot_sync(0xffffffffu, in && v == 0u);
                    const uint32_t mout = __ballot_sync(0xffffffffu, !in);
                    if (m2)
                    {
                        const int c2 = __ffs(m2) - 1;
                        if ((m0 & ((1u << c2) - 1u)) == 0u)
                        {
                            cut = c2;
                            incl_found = true;
                            ready = true;
                        }
                    }
                    else if (m0 == 0u && mout == 0u)
                    {
                        cut = 32;
                        ready = true;
                    }
                    if (!ready)
                        __nanosleep(64);
                }
                if (lane == 0)
                {
                    // bits 0-7: aggregates to fold; bit 8: the walk ends here;
                    // bit 9: also fold the inclusive prefix of band j - cut
                    if (!ready)
                    {
                        atomicOr(p.flags, 2u); // gave up: the exact passes recompute the table
                        s_state = 0x100u;
                    }
                    else
                        s_state = static_cast<uint32_t>(cut) | (incl_found ? 0x300u : 0u);
                }
            }
            __syncthreads();
            const uint32_t st = s_state;
            const int cut = static_cast<int>(st & 0xffu);
            const bool done = (st & 0x100u) != 0u;
            for (int i = 0; i < cut; ++i)
            {
                const int32_t* v = p.agg + (j - i) * W;
#pragma unroll
                for (int c = 0; c < C; ++c)
                    if (x0 + c < W)
                        carry[c] += __ldcg(v + x0 + c);
            }
            if (st & 0x200u)
            {
                const int32_t* v = p.incl + (j - cut) * W;
#pragma unroll
                for (int c = 0; c < C; ++c)
                    if (x0 + c < W)
                        carry[c] += __ldcg(v + x0 + c);
            }
            __syncthreads();
            if (done)
                break;
            j -= 32;
        }
#pragma unroll
        for (int c = 0; c < C; ++c)
            if (x0 + c < W)
                inclv[x0 + c] = carry[c] + agg[c];
        __syncthreads();
        if (tid == 0)
        {
            __threadfence();
            st_release_gpu(&p.status[band], 2u);
        }
    }

    // sweep 2: the band's rows, carries added, written once
    float* out = p.out + (view * p.H + y0) * W;
#pragma unroll
    for (int c = 0; c < C; ++c)
        col[c] = 0;
    for (int r = 0; r < rows; ++r)
    {
        int32_t run = 0;
        float v[C];
        load_run<DT, C>(tile, r * W, x0, W, p.vec_in != 0, v);
#pragma unroll
        for (int c = 0; c < C; ++c)
        {
            col[c] += v[c] == 1.f ? 1 : 0;
            run += col[c];
            lp[c] = run;
        }
        const int32_t ex = warp_exclusive_i32(run, lane) + woff[r][warp];
        float* orow = out + r * W + x0;
        if constexpr (C % 4 == 0)
        {
            if (p.vec_out && x0 + C <= W)
            {
#pragma unroll
                for (int c = 0; c < C; c += 4)
                    *reinterpret_cast<float4*>(orow + c) =
                            make_float4(static_cast<float>(carry[c] + ex + lp[c]),
                                        static_cast<float>(carry[c + 1] + ex + lp[c + 1]),
                                        static_cast<float>(carry[c + 2] + ex + lp[c + 2]),
                                        static_cast<float>(carry[c + 3] + ex + lp[c + 3]));
                continue;
            }
        }
#pragma unroll
        for (int c = 0; c < C; ++c)
            if (x0 + c < W)
                orow[c] = static_cast<float>(carry[c] + ex + lp[c]);
    }
}

struct BandShape
{
    int rows = 0, cols_per_thread = 0;
    int64_t bands_per_view = 0, smem = 0;
};

const int kElemBytes[] = { 1, 1, 1, 2, 4, 8, 2, 4, 8 }; // by dtype code

// Band shape of the single pass, or rows == 0 when it does not apply.
BandShape band_shape(int64_t B, int64_t H, int64_t W, int dtype)
{
    BandShape s;
    if (dtype < TH_UINT8 || dtype > TH_FLOAT64 || B <= 0 || H <= 0 || W <= 0)
        return s;
    if (H * W > (int64_t{ 1 } << 24) || W > 16 * kBandThreads)
        return s;
    // bands of about 64 KB (3 blocks per SM), at least 16 rows where 128 KB
    // allows it, else 8: fewer, taller bands shorten the look-back (its
    // carries are whole rows); smaller bands measured slower on GB300
    const int64_t row_bytes = W * kElemBytes[dtype];
    int64_t rows = std::min<int64_t>(kMaxBandRows, 65536 / row_bytes);
    if (rows < 16)
        rows = std::min<int64_t>(16, 131072 / row_bytes);
    if (rows < 8)
        return s;
    const int64_t need = (W + kBandThreads - 1) / kBandThreads;
    s.cols_per_thread = need <= 1 ? 1 : need <= 2 ? 2 : need <= 4 ? 4 : need <= 8 ? 8 : 16;
    s.rows = static_cast<int>(rows);
    s.bands_per_view = (H + rows - 1) / rows;
    s.smem = rows * row_bytes;
    return s;
}

constexpr int64_t kSchedBytes = 256;

int64_t status_bytes(int64_t nbands)
{
    return (nbands * 4 + 255) / 256 * 256;
}

template <int DT>
__global__ void convert_transforms_kernel(const void* __restrict__ tf, int64_t n, float* __restrict__ out)
{
    const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = load_f32<DT>(tf, i);
}

} // namespace

int64_t sat_scratch_bytes(int64_t B, int64_t H, int64_t W, int dtype)
{
    const BandShape bs = band_shape(B, H, W, dtype);
    if (bs.rows == 0)
        return 0;
    const int64_t nbands = B * bs.bands_per_view;
    return kSchedBytes + status_bytes(nbands) + 2 * nbands * W * 4;
}

namespace
{

template <int DT, int C, bool TMA>
void launch_bands(const SatBandPlan& plan, int64_t nbands, int64_t smem, cudaStream_t s)
{
    auto kernel = sat_bands_kernel<DT, C, TMA>;
    // the shared-memory limit is raised once per device (a second call is harmless)
    static std::atomic<uint64_t> configured{ 0 };
    int dev = 0;
    TH_CUDA(cudaGetDevice(&dev));
    const uint64_t bit = uint64_t{ 1 } << (dev & 63);
    if (!(configured.load() & bit))
    {
        TH_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 131072));
        configured.fetch_or(bit);
    }
    kernel<<<static_cast<unsigned>(nbands), kBandThreads, static_cast<size_t>(smem), s>>>(plan);
}

template <int DT, bool TMA>
void launch_bands_c(int c, const SatBandPlan& plan, int64_t nbands, int64_t smem, cudaStream_t s)
{
    switch (c)
    {
    case 1:
        launch_bands<DT, 1, TMA>(plan, nbands, smem, s);
        break;
    case 2:
        launch_bands<DT, 2, TMA>(plan, nbands, smem, s);
        break;
    case 4:
        launch_bands<DT, 4, TMA>(plan, nbands, smem, s);
        break;
    case 8:
        launch_bands<DT, 8, TMA>(plan, nbands, smem, s);
        break;
    default:
        launch_bands<DT, 16, TMA>(plan, nbands, smem, s);
        break;
    }
}

} // namespace

void launch_integral_image(const void* masks,
                           int dtype,
                           int64_t B,
                           int64_t H,
                           int64_t W,
                           float* out,
                           cudaStream_t s,
                           unsigned int* nonbinary,
                           SatScratch scratch)
{
    if (B * H * W == 0)
        return;
    const unsigned int* gate = nullptr;
    const BandShape bs = band_shape(B, H, W, dtype);
    if (bs.rows > 0 && scratch.p && nonbinary)
    {
        const int64_t nbands = B * bs.bands_per_view;
        auto* base = static_cast<unsigned char*>(scratch.p);
        SatBandPlan plan{};
        plan.masks = masks;
        plan.out = out;
        plan.flags = nonbinary;
        plan.sched = reinterpret_cast<uint32_t*>(base);
        plan.status = reinterpret_cast<uint32_t*>(base + kSchedBytes);
        plan.agg = reinterpret_cast<int32_t*>(base + kSchedBytes + status_bytes(nbands));
        plan.incl = plan.agg + nbands * W;
        plan.H = H;
        plan.W = W;
        plan.rows = bs.rows;
        plan.bands_per_view = static_cast<int32_t>(bs.bands_per_view);
        plan.nbands = nbands;
        plan.vec_out = (reinterpret_cast<uintptr_t>(out) % 16 == 0) && (W % 4 == 0);
        const int64_t run_bytes = std::min<int64_t>(int64_t{ bs.cols_per_thread } * kElemBytes[dtype], 16);
        plan.vec_in = (W * kElemBytes[dtype]) % run_bytes == 0;
        // the ticket counter and this launch's status words start at zero (row
        // vectors of earlier launches of other shapes may lie where they are now)
        launch_zero(base, static_cast<size_t>(kSchedBytes + status_bytes(nbands)), s);
        const bool tma = (reinterpret_cast<uintptr_t>(masks) % 16 == 0) && ((W * kElemBytes[dtype]) % 16 == 0);
        const bool ok = dispatch_image_dtype(dtype, [&]<int DT>() {
            if (tma)
                launch_bands_c<DT, true>(bs.cols_per_thread, plan, nbands, bs.smem, s);
            else
                launch_bands_c<DT, false>(bs.cols_per_thread, plan, nbands, bs.smem, s);
        });
        if (!ok)
            throw CudaError{ cudaErrorInvalidValue, "integral image: unsupported mask dtype" };
        TH_LAUNCH_CHECK();
        gate = nonbinary; // the exact passes below run only if the single pass could not be used
    }
    const int64_t cols = B * W;
    const unsigned grid = static_cast<unsigned>((cols + 255) / 256);
    bool ok = dispatch_image_dtype(dtype, [&]<int DT>() {
        sat_columns_kernel<DT><<<grid, 256, 0, s>>>(masks, out, B, H, W, nonbinary, gate);
    });
    if (!ok)
        throw CudaError{ cudaErrorInvalidValue, "integral image: unsupported mask dtype" };
    TH_LAUNCH_CHECK();
    const int64_t rows = B * H;
    const unsigned grid_rows = static_cast<unsigned>((rows + 32 * kRowWarps - 1) / (32 * kRowWarps));
    sat_rows_kernel<<<grid_rows, 32 * kRowWarps, 0, s>>>(out, rows, W, gate);
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
