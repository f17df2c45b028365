// Leaf corners, hull field and sparse marching cubes.
//
// Corner set.  The reference turns the leaf cells into 8 corner ids each, then
// radix-sorts and uniques them (visual_hull_cuda.cu:770-825).  Here each leaf
// sets its corners in a bitmap over the (2^L+1)^3 grid, laid out row by row
// (x fastest, one row = WR 64-bit words) so that scanning the set bits in
// memory order yields the ids already ascending and unique.  A second bitmap
// flags the rows that hold any bit, so only those rows are scanned and later
// cleared.  The scan also stores, per word, the rank of its first bit, which
// turns "index of corner v in the sorted list" into one word load, one rank
// load and a popcount: this replaces the hash map the reference builds for its
// marching cubes (marching_cubes_cuda.cu:66-70, :133-144).
//
// Hull field.  One thread per corner multiplies the bilinear mask samples of
// all views in ascending view order, the order in which the reference's
// per-view launches (visual_hull_cuda.cu:827-888) multiply them.
//
// Marching cubes.  A corner g is a cell when all 8 cube corners are present
// (marching_cubes_cuda.cu:180-223).  Its code selects triangles from the
// table; every edge a triangle uses is marked on the edge's lower corner (3
// bits per corner, one per axis).  A scan over corners then numbers the marked
// edges in (corner, axis) order, which is exactly the reference's vertex order
// after torch::unique_dim over the edge ids (ravel(p1) << 3 | 1 << axis),
// (:99-112, :674-693), without a sort.  Faces are emitted per cell in
// ascending corner order and table order, as the reference's soup is.

#include "mc_tables.h"
#include "th_hull.cuh"
#include "th_internal.h"

namespace th
{

namespace
{

__device__ const uint8_t g_mc_count[256] = TH_MC_TRI_COUNT_INIT;
__device__ const uint8_t g_mc_edges[256][15] = TH_MC_TRI_EDGES_INIT;

struct TableCache
{
    uint8_t count[256];
    uint8_t edges[256][16];
};

__device__ __forceinline__ void load_tables(TableCache& t)
{
    for (int i = threadIdx.x; i < 256; i += blockDim.x)
    {
        t.count[i] = g_mc_count[i];
#pragma unroll
        for (int j = 0; j < 15; ++j)
            t.edges[i][j] = g_mc_edges[i][j];
    }
    __syncthreads();
}

// Rank of grid point (x,y,z) among the set corners, or false if not set.
__device__ __forceinline__ bool corner_rank(const HullPlan& p, int64_t x, int64_t y, int64_t z, uint32_t& rank)
{
    const int64_t row = y + z * p.R;
    const int64_t w = row * p.WR + (x >> 6);
    const uint64_t word = p.bitmap[w];
    const uint64_t bit = 1ull << (x & 63);
    if (!(word & bit))
        return false;
    rank = p.word_rank[w] + static_cast<uint32_t>(__popcll(word & (bit - 1)));
    return true;
}

__global__ void __launch_bounds__(256) mark_corners_kernel(HullPlan p)
{
    const DevCounters* c = p.ctr;
    const int L = p.level;
    const int64_t n = c->level_count[L];
    const int64_t* leaves = p.nodes + c->level_off[L];
    const int64_t r = int64_t{ 1 } << L;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += stride)
    {
        const int64_t idx = leaves[t];
        const int64_t x = idx & (r - 1), y = (idx >> L) & (r - 1), z = idx >> (2 * L);
        mark_cell_corners(p.bitmap, p.rowbits, p.R, p.WR, x, y, z);
    }
}

struct RowCount
{
    const uint32_t* rowbits;
    __device__ unsigned long long operator()(int64_t i) const
    {
        return static_cast<unsigned long long>(__popc(rowbits[i]));
    }
};

struct RowEmit
{
    const uint32_t* rowbits;
    uint32_t* rows;
    __device__ void operator()(int64_t i, unsigned long long off, unsigned long long cnt) const
    {
        uint32_t w = rowbits[i];
        while (w)
        {
            const int bit = __ffs(w) - 1;
            rows[off++] = static_cast<uint32_t>(i * 32 + bit);
            w &= w - 1;
        }
    }
};

struct RowEpilogue
{
    DevCounters* ctr;
    __device__ void operator()(unsigned long long total) const
    {
        ctr->rows = static_cast<int64_t>(total);
    }
};

struct CornerCount
{
    HullPlan p;
    __device__ unsigned long long operator()(int64_t k) const
    {
        const int64_t base = static_cast<int64_t>(p.rows[k]) * p.WR;
        unsigned long long s = 0;
        for (int64_t w = 0; w < p.WR; ++w)
            s += __popcll(p.bitmap[base + w]);
        return s;
    }
};

struct CornerEmit
{
    HullPlan p;
    __device__ void operator()(int64_t k, unsigned long long off, unsigned long long) const
    {
        const int64_t row = p.rows[k];
        const int64_t base = row * p.WR;
        const uint32_t ry = static_cast<uint32_t>(row) % static_cast<uint32_t>(p.R);
        const uint32_t rz = static_cast<uint32_t>(row) / static_cast<uint32_t>(p.R);
        uint64_t out = off;
        for (int64_t w = 0; w < p.WR; ++w)
        {
            uint64_t word = p.bitmap[base + w];
            p.word_rank[base + w] = static_cast<uint32_t>(out);
            while (word)
            {
                const int bit = __ffsll(static_cast<long long>(word)) - 1;
                if (static_cast<int64_t>(out) < p.corner_cap)
                {
                    p.corners[out] = pack_corner(w * 64 + bit, ry, rz);
                    p.emask[out] = 0;
                }
                ++out;
                word &= word - 1;
            }
        }
    }
};

struct CornerEpilogue
{
    DevCounters* ctr;
    int64_t cap;
    __device__ void operator()(unsigned long long total) const
    {
        int64_t n = static_cast<int64_t>(total);
        if (n > cap)
        {
            ctr->overflow |= kOverflowCorners;
            n = cap;
        }
        ctr->corners = n;
    }
};

template <int DT>
__device__ __forceinline__ float mask_sample(const HullPlan& p, const void* masks, int64_t b, int64_t y, int64_t x, float pad)
{
    // 0 <= y < H and 0 <= x < W, as unsigned compares
    return (static_cast<uint64_t>(y) < static_cast<uint64_t>(p.H) && static_cast<uint64_t>(x) < static_cast<uint64_t>(p.W))
                   ? load_f32<DT>(masks, (b * p.H + y) * p.W + x)
                   : pad;
}

// Factor of view b for the corner at world point (wx, wy, wz): the bilinear
// mask sample (image_utils.h:162-214), or exactly 1 when partial mode skips
// the view (x * 1 == x, so multiplying by it equals skipping it).
//
// The reference converts the rounded pixel to int64.  Near the image the
// rounding and the conversion are done exactly with float adds (the
// conversion instructions run on narrow pipes, the 64-bit ones on GB300's
// FP64 pipe); far from it (|coordinate| >= 2^22, or NaN) the saturating int32
// conversion stands in: the in-image tests decide identically, and where its
// value differs from the int64 one (|coordinate| >= 2^31) all four samples
// are padding, for which the interpolation gives the same result (0, 1 or
// NaN) for either weight.
template <int DT, bool PARTIAL>
__device__ __forceinline__ float view_factor(const HullPlan& p, const void* masks, int64_t b, const float4 (&rows)[3], float wx, float wy, float wz, float Hf, float Wf)
{
    float px, py;
    to_pixel_rows(rows[0], rows[1], rows[2], wx, wy, wz, p.opengl, Hf, Wf, px, py);
    const float pad = PARTIAL ? 1.f : 0.f;
    // 1 <= round(q) < size - 1 (half away from zero) exactly when 0.5 <= q < size - 1.5
    if (PARTIAL && !(px >= 0.5f && px < __fsub_rn(Wf, 1.5f) && py >= 0.5f && py < __fsub_rn(Hf, 1.5f)))
        return 1.f;
    Snapped ry, rx;
    if (!round_small(__fadd_rn(py, -0.5f), ry))
    {
        ry.i = __float2int_rz(roundf(__fadd_rn(py, -0.5f)));
        ry.f = __int2float_rn(ry.i);
    }
    if (!round_small(__fadd_rn(px, -0.5f), rx))
    {
        rx.i = __float2int_rz(roundf(__fadd_rn(px, -0.5f)));
        rx.f = __int2float_rn(rx.i);
    }
    const int64_t y0 = ry.i, x0 = rx.i;
    // All-ones footprint: the sample is exactly 1.  The weights q - round(q
    // - 0.5) lie in [0, 1] whenever the footprint starts inside the image
    // (q - 0.5 is exact for q >= 0.5; below, a start of 0 means q in (0,
    // 0.5)), except for q = NaN, whose sample is NaN.
    if (p.field_ones && static_cast<uint64_t>(y0) < static_cast<uint64_t>(p.H) &&
        static_cast<uint64_t>(x0) < static_cast<uint64_t>(p.W) && px == px && py == py)
    {
        const uint32_t word = __ldg(p.ones + (b * p.H + y0) * p.WW + (x0 >> 5));
        if ((word >> (x0 & 31)) & 1u)
            return 1.f;
    }
    float v00, v10, v01, v11;
    if (PARTIAL)
    {
        // in frame: round(q - 0.5) lies in [0, size - 2], so all four samples are inside
        const int64_t i = (b * p.H + y0) * p.W + x0;
        v00 = load_f32<DT>(masks, i);
        v01 = load_f32<DT>(masks, i + 1);
        v10 = load_f32<DT>(masks, i + p.W);
        v11 = load_f32<DT>(masks, i + p.W + 1);
    }
    else
    {
        v00 = mask_sample<DT>(p, masks, b, y0, x0, pad);
        v10 = mask_sample<DT>(p, masks, b, y0 + 1, x0, pad);
        v01 = mask_sample<DT>(p, masks, b, y0, x0 + 1, pad);
        v11 = mask_sample<DT>(p, masks, b, y0 + 1, x0 + 1, pad);
    }
    const float ty = __fsub_rn(py, ry.f);
    const float tx = __fsub_rn(px, rx.f);
    return bilerp(v00, v10, v01, v11, ty, tx);
}

// The all-ones footprint bitmap of the masks (HullPlan::ones): one warp per
// mask row y, 32 columns per step; a lane tests its column in rows y and y+1
// and takes its right neighbour's result by a shuffle (the last lane loads
// the column after the step).  Columns x = W-1 and rows y = H-1 have no 2x2
// footprint and get 0.
template <int DT>
__global__ void __launch_bounds__(256) ones_kernel(HullPlan p)
{
    const void* masks = p.rq->masks;
    const int64_t H = p.H, W = p.W, rows = p.B * H;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t row = warp; row < rows; row += nwarps)
    {
        const int64_t y = row % H;
        const bool below = y + 1 < H;
        const int64_t base = row * W;
        for (int64_t x0 = 0; x0 < W; x0 += 32)
        {
            const int64_t x = x0 + lane;
            bool col = false; // column x is 1 in rows y and y+1
            if (x < W && below)
                col = load_f32<DT>(masks, base + x) == 1.f && load_f32<DT>(masks, base + W + x) == 1.f;
            bool next = __shfl_down_sync(0xffffffffu, col, 1);
            if (lane == 31)
                next = x + 1 < W && below && load_f32<DT>(masks, base + x + 1) == 1.f &&
                       load_f32<DT>(masks, base + W + x + 1) == 1.f;
            const uint32_t word = __ballot_sync(0xffffffffu, col && next);
            if (lane == 0)
                p.ones[row * p.WW + (x0 >> 5)] = word;
        }
    }
}

// accumulate_hull_counts_{full,partial} (visual_hull_cuda.cu:419-520): the
// views [b0, b1) multiplied into each corner's running product in ascending
// view order (b0 == 0 starts it at 1).  Views go in chunks of kFieldViews, one
// launch each, so that all resident threads read the masks of the same few
// views and those stay in L2; the product is the same sequence of roundings.
constexpr int64_t kFieldViews = 16;

template <int DT, bool PARTIAL>
__global__ void __launch_bounds__(256) field_kernel(HullPlan p, int64_t b0, int64_t b1)
{
    // the projection rows of the chunk's views, read from shared memory by
    // every (corner, view) pair instead of twelve global loads each
    __shared__ float4 rows[kFieldViews][3];
    const int nv = static_cast<int>(b1 - b0);
    for (int i = threadIdx.x; i < 3 * nv; i += blockDim.x)
    {
        const int v = i / 3, r = i - 3 * (i / 3);
        const int row = r < 2 ? r : (p.opengl ? 3 : 2);
        rows[v][r] = *reinterpret_cast<const float4*>(p.tf + 16 * (b0 + v) + 4 * row);
    }
    __syncthreads();
    const int64_t n = p.ctr->corners;
    const int64_t R = p.R;
    const float inv_rc = __fdiv_rn(1.f, static_cast<float>(R - 1)); // exact: a power of two
    const float Hf = small_i2f(static_cast<int32_t>(p.H)), Wf = small_i2f(static_cast<int32_t>(p.W));
    const float cx = p.rq->corner[0], cy = p.rq->corner[1], cz = p.rq->corner[2], length = p.rq->length;
    const void* masks = p.rq->masks;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += stride)
    {
        const int64_t idx = p.corners[t];
        int64_t gx, gy, gz;
        unpack_corner(idx, gx, gy, gz);
        // c + v/r * L fused (visual_hull_cuda.cu:444-448); v/r == v * (1/r) exactly
        // corner coordinates are at most 2^12
        const float wx = __fmaf_rn(__fmul_rn(small_i2f(static_cast<int32_t>(gx)), inv_rc), length, cx);
        const float wy = __fmaf_rn(__fmul_rn(small_i2f(static_cast<int32_t>(gy)), inv_rc), length, cy);
        const float wz = __fmaf_rn(__fmul_rn(small_i2f(static_cast<int32_t>(gz)), inv_rc), length, cz);
        float value = b0 == 0 ? 1.f : p.values[t];
#pragma unroll 4
        for (int v = 0; v < nv; ++v)
            value = __fmul_rn(value, view_factor<DT, PARTIAL>(p, masks, b0 + v, rows[v], wx, wy, wz, Hf, Wf));
        p.values[t] = value;
    }
}

// Ranks of the 8 corners of the cell with base corner t; false if incomplete.
// Ranks at or beyond n (possible only when the corner pool overflowed and the
// request is about to be rerun) count as missing, so no access leaves the pools.
__device__ __forceinline__ bool cell_ranks(const HullPlan& p,
                                           int64_t t,
                                           int64_t n,
                                           int64_t gx,
                                           int64_t gy,
                                           int64_t gz,
                                           uint32_t rk[8])
{
    const int64_t R = p.R;
    if (!(gx < R - 1 && gy < R - 1 && gz < R - 1))
        return false;
    rk[0] = static_cast<uint32_t>(t);
#pragma unroll
    for (int i = 1; i < 8; ++i)
        if (!corner_rank(p, gx + (i & 1), gy + (i >> 1 & 1), gz + (i >> 2 & 1), rk[i]) || rk[i] >= n)
            return false;
    return true;
}

// classify_voxels_sparse (marching_cubes_cuda.cu:180-223) plus edge marking.
__global__ void __launch_bounds__(256) mc_cells_kernel(HullPlan p)
{
    __shared__ TableCache tab;
    load_tables(tab);
    const int64_t n = p.ctr->corners;
    const float iso = 0.5f;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += stride)
    {
        const int64_t idx = p.corners[t];
        int64_t gx, gy, gz;
        unpack_corner(idx, gx, gy, gz);
        uint32_t rk[8];
        uint32_t code = 0;
        if (cell_ranks(p, t, n, gx, gy, gz, rk))
        {
#pragma unroll
            for (int i = 0; i < 8; ++i)
                if (p.values[rk[i]] < iso)
                    code |= 1u << i;
            const int cnt = tab.count[code];
            uint32_t used = 0; // bit (lo * 3 + axis)
            for (int j = 0; j < cnt; ++j)
            {
                const uint32_t e = tab.edges[code][j];
                used |= 1u << ((e & 7u) * 3u + (e >> 3));
            }
            while (used)
            {
                const int k = __ffs(used) - 1;
                used &= used - 1;
                const uint32_t r1 = rk[k / 3];
                const uint32_t bit = (1u << (k % 3)) << (8u * (r1 & 3u));
                unsigned int* word = reinterpret_cast<unsigned int*>(p.emask) + (r1 >> 2);
                if ((*word & bit) != bit)
                    atomicOr(word, bit);
            }
        }
        p.codes[t] = static_cast<uint8_t>(code);
    }
}

struct VertCount
{
    const uint8_t* codes;
    const uint8_t* emask;
    __device__ unsigned long long operator()(int64_t t) const
    {
        return (static_cast<unsigned long long>(g_mc_count[codes[t]]) << 32) |
               static_cast<unsigned long long>(__popc(emask[t]));
    }
};

struct VertEmit
{
    uint32_t* soup_off;
    uint32_t* vbase;
    __device__ void operator()(int64_t t, unsigned long long off, unsigned long long) const
    {
        soup_off[t] = static_cast<uint32_t>(off >> 32);
        vbase[t] = static_cast<uint32_t>(off & 0xffffffffull);
    }
};

struct VertEpilogue
{
    DevCounters* ctr;
    __device__ void operator()(unsigned long long total) const
    {
        ctr->soup = static_cast<int64_t>(total >> 32);
        ctr->verts = static_cast<int64_t>(total & 0xffffffffull);
    }
};

// interpolate_vertex (marching_cubes_cuda.cu:72-97) followed by the world
// transform of to_global_coordinates (visual_hull_cuda.cu:916-939).
__device__ __forceinline__ void edge_vertex(const HullPlan& p,
                                            int64_t x1,
                                            int64_t y1,
                                            int64_t z1,
                                            int axis,
                                            float v1,
                                            float v2,
                                            float scale,
                                            float* out)
{
    const float iso = 0.5f, eps = 1e-5f;
    const int64_t x2 = x1 + (axis == 0), y2 = y1 + (axis == 1), z2 = z1 + (axis == 2);
    // 1: snap to p1, 2: snap to p2, 0: interpolate (the reference's check order)
    int snap = 0;
    if (fabsf(__fsub_rn(iso, v1)) < eps)
        snap = 1;
    else if (fabsf(__fsub_rn(iso, v2)) < eps)
        snap = 2;
    else if (fabsf(__fsub_rn(v1, v2)) < eps)
        snap = 1;
    float q[3];
    if (snap == 1)
    {
        q[0] = static_cast<float>(x1);
        q[1] = static_cast<float>(y1);
        q[2] = static_cast<float>(z1);
    }
    else if (snap == 2)
    {
        q[0] = static_cast<float>(x2);
        q[1] = static_cast<float>(y2);
        q[2] = static_cast<float>(z2);
    }
    else
    {
        const float t = __fdiv_rn(__fsub_rn(iso, v1), __fsub_rn(v2, v1));
        q[0] = lerp(static_cast<float>(x1), static_cast<float>(x2), t);
        q[1] = lerp(static_cast<float>(y1), static_cast<float>(y2), t);
        q[2] = lerp(static_cast<float>(z1), static_cast<float>(z2), t);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
        out[a] = __fmaf_rn(scale, q[a], p.corner[a]);
}

__global__ void __launch_bounds__(256) export_verts_kernel(HullPlan p, float* __restrict__ verts)
{
    const int64_t n = p.ctr->corners;
    const float scale = __fdiv_rn(p.length, static_cast<float>(int64_t{ 1 } << p.level));
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += stride)
    {
        const uint32_t bits = p.emask[t];
        if (!bits)
            continue;
        const int64_t idx = p.corners[t];
        int64_t gx, gy, gz;
        unpack_corner(idx, gx, gy, gz);
        const float v1 = p.values[t];
        int64_t out = p.vbase[t];
#pragma unroll
        for (int a = 0; a < 3; ++a)
        {
            if (!(bits >> a & 1u))
                continue;
            uint32_t r2 = 0;
            corner_rank(p, gx + (a == 0), gy + (a == 1), gz + (a == 2), r2);
            float v[3];
            edge_vertex(p, gx, gy, gz, a, v1, p.values[r2], scale, v);
            verts[3 * out + 0] = v[0];
            verts[3 * out + 1] = v[1];
            verts[3 * out + 2] = v[2];
            ++out;
        }
    }
}

// Faces in soup order; with unique vertices they index the edge-numbered
// vertex list, without they index the soup, which this kernel also writes.
// Columns 1 and 2 are swapped as flip_faces does (visual_hull_cuda.cu:941-956).
__global__ void __launch_bounds__(256) export_faces_kernel(HullPlan p, float* __restrict__ verts, int64_t* __restrict__ faces)
{
    __shared__ TableCache tab;
    load_tables(tab);
    const int64_t n = p.ctr->corners;
    const float scale = __fdiv_rn(p.length, static_cast<float>(int64_t{ 1 } << p.level));
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += stride)
    {
        const uint32_t code = p.codes[t];
        const int cnt = tab.count[code];
        if (cnt == 0)
            continue;
        const int64_t idx = p.corners[t];
        int64_t gx, gy, gz;
        unpack_corner(idx, gx, gy, gz);
        uint32_t rk[8];
        cell_ranks(p, t, n, gx, gy, gz, rk);
        const int64_t base = p.soup_off[t];
        for (int j = 0; j < cnt; ++j)
        {
            const uint32_t e = tab.edges[code][j];
            const int lo = static_cast<int>(e & 7u), axis = static_cast<int>(e >> 3);
            const int64_t f = base + j;
            const int slot = static_cast<int>(f % 3);
            const int64_t dst = f - slot + (slot == 0 ? 0 : 3 - slot);
            if (p.unique)
            {
                const uint32_t r1 = rk[lo];
                faces[dst] = static_cast<int64_t>(p.vbase[r1]) + __popc(p.emask[r1] & ((1u << axis) - 1u));
            }
            else
            {
                float v[3];
                const int hi = lo | (1 << axis);
                edge_vertex(p, gx + (lo & 1), gy + (lo >> 1 & 1), gz + (lo >> 2 & 1), axis, p.values[rk[lo]],
                            p.values[rk[hi]], scale, v);
                verts[3 * f + 0] = v[0];
                verts[3 * f + 1] = v[1];
                verts[3 * f + 2] = v[2];
                faces[dst] = f;
            }
        }
    }
}

__global__ void __launch_bounds__(256) clear_rows_kernel(HullPlan p)
{
    const int64_t n = p.ctr->rows;
    const int64_t total = n * p.WR;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += stride)
    {
        const int64_t k = i / p.WR, w = i - k * p.WR;
        p.bitmap[static_cast<int64_t>(p.rows[k]) * p.WR + w] = 0;
    }
}

} // namespace

void launch_corners(const HullPlan& p, cudaStream_t s)
{
    const int64_t max_leaves = p.node_cap;
    mark_corners_kernel<<<grid_for(max_leaves, 256), 256, 0, s>>>(p);
    TH_LAUNCH_CHECK();
    launch_rank_corners(p, s);
}

void launch_rank_corners(const HullPlan& p, cudaStream_t s)
{
    const int64_t row_words = (p.R * p.R + 31) / 32;
    run_scan(RowCount{ p.rowbits }, RowEmit{ p.rowbits, p.rows }, RowEpilogue{ p.ctr }, Count{ nullptr, row_words },
             row_words, p.tile_sums, &p.ctr->scan, s);
    run_scan(CornerCount{ p }, CornerEmit{ p }, CornerEpilogue{ p.ctr, p.corner_cap }, Count{ &p.ctr->rows, 0 },
             p.R * p.R, p.tile_sums, &p.ctr->scan, s);
}

void launch_field(const HullPlan& p, cudaStream_t s)
{
    if (p.field_ones)
    {
        bool ok = dispatch_image_dtype(p.masks_dtype, [&]<int DT>() {
            ones_kernel<DT><<<grid_for(p.B * p.H * 32, 256), 256, 0, s>>>(p);
        });
        if (!ok)
            throw CudaError{ cudaErrorInvalidValue, "hull field: unsupported mask dtype" };
        TH_LAUNCH_CHECK();
    }
    const int grid = grid_for(p.corner_cap, 256);
    // at least one launch, so that B == 0 still writes the empty product 1
    for (int64_t b0 = 0; b0 == 0 || b0 < p.B; b0 += kFieldViews)
    {
        const int64_t b1 = b0 + kFieldViews < p.B ? b0 + kFieldViews : p.B;
        bool ok = dispatch_image_dtype(p.masks_dtype, [&]<int DT>() {
            if (p.partial)
                field_kernel<DT, true><<<grid, 256, 0, s>>>(p, b0, b1);
            else
                field_kernel<DT, false><<<grid, 256, 0, s>>>(p, b0, b1);
        });
        if (!ok)
            throw CudaError{ cudaErrorInvalidValue, "hull field: unsupported mask dtype" };
        TH_LAUNCH_CHECK();
    }
}

void launch_marching_cubes(const HullPlan& p, cudaStream_t s)
{
    mc_cells_kernel<<<grid_for(p.corner_cap, 256), 256, 0, s>>>(p);
    TH_LAUNCH_CHECK();
    run_scan(VertCount{ p.codes, p.emask }, VertEmit{ p.soup_off, p.vbase }, VertEpilogue{ p.ctr },
             Count{ &p.ctr->corners, 0 }, p.corner_cap, p.tile_sums, &p.ctr->scan, s);
}

void launch_export(const HullPlan& p, float* verts, int64_t* faces, cudaStream_t s)
{
    const int grid = grid_for(p.corner_cap, 256);
    if (p.unique)
    {
        export_verts_kernel<<<grid, 256, 0, s>>>(p, verts);
        TH_LAUNCH_CHECK();
    }
    export_faces_kernel<<<grid, 256, 0, s>>>(p, verts, faces);
    TH_LAUNCH_CHECK();
}

namespace
{

__global__ void __launch_bounds__(256) export_field_kernel(HullPlan p, int64_t n, int64_t* __restrict__ indices, float* __restrict__ values)
{
    const int64_t R = p.R;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += stride)
    {
        int64_t x, y, z;
        unpack_corner(p.corners[t], x, y, z);
        indices[t] = x + y * R + z * R * R;
        values[t] = p.values[t];
    }
}

} // namespace

void launch_export_field(const HullPlan& p, int64_t n, int64_t* indices, float* values, cudaStream_t s)
{
    if (n <= 0)
        return;
    export_field_kernel<<<grid_for(n, 256), 256, 0, s>>>(p, n, indices, values);
    TH_LAUNCH_CHECK();
}

void launch_cleanup(const HullPlan& p, cudaStream_t s)
{
    clear_rows_kernel<<<grid_for(p.R * p.R * p.WR, 256), 256, 0, s>>>(p);
    TH_LAUNCH_CHECK();
    TH_CUDA(cudaMemsetAsync(p.rowbits, 0, sizeof(uint32_t) * ((p.R * p.R + 31) / 32), s));
}

} // namespace th
