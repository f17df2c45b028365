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

// Rank of a corner known to be set: the bitmap word and its rank word are
// loaded together (no check of the bit in between).
__device__ __forceinline__ uint32_t rank_of(const HullPlan& p, int64_t x, int64_t y, int64_t z)
{
    const int64_t w = (y + z * p.R) * p.WR + (x >> 6);
    const uint64_t word = p.bitmap[w];
    const uint32_t base = p.word_rank[w];
    return base + static_cast<uint32_t>(__popcll(word & ((1ull << (x & 63)) - 1ull)));
}

__global__ void __launch_bounds__(256) mark_corners_kernel(HullPlan p)
{
    const DevCounters* c = p.ctr;
    const int L = p.level;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    const int64_t t0 = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (L == 0)
    {
        // the root is the only leaf
        if (t0 == 0 && c->level_count[0] > 0)
            mark_cell_corners(p.bitmap, p.rowbits, p.R, p.WR, 0, 0, 0);
        return;
    }
    // the leaves are the refined children of the level L-1 cells (their
    // child masks), which the carve does not write out
    if (c->level_count[L] == 0)
        return;
    const int li = L - 1;
    const int64_t n = c->level_count[li];
    const int64_t* parents = p.nodes + c->level_off[li];
    const int64_t r = int64_t{ 1 } << li;
    for (int64_t t = t0; t < n; t += stride)
    {
        uint32_t m = p.child_masks[t];
        if (!m)
            continue;
        const int64_t idx = parents[t];
        mark_children_corners(p.bitmap, p.rowbits, p.R, p.WR, 2 * (idx & (r - 1)), 2 * ((idx >> li) & (r - 1)),
                              2 * (idx >> (2 * li)), m);
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

// One scan item per bitmap word of the touched rows (item k: word k % WR of
// row rows[k / WR]), so that a thread emits the corners of a few words, not
// of several whole rows.
struct CornerCount
{
    HullPlan p;
    __device__ unsigned long long operator()(int64_t k) const
    {
        const uint32_t wr = static_cast<uint32_t>(p.WR), kk = static_cast<uint32_t>(k);
        const int64_t w = static_cast<int64_t>(p.rows[kk / wr]) * p.WR + (kk % wr);
        return static_cast<unsigned long long>(__popcll(p.bitmap[w]));
    }
};


// Position of the set bit of the 64-bit word w with j set bits below it.
__device__ __forceinline__ int nth_set_bit64(uint64_t w, int j)
{
    const uint32_t lo = static_cast<uint32_t>(w);
    const int c = __popc(lo);
    return j < c ? nth_set_bit(lo, j) : 32 + nth_set_bit(static_cast<uint32_t>(w >> 32), j - c);
}

// Pass 2 of the corner scan (the counts come from CornerCount's tile sums):
// a block owns one scan tile of kScanTile words, a warp 8 chunks of 32
// consecutive words.  Per chunk the warp numbers the words' corners by a
// warp scan and writes them with all lanes: corner k of the chunk belongs to
// the word whose offset is the last one <= k, so the stores are coalesced.
// Also stores each word's rank (word_rank).
__global__ void __launch_bounds__(kScanThreads) corner_emit_kernel(HullPlan p, const unsigned long long* __restrict__ tile_offsets)
{
    static_assert(kScanThreads == 256 && kScanItems == 8, "one warp chunk per 32 items");
    __shared__ unsigned long long warp_totals[kScanThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t n = p.ctr->rows * p.WR;
    const int64_t ntiles = (n + kScanTile - 1) / kScanTile;
    const uint32_t wr = static_cast<uint32_t>(p.WR), R = static_cast<uint32_t>(p.R);
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
    {
        const int64_t first = tile * kScanTile + static_cast<int64_t>(w) * 256;
        uint64_t words[8];
        unsigned long long wsum = 0;
#pragma unroll
        for (int c = 0; c < 8; ++c)
        {
            const int64_t k = first + c * 32 + lane;
            words[c] = 0;
            if (k < n)
            {
                const uint32_t kk = static_cast<uint32_t>(k);
                words[c] = p.bitmap[static_cast<int64_t>(p.rows[kk / wr]) * p.WR + kk % wr];
            }
            wsum += __popcll(words[c]);
        }
        // this warp's corners come after those of the tile's earlier warps
        unsigned long long wtot = wsum;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1)
            wtot += __shfl_xor_sync(0xffffffffu, wtot, d);
        if (lane == 0)
            warp_totals[w] = wtot;
        __syncthreads();
        unsigned long long running = tile_offsets[tile];
        for (int v = 0; v < w; ++v)
            running += warp_totals[v];
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 8; ++c)
        {
            const int64_t k = first + c * 32 + lane;
            const int cnt = __popcll(words[c]);
            const int incl = warp_inclusive_scan(cnt);
            const int excl = incl - cnt;
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            uint32_t row = 0, wi = 0;
            if (k < n)
            {
                const uint32_t kk = static_cast<uint32_t>(k);
                row = p.rows[kk / wr];
                wi = kk % wr;
                p.word_rank[static_cast<int64_t>(row) * p.WR + wi] = static_cast<uint32_t>(running + excl);
            }
            for (int k0 = 0; k0 < total; k0 += 32)
            {
                const int kk = k0 + lane;
                const int s = item_slot(excl, kk);
                const int es = __shfl_sync(0xffffffffu, excl, s);
                const uint64_t ws = __shfl_sync(0xffffffffu, words[c], s);
                const uint32_t rs = __shfl_sync(0xffffffffu, row, s);
                const uint32_t wis = __shfl_sync(0xffffffffu, wi, s);
                if (kk < total)
                {
                    const int bit = nth_set_bit64(ws, kk - es);
                    const int64_t out = static_cast<int64_t>(running) + kk;
                    if (out < p.corner_cap)
                    {
                        p.corners[out] = pack_corner(static_cast<int64_t>(wis) * 64 + bit, rs % R, rs / R);
                        p.emask[out] = 0;
                    }
                }
            }
            running += static_cast<unsigned long long>(total);
        }
    }
}

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
    if constexpr (PARTIAL)
    {
        // 1 <= round(q) < size - 1 (half away from zero) exactly when 0.5 <= q < size - 1.5
        if (!(px >= 0.5f && px < __fsub_rn(Wf, 1.5f) && py >= 0.5f && py < __fsub_rn(Hf, 1.5f)))
            return 1.f;
        // In frame q - 0.5 is exact and >= 0, so round(q - 0.5) = floor(q), in
        // [0, size - 2]; q + 2^23 rounded down is 2^23 + floor(q) (the floats
        // in [2^23, 2^24) are the integers).
        const float sy = __fadd_rd(py, kTwo23), sx = __fadd_rd(px, kTwo23);
        const int64_t y0 = __float_as_int(sy) - kTwo23Bits, x0 = __float_as_int(sx) - kTwo23Bits;
        // all-ones footprint: exactly 1 (the weights below are in [0, 1])
        if (p.field_ones)
        {
            const uint32_t word = __ldg(p.ones + (b * p.H + y0) * p.WW + (x0 >> 5));
            if ((word >> (x0 & 31)) & 1u)
                return 1.f;
        }
        const int64_t i = (b * p.H + y0) * p.W + x0;
        const float v00 = load_f32<DT>(masks, i);
        const float v01 = load_f32<DT>(masks, i + 1);
        const float v10 = load_f32<DT>(masks, i + p.W);
        const float v11 = load_f32<DT>(masks, i + p.W + 1);
        return bilerp(v00, v10, v01, v11, __fsub_rn(py, __fsub_rn(sy, kTwo23)), __fsub_rn(px, __fsub_rn(sx, kTwo23)));
    }
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
    const float v00 = mask_sample<DT>(p, masks, b, y0, x0, pad);
    const float v10 = mask_sample<DT>(p, masks, b, y0 + 1, x0, pad);
    const float v01 = mask_sample<DT>(p, masks, b, y0, x0 + 1, pad);
    const float v11 = mask_sample<DT>(p, masks, b, y0 + 1, x0 + 1, pad);
    const float ty = __fsub_rn(py, ry.f);
    const float tx = __fsub_rn(px, rx.f);
    return bilerp(v00, v10, v01, v11, ty, tx);
}

// The all-ones footprint bitmap of the masks (HullPlan::ones).  A warp owns
// 32 columns of a band of kOnesBand rows of one view: it loads the band's
// rows and the row below at once (the last lane also the column after the
// chunk), then per row a lane tests its column, takes its right neighbour's
// result by a shuffle, and a ballot gives the row's "this column and the next
// are 1" bits; a footprint word is the AND of two consecutive rows' bits.
// Each mask row is read once, plus one row per band of 8.  Columns x = W-1 and the
// last row have no 2x2 footprint and get 0.
constexpr int kOnesBand = 8;

template <int DT>
__global__ void __launch_bounds__(256) ones_kernel(HullPlan p)
{
    const void* masks = p.rq->masks;
    const int64_t H = p.H, W = p.W, WW = p.WW;
    const int64_t bands = (H + kOnesBand - 1) / kOnesBand;
    const int64_t units = p.B * bands * WW;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t u = warp; u < units; u += nwarps)
    {
        // chunk fastest: neighbouring warps read neighbouring segments of a row
        const int64_t chunk = u % WW, vb = u / WW;
        const int64_t band = vb % bands, b = vb / bands;
        const int64_t y0 = band * kOnesBand;
        const int64_t x = chunk * 32 + lane;
        const int64_t view = b * H;
        float own[kOnesBand + 1], right[kOnesBand + 1];
#pragma unroll
        for (int i = 0; i <= kOnesBand; ++i)
        {
            const bool row = y0 + i < H;
            own[i] = row && x < W ? load_f32<DT>(masks, (view + y0 + i) * W + x) : 0.f;
            right[i] = row && lane == 31 && x + 1 < W ? load_f32<DT>(masks, (view + y0 + i) * W + x + 1) : 0.f;
        }
        uint32_t prev = 0;
#pragma unroll
        for (int i = 0; i <= kOnesBand; ++i)
        {
            const bool one = own[i] == 1.f;
            bool next = __shfl_down_sync(0xffffffffu, one, 1);
            if (lane == 31)
                next = right[i] == 1.f;
            const uint32_t pair = __ballot_sync(0xffffffffu, one && next);
            if (i > 0 && lane == 0 && y0 + i - 1 < H)
                p.ones[(view + y0 + i - 1) * WW + chunk] = prev & pair;
            prev = pair;
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
        const unsigned nact = __popc(__activemask());
        if ((threadIdx.x & 31) == __ffs(__activemask()) - 1)
            atomicAdd(&p.ctr->field_items, static_cast<unsigned long long>(nact) * nv);
#pragma unroll 4
        for (int v = 0; v < nv; ++v)
            value = __fmul_rn(value, view_factor<DT, PARTIAL>(p, masks, b0 + v, rows[v], wx, wy, wz, Hf, Wf));
        p.values[t] = value;
    }
}

// The cell-mask table (HullPlan::cell_masks): every cell of level L-1
// writes its skip and out-of-frame views (set) or 0 (clear).
__global__ void __launch_bounds__(256) cell_masks_kernel(HullPlan p, bool set)
{
    const DevCounters* c = p.ctr;
    const int li = p.level - 1;
    const int64_t n = c->level_count[li];
    const int64_t off = c->level_off[li];
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t k = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride)
        p.cell_masks[p.nodes[off + k]] = set ? (p.node_skip[off + k] | p.node_out[off + k]) : 0u;
}

// Views of a corner whose field factor is exactly 1: the OR of the cell-mask
// entries of the level L-1 cells whose lattice holds the corner (x >> 1, and
// also (x - 1) >> 1 for an even x > 0, per axis; cells beyond the grid and
// cells that are no node hold 0).
__device__ __forceinline__ uint32_t corner_view_mask(const HullPlan& p, int64_t gx, int64_t gy, int64_t gz)
{
    const int li = p.level - 1;
    const int64_t r = int64_t{ 1 } << li;
    const int64_t x0 = gx >> 1, y0 = gy >> 1, z0 = gz >> 1;
    const int64_t x1 = (gx - 1) >> 1, y1 = (gy - 1) >> 1, z1 = (gz - 1) >> 1;
    const bool two_x = x1 != x0 && gx > 0, two_y = y1 != y0 && gy > 0, two_z = z1 != z0 && gz > 0;
    // up to eight cells, a fixed unrolled pattern of predicated loads (issued together)
    uint32_t m = 0;
#pragma unroll
    for (int k = 0; k < 2; ++k)
    {
#pragma unroll
        for (int j = 0; j < 2; ++j)
        {
#pragma unroll
            for (int i = 0; i < 2; ++i)
            {
                const int64_t cx = i ? x1 : x0, cy = j ? y1 : y0, cz = k ? z1 : z0;
                const bool use = (i == 0 || two_x) && (j == 0 || two_y) && (k == 0 || two_z) && cx < r && cy < r &&
                                 cz < r;
                if (use)
                    m |= __ldg(p.cell_masks + (cx | (cy << li) | (cz << (2 * li))));
            }
        }
    }
    return m;
}

constexpr int kMaskedWarps = 8;

// The field with the cell masks, for the views [b0, b1) (at most 32): the
// views of a corner's mask are left out of its product (x * 1 == x); the
// remaining (corner, view) items of a warp's 32 corners are dealt out to its
// lanes, the factors parked in shared memory, and each lane multiplies its
// corner's factors in ascending view order, the reference's order.  A warp
// whose corners skip nothing walks the views directly, one corner per lane.
template <int DT, bool PARTIAL>
__global__ void __launch_bounds__(32 * kMaskedWarps) field_masked_kernel(HullPlan p, int64_t b0, int64_t b1)
{
    __shared__ float4 rows[32][3];
    __shared__ float fac_all[kMaskedWarps][32][33];
    const int nv = static_cast<int>(b1 - b0);
    for (int i = threadIdx.x; i < 3 * nv; i += blockDim.x)
    {
        const int v = i / 3, r = i - 3 * (i / 3);
        const int row = r < 2 ? r : (p.opengl ? 3 : 2);
        rows[v][r] = *reinterpret_cast<const float4*>(p.tf + 16 * (b0 + v) + 4 * row);
    }
    __syncthreads();
    float(*fac)[33] = fac_all[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int64_t n = p.ctr->corners;
    const float inv_rc = __fdiv_rn(1.f, static_cast<float>(p.R - 1)); // exact: a power of two
    const float Hf = small_i2f(static_cast<int32_t>(p.H)), Wf = small_i2f(static_cast<int32_t>(p.W));
    const float cx = p.rq->corner[0], cy = p.rq->corner[1], cz = p.rq->corner[2], length = p.rq->length;
    const void* masks = p.rq->masks;
    const uint32_t vb = nv >= 32 ? 0xffffffffu : ((1u << nv) - 1u);
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t base = warp * 32; base < n; base += nwarps * 32)
    {
        const int64_t t = base + lane;
        const bool valid = t < n;
        float wx = 0.f, wy = 0.f, wz = 0.f, value = 1.f;
        uint32_t skip = 0;
        if (valid)
        {
            int64_t gx, gy, gz;
            unpack_corner(p.corners[t], gx, gy, gz);
            // c + v/r * L fused (visual_hull_cuda.cu:444-448), as in field_kernel
            wx = __fmaf_rn(__fmul_rn(small_i2f(static_cast<int32_t>(gx)), inv_rc), length, cx);
            wy = __fmaf_rn(__fmul_rn(small_i2f(static_cast<int32_t>(gy)), inv_rc), length, cy);
            wz = __fmaf_rn(__fmul_rn(small_i2f(static_cast<int32_t>(gz)), inv_rc), length, cz);
            if (b0 == 0)
                skip = corner_view_mask(p, gx, gy, gz) & vb;
            else
                value = p.values[t];
        }
        if (!__any_sync(0xffffffffu, skip != 0))
        {
            const unsigned nvalid = __popc(__ballot_sync(0xffffffffu, valid));
            if (lane == 0)
                atomicAdd(&p.ctr->field_items, static_cast<unsigned long long>(nvalid) * nv);
            if (valid)
            {
#pragma unroll 4
                for (int v = 0; v < nv; ++v)
                    value = __fmul_rn(value, view_factor<DT, PARTIAL>(p, masks, b0 + v, rows[v], wx, wy, wz, Hf, Wf));
                p.values[t] = value;
            }
            continue;
        }
        const uint32_t active = valid ? (vb & ~skip) : 0u;
        const int count = __popc(active);
        const int incl = warp_inclusive_scan(count);
        const int excl = incl - count;
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        if (lane == 0 && total > 0)
            atomicAdd(&p.ctr->field_items, static_cast<unsigned long long>(total));
        for (int k0 = 0; k0 < total; k0 += 32)
        {
            const int k = k0 + lane;
            const int s = item_slot(excl, k);
            const int es = __shfl_sync(0xffffffffu, excl, s);
            const uint32_t as = __shfl_sync(0xffffffffu, active, s);
            const float sx = __shfl_sync(0xffffffffu, wx, s);
            const float sy = __shfl_sync(0xffffffffu, wy, s);
            const float sz = __shfl_sync(0xffffffffu, wz, s);
            if (k < total)
            {
                const int j = k - es;
                const int v = nth_set_bit(as, j);
                fac[s][j] = view_factor<DT, PARTIAL>(p, masks, b0 + v, rows[v], sx, sy, sz, Hf, Wf);
            }
        }
        __syncwarp();
        for (int j = 0; j < count; ++j)
            value = __fmul_rn(value, fac[lane][j]);
        __syncwarp();
        if (valid)
            p.values[t] = value;
    }
}

// Ranks of the 8 corners of the cell with base corner t; false if incomplete.
// Ranks at or beyond n (possible only when the corner pool overflowed and the
// request is about to be rerun) count as missing, so no access leaves the pools.
// The points (x, row) and (x + 1, row) are neighbours in the bitmap's order,
// so when both are set their ranks are consecutive: one rank lookup per row
// of the cell (three, the base row's rank being t) instead of seven.
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
    const int b = static_cast<int>(gx & 63);
    // the four rows of corners (dy, dz) = (q & 1, q >> 1): their bitmap words
    // and rank words are loaded together (independent loads), then checked
    int64_t w[4];
    uint64_t word[4], nextw[4];
    uint32_t wrank[4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
    {
        w[q] = ((gy + (q & 1)) + (gz + (q >> 1)) * R) * p.WR + (gx >> 6);
        word[q] = p.bitmap[w[q]];
        wrank[q] = q > 0 ? p.word_rank[w[q]] : 0u;
        // x + 1 < R stays in the row; at bit 63 the +x corner is bit 0 of the next word
        nextw[q] = b == 63 ? p.bitmap[w[q] + 1] : 0ull;
    }
    bool ok = true;
#pragma unroll
    for (int q = 0; q < 4; ++q)
    {
        const bool next = b < 63 ? ((word[q] >> (b + 1)) & 1ull) != 0 : (nextw[q] & 1ull) != 0;
        ok = ok && next && (q == 0 || ((word[q] >> b) & 1ull) != 0);
    }
    if (!ok)
        return false;
#pragma unroll
    for (int q = 0; q < 4; ++q)
    {
        const uint32_t r = q == 0 ? static_cast<uint32_t>(t)
                                  : wrank[q] + static_cast<uint32_t>(__popcll(word[q] & ((1ull << b) - 1ull)));
        if (r + 1 >= n)
            return false;
        rk[2 * q] = r;
        rk[2 * q + 1] = r + 1;
    }
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
            // the vertex-edge bits of each lower corner, one word read and at
            // most one atomic per corner (the reads are independent)
            unsigned int* words[8];
            uint32_t bits[8], cur[8];
#pragma unroll
            for (int i = 0; i < 8; ++i)
            {
                const uint32_t r1 = rk[i];
                bits[i] = ((used >> (3 * i)) & 7u) << (8u * (r1 & 3u));
                words[i] = reinterpret_cast<unsigned int*>(p.emask) + (r1 >> 2);
                cur[i] = bits[i] ? *words[i] : 0u;
            }
#pragma unroll
            for (int i = 0; i < 8; ++i)
                if ((cur[i] & bits[i]) != bits[i])
                    atomicOr(words[i], bits[i]);
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
    // grid coordinates are below 2^13: exact float conversions by adds (the
    // 64-bit integer conversions run on GB300's FP64 pipe)
    const float fx1 = small_i2f(static_cast<int32_t>(x1)), fy1 = small_i2f(static_cast<int32_t>(y1)),
                fz1 = small_i2f(static_cast<int32_t>(z1));
    const float fx2 = small_i2f(static_cast<int32_t>(x2)), fy2 = small_i2f(static_cast<int32_t>(y2)),
                fz2 = small_i2f(static_cast<int32_t>(z2));
    float q[3];
    if (snap == 1)
    {
        q[0] = fx1;
        q[1] = fy1;
        q[2] = fz1;
    }
    else if (snap == 2)
    {
        q[0] = fx2;
        q[1] = fy2;
        q[2] = fz2;
    }
    else
    {
        const float t = __fdiv_rn(__fsub_rn(iso, v1), __fsub_rn(v2, v1));
        q[0] = lerp(fx1, fx2, t);
        q[1] = lerp(fy1, fy2, t);
        q[2] = lerp(fz1, fz2, t);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
        out[a] = __fmaf_rn(scale, q[a], p.corner[a]);
}

// Faces in soup order; with unique vertices they index the edge-numbered
// vertex list, without they index the soup, which this kernel also writes.
// Columns 1 and 2 are swapped as flip_faces does (visual_hull_cuda.cu:941-956).
// A warp takes 32 consecutive corners, whose face entries form one contiguous
// range of the soup (soup_off is their exclusive prefix sum).  The range's
// entries are dealt out one per lane (entry k of the range belongs to the
// cell whose offset is the last one <= k; the cells' corner ranks are parked
// in shared memory), parked in shared memory at their flipped position, and
// stored with coalesced writes.  One thread per cell left three quarters of
// the lanes idle (a quarter of the corners start an active cell, with 1 to 15
// entries) and scattered each store over ~50 sectors.
constexpr int kExportWarps = 8;

__global__ void __launch_bounds__(32 * kExportWarps) export_faces_kernel(HullPlan p, float* __restrict__ verts, int64_t* __restrict__ faces)
{
    __shared__ TableCache tab;
    __shared__ int64_t stage_all[kExportWarps][32 * 15];
    __shared__ uint32_t ranks_all[kExportWarps][32][9];
    load_tables(tab);
    int64_t* stage = stage_all[threadIdx.x >> 5];
    uint32_t(*ranks)[9] = ranks_all[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int64_t n = p.ctr->corners;
    const float scale = __fdiv_rn(p.length, static_cast<float>(int64_t{ 1 } << p.level));
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t wb = warp * 32; wb < n; wb += nwarps * 32)
    {
        const int64_t t = wb + lane;
        const bool valid = t < n;
        const uint32_t code = valid ? p.codes[t] : 0u;
        const int cnt = tab.count[code];
        const unsigned act = __ballot_sync(0xffffffffu, cnt > 0);
        if (!act)
            continue;
        // the warp's range of the soup starts at lane 0's offset (a multiple of 3)
        const int64_t lo = __shfl_sync(0xffffffffu, valid ? static_cast<int64_t>(p.soup_off[t]) : int64_t{ 0 }, 0);
        const int64_t id = cnt > 0 ? p.corners[t] : 0;
        if (cnt > 0)
        {
            int64_t gx, gy, gz;
            unpack_corner(id, gx, gy, gz);
            uint32_t rk[8];
            cell_ranks(p, t, n, gx, gy, gz, rk);
#pragma unroll
            for (int i = 0; i < 8; ++i)
                ranks[lane][i] = rk[i];
        }
        const int incl = warp_inclusive_scan(cnt);
        const int excl = incl - cnt;
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        __syncwarp();
        for (int k0 = 0; k0 < total; k0 += 32)
        {
            const int k = k0 + lane;
            const int s = item_slot(excl, k);
            const int es = __shfl_sync(0xffffffffu, excl, s);
            const uint32_t cs = __shfl_sync(0xffffffffu, code, s);
            const int64_t ids = __shfl_sync(0xffffffffu, id, s);
            if (k < total)
            {
                const uint32_t e = tab.edges[cs][k - es];
                const int lo_corner = static_cast<int>(e & 7u), axis = static_cast<int>(e >> 3);
                const int64_t f = lo + k;
                const int slot = static_cast<int>(f % 3);
                const int dst = k - slot + (slot == 0 ? 0 : 3 - slot);
                const uint32_t r1 = ranks[s][lo_corner];
                if (p.unique)
                    stage[dst] = static_cast<int64_t>(p.vbase[r1]) + __popc(p.emask[r1] & ((1u << axis) - 1u));
                else
                {
                    int64_t gx, gy, gz;
                    unpack_corner(ids, gx, gy, gz);
                    float v[3];
                    const int hi_corner = lo_corner | (1 << axis);
                    edge_vertex(p, gx + (lo_corner & 1), gy + (lo_corner >> 1 & 1), gz + (lo_corner >> 2 & 1), axis,
                                p.values[r1], p.values[ranks[s][hi_corner]], scale, v);
                    verts[3 * f + 0] = v[0];
                    verts[3 * f + 1] = v[1];
                    verts[3 * f + 2] = v[2];
                    stage[dst] = f;
                }
            }
        }
        __syncwarp();
        for (int i = lane; i < total; i += 32)
            faces[lo + i] = stage[i];
        __syncwarp();
    }
}

// Unique vertices: vertices and faces in one pass.  A warp takes 128
// consecutive corners at a time: their data (code, edge bits, id, value) is
// staged in shared memory with coalesced loads, and their vertices (one per
// set edge bit, numbered by vbase) and face entries (numbered by soup_off)
// form two contiguous output ranges, dealt out one entry per lane (the owner
// of entry k is found by a binary search over the staged prefix sums), so the
// rank and value gathers run on all lanes although only about a quarter of
// the corners own any vertex or face.  The +x neighbour of a corner of the
// mesh has the next rank; other neighbours are looked up in the bitmap.
// Face columns 1 and 2 are swapped as flip_faces does
// (visual_hull_cuda.cu:941-956): entry k of a triangle goes to k's mirror.
constexpr int kExportPer = 4;                   // corners per lane
constexpr int kExportChunk = 32 * kExportPer;   // corners per warp and iteration

struct ExportStage
{
    int64_t id[kExportChunk];
    float val[kExportChunk];
    int32_t vpre[kExportChunk]; // exclusive prefix of the vertex counts over the chunk
    int32_t fpre[kExportChunk]; // exclusive prefix of the face-entry counts
    uint8_t code[kExportChunk], em[kExportChunk], nv[kExportChunk], nf[kExportChunk];
};

// Largest c in [0, kExportChunk) with pre[c] <= k (pre non-decreasing, pre[0] = 0).
__device__ __forceinline__ int stage_owner(const int32_t* pre, int k)
{
    int c = 0;
#pragma unroll
    for (int step = kExportChunk / 2; step > 0; step >>= 1)
        if (pre[c + step] <= k)
            c += step;
    return c;
}

__global__ void __launch_bounds__(32 * kExportWarps) export_mesh_kernel(HullPlan p, float* __restrict__ verts, int64_t* __restrict__ faces)
{
    __shared__ TableCache tab;
    __shared__ ExportStage stage_all[kExportWarps];
    load_tables(tab);
    __syncthreads();
    ExportStage& st = stage_all[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int64_t n = p.ctr->corners;
    const float scale = __fdiv_rn(p.length, static_cast<float>(int64_t{ 1 } << p.level));
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t wb = warp * kExportChunk; wb < n; wb += nwarps * kExportChunk)
    {
        // stage the chunk (coalesced: corner g * 32 + lane)
        bool any = false;
#pragma unroll
        for (int g = 0; g < kExportPer; ++g)
        {
            const int c = g * 32 + lane;
            const int64_t t = wb + c;
            const bool valid = t < n;
            const uint32_t code = valid ? p.codes[t] : 0u;
            const uint32_t em = valid ? p.emask[t] : 0u;
            const int nv = __popc(em), nf = tab.count[code];
            st.code[c] = static_cast<uint8_t>(code);
            st.em[c] = static_cast<uint8_t>(em);
            st.nv[c] = static_cast<uint8_t>(nv);
            st.nf[c] = static_cast<uint8_t>(nf);
            if (nv > 0 || nf > 0)
            {
                st.id[c] = p.corners[t];
                any = true;
            }
            if (nv > 0)
                st.val[c] = p.values[t];
        }
        if (!__any_sync(0xffffffffu, any))
            continue;
        __syncwarp();
        // prefix sums in corner order: lane l owns corners [4l, 4l + 4)
        int vloc[kExportPer], floc[kExportPer];
        int vt = 0, ft = 0;
#pragma unroll
        for (int g = 0; g < kExportPer; ++g)
        {
            const int c = lane * kExportPer + g;
            vloc[g] = vt;
            floc[g] = ft;
            vt += st.nv[c];
            ft += st.nf[c];
        }
        const int vin = warp_inclusive_scan(vt), fin = warp_inclusive_scan(ft);
        const int vex = vin - vt, fex = fin - ft;
        const int vtot = __shfl_sync(0xffffffffu, vin, 31), ftot = __shfl_sync(0xffffffffu, fin, 31);
#pragma unroll
        for (int g = 0; g < kExportPer; ++g)
        {
            st.vpre[lane * kExportPer + g] = vex + vloc[g];
            st.fpre[lane * kExportPer + g] = fex + floc[g];
        }
        __syncwarp();

        // vertices: the chunk's range starts at its first corner's vertex base.
        // Two entries per lane and iteration, their loads issued together;
        // every corner looked up here exists, so the rank needs no check.
        if (vtot > 0)
        {
            const int64_t vlo = p.vbase[wb];
            auto vertex_at = [&](int k, float v[3]) {
                const int c = stage_owner(st.vpre, k);
                const int a = nth_set_bit(st.em[c], k - st.vpre[c]);
                int64_t gx, gy, gz;
                unpack_corner(st.id[c], gx, gy, gz);
                // the edge's upper corner (for a = 0 the next rank, wb + c + 1)
                const uint32_t r2 = rank_of(p, gx + (a == 0), gy + (a == 1), gz + (a == 2));
                edge_vertex(p, gx, gy, gz, a, st.val[c], p.values[r2], scale, v);
            };
            for (int k = lane; k < vtot; k += 64)
            {
                const bool two = k + 32 < vtot;
                float v0[3], v1[3];
                vertex_at(k, v0);
                vertex_at(two ? k + 32 : k, v1);
                int64_t out = vlo + k;
                verts[3 * out + 0] = v0[0];
                verts[3 * out + 1] = v0[1];
                verts[3 * out + 2] = v0[2];
                if (two)
                {
                    out += 32;
                    verts[3 * out + 0] = v1[0];
                    verts[3 * out + 1] = v1[1];
                    verts[3 * out + 2] = v1[2];
                }
            }
        }

        // faces: the chunk's entries are one contiguous range of the soup
        // (soup_off is their exclusive prefix sum, a multiple of 3)
        if (ftot > 0)
        {
            const int64_t lo = p.soup_off[wb];
            auto face_at = [&](int k) -> int64_t {
                const int c = stage_owner(st.fpre, k);
                const uint32_t e = tab.edges[st.code[c]][k - st.fpre[c]];
                const int lo_corner = static_cast<int>(e & 7u), axis = static_cast<int>(e >> 3);
                int64_t gx, gy, gz;
                unpack_corner(st.id[c], gx, gy, gz);
                // the edge's lower corner (every corner of a cell with faces exists)
                const uint32_t r1 = rank_of(p, gx + (lo_corner & 1), gy + (lo_corner >> 1 & 1), gz + (lo_corner >> 2 & 1));
                return static_cast<int64_t>(p.vbase[r1]) + __popc(p.emask[r1] & ((1u << axis) - 1u));
            };
            for (int k = lane; k < ftot; k += 64)
            {
                const bool two = k + 32 < ftot;
                const int64_t f0 = face_at(k);
                const int64_t f1 = face_at(two ? k + 32 : k);
                // columns 1 and 2 swapped: entry k of a triangle goes to its mirror
                const int s0 = k % 3;
                faces[lo + k - s0 + (s0 == 0 ? 0 : 3 - s0)] = f0;
                if (two)
                {
                    const int k1 = k + 32, s1 = k1 % 3;
                    faces[lo + k1 - s1 + (s1 == 0 ? 0 : 3 - s1)] = f1;
                }
            }
        }
        __syncwarp();
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
    const int64_t max_words = p.R * p.R * p.WR;
    run_scan_reduce(CornerCount{ p }, CornerEpilogue{ p.ctr, p.corner_cap }, Count{ &p.ctr->rows, 0, p.WR }, max_words,
                    p.tile_sums, &p.ctr->scan, s);
    corner_emit_kernel<<<scan_grid(max_words), kScanThreads, 0, s>>>(p, p.tile_sums);
    TH_LAUNCH_CHECK();
}

void launch_field(const HullPlan& p, cudaStream_t s)
{
    if (p.field_ones)
    {
        bool ok = dispatch_image_dtype(p.masks_dtype, [&]<int DT>() {
            const int64_t units = p.B * ((p.H + kOnesBand - 1) / kOnesBand) * p.WW;
            ones_kernel<DT><<<grid_for(units * 32, 256), 256, 0, s>>>(p);
        });
        if (!ok)
            throw CudaError{ cudaErrorInvalidValue, "hull field: unsupported mask dtype" };
        TH_LAUNCH_CHECK();
    }
    if (p.cell_masks)
    {
        const int64_t cells = p.level >= 1 ? (int64_t{ 1 } << (3 * (p.level - 1))) : 1;
        const int mgrid = grid_for(cells < p.node_cap ? cells : p.node_cap, 256);
        if (p.own_cell_masks)
        {
            cell_masks_kernel<<<mgrid, 256, 0, s>>>(p, true);
            TH_LAUNCH_CHECK();
        }
        const int grid = grid_for(p.corner_cap, 32 * kMaskedWarps);
        // at least one launch, so that B == 0 still writes the empty product 1
        for (int64_t b0 = 0; b0 == 0 || b0 < p.B; b0 += 32)
        {
            const int64_t b1 = b0 + 32 < p.B ? b0 + 32 : p.B;
            bool ok = dispatch_image_dtype(p.masks_dtype, [&]<int DT>() {
                if (p.partial)
                    field_masked_kernel<DT, true><<<grid, 32 * kMaskedWarps, 0, s>>>(p, b0, b1);
                else
                    field_masked_kernel<DT, false><<<grid, 32 * kMaskedWarps, 0, s>>>(p, b0, b1);
            });
            if (!ok)
                throw CudaError{ cudaErrorInvalidValue, "hull field: unsupported mask dtype" };
            TH_LAUNCH_CHECK();
        }
        if (p.own_cell_masks)
        {
            cell_masks_kernel<<<mgrid, 256, 0, s>>>(p, false);
            TH_LAUNCH_CHECK();
        }
        return;
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
    const int grid = grid_for(p.corner_cap, 32 * kExportWarps);
    if (p.unique)
        export_mesh_kernel<<<grid, 32 * kExportWarps, 0, s>>>(p, verts, faces);
    else
        export_faces_kernel<<<grid, 32 * kExportWarps, 0, s>>>(p, verts, faces);
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
    launch_zero(p.rowbits, sizeof(uint32_t) * ((p.R * p.R + 31) / 32), s);
}

} // namespace th
