// Octree carving: one level per launch pair (classify, then compact).
//
// Reference: classify_children_full / _partial (visual_hull_cuda.cu:168-417)
// run one thread per child and project each of the child's 8 corners for
// every view; the level loop (:633-751) compacts the flags with cub and reads
// the count back to the host.
//
// Work items.  A warp takes 32 parents and turns them into (parent, view)
// items: every view of every parent except the views the parent's skip mask
// marks (below).  Its lanes walk the item list, so skipped views cost nothing
// and the kernel does not depend on the number of views.  A lane evaluates
// one item: it walks the parent's 3x3x3 lattice of child corners plane by
// plane (z), evaluating the nested fmas of the projection
// fma(a0,x,fma(a1,y,fma(a2,z,a3))) innermost-first so the z and (y,z) partial
// sums are shared between lattice points without changing a single rounding;
// each plane is reduced to the pixel boxes of its four 2x2 point cells, and
// the four children between two consecutive planes take the union of their
// two cells (27 projections per item where the reference makes 64).  Per child
// the per-view outcomes combine by OR (empty in any view, partial in any view,
// fully inside some frame), so items OR their 8-bit results into the parent's
// shared-memory slot and the result equals the reference's decision exactly.
//
// View skipping (binary masks).  When a child's pixel box grown by one pixel
// lies inside the image and holds only ones, the child's own children are
// "object" in that view too: their corners project into the child's box up to
// rounding errors far below a pixel, so their rounded boxes stay inside the
// grown box, every pixel there is 1, and "object" contributes nothing to the
// decision.  The child records that view in its skip mask and its children
// never evaluate it.  Before the last level in partial mode a skipped view
// must also report "fully inside", so there the rule additionally requires
// every corner of the child to round at least two pixels inside the frame.
// For leaves the mask tells the hull field that the view's bilinear factor is
// exactly 1.  All corners must be in front of the camera for any of this.
//
// Conversions: the reference converts the rounded pixel coordinates to int64
// (glm::i64vec2).  On GB300 64-bit float<->int conversions run on the FP64
// pipe, which made them the bottleneck, so the kernel converts to int32 with
// saturation instead.  Every use of those values is a clamp to [0, size-1] or
// an in-image test, whose outcome is the same for the int64 and the saturated
// int32 value (including +-inf and NaN).  The one exception is partial mode's
// unclamped box area; a child whose rounded box leaves the int32 range takes
// the exact int64 path for that view.
//
// The 8 child flags of a parent become one byte; a device-wide scan over the
// popcounts then writes the refined children (and their skip masks) in the
// reference's stable order (parent order, then child index), and its last
// block stores the level size on the device for the next level.

#include <cfloat>

#include "th_hull.cuh"
#include "th_internal.h"

namespace th
{

namespace
{

constexpr int kWarps = 8; // warps per block of the classify kernel

__global__ void hull_init_kernel(HullPlan p)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
    {
        DevCounters* c = p.ctr;
        c->level_count[0] = 1;
        c->level_off[0] = 0;
        c->level_off[1] = 1;
        p.nodes[0] = 0;
        p.node_skip[0] = 0;
    }
}

struct Box
{
    float minx, miny, maxx, maxy;
};

__device__ __forceinline__ Box merge(const Box& a, const Box& b)
{
    return Box{ fminf(a.minx, b.minx), fminf(a.miny, b.miny), fmaxf(a.maxx, b.maxx), fmaxf(a.maxy, b.maxy) };
}

// Saturating float -> int32 (NaN to a value outside every image).
__device__ __forceinline__ int32_t f2i32(float f)
{
    return __float2int_rz(f);
}

__device__ __forceinline__ bool fits_i32(float f)
{
    return f > -2147483648.0f && f < 2147483648.0f;
}

__device__ __forceinline__ float box_sum(const float* __restrict__ sat_b, int32_t W, int32_t x0, int32_t y0, int32_t x1, int32_t y1)
{
    // sample_zeros_padding at the four corners (image_utils.h:84-97); inputs are
    // clamped to the image, so only the -1 row/column can leave it.
    const float* row_hi = sat_b + static_cast<int64_t>(y1) * W;
    const float* row_lo = sat_b + static_cast<int64_t>(y0 - 1) * W;
    const float i11 = row_hi[x1];
    const float i10 = x0 > 0 ? row_hi[x0 - 1] : 0.f;
    const float i01 = y0 > 0 ? row_lo[x1] : 0.f;
    const float i00 = (x0 > 0 && y0 > 0) ? row_lo[x0 - 1] : 0.f;
    return __fsub_rn(__fsub_rn(__fadd_rn(i11, i00), i10), i01);
}

enum ViewClass : uint32_t
{
    kNone = 0,
    kEmpty = 1,
    kRefine = 2,
    kObject = 3,
};

struct ViewResult
{
    uint32_t cls;
    bool skip; // the child's children may skip this view
};

// One child in one view from its pixel box (visual_hull_cuda.cu:236-285 and
// :365-410).  The box starts the reference's min/max from +-FLT_MAX.
// want_skip: evaluate the skip rule (binary masks, corners in front, inside
// rule already checked by the caller).  H, W >= 1.
template <bool PARTIAL>
__device__ __forceinline__ ViewResult classify_view(const float* __restrict__ sat_b, int32_t H, int32_t W, Box bb, bool want_skip)
{
    const float margin = 0.5f - 0.1f; // isolevel - epsilon (visual_hull_cuda.cu:259-267)
    bb.minx = fminf(FLT_MAX, bb.minx);
    bb.miny = fminf(FLT_MAX, bb.miny);
    bb.maxx = fmaxf(-FLT_MAX, bb.maxx);
    bb.maxy = fmaxf(-FLT_MAX, bb.maxy);
    const float fminx = roundf(__fadd_rn(bb.minx, -0.5f));
    const float fminy = roundf(__fadd_rn(bb.miny, -0.5f));
    const float fmaxx = roundf(__fadd_rn(bb.maxx, 0.5f));
    const float fmaxy = roundf(__fadd_rn(bb.maxy, 0.5f));
    const int32_t cminx = min(max(f2i32(fminx), 0), W - 1);
    const int32_t cminy = min(max(f2i32(fminy), 0), H - 1);
    const int32_t cmaxx = min(max(f2i32(fmaxx), 0), W - 1);
    const int32_t cmaxy = min(max(f2i32(fmaxy), 0), H - 1);
    const int64_t area = static_cast<int64_t>(cmaxy - cminy + 1) * static_cast<int64_t>(cmaxx - cminx + 1);
    const float sum = box_sum(sat_b, W, cminx, cminy, cmaxx, cmaxy);
    bool whole = true;
    if (PARTIAL)
    {
        // full_area_bb (:377) from the unclamped rounded box, int64 arithmetic
        // wrapping like the device's; exact int64 values when int32 cannot hold them.
        int64_t rminx, rminy, rmaxx, rmaxy;
        if (fits_i32(fminx) && fits_i32(fminy) && fits_i32(fmaxx) && fits_i32(fmaxy))
        {
            rminx = f2i32(fminx);
            rminy = f2i32(fminy);
            rmaxx = f2i32(fmaxx);
            rmaxy = f2i32(fmaxy);
        }
        else
        {
            rminx = f2i64(fminx);
            rminy = f2i64(fminy);
            rmaxx = f2i64(fmaxx);
            rmaxy = f2i64(fmaxy);
        }
        const uint64_t fy = static_cast<uint64_t>(rmaxy) - static_cast<uint64_t>(rminy) + 1u;
        const uint64_t fx = static_cast<uint64_t>(rmaxx) - static_cast<uint64_t>(rminx) + 1u;
        whole = (static_cast<uint64_t>(area) == fy * fx);
    }
    const float area_f = (area >= INT32_MIN && area <= INT32_MAX) ? __int2float_rn(static_cast<int32_t>(area))
                                                                  : __ll2float_rn(area);
    ViewResult res{ kNone, false };
    if (sum <= 0.f + margin && whole)
        res.cls = kEmpty;
    else if (sum >= __fsub_rn(area_f, margin) && whole)
        res.cls = kObject;
    else if (!PARTIAL || (cmaxy - cminy > 1 && cmaxx - cminx > 1))
        res.cls = kRefine;
    if (want_skip && res.cls == kObject && fminx >= 1.f && fminy >= 1.f && fmaxx <= static_cast<float>(W - 2) &&
        fmaxy <= static_cast<float>(H - 2))
    {
        // the box grown by one pixel is inside the image: all ones there?
        const int32_t x0 = static_cast<int32_t>(fminx) - 1, y0 = static_cast<int32_t>(fminy) - 1;
        const int32_t x1 = static_cast<int32_t>(fmaxx) + 1, y1 = static_cast<int32_t>(fmaxy) + 1;
        const float grown = box_sum(sat_b, W, x0, y0, x1, y1);
        res.skip = grown == static_cast<float>((y1 - y0 + 1) * (x1 - x0 + 1));
    }
    return res;
}

struct ItemResult
{
    uint32_t empty, refine, inside, skip; // 8-bit child masks
};

// One (parent, view) item: the parent's lattice projected into view b.
// skip_inside: the skip rule also needs the child's corners two pixels inside.
template <bool PARTIAL, bool OPENGL>
__device__ __forceinline__ ItemResult classify_item(const HullPlan& p,
                                                    int64_t b,
                                                    const float wx[3],
                                                    const float wy[3],
                                                    const float wz[3],
                                                    bool want_skip,
                                                    bool skip_inside)
{
    const int32_t H = static_cast<int32_t>(p.H), W = static_cast<int32_t>(p.W);
    const float Hf = static_cast<float>(p.H), Wf = static_cast<float>(p.W);
    const float* m = p.tf + 16 * b;
    // rows x, y and the divisor row (w for OpenGL, z for OpenCV)
    const float4 rx = *reinterpret_cast<const float4*>(m);
    const float4 ry = *reinterpret_cast<const float4*>(m + 4);
    const float4 rd = *reinterpret_cast<const float4*>(m + (OPENGL ? 12 : 8));
    const float* sat_b = p.sat + b * p.H * p.W;
    ItemResult out{ 0, 0, 0, 0 };
    Box prev[4];
    uint32_t prev_in = 0, prev_in2 = 0, prev_front = 0;
#pragma unroll
    for (int z = 0; z < 3; ++z)
    {
        const float tzx = __fmaf_rn(rx.z, wz[z], rx.w);
        const float tzy = __fmaf_rn(ry.z, wz[z], ry.w);
        const float tzd = __fmaf_rn(rd.z, wz[z], rd.w);
        float px[9], py[9];
        uint32_t in9 = 0, in9b = 0, front9 = 0;
#pragma unroll
        for (int y = 0; y < 3; ++y)
        {
            const float tyx = __fmaf_rn(rx.y, wy[y], tzx);
            const float tyy = __fmaf_rn(ry.y, wy[y], tzy);
            const float tyd = __fmaf_rn(rd.y, wy[y], tzd);
#pragma unroll
            for (int x = 0; x < 3; ++x)
            {
                const int k = x + 3 * y;
                const float cx = __fmaf_rn(rx.x, wx[x], tyx);
                const float cy = __fmaf_rn(ry.x, wx[x], tyy);
                const float cd = __fmaf_rn(rd.x, wx[x], tyd);
                const float nx = __fdiv_rn(cx, cd);
                const float ny = __fdiv_rn(cy, cd);
                if (OPENGL)
                {
                    // (n + 1) * size / 2 - 0.5 (image_utils.h:67-71); /2 == *0.5 exactly
                    px[k] = __fsub_rn(__fmul_rn(__fmul_rn(__fadd_rn(nx, 1.f), Wf), 0.5f), 0.5f);
                    py[k] = __fsub_rn(__fmul_rn(__fmul_rn(__fadd_rn(ny, 1.f), Hf), 0.5f), 0.5f);
                }
                else
                {
                    px[k] = __fsub_rn(nx, 0.5f);
                    py[k] = __fsub_rn(ny, 0.5f);
                }
                if (want_skip && cd > 0.f)
                    front9 |= 1u << k;
                if (PARTIAL)
                {
                    const int32_t qx = f2i32(roundf(px[k]));
                    const int32_t qy = f2i32(roundf(py[k]));
                    if (1 <= qy && qy < H - 1 && 1 <= qx && qx < W - 1)
                        in9 |= 1u << k;
                    if (skip_inside && 2 <= qy && qy < H - 2 && 2 <= qx && qx < W - 2)
                        in9b |= 1u << k;
                }
            }
        }
        Box cur[4];
        uint32_t cur_in = 0, cur_in2 = 0, cur_front = 0;
#pragma unroll
        for (int c = 0; c < 4; ++c)
        {
            const int cx = c & 1, cy = c >> 1;
            const int k0 = cx + 3 * cy, k1 = k0 + 1, k2 = k0 + 3, k3 = k0 + 4;
            cur[c] = Box{ fminf(fminf(px[k0], px[k1]), fminf(px[k2], px[k3])),
                          fminf(fminf(py[k0], py[k1]), fminf(py[k2], py[k3])),
                          fmaxf(fmaxf(px[k0], px[k1]), fmaxf(px[k2], px[k3])),
                          fmaxf(fmaxf(py[k0], py[k1]), fmaxf(py[k2], py[k3])) };
            const uint32_t need = (1u << k0) | (1u << k1) | (1u << k2) | (1u << k3);
            if ((in9 & need) == need)
                cur_in |= 1u << c;
            if ((in9b & need) == need)
                cur_in2 |= 1u << c;
            if ((front9 & need) == need)
                cur_front |= 1u << c;
        }
        if (z > 0)
        {
#pragma unroll
            for (int c = 0; c < 4; ++c)
            {
                const uint32_t cbit = 1u << c;
                const uint32_t bit = 1u << (c + 4 * (z - 1));
                const bool front = (prev_front & cur_front & cbit) != 0;
                const bool in2 = (prev_in2 & cur_in2 & cbit) != 0;
                const ViewResult r = classify_view<PARTIAL>(sat_b, H, W, merge(prev[c], cur[c]),
                                                            want_skip && front && (!skip_inside || in2));
                if (r.cls == kEmpty)
                    out.empty |= bit;
                else if (r.cls == kRefine)
                    out.refine |= bit;
                if (r.skip)
                    out.skip |= bit;
                if (PARTIAL && (prev_in & cur_in & cbit))
                    out.inside |= bit;
            }
        }
#pragma unroll
        for (int c = 0; c < 4; ++c)
            prev[c] = cur[c];
        prev_in = cur_in;
        prev_in2 = cur_in2;
        prev_front = cur_front;
    }
    return out;
}

struct WarpSlots
{
    uint32_t empty[32], refine[32], inside[32];
    uint32_t cskip[32][8];
};

// Position of the j-th set bit of m (j < popc(m)).
__device__ __forceinline__ int select_bit(uint32_t m, int j)
{
    for (int t = 0; t < j; ++t)
        m &= m - 1;
    return __ffs(m) - 1;
}

template <bool PARTIAL, bool OPENGL>
__global__ void __launch_bounds__(32 * kWarps) classify_kernel(HullPlan p, int li)
{
    __shared__ WarpSlots slots_all[kWarps];
    WarpSlots& ws = slots_all[threadIdx.x >> 5];
    const DevCounters* ctr = p.ctr;
    const int64_t n = ctr->level_count[li];
    const int64_t lvl_off = ctr->level_off[li];
    const int64_t* parents = p.nodes + lvl_off;
    const uint32_t* parent_skip = p.node_skip + lvl_off;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const int64_t r = int64_t{ 1 } << li;
    const float inv_rc = __fdiv_rn(1.f, static_cast<float>(2 * r)); // exact: a power of two
    const bool last = (li == p.level - 1);
    const int B = static_cast<int>(p.B);
    const uint32_t view_bits = B >= 32 ? 0xffffffffu : ((1u << B) - 1u);
    // view skipping needs exact integer SAT sums (binary masks, H*W < 2^24)
    const bool skips = p.skip_ok && (*p.nonbinary == 0);
    // what the children's skip masks will be used for
    const bool skip_inside = PARTIAL && (li + 1 == p.level - 1);

    for (int64_t base = warp * 32; base < n; base += nwarps * 32)
    {
        const int64_t pi = base + lane;
        const bool valid = pi < n;
        const int64_t idx = valid ? parents[pi] : 0;
        const uint32_t skipm = (valid && skips) ? (parent_skip[pi] & view_bits) : 0u;
        const int count = valid ? (B - __popc(skipm)) : 0;
        ws.empty[lane] = 0;
        ws.refine[lane] = 0;
        // before the last level a skipped view (partial mode) is one where
        // every child is fully inside the frame
        ws.inside[lane] = (PARTIAL && last && skipm) ? 0xffu : 0u;
#pragma unroll
        for (int c = 0; c < 8; ++c)
            ws.cskip[lane][c] = 0;
        const int incl = warp_inclusive_scan(count);
        const int excl = incl - count;
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        __syncwarp();
        for (int k0 = 0; k0 < total; k0 += 32)
        {
            const int k = k0 + lane;
            // slot s: the last lane whose exclusive offset is <= k
            int s = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1)
            {
                const int e = __shfl_sync(0xffffffffu, excl, s + step);
                if (s + step < 32 && e <= k)
                    s += step;
            }
            const int es = __shfl_sync(0xffffffffu, excl, s);
            const uint32_t ms = __shfl_sync(0xffffffffu, skipm, s);
            const int64_t is = __shfl_sync(0xffffffffu, idx, s);
            if (k >= total)
                continue;
            const int j = k - es;
            const uint32_t active = view_bits & ~ms;
            const int na = __popc(active);
            const int b = j < na ? select_bit(active, j) : 32 + (j - na);
            const int64_t gx = is % r, gy = is / r % r, gz = is / (r * r);
            float wx[3], wy[3], wz[3];
#pragma unroll
            for (int d = 0; d < 3; ++d)
            {
                // c + v/r * L fused (visual_hull_cuda.cu:206-213); v/r == v * (1/r) exactly
                wx[d] = __fmaf_rn(__fmul_rn(static_cast<float>(2 * gx + d), inv_rc), p.length, p.corner[0]);
                wy[d] = __fmaf_rn(__fmul_rn(static_cast<float>(2 * gy + d), inv_rc), p.length, p.corner[1]);
                wz[d] = __fmaf_rn(__fmul_rn(static_cast<float>(2 * gz + d), inv_rc), p.length, p.corner[2]);
            }
            const ItemResult res =
                    classify_item<PARTIAL, OPENGL>(p, b, wx, wy, wz, skips && b < 32, skip_inside);
            if (res.empty)
                atomicOr(&ws.empty[s], res.empty);
            if (res.refine)
                atomicOr(&ws.refine[s], res.refine);
            if (res.inside)
                atomicOr(&ws.inside[s], res.inside);
            if (res.skip)
            {
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    if (res.skip >> c & 1u)
                        atomicOr(&ws.cskip[s][c], 1u << b);
            }
        }
        __syncwarp();
        if (valid)
        {
            uint32_t mask = ws.refine[lane] & ~ws.empty[lane];
            if (PARTIAL && last)
                mask &= ws.inside[lane];
            p.child_masks[pi] = static_cast<uint8_t>(mask);
            if (pi < p.parent_cap)
            {
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    p.child_skip[pi * 8 + c] = skips ? ws.cskip[lane][c] : 0u;
            }
        }
        __syncwarp();
    }
}

struct ChildCount
{
    const uint8_t* masks;
    __device__ unsigned long long operator()(int64_t i) const
    {
        return static_cast<unsigned long long>(__popc(masks[i]));
    }
};

struct ChildEmit
{
    HullPlan p;
    int li;
    __device__ void operator()(int64_t i, unsigned long long off, unsigned long long cnt) const
    {
        if (cnt == 0)
            return;
        const DevCounters* c = p.ctr;
        const int64_t r = int64_t{ 1 } << li, rc = 2 * r;
        const int64_t idx = p.nodes[c->level_off[li] + i];
        const int64_t gx = 2 * (idx % r), gy = 2 * (idx / r % r), gz = 2 * (idx / (r * r));
        const uint32_t m = p.child_masks[i];
        const bool has_skip = i < p.parent_cap;
        int64_t out = c->level_off[li + 1] + static_cast<int64_t>(off);
#pragma unroll
        for (int k = 0; k < 8; ++k)
        {
            if (m >> k & 1u)
            {
                if (out < p.node_cap)
                {
                    p.nodes[out] = (gx + (k & 1)) + (gy + (k >> 1 & 1)) * rc + (gz + (k >> 2 & 1)) * rc * rc;
                    p.node_skip[out] = has_skip ? p.child_skip[i * 8 + k] : 0u;
                }
                ++out;
            }
        }
    }
};

struct ChildEpilogue
{
    DevCounters* ctr;
    int li;
    int64_t node_cap;
    int64_t parent_cap;
    __device__ void operator()(unsigned long long total) const
    {
        const int64_t start = ctr->level_off[li + 1];
        int64_t n = static_cast<int64_t>(total);
        if (ctr->level_count[li] > parent_cap)
            ctr->overflow |= kOverflowParents; // skip masks were dropped; rerun with more room
        if (start + n > node_cap)
        {
            ctr->overflow |= kOverflowNodes;
            n = 0; // stop the octree here; the host retries with a larger pool
        }
        ctr->level_count[li + 1] = n;
        ctr->level_off[li + 2] = start + n;
    }
};

} // namespace

int grid_for(int64_t work_items, int threads)
{
    const int64_t blocks = (work_items + threads - 1) / threads;
    const int64_t cap = 8LL * sm_count();
    return static_cast<int>(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

void launch_hull_init(const HullPlan& p, cudaStream_t s)
{
    TH_CUDA(cudaMemsetAsync(p.ctr, 0, sizeof(DevCounters), s));
    hull_init_kernel<<<1, 32, 0, s>>>(p);
    TH_LAUNCH_CHECK();
}

void launch_carve_level(const HullPlan& p, int li, cudaStream_t s)
{
    // Upper bound of the parents at level li, for the grid size only.
    const int64_t bound = li < 10 ? (int64_t{ 1 } << (3 * li)) : p.node_cap;
    const int64_t max_parents = bound < p.node_cap ? bound : p.node_cap;
    const int grid = grid_for(max_parents * 8, 32 * kWarps);
    if (p.partial)
    {
        if (p.opengl)
            classify_kernel<true, true><<<grid, 32 * kWarps, 0, s>>>(p, li);
        else
            classify_kernel<true, false><<<grid, 32 * kWarps, 0, s>>>(p, li);
    }
    else
    {
        if (p.opengl)
            classify_kernel<false, true><<<grid, 32 * kWarps, 0, s>>>(p, li);
        else
            classify_kernel<false, false><<<grid, 32 * kWarps, 0, s>>>(p, li);
    }
    TH_LAUNCH_CHECK();
    run_scan(ChildCount{ p.child_masks }, ChildEmit{ p, li }, ChildEpilogue{ p.ctr, li, p.node_cap, p.parent_cap },
             Count{ &p.ctr->level_count[li], 0 }, max_parents, p.tile_sums, &p.ctr->scan, s);
}

} // namespace th
