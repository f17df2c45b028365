// Octree carving: one level per launch pair (classify, then compact).
//
// Reference: classify_children_full / _partial (visual_hull_cuda.cu:168-417)
// run one thread per child and project each of the child's 8 corners for
// every view; the level loop (:633-751) compacts the flags with cub and reads
// the count back to the host.
//
// Lattice.  For one parent and one view, a lane walks the parent's 3x3x3
// lattice of child corners plane by plane (z).  The nested fmas of the
// projection fma(a0,x,fma(a1,y,fma(a2,z,a3))) are evaluated innermost-first,
// so the z and (y,z) partial sums are shared between lattice points without
// changing a single rounding; each plane is reduced to the pixel boxes of its
// four 2x2 point cells, and the four children between two consecutive planes
// take the union of their two cells: 27 projections where the reference makes
// 64.  Per child the per-view outcomes combine by OR (empty in any view,
// partial in any view, fully inside some frame), so any split of the views
// across lanes, OR-reduced, gives the reference's decision exactly.
//
// Two kernels share that per-(parent, view) routine:
//  * views over lanes: a group of LANES lanes owns one parent, lane = view;
//    coherent and best while every view must be evaluated;
//  * (parent, view) items: a warp takes a chunk of parents, lists the views
//    each parent still needs (below) and deals the items out to its lanes;
//    results are OR-reduced over runs of lanes of the same parent, then
//    merged in shared memory.  Best when many views are skipped.
// The host picks one per level (autotuned by measuring both).
//
// View skipping (binary masks).  When a child's pixel box grown by two pixels
// lies inside the image and holds only ones, every descendant of the child is
// "object" in that view: the descendants' corners project into the child's
// box up to rounding errors far below a pixel, so their rounded boxes stay
// within one pixel of the child's, their boxes grown by one pixel stay inside
// the grown box, every pixel there is 1, and "object" contributes nothing to
// the decision.  The child records the view in its skip mask, its children
// inherit the mask, and the item kernel never evaluates the view for any of
// them.  In partial mode a skipped view must also report "fully inside" at the
// last level, so the rule also requires every corner of the child to round at
// least two pixels inside the frame.  All corners must be in front of the
// camera for any of this.
//
// Out-of-frame views (partial masks).  A child box more than two pixels
// outside the image (box_out) can change nothing for any descendant; the view
// goes into the child's out mask, is inherited and skipped the same way.
//
// Conversions: the reference converts the rounded pixel coordinates to int64
// (glm::i64vec2).  On GB300 64-bit float<->int conversions run on the FP64
// pipe, which made them the bottleneck, so the kernels convert to int32 with
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

#include "th_classify.cuh"
#include "th_hull.cuh"
#include "th_internal.h"

namespace th
{

namespace
{

#ifndef TH_CARVE_WARPS
#define TH_CARVE_WARPS 8
#endif
constexpr int kWarps = TH_CARVE_WARPS; // warps per block of the classify kernels
#ifndef TH_CARVE_MIN_BLOCKS
#define TH_CARVE_MIN_BLOCKS 2
#endif
// resident blocks per SM the classify kernels' register budget is cut for
constexpr int kMinBlocks = TH_CARVE_MIN_BLOCKS;

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
        p.node_out[0] = 0;
    }
}

// Per-level constants shared by both kernels.
struct LevelInfo
{
    int64_t n;
    const int64_t* parents;
    const uint32_t* parent_skip;
    const uint32_t* parent_out;
    float inv_rc;
    bool last;
    bool skips;       // binary masks: skip masks are valid and may be produced
    bool produce;     // compute the children's skip masks (the next level consumes them)
    bool skip_inside; // partial mode: the skip rule also wants the corners in frame
    bool produce_out; // compute the children's out-of-frame masks (partial; the next level consumes them)
    int skip_grow;    // margin of the children's skip rule: 1 when their children are leaves, else 2
};

__device__ __forceinline__ LevelInfo level_info(const HullPlan& p, int li, bool partial)
{
    LevelInfo L;
    const DevCounters* ctr = p.ctr;
    L.n = ctr->level_count[li];
    const int64_t off = ctr->level_off[li];
    L.parents = p.nodes + off;
    L.parent_skip = p.node_skip + off;
    L.parent_out = p.node_out + off;
    L.inv_rc = __int_as_float((127 - (li + 1)) << 23); // 2^-(li + 1), exact
    L.last = (li == p.level - 1);
    L.skips = p.skip_ok && (*p.nonbinary == 0);
    // the children are parents of the next level, which uses the item kernel
    L.produce = L.skips && (li + 1 < p.level) && p.carve_variant[li + 1] == 1;
    L.skip_inside = partial;
    L.produce_out = partial && (li + 1 < p.level) && p.carve_variant[li + 1] == 1;
    L.skip_grow = li + 2 == p.level ? 1 : 2;
    return L;
}

__device__ __forceinline__ void store_parent(const HullPlan& p, const LevelInfo& L, int64_t pi, uint32_t empty, uint32_t refine, uint32_t inside, bool partial)
{
    uint32_t mask = refine & ~empty;
    if (partial && L.last)
        mask &= inside;
    p.child_masks[pi] = static_cast<uint8_t>(mask);
}

// Views over lanes: a group of LANES lanes owns one parent.
template <int LANES, bool PARTIAL, bool OPENGL>
__global__ void __launch_bounds__(32 * kWarps, kMinBlocks) classify_views_kernel(HullPlan p, int li)
{
    constexpr int G = 32 / LANES;
    const LevelInfo L = level_info(p, li, PARTIAL);
    const int lane = threadIdx.x & 31;
    const int sub = lane % LANES, grp = lane / LANES;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    // skip masks can come out of a ballot only when lane == view (<= 32 views)
    const bool produce = L.produce && LANES == 32 && p.B <= 32;
    const bool produce_out = L.produce_out && LANES == 32 && p.B <= 32;
    for (int64_t base = warp * G; base < L.n; base += nwarps * G)
    {
        const int64_t pi = base + grp;
        const bool valid = pi < L.n;
        if (lane == 0)
            atomicAdd(&p.ctr->items[li],
                      static_cast<unsigned long long>(p.B * (L.n - base < G ? L.n - base : G)));
        uint32_t empty = 0, refine = 0, inside = 0, skip = 0, outb = 0;
        if (valid)
        {
            float wx[3], wy[3], wz[3];
            lattice_world(p.rq->corner, p.rq->length, L.parents[pi], li, L.inv_rc, wx, wy, wz);
            const ViewSource src = make_view_source(p.tf, p.sat, p.H, p.W);
            for (int64_t b = sub; b < p.B; b += LANES)
            {
                const ItemResult r = classify_item<PARTIAL, OPENGL>(src, b, wx, wy, wz, produce, L.skip_inside,
                                                                    produce_out, L.skip_grow, L.last);
                empty |= r.empty;
                refine |= r.refine;
                inside |= r.inside;
                skip |= r.skip;
                outb |= r.out;
            }
        }
        uint32_t cskip[8], cout[8];
        if (produce)
        {
#pragma unroll
            for (int c = 0; c < 8; ++c)
                cskip[c] = __ballot_sync(0xffffffffu, (skip >> c) & 1u);
        }
        if (produce_out)
        {
#pragma unroll
            for (int c = 0; c < 8; ++c)
                cout[c] = __ballot_sync(0xffffffffu, (outb >> c) & 1u);
        }
#pragma unroll
        for (int off = LANES / 2; off > 0; off >>= 1)
        {
            empty |= __shfl_xor_sync(0xffffffffu, empty, off);
            refine |= __shfl_xor_sync(0xffffffffu, refine, off);
            inside |= __shfl_xor_sync(0xffffffffu, inside, off);
        }
        if (valid && sub == 0)
        {
            store_parent(p, L, pi, empty, refine, inside, PARTIAL);
            if (pi < p.parent_cap && !L.last)
            {
                // the children inherit the parent's skip views (all descendants are object there)
                const uint32_t inherited = produce && L.skips ? L.parent_skip[pi] : 0u;
#pragma unroll
                for (int c = 0; c < 8; ++c)
                {
                    p.child_skip[pi * 8 + c] = produce ? (cskip[c] | inherited) : 0u;
                    p.child_out[pi * 8 + c] = produce_out ? cout[c] : 0u;
                }
            }
        }
    }
}

// (parent, view) items: a warp deals the unskipped views of a chunk of parents
// out to its lanes.
template <bool PARTIAL, bool OPENGL>
__global__ void __launch_bounds__(32 * kWarps, kMinBlocks) classify_items_kernel(HullPlan p, int li)
{
    __shared__ WarpSlots slots_all[kWarps];
    WarpSlots& ws = slots_all[threadIdx.x >> 5];
    const LevelInfo L = level_info(p, li, PARTIAL);
    const int lane = threadIdx.x & 31;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const int B = static_cast<int>(p.B);
    const uint32_t view_bits = B >= 32 ? 0xffffffffu : ((1u << B) - 1u);
    // parents per chunk: enough chunks for every warp, at most one per lane
    const int64_t per = (L.n + nwarps - 1) / nwarps;
    const int ppw = static_cast<int>(per < 1 ? 1 : (per > 32 ? 32 : per));

    for (int64_t base = warp * ppw; base < L.n; base += nwarps * ppw)
    {
        const int64_t pi = base + lane;
        const bool valid = lane < ppw && pi < L.n;
        const int64_t idx = valid ? L.parents[pi] : 0;
        const uint32_t skipm = (valid && L.skips) ? (L.parent_skip[pi] & view_bits) : 0u;
        // views that see the parent out of the frame for good (partial mode)
        const uint32_t outm = (valid && PARTIAL) ? (L.parent_out[pi] & view_bits) : 0u;
        const uint32_t skipall = skipm | outm;
        const int count = valid ? (B - __popc(skipall)) : 0;
        ws.empty[lane] = 0;
        ws.refine[lane] = 0;
        // a skipped view before the last level (partial mode) is one where
        // every child is fully inside the frame
        ws.inside[lane] = (PARTIAL && L.last && skipm) ? 0xffu : 0u;
#pragma unroll
        for (int c = 0; c < 8; ++c)
        {
            ws.cskip[lane][c] = 0;
            ws.cout[lane][c] = 0;
        }
        // the children inherit the parent's out-of-frame views
        ws.cout_all[lane] = outm;
        const int incl = warp_inclusive_scan(count);
        const int excl = incl - count;
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        if (lane == 0 && total > 0)
            atomicAdd(&p.ctr->items[li], static_cast<unsigned long long>(total));
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
            const uint32_t ms = __shfl_sync(0xffffffffu, skipall, s);
            const int64_t is = __shfl_sync(0xffffffffu, idx, s);
            ItemResult res{ 0, 0, 0, 0, 0 };
            int b = 0;
            const bool act = k < total;
            if (act)
            {
                const int j = k - es;
                const uint32_t active = view_bits & ~ms;
                const int na = __popc(active);
                b = j < na ? select_bit(active, j) : 32 + (j - na);
                float wx[3], wy[3], wz[3];
                lattice_world(p.rq->corner, p.rq->length, is, li, L.inv_rc, wx, wy, wz);
                const ViewSource src = make_view_source(p.tf, p.sat, p.H, p.W);
                res = classify_item<PARTIAL, OPENGL>(src, b, wx, wy, wz, L.produce && b < 32, L.skip_inside,
                                                     L.produce_out && b < 32, L.skip_grow, L.last);
                if (res.out == 0xffu)
                    atomicOr(&ws.cout_all[s], 1u << b);
                else
                    for (uint32_t o = res.out; o; o &= o - 1)
                        atomicOr(&ws.cout[s][__ffs(o) - 1], 1u << b);
                // merge into the slot's words: one shared atomic per non-zero
                // word (a slot's items sit in neighbouring lanes, so conflicts
                // are short)
                if (res.empty)
                    atomicOr(&ws.empty[s], res.empty);
                if (res.refine)
                    atomicOr(&ws.refine[s], res.refine);
                if (res.inside)
                    atomicOr(&ws.inside[s], res.inside);
                if (L.produce)
                    for (uint32_t m = res.skip; m; m &= m - 1)
                        atomicOr(&ws.cskip[s][__ffs(m) - 1], 1u << (b & 31));
            }
        }
        __syncwarp();
        if (valid)
        {
            store_parent(p, L, pi, ws.empty[lane], ws.refine[lane], ws.inside[lane], PARTIAL);
            if (pi < p.parent_cap && !L.last)
            {
#pragma unroll
                for (int c = 0; c < 8; ++c)
                {
                    p.child_skip[pi * 8 + c] = L.produce ? (ws.cskip[lane][c] | skipm) : 0u;
                    p.child_out[pi * 8 + c] = L.produce_out ? (ws.cout[lane][c] | ws.cout_all[lane]) : 0u;
                }
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
        const int64_t mask = (int64_t{ 1 } << li) - 1;
        // Read-only loads: this launch writes only the next level's slots
        // (from level_off[li + 1] on), never this level's nodes or the
        // parents' child masks, so the loads of one chunk of items need not
        // wait for the stores of the previous one.
        const int64_t idx = __ldg(p.nodes + c->level_off[li] + i);
        const int64_t gx = 2 * (idx & mask), gy = 2 * ((idx >> li) & mask), gz = 2 * (idx >> (2 * li));
        const int sh = li + 1; // children ravel at resolution 2^(li+1)
        const uint32_t m = __ldg(p.child_masks + i);
        // the masks of the children of the last level (the leaves) are never read
        const bool has_skip = i < p.parent_cap && li + 1 < p.level;
        int64_t out = c->level_off[li + 1] + static_cast<int64_t>(off);
#pragma unroll
        for (int k = 0; k < 8; ++k)
        {
            if (m >> k & 1u)
            {
                if (out < p.node_cap)
                {
                    p.nodes[out] = (gx + (k & 1)) | ((gy + (k >> 1 & 1)) << sh) | ((gz + (k >> 2 & 1)) << (2 * sh));
                    p.node_skip[out] = has_skip ? __ldg(p.child_skip + i * 8 + k) : 0u;
                    p.node_out[out] = has_skip ? __ldg(p.child_out + i * 8 + k) : 0u;
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
            ctr->overflow |= kOverflowParents; // skip masks were dropped for the excess
        if (start + n > node_cap)
        {
            ctr->overflow |= kOverflowNodes;
            n = 0; // stop the octree here; the host retries with a larger pool
        }
        ctr->level_count[li + 1] = n;
        ctr->level_off[li + 2] = start + n;
    }
};

template <bool PARTIAL, bool OPENGL>
void launch_classify(const HullPlan& p, int li, int64_t max_parents, cudaStream_t s)
{
    const int threads = 32 * kWarps;
    if (p.carve_variant[li] == 1)
    {
        // about one lane per (parent, view) item when the level is small
        classify_items_kernel<PARTIAL, OPENGL><<<grid_for(max_parents * p.B, threads), threads, 0, s>>>(p, li);
        return;
    }
    const int grid = grid_for(max_parents * 32, threads);
    if (p.B <= 4)
        classify_views_kernel<4, PARTIAL, OPENGL><<<grid, threads, 0, s>>>(p, li);
    else if (p.B <= 8)
        classify_views_kernel<8, PARTIAL, OPENGL><<<grid, threads, 0, s>>>(p, li);
    else if (p.B <= 16)
        classify_views_kernel<16, PARTIAL, OPENGL><<<grid, threads, 0, s>>>(p, li);
    else
        classify_views_kernel<32, PARTIAL, OPENGL><<<grid, threads, 0, s>>>(p, li);
}

} // namespace

int grid_for(int64_t work_items, int threads)
{
    const int64_t blocks = (work_items + threads - 1) / threads;
    const int64_t cap = 8LL * sm_count();
    return static_cast<int>(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

void launch_hull_init(const HullPlan& p, cudaStream_t s)
{
    launch_zero(p.ctr, sizeof(DevCounters), s);
    hull_init_kernel<<<1, 32, 0, s>>>(p);
    TH_LAUNCH_CHECK();
}

void launch_carve_level(const HullPlan& p, int li, cudaStream_t s)
{
    // Upper bound of the parents at level li, for the grid size only.
    const int64_t bound = li < 10 ? (int64_t{ 1 } << (3 * li)) : p.node_cap;
    const int64_t max_parents = bound < p.node_cap ? bound : p.node_cap;
    if (p.partial)
    {
        if (p.opengl)
            launch_classify<true, true>(p, li, max_parents, s);
        else
            launch_classify<true, false>(p, li, max_parents, s);
    }
    else
    {
        if (p.opengl)
            launch_classify<false, true>(p, li, max_parents, s);
        else
            launch_classify<false, false>(p, li, max_parents, s);
    }
    TH_LAUNCH_CHECK();
    if (li + 1 == p.level)
    {
        // The leaves are not written out: their corners are marked from the
        // parents' child masks (launch_corners), and the leaf list is emitted
        // only when the candidates of the last level are exported.  The count
        // (and the pool check) is still taken here.
        run_scan_reduce(ChildCount{ p.child_masks }, ChildEpilogue{ p.ctr, li, p.node_cap, p.parent_cap },
                        Count{ &p.ctr->level_count[li], 0 }, max_parents, p.tile_sums, &p.ctr->scan, s);
        return;
    }
    run_scan(ChildCount{ p.child_masks }, ChildEmit{ p, li }, ChildEpilogue{ p.ctr, li, p.node_cap, p.parent_cap },
             Count{ &p.ctr->level_count[li], 0 }, max_parents, p.tile_sums, &p.ctr->scan, s);
}

void launch_emit_leaves(const HullPlan& p, cudaStream_t s)
{
    const int li = p.level - 1;
    if (li < 0)
        return;
    const int64_t bound = li < 10 ? (int64_t{ 1 } << (3 * li)) : p.node_cap;
    const int64_t max_parents = bound < p.node_cap ? bound : p.node_cap;
    run_scan(ChildCount{ p.child_masks }, ChildEmit{ p, li }, NoEpilogue{}, Count{ &p.ctr->level_count[li], 0 },
             max_parents, p.tile_sums, &p.ctr->scan, s);
}

} // namespace th
