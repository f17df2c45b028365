// Octree carving: one level per launch pair (classify, then compact).
//
// Reference: classify_children_full / _partial (visual_hull_cuda.cu:168-417)
// run one thread per child and project each of the child's 8 corners for
// every view; the level loop (:633-751) compacts the flags with cub and reads
// the count back to the host.
//
// Here a group of LANES lanes of a warp owns one parent cell and its lanes
// split the views.  For each view a lane projects the 27 points of the
// parent's 3x3x3 child-corner lattice once (the reference projects 64 corner
// instances for the same 8 children), then derives each child's pixel bounding
// box, its four SAT corner samples and its class with the reference's exact
// arithmetic.  Per child the per-view outcomes combine by OR (empty in any
// view, partial in any view, fully inside some frame), so splitting views over
// lanes and OR-reducing with shuffles gives the reference's decision exactly.
// The 8 child flags of a parent become one byte; a device-wide scan over the
// popcounts then writes the refined children in the reference's stable order
// (parent order, then child index), and its last block stores the level size
// on the device for the next level.  No host round trip per level.

#include <cfloat>

#include "th_hull.cuh"
#include "th_internal.h"

namespace th
{

namespace
{

__global__ void hull_init_kernel(HullPlan p)
{
    if (threadIdx.x == 0 && blockIdx.x == 0)
    {
        DevCounters* c = p.ctr;
        c->level_count[0] = 1;
        c->level_off[0] = 0;
        c->level_off[1] = 1;
        p.nodes[0] = 0;
    }
}

__device__ __forceinline__ float sat_sample(const HullPlan& p, int64_t b, int64_t y, int64_t x)
{
    // sample_zeros_padding (image_utils.h:84-97)
    return in_image(y, x, p.H, p.W) ? p.sat[(b * p.H + y) * p.W + x] : 0.f;
}

template <int LANES, bool PARTIAL>
__global__ void __launch_bounds__(256) classify_kernel(HullPlan p, int li)
{
    constexpr int G = 32 / LANES;
    const DevCounters* ctr = p.ctr;
    const int64_t n = ctr->level_count[li];
    const int64_t* parents = p.nodes + ctr->level_off[li];
    const int lane = threadIdx.x & 31;
    const int sub = lane % LANES, grp = lane / LANES;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const int64_t r = int64_t{ 1 } << li;
    const float rcf = static_cast<float>(2 * r);
    const bool last = (li == p.level - 1);
    const float Hf = static_cast<float>(p.H), Wf = static_cast<float>(p.W);
    const float margin = 0.5f - 0.1f; // isolevel - epsilon (visual_hull_cuda.cu:259-267)

    for (int64_t base = warp * G; base < n; base += nwarps * G)
    {
        const int64_t pi = base + grp;
        const bool valid = pi < n;
        uint32_t empty = 0, refine = 0, inside = 0;
        if (valid)
        {
            const int64_t idx = parents[pi];
            const int64_t gx = idx % r, gy = idx / r % r, gz = idx / (r * r);
            float wx[3], wy[3], wz[3];
#pragma unroll
            for (int d = 0; d < 3; ++d)
            {
                wx[d] = world_coordinate(2 * gx + d, rcf, p.corner[0], p.length);
                wy[d] = world_coordinate(2 * gy + d, rcf, p.corner[1], p.length);
                wz[d] = world_coordinate(2 * gz + d, rcf, p.corner[2], p.length);
            }
            for (int64_t b = sub; b < p.B; b += LANES)
            {
                float m[16];
#pragma unroll
                for (int k = 0; k < 16; ++k)
                    m[k] = p.tf[16 * b + k];
                float px[27], py[27];
                uint32_t in27 = 0;
#pragma unroll
                for (int k = 0; k < 27; ++k)
                {
                    to_pixel(m, wx[k % 3], wy[k / 3 % 3], wz[k / 9], p.opengl, Hf, Wf, px[k], py[k]);
                    if (PARTIAL)
                    {
                        const int64_t rx = f2i64(roundf(px[k]));
                        const int64_t ry = f2i64(roundf(py[k]));
                        if (in_image(ry, rx, p.H, p.W, 1))
                            in27 |= 1u << k;
                    }
                }
#pragma unroll
                for (int c = 0; c < 8; ++c)
                {
                    const int cx = c & 1, cy = c >> 1 & 1, cz = c >> 2 & 1;
                    float bminx = FLT_MAX, bminy = FLT_MAX, bmaxx = -FLT_MAX, bmaxy = -FLT_MAX;
                    bool full_in = true;
#pragma unroll
                    for (int i = 0; i < 8; ++i)
                    {
                        const int k = (cx + (i & 1)) + 3 * (cy + (i >> 1 & 1)) + 9 * (cz + (i >> 2 & 1));
                        bminx = fminf(bminx, px[k]);
                        bminy = fminf(bminy, py[k]);
                        bmaxx = fmaxf(bmaxx, px[k]);
                        bmaxy = fmaxf(bmaxy, py[k]);
                        if (PARTIAL)
                            full_in = full_in && ((in27 >> k) & 1u);
                    }
                    // visual_hull_cuda.cu:236-257
                    const int64_t rminx = f2i64(roundf(__fadd_rn(bminx, -0.5f)));
                    const int64_t rminy = f2i64(roundf(__fadd_rn(bminy, -0.5f)));
                    const int64_t rmaxx = f2i64(roundf(__fadd_rn(bmaxx, 0.5f)));
                    const int64_t rmaxy = f2i64(roundf(__fadd_rn(bmaxy, 0.5f)));
                    const int64_t cminx = min(max(rminx, int64_t{ 0 }), p.W - 1);
                    const int64_t cminy = min(max(rminy, int64_t{ 0 }), p.H - 1);
                    const int64_t cmaxx = min(max(rmaxx, int64_t{ 0 }), p.W - 1);
                    const int64_t cmaxy = min(max(rmaxy, int64_t{ 0 }), p.H - 1);
                    const int64_t area = (cmaxy - cminy + 1) * (cmaxx - cminx + 1);
                    const float i00 = sat_sample(p, b, cminy - 1, cminx - 1);
                    const float i10 = sat_sample(p, b, cmaxy, cminx - 1);
                    const float i01 = sat_sample(p, b, cminy - 1, cmaxx);
                    const float i11 = sat_sample(p, b, cmaxy, cmaxx);
                    const float sum = __fsub_rn(__fsub_rn(__fadd_rn(i11, i00), i10), i01);
                    bool whole = true;
                    if (PARTIAL)
                    {
                        // full_area_bb with the device's wrapping int64 arithmetic (:377)
                        const uint64_t fy = static_cast<uint64_t>(rmaxy) - static_cast<uint64_t>(rminy) + 1u;
                        const uint64_t fx = static_cast<uint64_t>(rmaxx) - static_cast<uint64_t>(rminx) + 1u;
                        whole = (static_cast<uint64_t>(area) == fy * fx);
                    }
                    const uint32_t bit = 1u << c;
                    if (sum <= 0.f + margin && whole)
                        empty |= bit;
                    else if (sum >= __fsub_rn(__ll2float_rn(area), margin) && whole)
                    {
                    }
                    else if (!PARTIAL || (cmaxy - cminy > 1 && cmaxx - cminx > 1))
                        refine |= bit;
                    if (PARTIAL && full_in)
                        inside |= bit;
                }
            }
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
            uint32_t mask = refine & ~empty;
            if (PARTIAL && last)
                mask &= inside;
            p.child_masks[pi] = static_cast<uint8_t>(mask);
        }
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
        int64_t out = c->level_off[li + 1] + static_cast<int64_t>(off);
#pragma unroll
        for (int k = 0; k < 8; ++k)
        {
            if (m >> k & 1u)
            {
                if (out < p.node_cap)
                    p.nodes[out] = (gx + (k & 1)) + (gy + (k >> 1 & 1)) * rc + (gz + (k >> 2 & 1)) * rc * rc;
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
    __device__ void operator()(unsigned long long total) const
    {
        const int64_t start = ctr->level_off[li + 1];
        int64_t n = static_cast<int64_t>(total);
        if (start + n > node_cap)
        {
            ctr->overflow |= kOverflowNodes;
            n = 0; // stop the octree here; the host retries with a larger pool
        }
        ctr->level_count[li + 1] = n;
        ctr->level_off[li + 2] = start + n;
    }
};

template <int LANES>
void launch_classify(const HullPlan& p, int li, int grid, cudaStream_t s)
{
    if (p.partial)
        classify_kernel<LANES, true><<<grid, 256, 0, s>>>(p, li);
    else
        classify_kernel<LANES, false><<<grid, 256, 0, s>>>(p, li);
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
    TH_CUDA(cudaMemsetAsync(p.ctr, 0, sizeof(DevCounters), s));
    hull_init_kernel<<<1, 32, 0, s>>>(p);
    TH_LAUNCH_CHECK();
}

void launch_carve_level(const HullPlan& p, int li, cudaStream_t s)
{
    // Upper bound of the parents at level li, for the grid size only.
    const int64_t bound = li < 10 ? (int64_t{ 1 } << (3 * li)) : p.node_cap;
    const int64_t max_parents = bound < p.node_cap ? bound : p.node_cap;
    const int grid = grid_for(max_parents * 32, 256);
    if (p.B <= 4)
        launch_classify<4>(p, li, grid, s);
    else if (p.B <= 8)
        launch_classify<8>(p, li, grid, s);
    else if (p.B <= 16)
        launch_classify<16>(p, li, grid, s);
    else
        launch_classify<32>(p, li, grid, s);
    TH_LAUNCH_CHECK();
    run_scan(ChildCount{ p.child_masks }, ChildEmit{ p, li }, ChildEpilogue{ p.ctr, li, p.node_cap },
             Count{ &p.ctr->level_count[li], 0 }, max_parents, p.tile_sums, &p.ctr->scan, s);
}

} // namespace th
