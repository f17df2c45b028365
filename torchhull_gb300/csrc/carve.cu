// Octree carving: one level per launch pair (classify, then compact).
//
// Reference: classify_children_full / _partial (visual_hull_cuda.cu:168-417)
// run one thread per child and project each of the child's 8 corners for
// every view; the level loop (:633-751) compacts the flags with cub and reads
// the count back to the host.
//
// Here a group of LANES lanes of a warp owns one parent cell and its lanes
// split the views.  For each view a lane walks the parent's 3x3x3 lattice of
// child corners plane by plane (z): the nested fmas of the projection
// fma(a0,x,fma(a1,y,fma(a2,z,a3))) are evaluated innermost-first, so the z and
// (y,z) partial sums are shared between lattice points without changing a
// single rounding; each plane is reduced to the pixel boxes of its four 2x2
// point cells, and the four children between two consecutive planes take the
// union of their two cells.  The 27 projections per view replace the
// reference's 64, and only two planes of boxes are live at a time.
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
// Per child the per-view outcomes combine by OR (empty in any view, partial
// in any view, fully inside some frame), so splitting views over lanes and
// OR-reducing with shuffles gives the reference's decision exactly.  The 8
// child flags of a parent become one byte; a device-wide scan over the
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

// Classifies one child in one view from its pixel box; returns bit 0 = empty,
// bit 1 = refine (visual_hull_cuda.cu:236-285 and :365-410).  The box starts
// the reference's min/max from +-FLT_MAX.  sat_b: this view's SAT; H, W >= 1.
template <bool PARTIAL>
__device__ __forceinline__ uint32_t classify_view(const float* __restrict__ sat_b, int32_t H, int32_t W, Box bb)
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
    // sample_zeros_padding at the four box corners; after the clamps only the
    // -1 row/column can leave the image.
    const float* row_hi = sat_b + static_cast<int64_t>(cmaxy) * W;
    const float* row_lo = sat_b + static_cast<int64_t>(cminy - 1) * W;
    const float i11 = row_hi[cmaxx];
    const float i10 = cminx > 0 ? row_hi[cminx - 1] : 0.f;
    const float i01 = cminy > 0 ? row_lo[cmaxx] : 0.f;
    const float i00 = (cminx > 0 && cminy > 0) ? row_lo[cminx - 1] : 0.f;
    const float sum = __fsub_rn(__fsub_rn(__fadd_rn(i11, i00), i10), i01);
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
    if (sum <= 0.f + margin && whole)
        return 1u;
    if (sum >= __fsub_rn(area_f, margin) && whole)
        return 0u;
    if (!PARTIAL || (cmaxy - cminy > 1 && cmaxx - cminx > 1))
        return 2u;
    return 0u;
}

template <int LANES, bool PARTIAL, bool OPENGL>
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
    const int32_t H = static_cast<int32_t>(p.H), W = static_cast<int32_t>(p.W);
    const float Hf = static_cast<float>(p.H), Wf = static_cast<float>(p.W);
    const int64_t view_stride = p.H * p.W;

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
                const float* m = p.tf + 16 * b;
                // rows x, y and the divisor row (w for OpenGL, z for OpenCV)
                const float4 rx = *reinterpret_cast<const float4*>(m);
                const float4 ry = *reinterpret_cast<const float4*>(m + 4);
                const float4 rd = *reinterpret_cast<const float4*>(m + (OPENGL ? 12 : 8));
                const float* sat_b = p.sat + b * view_stride;
                Box prev[4];
                uint32_t prev_in = 0;
#pragma unroll
                for (int z = 0; z < 3; ++z)
                {
                    const float tzx = __fmaf_rn(rx.z, wz[z], rx.w);
                    const float tzy = __fmaf_rn(ry.z, wz[z], ry.w);
                    const float tzd = __fmaf_rn(rd.z, wz[z], rd.w);
                    float px[9], py[9];
                    uint32_t in9 = 0;
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
                            if (PARTIAL)
                            {
                                const int32_t qx = f2i32(roundf(px[k]));
                                const int32_t qy = f2i32(roundf(py[k]));
                                if (1 <= qy && qy < H - 1 && 1 <= qx && qx < W - 1)
                                    in9 |= 1u << k;
                            }
                        }
                    }
                    Box cur[4];
                    uint32_t cur_in = 0;
#pragma unroll
                    for (int c = 0; c < 4; ++c)
                    {
                        const int cx = c & 1, cy = c >> 1;
                        const int k0 = cx + 3 * cy, k1 = k0 + 1, k2 = k0 + 3, k3 = k0 + 4;
                        cur[c] = Box{ fminf(fminf(px[k0], px[k1]), fminf(px[k2], px[k3])),
                                      fminf(fminf(py[k0], py[k1]), fminf(py[k2], py[k3])),
                                      fmaxf(fmaxf(px[k0], px[k1]), fmaxf(px[k2], px[k3])),
                                      fmaxf(fmaxf(py[k0], py[k1]), fmaxf(py[k2], py[k3])) };
                        if (PARTIAL)
                        {
                            const uint32_t need = (1u << k0) | (1u << k1) | (1u << k2) | (1u << k3);
                            if ((in9 & need) == need)
                                cur_in |= 1u << c;
                        }
                    }
                    if (z > 0)
                    {
#pragma unroll
                        for (int c = 0; c < 4; ++c)
                        {
                            const uint32_t bit = 1u << (c + 4 * (z - 1));
                            const uint32_t cls = classify_view<PARTIAL>(sat_b, H, W, merge(prev[c], cur[c]));
                            if (cls & 1u)
                                empty |= bit;
                            if (cls & 2u)
                                refine |= bit;
                            if (PARTIAL && (prev_in & cur_in & (1u << c)))
                                inside |= bit;
                        }
                    }
#pragma unroll
                    for (int c = 0; c < 4; ++c)
                        prev[c] = cur[c];
                    prev_in = cur_in;
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
    {
        if (p.opengl)
            classify_kernel<LANES, true, true><<<grid, 256, 0, s>>>(p, li);
        else
            classify_kernel<LANES, true, false><<<grid, 256, 0, s>>>(p, li);
    }
    else
    {
        if (p.opengl)
            classify_kernel<LANES, false, true><<<grid, 256, 0, s>>>(p, li);
        else
            classify_kernel<LANES, false, false><<<grid, 256, 0, s>>>(p, li);
    }
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
