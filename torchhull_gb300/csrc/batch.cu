// Batched form: the octrees of many requests, carved by one persistent launch.
//
// The plain path launches a classify kernel and a compaction per level and
// request.  Here one cooperative kernel, resident on every SM, walks the
// levels of all requests at once: level i is one list of request-tagged cells
// (the device work queue).  Warps take chunks of it from an atomic head,
// deal the chunk's unskipped (cell, view) items to their lanes with the same
// per-item routine as the plain kernels (th_classify.cuh), and record each
// cell's refined children; after a grid-wide barrier every block writes the
// children of a contiguous range of cells, in cell order, at offsets from a
// grid-wide scan (two more barriers).  Lists stay in the order of the plain
// path's compaction: requests in order, neighbouring cells together.
// Requests with different view counts, sizes, levels and modes share warps; a
// cell whose request ends at level i is a leaf and produces no items.  Each
// request's mesh is bit-identical to the plain path's: the corner set is built
// in a bitmap and comes out sorted.
//
// Afterwards one launch marks the corners of every request's leaves in that
// request's bitmap; the remaining stages (corner ranks, field, marching cubes)
// run per request on the host's streams.

#include <cooperative_groups.h>

#include "th_batch.cuh"
#include "th_classify.cuh"
#include "th_hull.cuh"
#include "th_internal.h"

namespace cg = cooperative_groups;

namespace th
{

namespace
{

constexpr int kBatchWarps = 8;
constexpr int64_t kCellMask = (int64_t{ 1 } << kTagShift) - 1;

__global__ void batch_init_kernel(BatchPlan bp)
{
    for (int i = threadIdx.x; i < bp.nreq; i += blockDim.x)
    {
        bp.nodes[i] = static_cast<int64_t>(i) << kTagShift;
        bp.node_skip[i] = 0;
        bp.node_out[i] = 0;
    }
    if (threadIdx.x == 0)
        bp.ctr->count[0] = bp.nreq;
}

// VARIANT: (partial << 1) | opengl shared by every request of the batch, or
// -1 to branch per request.
template <int VARIANT>
__device__ __forceinline__ ItemResult batch_item(const BatchReq& q,
                                                 int64_t b,
                                                 const float wx[3],
                                                 const float wy[3],
                                                 const float wz[3],
                                                 bool want_skip,
                                                 bool skip_inside,
                                                 bool want_out,
                                                 int grow,
                                                 bool want_inside)
{
    const ViewSource src = make_view_source(q.tf, q.sat, q.H, q.W);
    if constexpr (VARIANT >= 0)
        return classify_item<(VARIANT >> 1) != 0, (VARIANT & 1) != 0>(src, b, wx, wy, wz, want_skip, skip_inside,
                                                                      want_out, grow, want_inside);
    if (q.partial)
        return q.opengl ? classify_item<true, true>(src, b, wx, wy, wz, want_skip, skip_inside, want_out, grow,
                                                    want_inside)
                        : classify_item<true, false>(src, b, wx, wy, wz, want_skip, skip_inside, want_out, grow,
                                                     want_inside);
    return q.opengl ? classify_item<false, true>(src, b, wx, wy, wz, want_skip, skip_inside, want_out, grow,
                                                 want_inside)
                    : classify_item<false, false>(src, b, wx, wy, wz, want_skip, skip_inside, want_out, grow,
                                                  want_inside);
}

// Entries of level li that were written (a pool overflow drops the rest).
__device__ __forceinline__ int64_t level_entries(const BatchPlan& bp, int li, int64_t start)
{
    const int64_t n = bp.ctr->count[li];
    const int64_t room = bp.node_cap - start;
    return n < room ? n : (room > 0 ? room : 0);
}

template <int VARIANT>
__global__ void __launch_bounds__(32 * kBatchWarps, 2) batch_carve_kernel(BatchPlan bp)
{
    cg::grid_group grid = cg::this_grid();
    __shared__ WarpSlots slots_all[kBatchWarps];
    WarpSlots& ws = slots_all[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    BatchCounters* ctr = bp.ctr;
    const int64_t nwarps = static_cast<int64_t>(gridDim.x) * kBatchWarps;
    int64_t start = 0;
    for (int li = 0; li < bp.max_level; ++li)
    {
        const int64_t n = level_entries(bp, li, start);
        const int64_t next = start + n;
        const float inv_rc = __int_as_float((127 - (li + 1)) << 23); // 2^-(li + 1), exact
        const int64_t per = (n + nwarps - 1) / nwarps;
        const int ppw = static_cast<int>(per < 1 ? 1 : (per > 32 ? 32 : per));
        // Warps take chunks from an atomic head: cells differ widely in work
        // (skipped views, requests of different sizes), and a static
        // round-robin deal left the level's tail 6 % longer on the 4 x
        // level-9 batch although it shares L1 lines better.
        for (;;)
        {
            unsigned long long got = 0;
            if (lane == 0)
                got = atomicAdd(&ctr->head[li], static_cast<unsigned long long>(ppw));
            const int64_t base = static_cast<int64_t>(__shfl_sync(0xffffffffu, got, 0));
            if (base >= n)
                break;
            const int64_t pi = base + lane;
            const bool valid = lane < ppw && pi < n;
            const int64_t node = valid ? bp.nodes[start + pi] : 0;
            const BatchReq& q = bp.reqs[static_cast<int>(node >> kTagShift)];
            const bool work = valid && q.level > li && !q.no_carve;
            const bool skips = work && q.skip_ok && (*q.nonbinary == 0);
            const uint32_t view_bits = q.B >= 32 ? 0xffffffffu : ((1u << q.B) - 1u);
            const uint32_t skipm = skips ? (bp.node_skip[start + pi] & view_bits) : 0u;
            // views that see the cell out of the frame for good (partial requests)
            const uint32_t outm = (work && q.partial) ? (bp.node_out[start + pi] & view_bits) : 0u;
            const uint32_t skipall = skipm | outm;
            const int count = work ? (q.B - __popc(skipall)) : 0;
            const bool last = (li == q.level - 1);
            ws.empty[lane] = 0;
            ws.refine[lane] = 0;
            ws.inside[lane] = (work && q.partial && last && skipm) ? 0xffu : 0u;
#pragma unroll
            for (int c = 0; c < 8; ++c)
            {
                ws.cskip[lane][c] = 0;
                ws.cout[lane][c] = 0;
            }
            // the children inherit the cell's out-of-frame views
            ws.cout_all[lane] = outm;
            const int incl = warp_inclusive_scan(count);
            const int excl = incl - count;
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            __syncwarp();
            for (int k0 = 0; k0 < total; k0 += 32)
            {
                const int k = k0 + lane;
                const int s = item_slot(excl, k);
                const int es = __shfl_sync(0xffffffffu, excl, s);
                const uint32_t ms = __shfl_sync(0xffffffffu, skipall, s);
                const int64_t is = __shfl_sync(0xffffffffu, node, s);
                const bool act = k < total;
                ItemResult res{ 0, 0, 0, 0, 0 };
                int b = 0;
                bool produce = false;
                if (act)
                {
                    const BatchReq& qq = bp.reqs[static_cast<int>(is >> kTagShift)];
                    const uint32_t vb = qq.B >= 32 ? 0xffffffffu : ((1u << qq.B) - 1u);
                    const uint32_t active = vb & ~ms;
                    const int na = __popc(active);
                    const int j = k - es;
                    b = j < na ? select_bit(active, j) : 32 + (j - na);
                    float wx[3], wy[3], wz[3];
                    lattice_world(qq.corner, qq.length, is & kCellMask, li, inv_rc, wx, wy, wz);
                    produce = qq.skip_ok && (*qq.nonbinary == 0) && (li + 1 < qq.level);
                    const bool skip_inside = qq.partial != 0;
                    const bool want_out = qq.partial && (li + 1 < qq.level) && b < 32;
                    const int grow = li + 2 == qq.level ? 1 : 2;
                    res = batch_item<VARIANT>(qq, b, wx, wy, wz, produce && b < 32, skip_inside, want_out, grow,
                                              li + 1 == qq.level);
                    if (res.out == 0xffu)
                        atomicOr(&ws.cout_all[s], 1u << b);
                    else
                        for (uint32_t o = res.out; o; o &= o - 1)
                            atomicOr(&ws.cout[s][__ffs(o) - 1], 1u << b);
                    // merge into the slot's words: one shared atomic per non-zero word
                    if (res.empty)
                        atomicOr(&ws.empty[s], res.empty);
                    if (res.refine)
                        atomicOr(&ws.refine[s], res.refine);
                    if (res.inside)
                        atomicOr(&ws.inside[s], res.inside);
                    if (produce)
                        for (uint32_t m = res.skip; m; m &= m - 1)
                            atomicOr(&ws.cskip[s][__ffs(m) - 1], 1u << (b & 31));
                }
            }
            __syncwarp();
            // the refined children of every slot, appended to level li+1
            uint32_t mask = 0;
            if (work)
            {
                mask = ws.refine[lane] & ~ws.empty[lane];
                if (q.partial && last)
                    mask &= ws.inside[lane];
            }
            if (valid)
            {
                // the children come out in phase B, in parent order
                bp.child_masks[pi] = static_cast<uint8_t>(mask);
                if (pi < bp.skip_cap)
                {
                    const bool produce_me = skips && (li + 1 < q.level);
                    const bool produce_out = work && q.partial && (li + 1 < q.level);
#pragma unroll
                    for (int c = 0; c < 8; ++c)
                    {
                        bp.child_skip[pi * 8 + c] = produce_me ? (ws.cskip[lane][c] | skipm) : 0u;
                        bp.child_out[pi * 8 + c] = produce_out ? (ws.cout[lane][c] | ws.cout_all[lane]) : 0u;
                    }
                }
            }
            __syncwarp();
        }
        // The children of the last level are the leaves of the requests that
        // end there: batch_mark_kernel marks their corners from child_masks,
        // so they are not written out.
        if (li + 1 == bp.max_level)
            break;
        grid.sync();
        // Phase B: the refined children of level li, in parent order (like
        // the plain path's compaction), so that neighbouring cells stay
        // neighbours in the list and their integral-image reads hit L1/L2.
        // Each block owns a contiguous range of parents.
        const int64_t per_block = (n + gridDim.x - 1) / gridDim.x;
        const int64_t lo = static_cast<int64_t>(blockIdx.x) * per_block;
        const int64_t hi = lo + per_block < n ? lo + per_block : n;
        {
            unsigned long long c = 0;
            for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x)
                c += __popc(bp.child_masks[i]);
            unsigned long long tot;
            block_exclusive_scan(c, &tot);
            if (threadIdx.x == 0)
                bp.block_sums[blockIdx.x] = tot;
        }
        grid.sync();
        {
            unsigned long long c = 0;
            for (int64_t b = threadIdx.x; b < static_cast<int64_t>(blockIdx.x); b += blockDim.x)
                c += bp.block_sums[b];
            unsigned long long prefix;
            block_exclusive_scan(c, &prefix);
            if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0)
                ctr->count[li + 1] = static_cast<int64_t>(prefix + bp.block_sums[blockIdx.x]);
            int64_t carry = next + static_cast<int64_t>(prefix);
            const int64_t m = (int64_t{ 1 } << li) - 1;
            const int sh = li + 1;
            for (int64_t c0 = lo; c0 < hi; c0 += blockDim.x)
            {
                const int64_t i = c0 + threadIdx.x;
                const uint32_t mask = i < hi ? bp.child_masks[i] : 0u;
                unsigned long long tot;
                const int64_t out0 = carry + static_cast<int64_t>(block_exclusive_scan(
                                                     static_cast<unsigned long long>(__popc(mask)), &tot));
                carry += static_cast<int64_t>(tot);
                if (!mask)
                    continue;
                const int64_t node = bp.nodes[start + i];
                const int64_t cell = node & kCellMask;
                const int64_t gx = 2 * (cell & m), gy = 2 * ((cell >> li) & m), gz = 2 * (cell >> (2 * li));
                const int64_t tag = node & ~kCellMask;
                int64_t out = out0;
#pragma unroll
                for (int c = 0; c < 8; ++c)
                {
                    if (!(mask >> c & 1u))
                        continue;
                    if (out < bp.node_cap)
                    {
                        bp.nodes[out] = tag | (gx + (c & 1)) | ((gy + (c >> 1 & 1)) << sh) | ((gz + (c >> 2 & 1)) << (2 * sh));
                        bp.node_skip[out] = i < bp.skip_cap ? bp.child_skip[i * 8 + c] : 0u;
                        bp.node_out[out] = i < bp.skip_cap ? bp.child_out[i * 8 + c] : 0u;
                    }
                    else
                        atomicOr(&ctr->overflow, 1ull);
                    ++out;
                }
            }
        }
        grid.sync();
        start = next;
    }
}

__global__ void __launch_bounds__(256) batch_mark_kernel(BatchPlan bp)
{
    int64_t starts[kMaxLevel + 2];
    int64_t s = 0;
    for (int li = 0; li <= bp.max_level; ++li)
    {
        starts[li] = s;
        s += level_entries(bp, li, s);
    }
    starts[bp.max_level + 1] = s;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    // only the lists of the levels some request ends at; the carve writes no
    // list for the last level (max_level > 0)
    for (int li = 0; li <= bp.max_level; ++li)
    {
        if (!((bp.leaf_levels >> li) & 1u) || (li == bp.max_level && li > 0))
            continue;
        const int64_t m = (int64_t{ 1 } << li) - 1;
        for (int64_t t = starts[li] + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < starts[li + 1];
             t += stride)
        {
            const int64_t node = bp.nodes[t];
            const BatchReq& q = bp.reqs[static_cast<int>(node >> kTagShift)];
            if (q.level != li)
                continue;
            const int64_t cell = node & kCellMask;
            mark_cell_corners(q.bitmap, q.rowbits, q.R, q.WR, cell & m, (cell >> li) & m, cell >> (2 * li));
        }
    }
    // the leaves of the requests that end at max_level: the refined children
    // of the last carved level's cells, from their child masks
    if (bp.max_level > 0)
    {
        const int li = bp.max_level - 1;
        const int64_t m = (int64_t{ 1 } << li) - 1;
        for (int64_t t = starts[li] + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < starts[li + 1];
             t += stride)
        {
            const uint32_t mask = bp.child_masks[t - starts[li]];
            if (!mask)
                continue;
            const int64_t node = bp.nodes[t];
            const BatchReq& q = bp.reqs[static_cast<int>(node >> kTagShift)];
            if (q.level != bp.max_level)
                continue;
            const int64_t cell = node & kCellMask;
            mark_children_corners(q.bitmap, q.rowbits, q.R, q.WR, 2 * (cell & m), 2 * ((cell >> li) & m),
                                  2 * (cell >> (2 * li)), mask);
        }
    }
}

// The cells of level L-1 of every request with a cell-mask table write their
// skip and out-of-frame views into it (set) or 0 (clear).
__global__ void __launch_bounds__(256) batch_cell_masks_kernel(BatchPlan bp, bool set)
{
    int64_t starts[kMaxLevel + 2];
    int64_t s = 0;
    for (int li = 0; li <= bp.max_level; ++li)
    {
        starts[li] = s;
        s += level_entries(bp, li, s);
    }
    starts[bp.max_level + 1] = s;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    // only the lists of the levels L-1 of requests with a table
    for (int li = 0; li <= bp.max_level; ++li)
    {
        if (!((bp.mask_levels >> li) & 1u))
            continue;
        for (int64_t t = starts[li] + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < starts[li + 1];
             t += stride)
        {
            const int64_t node = bp.nodes[t];
            const BatchReq& q = bp.reqs[static_cast<int>(node >> kTagShift)];
            if (q.cell_masks && li == q.level - 1)
                q.cell_masks[node & kCellMask] = set ? (bp.node_skip[t] | bp.node_out[t]) : 0u;
        }
    }
}

} // namespace

void launch_batch_init(const BatchPlan& bp, cudaStream_t s)
{
    launch_zero(bp.ctr, sizeof(BatchCounters), s);
    batch_init_kernel<<<1, 256, 0, s>>>(bp);
    TH_LAUNCH_CHECK();
}

void launch_batch_carve(const BatchPlan& bp, cudaStream_t s)
{
    if (bp.max_level <= 0)
        return;
    void (*kernel)(BatchPlan) = batch_carve_kernel<-1>;
    switch (bp.variant)
    {
    case 0:
        kernel = batch_carve_kernel<0>;
        break;
    case 1:
        kernel = batch_carve_kernel<1>;
        break;
    case 2:
        kernel = batch_carve_kernel<2>;
        break;
    case 3:
        kernel = batch_carve_kernel<3>;
        break;
    default:
        break;
    }
    int per_sm = 0;
    TH_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 32 * kBatchWarps, 0));
    if (per_sm < 1)
        throw CudaError{ cudaErrorLaunchOutOfResources, "batch carve kernel does not fit on an SM" };
    BatchPlan arg = bp;
    void* args[] = { &arg };
    TH_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<void*>(kernel), dim3(per_sm * sm_count()),
                                        dim3(32 * kBatchWarps), args, 0, s));
    note_launches(1);
}

void launch_batch_mark(const BatchPlan& bp, cudaStream_t s)
{
    batch_mark_kernel<<<grid_for(bp.node_cap, 256), 256, 0, s>>>(bp);
    TH_LAUNCH_CHECK();
}

void launch_batch_cell_masks(const BatchPlan& bp, bool set, cudaStream_t s)
{
    batch_cell_masks_kernel<<<grid_for(bp.node_cap, 256), 256, 0, s>>>(bp, set);
    TH_LAUNCH_CHECK();
}

} // namespace th
