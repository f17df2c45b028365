// C ABI: contexts with resident device pools, request orchestration and
// argument validation with the reference's error behaviour.
//
// One request enqueues every stage on the caller's stream and reads back one
// small counter block at the end (the reference synchronises after every
// kernel and reads counts back per level, visual_hull_cuda.cu:742, :820 and
// marching_cubes_cuda.cu:600-634).  Pools only grow: a request whose octree or
// corner set outgrows them is detected on the device, the pools grow fourfold
// and the request runs again, so repeated requests of similar size never allocate.

#include <algorithm>
#include <array>
#include <atomic>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <sstream>

#include "th_batch.cuh"
#include "th_hull.cuh"
#include "th_internal.h"
#include "th_mc.cuh"

namespace th
{

namespace
{
std::atomic<int64_t> g_launches{ 0 };
}

// Kernels enqueued while this thread captures a graph are counted when the
// graph is replayed, not when captured.
thread_local bool t_capturing = false;
thread_local int64_t t_captured = 0;

void note_launches(int n)
{
    if (t_capturing)
        t_captured += n;
    else
        g_launches.fetch_add(n, std::memory_order_relaxed);
}

void check_launch(const char* what)
{
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        throw CudaError{ e, std::string("kernel launch: ") + what };
}

int sm_count()
{
    static int cache[64] = { 0 };
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return 148;
    if (cache[dev] == 0)
    {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            n = 148;
        cache[dev] = n;
    }
    return cache[dev];
}

namespace
{

// Small host <-> device transfers (request constants in, counters out) run
// as a one-block kernel over mapped pinned host memory instead of
// cudaMemcpyAsync: a copy engine may be busy with a caller's bulk copy on
// another stream (a previous mesh going out, the next request's masks coming
// in), and a small copy queued behind it would stall the whole pipeline.
__global__ void small_copy_kernel(const unsigned char* __restrict__ src, unsigned char* __restrict__ dst, int64_t n)
{
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
        dst[i] = src[i];
    __threadfence_system();
}

__global__ void zero_kernel(unsigned char* __restrict__ p, int64_t n)
{
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
        p[i] = 0;
}

// dst and src are device addresses (device memory, or mapped host memory's device address).
void small_copy(void* dst, const void* src, size_t bytes, cudaStream_t st)
{
    small_copy_kernel<<<1, 256, 0, st>>>(static_cast<const unsigned char*>(src), static_cast<unsigned char*>(dst),
                                          static_cast<int64_t>(bytes));
    TH_LAUNCH_CHECK();
}

// Pinned host memory for count objects of T, mapped into the device's address space.
template <typename T>
void alloc_mapped(T** host, T** dev, size_t count = 1)
{
    void* h = nullptr;
    TH_CUDA(cudaHostAlloc(&h, sizeof(T) * count, cudaHostAllocMapped));
    void* d = nullptr;
    const cudaError_t e = cudaHostGetDevicePointer(&d, h, 0);
    if (e != cudaSuccess)
    {
        cudaFreeHost(h);
        throw CudaError{ e, "cudaHostGetDevicePointer" };
    }
    *host = static_cast<T*>(h);
    *dev = static_cast<T*>(d);
}

}  // namespace

void launch_zero(void* p, size_t bytes, cudaStream_t s)
{
    if (bytes == 0)
        return;
    const int64_t n = static_cast<int64_t>(bytes);
    const unsigned grid = static_cast<unsigned>(std::min<int64_t>((n + 255) / 256, 64));
    zero_kernel<<<grid, 256, 0, s>>>(static_cast<unsigned char*>(p), n);
    TH_LAUNCH_CHECK();
}

namespace
{

struct DevBuf
{
    void* p = nullptr;
    size_t bytes = 0;

    // Returns true when fresh memory was allocated (contents undefined).
    bool ensure(size_t need)
    {
        if (need <= bytes && p)
            return false;
        if (p)
            TH_CUDA(cudaFree(p));
        p = nullptr;
        bytes = 0;
        size_t sz = std::max<size_t>(need, 256);
        TH_CUDA(cudaMalloc(&p, sz));
        bytes = sz;
        return true;
    }
    void release()
    {
        if (p)
            cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T* as() const
    {
        return static_cast<T*>(p);
    }
};

struct ArgError
{
    th_status status;
    std::string msg;
};

const char* dtype_name(int d)
{
    static const char* names[] = { "Bool", "Byte", "Char", "Short", "Int", "Long", "Half", "Float", "Double", "BFloat16" };
    return (d >= 0 && d <= 9) ? names[d] : "Unknown";
}

bool is_image_dtype(int d)
{
    return d >= TH_UINT8 && d <= TH_FLOAT64;
}

// Pools and the state of the last request of one context.
struct HullSlot
{
    DevBuf tf, sat, ones, cell_masks, nodes, node_skip, node_out, child_masks, child_skip, child_out, tile_sums, bitmap,
            word_rank, rowbits, rows, corners, values, codes, emask, soup_off, vbase, counters, flags, sat_scratch;
    int64_t node_cap = 0, corner_cap = 0, parent_cap = 0;
    HullPlan plan{};
    DevCounters* host = nullptr; // pinned, mapped copy of the counters
    DevCounters* host_d = nullptr; // its device address
    DevBuf rq;                   // ReqConsts of the running request (device)
    ReqConsts* host_rq = nullptr; // pinned, mapped source of rq
    ReqConsts* host_rq_d = nullptr; // its device address
    th_hull_info info{};
    bool has_result = false;
    bool dirty = false; // bitmap rows of the last request still set
    cudaEvent_t done = nullptr;

    // Captured pipelines, keyed by the plan with the per-request fields cleared.
    struct Graph
    {
        HullPlan key;
        cudaGraphExec_t exec = nullptr;
        int64_t kernels = 0;
    };
    std::vector<Graph> graphs;
    cudaStream_t capture_stream = nullptr; // capture only (graphs launch on the caller's stream)

    void drop_graphs()
    {
        for (auto& g : graphs)
            if (g.exec)
                cudaGraphExecDestroy(g.exec);
        graphs.clear();
    }

    std::vector<const DevBuf*> buffers() const
    {
        return { &tf,     &sat,  &ones,  &cell_masks,   &nodes,     &node_skip,   &node_out,  &child_masks, &child_skip, &child_out, &tile_sums,
                 &bitmap, &word_rank, &rowbits, &rows, &corners,    &values,     &codes,
                 &emask,  &soup_off, &vbase,   &counters, &flags, &sat_scratch, &rq };
    }

    void release()
    {
        drop_graphs();
        for (const DevBuf* b : buffers())
            const_cast<DevBuf*>(b)->release();
        if (host)
            cudaFreeHost(host);
        host = nullptr;
        host_d = nullptr;
        if (host_rq)
            cudaFreeHost(host_rq);
        host_rq = nullptr;
        host_rq_d = nullptr;
        if (capture_stream)
            cudaStreamDestroy(capture_stream);
        capture_stream = nullptr;
        if (done)
            cudaEventDestroy(done);
        done = nullptr;
    }
};

} // namespace
} // namespace th

namespace th
{
namespace
{

// CUDA events between the stages of one request (th_context_set_profiling).
struct StageEvents
{
    static constexpr int kCount = TH_MAX_LEVEL + 6;
    cudaEvent_t ev[kCount] = {};
    bool ready = false;

    void create()
    {
        if (ready)
            return;
        for (auto& e : ev)
            TH_CUDA(cudaEventCreate(&e));
        ready = true;
    }
    void destroy()
    {
        if (!ready)
            return;
        for (auto& e : ev)
            cudaEventDestroy(e);
        ready = false;
    }
    void record(int i, cudaStream_t s)
    {
        TH_CUDA(cudaEventRecord(ev[i], s));
    }
    float between(int a, int b) const
    {
        float ms = 0.f;
        TH_CUDA(cudaEventElapsedTime(&ms, ev[a], ev[b]));
        return ms;
    }
};

} // namespace
} // namespace th

namespace th
{
namespace
{

// Request signature for the carve-kernel autotuner.
using TuneKey = std::array<int64_t, 8>;
using CarveVariants = std::array<uint8_t, kMaxLevel>;

TuneKey tune_key(const th_hull_args* a)
{
    return { a->batch, a->height, a->width, a->level, a->masks_partial, a->transforms_opengl, a->masks_dtype, 0 };
}

CarveVariants views_everywhere()
{
    CarveVariants v{};
    return v;
}

// Work items from level 4 on (levels below have at most 8^3 parents).
CarveVariants items_from_level4()
{
    CarveVariants v{};
    for (int i = 4; i < kMaxLevel; ++i)
        v[i] = 1;
    return v;
}

} // namespace
} // namespace th

namespace th
{
namespace
{

// Shared state of the batched form: the tagged node pool of the persistent
// carve, the request table, and the streams the per-request stages run on.
struct BatchState
{
    DevBuf reqs, nodes, node_skip, node_out, ctr, child_masks, child_skip, child_out, block_sums;
    BatchReq* host_reqs = nullptr; // pinned, mapped
    BatchReq* host_reqs_d = nullptr; // its device address
    int32_t host_reqs_cap = 0;
    BatchCounters* host_ctr = nullptr; // pinned, mapped
    BatchCounters* host_ctr_d = nullptr; // its device address
    int64_t node_cap = 0;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> joins;
    cudaEvent_t fork = nullptr;

    void release()
    {
        for (DevBuf* b : { &reqs, &nodes, &node_skip, &node_out, &ctr, &child_masks, &child_skip, &child_out, &block_sums })
            b->release();
        if (host_reqs)
            cudaFreeHost(host_reqs);
        if (host_ctr)
            cudaFreeHost(host_ctr);
        host_reqs = nullptr;
        host_ctr = nullptr;
        host_reqs_d = nullptr;
        host_ctr_d = nullptr;
        for (auto s : streams)
            cudaStreamDestroy(s);
        for (auto e : joins)
            cudaEventDestroy(e);
        if (fork)
            cudaEventDestroy(fork);
        streams.clear();
        joins.clear();
        fork = nullptr;
    }
};

} // namespace
} // namespace th

namespace th
{
namespace
{

// Pools and the last result of the public marching cubes.
struct McSlot
{
    DevBuf groups, keys, slots, codes, used, vbase, tiles_soup, tiles_verts, tiles_scan, active, active_soup, ctr;
    McCounters* host = nullptr; // pinned, mapped copy of the counters
    McCounters* host_d = nullptr; // its device address
    McPlan plan{};
    th_mc_info info{};
    bool has_result = false;

    std::vector<const DevBuf*> buffers() const
    {
        return { &groups, &keys, &slots, &codes, &used, &vbase, &tiles_soup, &tiles_verts, &tiles_scan, &active,
                 &active_soup, &ctr };
    }

    void release()
    {
        for (const DevBuf* b : buffers())
            const_cast<DevBuf*>(b)->release();
        if (host)
            cudaFreeHost(host);
        host = nullptr;
    }
};

} // namespace
} // namespace th

struct th_context
{
    int device = 0;
    std::string error;
    th::HullSlot hull;
    std::vector<th::HullSlot> batch;
    th::BatchState bstate;
    th::DevBuf blur_scratch;
    th::DevBuf blurred; // masks blurred by th_visual_hull_blurred
    th::DevBuf sat_aux; // th_integral_image: its 0/1 flag word, then the single pass's scratch
    cudaEvent_t sat_aux_done = nullptr; // the last th_integral_image that used sat_aux
    th::McSlot mc;
    bool profiling = false;
    th::StageEvents events;
    th_stage_times times{};
    int carve_mode = 0; // TH_OPTION_CARVE_KERNEL
    bool graphs = true;  // TH_OPTION_GRAPHS
    bool batch_route = false; // TH_OPTION_BATCH_ROUTE
    bool field_ones = true;   // TH_OPTION_FIELD_ONES
    bool field_masks = true;  // TH_OPTION_FIELD_MASKS
    bool sat_single_pass = true; // TH_OPTION_SAT_SINGLE_PASS
    std::map<th::TuneKey, th::CarveVariants> carve_tuned;
    cudaEvent_t tune_ev[2] = { nullptr, nullptr };
};

namespace th
{
namespace
{

int64_t pool_bytes(const th_context* ctx)
{
    auto sum = [](const HullSlot& s) {
        int64_t b = 0;
        for (const DevBuf* d : s.buffers())
            b += static_cast<int64_t>(d->bytes);
        return b;
    };
    int64_t total = sum(ctx->hull) + static_cast<int64_t>(ctx->blur_scratch.bytes) +
                    static_cast<int64_t>(ctx->blurred.bytes) + static_cast<int64_t>(ctx->sat_aux.bytes);
    for (const DevBuf* d : ctx->mc.buffers())
        total += static_cast<int64_t>(d->bytes);
    for (const auto& s : ctx->batch)
        total += sum(s);
    return total;
}

void validate(const th_hull_args* a)
{
    if (!a)
        throw ArgError{ TH_ERR_INVALID_ARGUMENT, "args is NULL" };
    // visual_hull_cuda.cu:591-613
    if (a->batch < 0 || a->height < 0 || a->width < 0)
        throw ArgError{ TH_ERR_INVALID_ARGUMENT, "Check failed: masks sizes must be non-negative" };
    if (a->level < 0)
        throw ArgError{ TH_ERR_INVALID_ARGUMENT, "Check failed: level >= 0 (" + std::to_string(a->level) + " vs. 0)" };
    if (a->level > TH_MAX_LEVEL)
        throw ArgError{ TH_ERR_INVALID_ARGUMENT,
                        "level " + std::to_string(a->level) + " exceeds the supported maximum " +
                                std::to_string(TH_MAX_LEVEL) };
    if (!(a->cube_length > 0.f))
        throw ArgError{ TH_ERR_INVALID_ARGUMENT, "Check failed: cube_length > 0.f" };
    // AT_DISPATCH_FLOATING_TYPES_AND_HALF over transforms (:646) and
    // AT_DISPATCH_ALL_TYPES_AND(Half) over masks (:832)
    if (!(a->transforms_dtype == TH_FLOAT16 || a->transforms_dtype == TH_FLOAT32 || a->transforms_dtype == TH_FLOAT64))
        throw ArgError{ TH_ERR_UNSUPPORTED_DTYPE,
                        std::string("\"classify_children\" not implemented for '") + dtype_name(a->transforms_dtype) +
                                "'" };
    if (!is_image_dtype(a->masks_dtype))
        throw ArgError{ TH_ERR_UNSUPPORTED_DTYPE,
                        std::string("\"accumulate_hull_counts\" not implemented for '") + dtype_name(a->masks_dtype) +
                                "'" };
    if (a->batch * a->height * a->width > 0 && (!a->masks || !a->transforms))
        throw ArgError{ TH_ERR_INVALID_ARGUMENT, "masks or transforms pointer is NULL" };
    // Flagged/Unique/stdgpu use 32-bit indices (visual_hull_cuda.cu:716, :798)
    if (a->batch * a->height * a->width >= (int64_t{ 1 } << 40))
        throw ArgError{ TH_ERR_INVALID_ARGUMENT, "masks too large" };
    // pixel indices are carried exactly in float mantissas by the carve
    if (a->height >= (int64_t{ 1 } << 23) || a->width >= (int64_t{ 1 } << 23))
        throw ArgError{ TH_ERR_INVALID_ARGUMENT, "mask height and width must be below 2^23" };
}

int64_t max_nodes(int level)
{
    // sum over levels of 8^i, the most the octree can hold
    int64_t s = 0;
    for (int i = 0; i <= level && i <= 12; ++i)
        s += int64_t{ 1 } << (3 * i);
    return s;
}

// Sizes the pools of slot s for request a and fills its plan.
// batch_slot: the request is part of a batch, whose octree lives in the
// batch's shared node pool, so the slot keeps no octree pools of its own.
void prepare(HullSlot& s, const th_hull_args* a, cudaStream_t st, bool field_ones, bool field_masks, bool batch_slot = false)
{
    const int L = a->level;
    const int64_t B = a->batch, H = a->height, W = a->width;
    const int64_t R = (int64_t{ 1 } << L) + 1;
    const int64_t WR = (R + 63) / 64;
    // Every request starts from at least the capacity its level could need up
    // to 16 M nodes and corners (about 0.5 GB; a level-9 hull of 32 megapixel
    // views fits without a rerun), whatever smaller requests the context
    // served before; beyond that the pools grow x4 per rerun.  Batch slots
    // keep no octree of their own and start at 4 M corners.
    if (batch_slot)
    {
        s.node_cap = std::max<int64_t>(s.node_cap, 1);
        s.parent_cap = std::max<int64_t>(s.parent_cap, 1);
    }
    else
    {
        s.node_cap = std::max<int64_t>(s.node_cap, std::min<int64_t>(max_nodes(L), int64_t{ 1 } << 24));
        s.parent_cap = std::max<int64_t>(s.parent_cap, std::min<int64_t>(max_nodes(L), int64_t{ 1 } << 22));
    }
    s.corner_cap = std::max<int64_t>(s.corner_cap, std::min<int64_t>(R * R * R, int64_t{ 1 } << (batch_slot ? 22 : 24)));
    const int64_t node_cap = std::min<int64_t>(s.node_cap, max_nodes(L));
    const int64_t corner_cap = std::min<int64_t>(s.corner_cap, R * R * R);
    const int64_t parent_cap = std::min<int64_t>(s.parent_cap, node_cap);

    s.tf.ensure(sizeof(float) * std::max<int64_t>(B, 1) * 16);
    s.sat.ensure(sizeof(float) * std::max<int64_t>(B * H * W, 1));
    const int64_t sat_scratch = sat_scratch_bytes(B, H, W, a->masks_dtype);
    if (sat_scratch > 0)
        s.sat_scratch.ensure(static_cast<size_t>(sat_scratch));
    const int64_t WW = (W + 31) / 32;
    // the field's cell-mask table of level L-1 (up to 2^27 cells, 512 MB:
    // level 10) skips most pairs; the all-ones bitmap only pays without it
    const bool cell_masks = field_masks && L >= 1 && 3 * (L - 1) <= 27 &&
                            (a->masks_partial != 0 || (B > 0 && H > 0 && W > 0 && H * W <= (int64_t{ 1 } << 23)));
    field_ones = field_ones && !cell_masks;
    if (field_ones)
        s.ones.ensure(sizeof(uint32_t) * std::max<int64_t>(B * H * WW, 1));
    s.nodes.ensure(sizeof(int64_t) * node_cap);
    s.node_skip.ensure(sizeof(uint32_t) * node_cap);
    s.node_out.ensure(sizeof(uint32_t) * node_cap);
    s.child_masks.ensure(node_cap);
    s.child_skip.ensure(sizeof(uint32_t) * 8 * parent_cap);
    s.child_out.ensure(sizeof(uint32_t) * 8 * parent_cap);
    s.flags.ensure(sizeof(unsigned int) * 4);
    const int64_t scan_items = std::max({ node_cap, corner_cap, R * R * WR });
    s.tile_sums.ensure(sizeof(unsigned long long) * ((scan_items + kScanTile - 1) / kScanTile + 1));
    const int64_t words = R * R * WR;
    const int64_t rwords = (R * R + 31) / 32;
    if (s.bitmap.ensure(sizeof(uint64_t) * words))
        TH_CUDA(cudaMemsetAsync(s.bitmap.p, 0, s.bitmap.bytes, st));
    s.word_rank.ensure(sizeof(uint32_t) * words);
    if (s.rowbits.ensure(sizeof(uint32_t) * rwords))
        TH_CUDA(cudaMemsetAsync(s.rowbits.p, 0, s.rowbits.bytes, st));
    s.rows.ensure(sizeof(uint32_t) * R * R);
    s.corners.ensure(sizeof(int64_t) * corner_cap);
    s.values.ensure(sizeof(float) * corner_cap);
    s.codes.ensure(corner_cap);
    s.emask.ensure((corner_cap + 3) / 4 * 4);
    s.soup_off.ensure(sizeof(uint32_t) * corner_cap);
    s.vbase.ensure(sizeof(uint32_t) * corner_cap);
    if (s.counters.ensure(sizeof(DevCounters)))
        TH_CUDA(cudaMemsetAsync(s.counters.p, 0, sizeof(DevCounters), st));
    if (!s.host)
        alloc_mapped(&s.host, &s.host_d);
    if (!s.done)
        TH_CUDA(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));

    HullPlan& p = s.plan;
    std::memset(&p, 0, sizeof(HullPlan)); // zero padding too: plans are compared bytewise
    p.masks = a->masks;
    p.masks_dtype = a->masks_dtype;
    p.B = B;
    p.H = H;
    p.W = W;
    p.tf = s.tf.as<float>();
    p.sat = s.sat.as<float>();
    p.opengl = a->transforms_opengl != 0;
    p.partial = a->masks_partial != 0;
    p.unique = a->unique_verts != 0;
    p.corner[0] = a->cube_corner_bfl[0];
    p.corner[1] = a->cube_corner_bfl[1];
    p.corner[2] = a->cube_corner_bfl[2];
    p.length = a->cube_length;
    p.level = L;
    p.nodes = s.nodes.as<int64_t>();
    p.node_cap = node_cap;
    p.child_masks = s.child_masks.as<uint8_t>();
    p.tile_sums = s.tile_sums.as<unsigned long long>();
    p.node_skip = s.node_skip.as<uint32_t>();
    p.child_skip = s.child_skip.as<uint32_t>();
    p.node_out = s.node_out.as<uint32_t>();
    p.child_out = s.child_out.as<uint32_t>();
    p.parent_cap = parent_cap;
    p.nonbinary = s.flags.as<unsigned int>();
    // exact integer box sums need every SAT sum of two entries below 2^24
    p.skip_ok = B > 0 && H > 0 && W > 0 && H * W <= (int64_t{ 1 } << 23);
    p.field_ones = field_ones && B > 0 && H > 0 && W > 0;
    p.cell_masks = nullptr;
    p.own_cell_masks = !batch_slot;
    if (cell_masks)
    {
        if (s.cell_masks.ensure(sizeof(uint32_t) * (int64_t{ 1 } << (3 * (L - 1)))))
            TH_CUDA(cudaMemsetAsync(s.cell_masks.p, 0, s.cell_masks.bytes, st));
        p.cell_masks = s.cell_masks.as<uint32_t>();
    }
    p.ones = field_ones ? s.ones.as<uint32_t>() : nullptr;
    p.WW = WW;
    p.R = R;
    p.WR = WR;
    p.bitmap = s.bitmap.as<uint64_t>();
    p.word_rank = s.word_rank.as<uint32_t>();
    p.rowbits = s.rowbits.as<uint32_t>();
    p.rows = s.rows.as<uint32_t>();
    p.corners = s.corners.as<int64_t>();
    p.values = s.values.as<float>();
    p.codes = s.codes.as<uint8_t>();
    p.emask = s.emask.as<uint8_t>();
    p.soup_off = s.soup_off.as<uint32_t>();
    p.vbase = s.vbase.as<uint32_t>();
    p.corner_cap = corner_cap;
    p.ctr = s.counters.as<DevCounters>();
    // the per-request inputs the carve and field kernels read from the device
    s.rq.ensure(sizeof(ReqConsts));
    if (!s.host_rq)
        alloc_mapped(&s.host_rq, &s.host_rq_d);
    *s.host_rq = ReqConsts{ { p.corner[0], p.corner[1], p.corner[2] }, p.length, p.masks };
    small_copy(s.rq.p, s.host_rq_d, sizeof(ReqConsts), st);
    p.rq = s.rq.as<ReqConsts>();
}

void fill_info(const HullSlot& s, th_hull_info* info)
{
    const DevCounters& c = *s.host;
    th_hull_info out{};
    const HullPlan& p = s.plan;
    // candidates_octree: levels up to and including the first empty one
    int n = 1;
    out.level_sizes[0] = c.level_count[0];
    for (int i = 1; i <= p.level; ++i)
    {
        out.level_sizes[i] = c.level_count[i];
        n = i + 1;
        if (c.level_count[i] == 0)
            break;
    }
    out.num_levels = n;
    const bool empty = c.level_count[p.level] == 0;
    out.num_corners = empty ? 0 : c.corners;
    if (empty || c.soup == 0)
    {
        out.num_verts = 0;
        out.num_faces = 0;
    }
    else
    {
        out.num_verts = p.unique ? c.verts : c.soup;
        out.num_faces = c.soup / 3;
    }
    *info = out;
}

// Everything of a run after the integral image: octree levels, corners,
// field, marching cubes and the read-back of the counters (stream-ordered
// only, so that it can be captured as a graph).
void enqueue_core(th_context* ctx, HullSlot& s, cudaStream_t st, StageEvents* ev, bool tune)
{
    const HullPlan& p = s.plan;
    const int L = p.level;
    launch_hull_init(p, st);
    // With an empty image every child is empty in the first view (the
    // reference samples zeros everywhere), so the octree stops at the root;
    // without views nothing is refined either.  Skip the carve in both cases.
    const bool carve = p.B > 0 && p.H > 0 && p.W > 0;
    if (tune)
        TH_CUDA(cudaEventRecord(ctx->tune_ev[0], st));
    for (int li = 0; li < p.level; ++li)
    {
        if (carve)
            launch_carve_level(p, li, st);
        if (ev)
            ev->record(2 + li, st);
    }
    if (tune)
        TH_CUDA(cudaEventRecord(ctx->tune_ev[1], st));
    if (ev)
        ev->record(L + 2, st);
    launch_corners(p, st);
    if (ev)
        ev->record(L + 3, st);
    launch_field(p, st);
    if (ev)
        ev->record(L + 4, st);
    launch_marching_cubes(p, st);
    if (ev)
        ev->record(L + 5, st);
    small_copy(s.host_d, p.ctr, sizeof(DevCounters), st);
}

// enqueue_core as a graph: captured once per plan (the per-request corner,
// length and masks come through p.rq, uploaded by prepare), replayed after.
void replay_core(HullSlot& s, cudaStream_t st)
{
    HullPlan key;
    std::memcpy(&key, &s.plan, sizeof(HullPlan));
    key.masks = nullptr;
    key.corner[0] = key.corner[1] = key.corner[2] = 0.f;
    key.length = 0.f;
    HullSlot::Graph* g = nullptr;
    for (auto& e : s.graphs)
        if (std::memcmp(&e.key, &key, sizeof(HullPlan)) == 0)
            g = &e;
    if (!g)
    {
        if (s.graphs.size() >= 8)
            s.drop_graphs();
        // captured on a private stream (the caller's may be the legacy
        // default stream, which cannot capture); nothing runs while capturing
        if (!s.capture_stream)
            TH_CUDA(cudaStreamCreateWithFlags(&s.capture_stream, cudaStreamNonBlocking));
        const cudaStream_t cs = s.capture_stream;
        cudaGraph_t graph = nullptr;
        TH_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        t_capturing = true;
        t_captured = 0;
        try
        {
            enqueue_core(nullptr, s, cs, nullptr, false);
        }
        catch (...)
        {
            t_capturing = false;
            cudaStreamEndCapture(cs, &graph);
            if (graph)
                cudaGraphDestroy(graph);
            throw;
        }
        t_capturing = false;
        TH_CUDA(cudaStreamEndCapture(cs, &graph));
        cudaGraphExec_t exec = nullptr;
        const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        TH_CUDA(e);
        s.graphs.push_back(HullSlot::Graph{ key, exec, t_captured });
        g = &s.graphs.back();
    }
    TH_CUDA(cudaGraphLaunch(g->exec, st));
    note_launches(static_cast<int>(g->kernels));
}

// One complete run of a request with the given carve kernels.  carve_ms
// (optional) receives the time of the carve stage, for the autotuner.
void run_hull_once(th_context* ctx,
                   HullSlot& s,
                   const th_hull_args* a,
                   cudaStream_t st,
                   StageEvents* ev,
                   const CarveVariants& variants,
                   float* carve_ms)
{
    if (s.dirty)
    {
        TH_CUDA(cudaStreamWaitEvent(st, s.done, 0));
        launch_cleanup(s.plan, st);
        s.dirty = false;
    }
    s.has_result = false;
    const int L = a->level;
    for (int attempt = 0; attempt < 8; ++attempt)
    {
        prepare(s, a, st, ctx->field_ones, ctx->field_masks);
        for (int i = 0; i < kMaxLevel; ++i)
            s.plan.carve_variant[i] = variants[i];
        const HullPlan& p = s.plan;
        if (attempt == 0)
        {
            if (ev)
                ev->record(0, st);
            launch_convert_transforms(a->transforms, a->transforms_dtype, a->batch, s.tf.as<float>(), st);
            launch_zero(s.flags.p, sizeof(unsigned int), st);
            launch_integral_image(a->masks, a->masks_dtype, a->batch, a->height, a->width, s.sat.as<float>(), st,
                                  s.flags.as<unsigned int>(),
                                  ctx->sat_single_pass ? SatScratch{ s.sat_scratch.p } : SatScratch{});
            if (ev)
                ev->record(1, st);
        }
        if (ctx->graphs && !ev && !carve_ms)
            replay_core(s, st);
        else
            enqueue_core(ctx, s, st, ev, carve_ms != nullptr);
        TH_CUDA(cudaStreamSynchronize(st));
        s.dirty = true;
        const int64_t ovf = s.host->overflow;
        // A level wider than the skip-mask scratch only loses view skipping
        // for its excess parents (results are unchanged): keep the result and
        // grow the scratch for the next request.
        if (ovf & kOverflowParents)
            s.parent_cap *= 4;
        if ((ovf & ~int64_t{ kOverflowParents }) == 0)
            break;
        launch_cleanup(p, st);
        s.dirty = false;
        if (ovf & kOverflowNodes)
            s.node_cap *= 4;
        if (ovf & kOverflowCorners)
            s.corner_cap *= 4;
        if (attempt == 7)
        {
            const DevCounters& c = *s.host;
            std::string counts;
            for (int i = 0; i <= L; ++i)
                counts += (i ? "," : "") + std::to_string(c.level_count[i]);
            throw ArgError{ TH_ERR_OUT_OF_MEMORY,
                            "visual hull pools could not be grown enough (overflow " + std::to_string(ovf) +
                                    ", level counts " + counts + ", corners " + std::to_string(c.corners) + ", rows " +
                                    std::to_string(c.rows) + ", node cap " + std::to_string(p.node_cap) +
                                    ", corner cap " + std::to_string(p.corner_cap) + ")" };
        }
    }
    fill_info(s, &s.info);
    s.has_result = true;
    if (ev)
    {
        th_stage_times t{};
        t.levels = L;
        t.integral_image_ms = ev->between(0, 1);
        for (int li = 0; li < L; ++li)
            t.carve_ms[li] = ev->between(1 + li, 2 + li);
        t.corners_ms = ev->between(L + 2, L + 3);
        t.field_ms = ev->between(L + 3, L + 4);
        t.marching_cubes_ms = ev->between(L + 4, L + 5);
        t.total_ms = ev->between(0, L + 5);
        for (int li = 0; li < L; ++li)
            t.carve_items[li] = static_cast<int64_t>(s.host->items[li]);
        t.field_items = static_cast<int64_t>(s.host->field_items);
        ctx->times = t;
    }
    if (carve_ms)
        TH_CUDA(cudaEventElapsedTime(carve_ms, ctx->tune_ev[0], ctx->tune_ev[1]));
}

// Runs request a on slot s.  With the autotuner on, the first request of a
// signature runs with both carve kernels (the results are identical) and the
// faster choice is kept for later requests of that signature.
void run_hull(th_context* ctx, HullSlot& s, const th_hull_args* a, cudaStream_t st, StageEvents* ev)
{
    validate(a);
    if (ctx->carve_mode == 1)
        return run_hull_once(ctx, s, a, st, ev, views_everywhere(), nullptr);
    if (ctx->carve_mode == 2)
        return run_hull_once(ctx, s, a, st, ev, items_from_level4(), nullptr);
    const TuneKey key = tune_key(a);
    auto it = ctx->carve_tuned.find(key);
    if (it != ctx->carve_tuned.end())
        return run_hull_once(ctx, s, a, st, ev, it->second, nullptr);
    if (a->level <= 4)
    {
        ctx->carve_tuned[key] = views_everywhere(); // both choices coincide
        return run_hull_once(ctx, s, a, st, ev, views_everywhere(), nullptr);
    }
    for (auto& e : ctx->tune_ev)
        if (!e)
            TH_CUDA(cudaEventCreate(&e));
    float t_views = 0.f, t_items = 0.f;
    run_hull_once(ctx, s, a, st, nullptr, views_everywhere(), &t_views);
    run_hull_once(ctx, s, a, st, ev, items_from_level4(), &t_items);
    ctx->carve_tuned[key] = (t_items < t_views) ? items_from_level4() : views_everywhere();
}

// Batched form: every request's SAT, then one persistent carve over all
// octrees, one launch marking all leaves' corners, then the per-request
// stages spread over a few streams; one device->host read at the end.
void run_batch(th_context* ctx, const th_hull_args* args, int32_t n, cudaStream_t st, th_hull_info* infos)
{
    for (int32_t r = 0; r < n; ++r)
        validate(&args[r]);
    if (n == 0)
        return;
    BatchState& bs = ctx->bstate;
    if (static_cast<int32_t>(ctx->batch.size()) < n)
        ctx->batch.resize(n);
    const int nstreams = std::min<int32_t>(n, 8);
    while (static_cast<int>(bs.streams.size()) < nstreams)
    {
        cudaStream_t s = nullptr;
        cudaEvent_t e = nullptr;
        TH_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        TH_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        bs.streams.push_back(s);
        bs.joins.push_back(e);
    }
    if (!bs.fork)
        TH_CUDA(cudaEventCreateWithFlags(&bs.fork, cudaEventDisableTiming));
    if (bs.host_reqs_cap < n)
    {
        if (bs.host_reqs)
            TH_CUDA(cudaFreeHost(bs.host_reqs));
        alloc_mapped(&bs.host_reqs, &bs.host_reqs_d, n);
        bs.host_reqs_cap = n;
    }
    if (!bs.host_ctr)
        alloc_mapped(&bs.host_ctr, &bs.host_ctr_d);
    int max_level = 0;
    int64_t want_nodes = 0;
    for (int32_t r = 0; r < n; ++r)
    {
        max_level = std::max(max_level, args[r].level);
        want_nodes += std::min<int64_t>(max_nodes(args[r].level), int64_t{ 1 } << 24);
    }
    if (bs.node_cap == 0)
        bs.node_cap = std::min<int64_t>(want_nodes, int64_t{ 1 } << 26);
    bs.node_cap = std::max<int64_t>(bs.node_cap, n);

    for (int32_t r = 0; r < n; ++r)
    {
        HullSlot& s = ctx->batch[r];
        if (s.dirty)
        {
            TH_CUDA(cudaStreamWaitEvent(st, s.done, 0));
            launch_cleanup(s.plan, st);
            s.dirty = false;
        }
        s.has_result = false;
    }
    for (int attempt = 0; attempt < 8; ++attempt)
    {
        bs.reqs.ensure(sizeof(BatchReq) * n);
        bs.nodes.ensure(sizeof(int64_t) * bs.node_cap);
        bs.node_skip.ensure(sizeof(uint32_t) * bs.node_cap);
        bs.node_out.ensure(sizeof(uint32_t) * bs.node_cap);
        // view-skip masks for up to a quarter of the pool's cells in one level
        const int64_t skip_cap = std::max<int64_t>(bs.node_cap / 4, 1);
        bs.child_masks.ensure(static_cast<size_t>(bs.node_cap));
        bs.child_skip.ensure(sizeof(uint32_t) * 8 * skip_cap);
        bs.child_out.ensure(sizeof(uint32_t) * 8 * skip_cap);
        bs.block_sums.ensure(sizeof(unsigned long long) * 8 * sm_count());
        bs.ctr.ensure(sizeof(BatchCounters));
        for (int32_t r = 0; r < n; ++r)
        {
            const th_hull_args* a = &args[r];
            HullSlot& s = ctx->batch[r];
            prepare(s, a, st, ctx->field_ones, ctx->field_masks, true);
            launch_zero(s.plan.ctr, sizeof(DevCounters), st);
            const HullPlan& p = s.plan;
            BatchReq& q = bs.host_reqs[r];
            q = BatchReq{};
            q.tf = p.tf;
            q.sat = p.sat;
            q.H = p.H;
            q.W = p.W;
            q.B = static_cast<int32_t>(p.B);
            q.level = p.level;
            q.partial = p.partial ? 1 : 0;
            q.opengl = p.opengl ? 1 : 0;
            q.skip_ok = p.skip_ok ? 1 : 0;
            // empty images or no views: the octree stops at the root (see run_hull_once)
            q.no_carve = (p.B > 0 && p.H > 0 && p.W > 0) ? 0 : 1;
            q.nonbinary = p.nonbinary;
            q.corner[0] = p.corner[0];
            q.corner[1] = p.corner[1];
            q.corner[2] = p.corner[2];
            q.length = p.length;
            q.bitmap = p.bitmap;
            q.rowbits = p.rowbits;
            q.R = p.R;
            q.WR = p.WR;
            q.cell_masks = p.cell_masks;
        }
        if (attempt == 0)
        {
            // the requests' integral images side by side on the streams (each
            // walks its columns and rows sequentially and leaves the GPU idle)
            TH_CUDA(cudaEventRecord(bs.fork, st));
            for (int i = 0; i < nstreams; ++i)
                TH_CUDA(cudaStreamWaitEvent(bs.streams[i], bs.fork, 0));
            for (int32_t r = 0; r < n; ++r)
            {
                const th_hull_args* a = &args[r];
                HullSlot& s = ctx->batch[r];
                cudaStream_t sr = bs.streams[r % nstreams];
                launch_convert_transforms(a->transforms, a->transforms_dtype, a->batch, s.tf.as<float>(), sr);
                launch_zero(s.flags.p, sizeof(unsigned int), sr);
                launch_integral_image(a->masks, a->masks_dtype, a->batch, a->height, a->width, s.sat.as<float>(), sr,
                                      s.flags.as<unsigned int>(),
                                      ctx->sat_single_pass ? SatScratch{ s.sat_scratch.p } : SatScratch{});
            }
            for (int i = 0; i < nstreams; ++i)
            {
                TH_CUDA(cudaEventRecord(bs.joins[i], bs.streams[i]));
                TH_CUDA(cudaStreamWaitEvent(st, bs.joins[i], 0));
            }
        }
        small_copy(bs.reqs.p, bs.host_reqs_d, sizeof(BatchReq) * n, st);
        BatchPlan bp{};
        bp.reqs = bs.reqs.as<BatchReq>();
        bp.nreq = n;
        bp.max_level = max_level;
        bp.nodes = bs.nodes.as<int64_t>();
        bp.node_skip = bs.node_skip.as<uint32_t>();
        bp.node_out = bs.node_out.as<uint32_t>();
        bp.node_cap = bs.node_cap;
        bp.ctr = bs.ctr.as<BatchCounters>();
        bp.child_masks = bs.child_masks.as<uint8_t>();
        bp.child_skip = bs.child_skip.as<uint32_t>();
        bp.child_out = bs.child_out.as<uint32_t>();
        bp.skip_cap = skip_cap;
        bp.block_sums = bs.block_sums.as<unsigned long long>();
        bp.leaf_levels = 0;
        bp.mask_levels = 0;
        for (int32_t r = 0; r < n; ++r)
        {
            const BatchReq& q = bs.host_reqs[r];
            bp.leaf_levels |= 1u << q.level;
            if (q.cell_masks && q.level >= 1)
                bp.mask_levels |= 1u << (q.level - 1);
        }
        bp.variant = -1;
        for (int32_t r = 0; r < n; ++r)
        {
            const BatchReq& q = bs.host_reqs[r];
            const int32_t v = (q.partial << 1) | q.opengl;
            bp.variant = (r == 0 || bp.variant == v) ? v : -2;
        }
        if (bp.variant < 0)
            bp.variant = -1;
        launch_batch_init(bp, st);
        launch_batch_carve(bp, st);
        launch_batch_mark(bp, st);
        launch_batch_cell_masks(bp, true, st);
        // per-request stages, spread over the streams
        TH_CUDA(cudaEventRecord(bs.fork, st));
        for (int i = 0; i < nstreams; ++i)
            TH_CUDA(cudaStreamWaitEvent(bs.streams[i], bs.fork, 0));
        for (int32_t r = 0; r < n; ++r)
        {
            const HullPlan& p = ctx->batch[r].plan;
            cudaStream_t sr = bs.streams[r % nstreams];
            launch_rank_corners(p, sr);
            launch_field(p, sr);
            launch_marching_cubes(p, sr);
        }
        for (int i = 0; i < nstreams; ++i)
        {
            TH_CUDA(cudaEventRecord(bs.joins[i], bs.streams[i]));
            TH_CUDA(cudaStreamWaitEvent(st, bs.joins[i], 0));
        }
        launch_batch_cell_masks(bp, false, st);
        small_copy(bs.host_ctr_d, bp.ctr, sizeof(BatchCounters), st);
        for (int32_t r = 0; r < n; ++r)
            small_copy(ctx->batch[r].host_d, ctx->batch[r].plan.ctr, sizeof(DevCounters), st);
        TH_CUDA(cudaStreamSynchronize(st));
        bool retry = false;
        if (bs.host_ctr->overflow)
        {
            bs.node_cap *= 4;
            retry = true;
        }
        for (int32_t r = 0; r < n; ++r)
        {
            HullSlot& s = ctx->batch[r];
            s.dirty = true;
            if (s.host->overflow & kOverflowCorners)
            {
                s.corner_cap *= 4;
                retry = true;
            }
        }
        if (!retry)
            break;
        for (int32_t r = 0; r < n; ++r)
        {
            launch_cleanup(ctx->batch[r].plan, st);
            ctx->batch[r].dirty = false;
        }
        if (attempt == 7)
            throw ArgError{ TH_ERR_OUT_OF_MEMORY, "batch pools could not be grown enough" };
    }
    for (int32_t r = 0; r < n; ++r)
    {
        HullSlot& s = ctx->batch[r];
        const DevCounters& c = *s.host;
        th_hull_info info{};
        info.num_corners = c.corners;
        info.num_levels = 0; // per-level candidates are not kept by the batched form
        if (c.soup > 0)
        {
            info.num_verts = s.plan.unique ? c.verts : c.soup;
            info.num_faces = c.soup / 3;
        }
        s.info = info;
        s.has_result = true;
        infos[r] = info;
    }
}

// With routing on, a request whose octree alone fills the GPU (level >= 8
// and at least 16 M mask pixels) runs through the per-request pipeline (graph
// replay, autotuned carve kernels) and the others share the persistent carve.
// Off by default: on a batch of four such requests routing gained 2 %, on a
// mixed batch it lost 16 % (the routed requests no longer overlap the
// others).  Results are identical either way.
bool fills_gpu(const th_hull_args& a)
{
    return a.level >= 8 && a.batch * a.height * a.width >= (int64_t{ 1 } << 24);
}

void run_batch_routed(th_context* ctx, const th_hull_args* args, int32_t n, cudaStream_t st, th_hull_info* infos)
{
    for (int32_t r = 0; r < n; ++r)
        validate(&args[r]);
    std::vector<int32_t> shared, solo;
    for (int32_t r = 0; r < n; ++r)
        (ctx->batch_route && fills_gpu(args[r]) ? solo : shared).push_back(r);
    if (static_cast<int32_t>(ctx->batch.size()) < n)
        ctx->batch.resize(n);
    if (!shared.empty())
    {
        std::vector<th_hull_args> sub(shared.size());
        std::vector<th_hull_info> sub_infos(shared.size());
        for (size_t j = 0; j < shared.size(); ++j)
            sub[j] = args[shared[j]];
        run_batch(ctx, sub.data(), static_cast<int32_t>(sub.size()), st, sub_infos.data());
        // results of shared[j] sit in slot j <= shared[j]: move them into place,
        // last first, so no placed result is moved again
        for (size_t j = shared.size(); j-- > 0;)
        {
            std::swap(ctx->batch[j], ctx->batch[shared[j]]);
            infos[shared[j]] = sub_infos[j];
        }
    }
    for (int32_t r : solo)
    {
        run_hull(ctx, ctx->batch[r], &args[r], st, nullptr);
        infos[r] = ctx->batch[r].info;
    }
}

th_status fail(th_context* ctx, th_status st, const std::string& msg)
{
    if (ctx)
        ctx->error = msg;
    return st;
}

template <class F>
th_status guarded(th_context* ctx, F&& f)
{
    if (!ctx)
        return TH_ERR_INVALID_ARGUMENT;
    ctx->error.clear();
    try
    {
        TH_CUDA(cudaSetDevice(ctx->device));
        f();
        return TH_OK;
    }
    catch (const ArgError& e)
    {
        return fail(ctx, e.status, e.msg);
    }
    catch (const CudaError& e)
    {
        const th_status st = (e.code == cudaErrorMemoryAllocation) ? TH_ERR_OUT_OF_MEMORY : TH_ERR_CUDA;
        return fail(ctx, st, std::string(cudaGetErrorString(e.code)) + " (" + e.where + ")");
    }
    catch (const std::exception& e)
    {
        return fail(ctx, TH_ERR_CUDA, e.what());
    }
}

} // namespace
} // namespace th

namespace th
{
namespace
{

// gaussian_blur_cuda.cu:294-305 and :79-81, in the reference's order.
void check_blur_args(int32_t images_dtype, int32_t kernel_size, float sigma, int32_t out_dtype)
{
    if (kernel_size <= 0)
        throw ArgError{ TH_ERR_INVALID_ARGUMENT,
                        "Check failed: kernel_size > 0 (" + std::to_string(kernel_size) + " vs. 0)" };
    if (kernel_size % 2 != 1)
        throw ArgError{ TH_ERR_INVALID_ARGUMENT,
                        "Check failed: kernel_size % 2 == 1 (" + std::to_string(kernel_size % 2) + " vs. 1)" };
    if (!(sigma > 0.f))
        throw ArgError{ TH_ERR_INVALID_ARGUMENT, "Check failed: sigma > 0.f" };
    if (!(out_dtype == TH_FLOAT16 || out_dtype == TH_FLOAT32 || out_dtype == TH_FLOAT64))
    {
        if (out_dtype == TH_BFLOAT16)
            throw ArgError{ TH_ERR_UNSUPPORTED_DTYPE, "\"tile_convolution_kernel\" not implemented for 'BFloat16'" };
        throw ArgError{ TH_ERR_INVALID_ARGUMENT, "Check failed: torch::isFloatingType(dtype_result) == true" };
    }
    if (!is_image_dtype(images_dtype))
        throw ArgError{ TH_ERR_UNSUPPORTED_DTYPE,
                        std::string("\"edge_kernel\" not implemented for '") + dtype_name(images_dtype) + "'" };
}

// Element size of a float dtype code.
size_t float_size(int32_t dt)
{
    return dt == TH_FLOAT64 ? 8 : (dt == TH_FLOAT32 ? 4 : 2);
}

std::string float_text(float v)
{
    std::ostringstream os;
    os << v;
    return os.str();
}

// Argument checks of marching_cubes_cuda_{dense,sparse} (:382-385, :758-764,
// :789-795) that reach the C ABI; the tensor-layout checks live in the torch layer.
void run_mc(McSlot& s, const th_mc_args* a, cudaStream_t st)
{
    s.has_result = false;
    if (!a)
        throw ArgError{ TH_ERR_INVALID_ARGUMENT, "args is NULL" };
    if (a->depth < 0 || a->height < 0 || a->width < 0 || a->nnz < 0)
        throw ArgError{ TH_ERR_INVALID_ARGUMENT, "volume sizes must be non-negative" };
    if (!(a->isolevel >= 0.f))
        throw ArgError{ TH_ERR_INVALID_ARGUMENT, "Check failed: isolevel >= 0 (" + float_text(a->isolevel) + " vs. 0)" };
    const char* kernel = a->sparse ? "classify_voxels_sparse" : "classify_voxels_dense";
    if (!(a->dtype == TH_FLOAT16 || a->dtype == TH_FLOAT32 || a->dtype == TH_FLOAT64))
        throw ArgError{ TH_ERR_UNSUPPORTED_DTYPE,
                        std::string("\"") + kernel + "\" not implemented for '" + dtype_name(a->dtype) + "'" };
    const int64_t D = a->depth, H = a->height, W = a->width;
    McPlan p{};
    p.dtype = a->dtype;
    p.sparse = a->sparse != 0;
    p.unique = a->unique_verts != 0;
    p.local = a->return_local_coords != 0;
    p.D = D;
    p.H = H;
    p.W = W;
    p.iso = a->isolevel;
    // 2.f / static_cast<float>(size - 1) (:515-517), x along W
    p.scale[0] = 2.f / static_cast<float>(W - 1);
    p.scale[1] = 2.f / static_cast<float>(H - 1);
    p.scale[2] = 2.f / static_cast<float>(D - 1);
    if (p.sparse)
    {
        if (a->nnz >= (int64_t{ 1 } << 31))
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "sparse volumes hold fewer than 2^31 values" };
        if (a->nnz > 0 && (!a->indices || !a->values))
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "indices or values pointer is NULL" };
        p.indices = a->indices;
        p.values = a->values;
        p.nnz = a->nnz;
    }
    else
    {
        // the dense driver sizes its cell arrays (D-1)(H-1)(W-1) and reads the
        // last scan entry back (:392-397, :421-423)
        const int64_t cells = (D - 1) * (H - 1) * (W - 1);
        if (D < 1 || H < 1 || W < 1)
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "Trying to create tensor with negative dimension " +
                                                             std::to_string(cells) + ": [" + std::to_string(cells) + "]" };
        if (cells == 0)
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "index -1 is out of bounds for dimension 0 with size 0" };
        if (!a->volume)
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "volume pointer is NULL" };
        p.volume = a->volume;
        p.points = D * H * W;
        p.wide = p.points >= (int64_t{ 1 } << 32);
        if (!p.wide)
        {
            p.div_w = make_fastdiv(static_cast<uint32_t>(W));
            p.div_h = make_fastdiv(static_cast<uint32_t>(H));
        }
        p.ngroups = (p.points + 31) / 32;
    }

    if (!s.host)
        alloc_mapped(&s.host, &s.host_d);
    s.ctr.ensure(sizeof(McCounters));
    p.ctr = s.ctr.as<McCounters>();
    if (p.sparse)
    {
        const int64_t n = p.nnz;
        uint64_t cap = 64;
        while (cap < 2 * static_cast<uint64_t>(n))
            cap <<= 1;
        s.keys.ensure(sizeof(unsigned long long) * cap);
        s.slots.ensure(sizeof(int32_t) * cap);
        s.codes.ensure(static_cast<size_t>(n));
        s.tiles_soup.ensure(sizeof(unsigned long long) * mc_scan_tiles(n));
        p.keys = s.keys.as<unsigned long long>();
        p.slots = s.slots.as<int32_t>();
        p.hmask = cap - 1;
        p.codes = s.codes.as<uint8_t>();
        p.tiles_soup = s.tiles_soup.as<unsigned long long>();
        if (p.unique)
        {
            s.used.ensure(sizeof(uint32_t) * n);
            s.vbase.ensure(sizeof(unsigned long long) * n);
            s.tiles_verts.ensure(sizeof(unsigned long long) * mc_scan_tiles(n));
            p.used = s.used.as<uint32_t>();
            p.vbase = s.vbase.as<unsigned long long>();
            p.tiles_verts = s.tiles_verts.as<unsigned long long>();
        }
    }
    else
    {
        s.tiles_soup.ensure(sizeof(unsigned long long) * mc_scan_tiles(p.points));
        s.codes.ensure(static_cast<size_t>(p.points));
        s.tiles_scan.ensure(sizeof(unsigned long long) * mc_scan_tiles(mc_scan_tiles(p.points)));
        p.tiles_soup = s.tiles_soup.as<unsigned long long>();
        p.tiles_scan = s.tiles_scan.as<unsigned long long>();
        p.codes = s.codes.as<uint8_t>();
        if (p.unique)
        {
            s.groups.ensure(sizeof(McGroup) * p.ngroups);
            s.tiles_verts.ensure(sizeof(unsigned long long) * mc_scan_tiles(p.ngroups));
            p.groups = s.groups.as<McGroup>();
            p.tiles_verts = s.tiles_verts.as<unsigned long long>();
        }
    }

    launch_mc_count(p, st);
    small_copy(s.host_d, p.ctr, sizeof(McCounters), st);
    TH_CUDA(cudaStreamSynchronize(st));
    const McCounters& c = *s.host;
    if (c.flags & kMcBadIndex)
        throw ArgError{ TH_ERR_INVALID_ARGUMENT, "sparse volume indices lie outside the volume" };
    if (c.flags & kMcUnsorted)
        throw ArgError{ TH_ERR_INVALID_ARGUMENT,
                        "sparse volume indices must be coalesced (strictly ascending in (z, y, x))" };
    if (!p.sparse)
    {
        // packed (soup << 32 | active) tile sums: both totals below 2^32
        if (c.active >= (1ull << 28))
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "marching cubes: more than 2^28 active cells" };
        p.nactive = static_cast<int64_t>(c.active);
        s.active.ensure(sizeof(int64_t) * std::max<int64_t>(p.nactive, 1));
        s.active_soup.ensure(sizeof(unsigned long long) * std::max<int64_t>(p.nactive, 1));
        p.active = s.active.as<int64_t>();
        p.active_soup = s.active_soup.as<unsigned long long>();
    }
    s.plan = p;
    s.info.num_faces = static_cast<int64_t>(c.soup / 3);
    s.info.num_verts = static_cast<int64_t>(p.unique ? c.verts : c.soup);
    s.has_result = true;
}

} // namespace
} // namespace th

using namespace th;

extern "C" {

th_status th_context_create(int32_t device, th_context** out)
{
    if (!out)
        return TH_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0)
        return TH_ERR_NO_DEVICE;
    if (device < 0 || device >= n)
        return TH_ERR_INVALID_ARGUMENT;
    auto* ctx = new th_context;
    ctx->device = device;
    *out = ctx;
    return TH_OK;
}

void th_context_destroy(th_context* ctx)
{
    if (!ctx)
        return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(ctx->device);
    cudaDeviceSynchronize();
    ctx->hull.release();
    for (auto& s : ctx->batch)
        s.release();
    ctx->blur_scratch.release();
    ctx->blurred.release();
    ctx->sat_aux.release();
    if (ctx->sat_aux_done)
        cudaEventDestroy(ctx->sat_aux_done);
    ctx->mc.release();
    ctx->bstate.release();
    ctx->events.destroy();
    for (auto& e : ctx->tune_ev)
        if (e)
            cudaEventDestroy(e);
    cudaSetDevice(prev);
    delete ctx;
}

const char* th_context_error(const th_context* ctx)
{
    return ctx ? ctx->error.c_str() : "";
}

const char* th_status_string(th_status status)
{
    switch (status)
    {
    case TH_OK:
        return "ok";
    case TH_ERR_INVALID_ARGUMENT:
        return "invalid argument";
    case TH_ERR_UNSUPPORTED_DTYPE:
        return "unsupported dtype";
    case TH_ERR_CUDA:
        return "CUDA error";
    case TH_ERR_OUT_OF_MEMORY:
        return "out of memory";
    case TH_ERR_STATE:
        return "invalid call order";
    case TH_ERR_NO_DEVICE:
        return "no CUDA device";
    }
    return "unknown status";
}

int64_t th_context_device_bytes(const th_context* ctx)
{
    return ctx ? pool_bytes(ctx) : 0;
}

th_status th_context_set_option(th_context* ctx, int32_t option, int64_t value)
{
    return guarded(ctx, [&] {
        if (option == TH_OPTION_CARVE_KERNEL && value >= 0 && value <= 2)
            ctx->carve_mode = static_cast<int>(value);
        else if (option == TH_OPTION_GRAPHS && (value == 0 || value == 1))
            ctx->graphs = value != 0;
        else if (option == TH_OPTION_BATCH_ROUTE && (value == 0 || value == 1))
            ctx->batch_route = value != 0;
        else if (option == TH_OPTION_FIELD_ONES && (value == 0 || value == 1))
            ctx->field_ones = value != 0;
        else if (option == TH_OPTION_FIELD_MASKS && (value == 0 || value == 1))
            ctx->field_masks = value != 0;
        else if (option == TH_OPTION_SAT_SINGLE_PASS && (value == 0 || value == 1))
            ctx->sat_single_pass = value != 0;
        else
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "unknown option or value" };
    });
}

th_status th_context_set_profiling(th_context* ctx, int32_t enable)
{
    return guarded(ctx, [&] {
        if (enable)
            ctx->events.create();
        ctx->profiling = enable != 0;
    });
}

th_status th_context_stage_times(const th_context* ctx, th_stage_times* out)
{
    if (!ctx || !out)
        return TH_ERR_INVALID_ARGUMENT;
    *out = ctx->times;
    return TH_OK;
}

int64_t th_launch_count(void)
{
    return g_launches.load(std::memory_order_relaxed);
}

namespace th
{
namespace
{

// 16-byte words, then the tail bytes.  Reads of host memory are latency
// bound: each thread keeps kCopyUnroll independent 16-byte loads in flight.
constexpr int kCopyUnroll = 8;

__global__ void __launch_bounds__(256) sm_copy_kernel(const unsigned char* __restrict__ src,
                                                      unsigned char* __restrict__ dst,
                                                      int64_t n,
                                                      int vec)
{
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    const int64_t t0 = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t done = 0;
    if (vec)
    {
        const int64_t nv = n / 16;
        const uint4* s4 = reinterpret_cast<const uint4*>(src);
        uint4* d4 = reinterpret_cast<uint4*>(dst);
        int64_t i = t0;
        for (; i + (kCopyUnroll - 1) * stride < nv; i += kCopyUnroll * stride)
        {
            uint4 r[kCopyUnroll];
#pragma unroll
            for (int k = 0; k < kCopyUnroll; ++k)
                r[k] = s4[i + k * stride];
#pragma unroll
            for (int k = 0; k < kCopyUnroll; ++k)
                d4[i + k * stride] = r[k];
        }
        for (; i < nv; i += stride)
            d4[i] = s4[i];
        done = nv * 16;
    }
    for (int64_t i = done + t0; i < n; i += stride)
        dst[i] = src[i];
}

// The device address of a copy operand for a kernel on the current device:
// its own device memory and managed memory as they are, pinned host memory
// through its mapping (host = true); nullptr for another device's memory and
// for host memory the device cannot address.
const void* device_address(const void* p, bool& host)
{
    host = false;
    cudaPointerAttributes a{};
    int current = -1;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess || cudaGetDevice(&current) != cudaSuccess)
    {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeManaged)
        return p;
    if (a.type == cudaMemoryTypeDevice)
        return a.device == current ? p : nullptr;
    if (a.type == cudaMemoryTypeHost)
    {
        host = true;
        return a.devicePointer;
    }
    return nullptr;
}

} // namespace
} // namespace th

th_status th_copy(void* dst, const void* src, int64_t bytes, void* stream)
{
    if (bytes < 0 || ((!dst || !src) && bytes > 0))
        return TH_ERR_INVALID_ARGUMENT;
    if (bytes == 0)
        return TH_OK;
    bool src_host = false, dst_host = false;
    const void* s = th::device_address(src, src_host);
    void* d = const_cast<void*>(th::device_address(dst, dst_host));
    if (!s || !d)
        return TH_ERR_INVALID_ARGUMENT;
    const int vec = (reinterpret_cast<uintptr_t>(d) % 16 == 0) && (reinterpret_cast<uintptr_t>(s) % 16 == 0);
    // A copy to or from host memory runs beside the hull kernels on a few
    // blocks: on GB300 eight blocks read host memory at ~130 GB/s and six
    // write it at ~190 GB/s (the link's rate), while a grid over all SMs
    // slows the concurrent hulls.  Device-to-device copies take every SM.
    const int grid = src_host ? 8 : dst_host ? 6 : 2 * th::sm_count();
    th::sm_copy_kernel<<<static_cast<unsigned>(grid), 256, 0, static_cast<cudaStream_t>(stream)>>>(
            static_cast<const unsigned char*>(s), static_cast<unsigned char*>(d), bytes, vec);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError() == cudaSuccess ? TH_OK : TH_ERR_CUDA;
}

th_status th_visual_hull(th_context* ctx, const th_hull_args* args, void* stream, th_hull_info* info)
{
    return guarded(ctx, [&] {
        run_hull(ctx, ctx->hull, args, static_cast<cudaStream_t>(stream), ctx->profiling ? &ctx->events : nullptr);
        if (info)
            *info = ctx->hull.info;
    });
}

th_status th_visual_hull_blurred(th_context* ctx,
                                 const th_hull_args* args,
                                 int32_t kernel_size,
                                 float sigma,
                                 void* stream,
                                 th_hull_info* info)
{
    return guarded(ctx, [&] {
        if (!args)
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "args is NULL" };
        // gaussian_blur(masks, kernel_size, sigma) first: its checks come first
        check_blur_args(args->masks_dtype, kernel_size, sigma, args->masks_dtype);
        validate(args);
        auto st = static_cast<cudaStream_t>(stream);
        th_hull_args a = *args;
        const int64_t n = args->batch * args->height * args->width;
        if (n > 0)
        {
            ctx->blurred.ensure(float_size(args->masks_dtype) * static_cast<size_t>(n));
            const int64_t bytes = blur_tile_bytes(args->batch, args->height, args->width, kernel_size);
            if (bytes > 0)
                ctx->blur_scratch.ensure(static_cast<size_t>(bytes));
            launch_gaussian_blur(args->masks, args->masks_dtype, args->batch, args->height, args->width, kernel_size,
                                 sigma, true, ctx->blurred.p, args->masks_dtype, ctx->blur_scratch.as<uint8_t>(), st);
            a.masks = ctx->blurred.p;
        }
        run_hull(ctx, ctx->hull, &a, st, ctx->profiling ? &ctx->events : nullptr);
        if (info)
            *info = ctx->hull.info;
    });
}

th_status th_visual_hull_export(th_context* ctx, float* verts, int64_t* faces, void* stream)
{
    return guarded(ctx, [&] {
        HullSlot& s = ctx->hull;
        if (!s.has_result)
            throw ArgError{ TH_ERR_STATE, "th_visual_hull_export called without a successful th_visual_hull" };
        auto st = static_cast<cudaStream_t>(stream);
        if (s.info.num_faces > 0)
        {
            if (!verts || !faces)
                throw ArgError{ TH_ERR_INVALID_ARGUMENT, "verts or faces pointer is NULL" };
            launch_export(s.plan, verts, faces, st);
        }
        TH_CUDA(cudaEventRecord(s.done, st));
    });
}

th_status th_visual_hull_export_candidates(th_context* ctx, int32_t level, int64_t* dst, void* stream)
{
    return guarded(ctx, [&] {
        HullSlot& s = ctx->hull;
        if (!s.has_result)
            throw ArgError{ TH_ERR_STATE, "export called without a successful th_visual_hull" };
        if (level < 0 || level >= s.info.num_levels)
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "candidate level out of range" };
        const int64_t n = s.info.level_sizes[level];
        if (n > 0)
        {
            if (!dst)
                throw ArgError{ TH_ERR_INVALID_ARGUMENT, "dst is NULL" };
            // the leaves are written out on demand
            if (level == s.plan.level)
                launch_emit_leaves(s.plan, static_cast<cudaStream_t>(stream));
            TH_CUDA(cudaMemcpyAsync(dst, s.plan.nodes + s.host->level_off[level], sizeof(int64_t) * n,
                                    cudaMemcpyDeviceToDevice, static_cast<cudaStream_t>(stream)));
        }
        TH_CUDA(cudaEventRecord(s.done, static_cast<cudaStream_t>(stream)));
    });
}

th_status th_visual_hull_export_field(th_context* ctx, int64_t* indices, float* values, void* stream)
{
    return guarded(ctx, [&] {
        HullSlot& s = ctx->hull;
        if (!s.has_result)
            throw ArgError{ TH_ERR_STATE, "export called without a successful th_visual_hull" };
        const int64_t n = s.info.num_corners;
        auto st = static_cast<cudaStream_t>(stream);
        if (n > 0)
        {
            if (!indices || !values)
                throw ArgError{ TH_ERR_INVALID_ARGUMENT, "indices or values pointer is NULL" };
            launch_export_field(s.plan, n, indices, values, st);
        }
        TH_CUDA(cudaEventRecord(s.done, st));
    });
}

th_status th_gaussian_blur(th_context* ctx,
                           const void* images,
                           int32_t images_dtype,
                           int64_t batch,
                           int64_t height,
                           int64_t width,
                           int32_t kernel_size,
                           float sigma,
                           int32_t sparse,
                           void* out,
                           int32_t out_dtype,
                           void* stream)
{
    return guarded(ctx, [&] {
        check_blur_args(images_dtype, kernel_size, sigma, out_dtype);
        if (batch < 0 || height < 0 || width < 0)
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "image sizes must be non-negative" };
        const int64_t n = batch * height * width;
        if (n == 0)
            return;
        if (!images || !out)
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "images or out pointer is NULL" };
        const int64_t bytes = blur_tile_bytes(batch, height, width, kernel_size);
        if (bytes > 0)
            ctx->blur_scratch.ensure(static_cast<size_t>(bytes));
        launch_gaussian_blur(images, images_dtype, batch, height, width, kernel_size, sigma, sparse != 0, out, out_dtype,
                             ctx->blur_scratch.as<uint8_t>(), static_cast<cudaStream_t>(stream));
    });
}

th_status th_integral_image(th_context* ctx,
                            const void* masks,
                            int32_t masks_dtype,
                            int64_t batch,
                            int64_t height,
                            int64_t width,
                            float* out,
                            void* stream)
{
    return guarded(ctx, [&] {
        if (!is_image_dtype(masks_dtype))
            throw ArgError{ TH_ERR_UNSUPPORTED_DTYPE,
                            std::string("integral image not implemented for '") + dtype_name(masks_dtype) + "'" };
        if (batch < 0 || height < 0 || width < 0)
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "mask sizes must be non-negative" };
        if (batch * height * width == 0)
            return;
        if (!masks || !out)
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "masks or out pointer is NULL" };
        const cudaStream_t st = static_cast<cudaStream_t>(stream);
        const int64_t sb = ctx->sat_single_pass ? sat_scratch_bytes(batch, height, width, masks_dtype) : 0;
        unsigned int* flag = nullptr;
        SatScratch sc{};
        if (sb > 0)
        {
            constexpr int64_t kFlagBytes = 256;
            // calls on different streams share sat_aux: each waits for the previous one
            if (!ctx->sat_aux_done)
                TH_CUDA(cudaEventCreateWithFlags(&ctx->sat_aux_done, cudaEventDisableTiming));
            else
                TH_CUDA(cudaStreamWaitEvent(st, ctx->sat_aux_done, 0));
            ctx->sat_aux.ensure(static_cast<size_t>(kFlagBytes + sb));
            flag = ctx->sat_aux.as<unsigned int>();
            launch_zero(flag, sizeof(unsigned int), st);
            sc = SatScratch{ static_cast<unsigned char*>(ctx->sat_aux.p) + kFlagBytes };
        }
        launch_integral_image(masks, masks_dtype, batch, height, width, out, st, flag, sc);
        if (sb > 0)
            TH_CUDA(cudaEventRecord(ctx->sat_aux_done, st));
    });
}

th_status th_marching_cubes(th_context* ctx, const th_mc_args* args, void* stream, th_mc_info* info)
{
    return guarded(ctx, [&] {
        run_mc(ctx->mc, args, static_cast<cudaStream_t>(stream));
        if (info)
            *info = ctx->mc.info;
    });
}

th_status th_marching_cubes_export(th_context* ctx, float* verts, int64_t* faces, void* stream)
{
    return guarded(ctx, [&] {
        McSlot& s = ctx->mc;
        if (!s.has_result)
            throw ArgError{ TH_ERR_STATE, "th_marching_cubes_export called without a successful th_marching_cubes" };
        if (s.info.num_faces > 0)
        {
            if (!verts || !faces)
                throw ArgError{ TH_ERR_INVALID_ARGUMENT, "verts or faces pointer is NULL" };
            launch_mc_emit(s.plan, verts, faces, static_cast<cudaStream_t>(stream));
        }
    });
}

th_status th_candidate_wireframe(th_context* ctx,
                                 const int64_t* candidates,
                                 int64_t n,
                                 int32_t level_index,
                                 const float cube_corner_bfl[3],
                                 float cube_length,
                                 float* verts,
                                 int64_t* edges,
                                 void* stream)
{
    return guarded(ctx, [&] {
        if (n < 0 || level_index < 0 || level_index > 20 || !cube_corner_bfl)
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "invalid wireframe arguments" };
        if (n > 0 && (!candidates || !verts || !edges))
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "candidates, verts or edges pointer is NULL" };
        launch_wireframe(candidates, n, level_index, cube_corner_bfl, cube_length, verts, edges,
                         static_cast<cudaStream_t>(stream));
    });
}

th_status th_store_curve_network(th_context* ctx,
                                 const char* filename,
                                 const float* verts,
                                 int64_t nv,
                                 const int64_t* edges,
                                 int64_t ne,
                                 int32_t verbose)
{
    // host only: no device is needed, ctx (may be NULL) only receives the message
    if (ctx)
        ctx->error.clear();
    if (!filename || nv < 0 || ne < 0 || (nv > 0 && !verts) || (ne > 0 && !edges))
        return fail(ctx, TH_ERR_INVALID_ARGUMENT, "invalid curve network arguments");
    const std::string name(filename);
    try
    {
        if (!store_curve_network(name, verts, nv, edges, ne, verbose != 0))
            return fail(ctx, TH_ERR_INVALID_ARGUMENT,
                        "No implementation for file extension \"" + file_extension(name) + "\".");
    }
    catch (const std::exception& e)
    {
        return fail(ctx, TH_ERR_INVALID_ARGUMENT, e.what());
    }
    return TH_OK;
}

th_status th_visual_hull_batch(th_context* ctx, const th_hull_args* args, int32_t n, void* stream, th_hull_info* infos)
{
    return guarded(ctx, [&] {
        if (n < 0 || (n > 0 && (!args || !infos)))
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "invalid batch arguments" };
        run_batch_routed(ctx, args, n, static_cast<cudaStream_t>(stream), infos);
    });
}

th_status th_visual_hull_batch_export(th_context* ctx, int32_t index, float* verts, int64_t* faces, void* stream)
{
    return guarded(ctx, [&] {
        if (index < 0 || index >= static_cast<int32_t>(ctx->batch.size()) || !ctx->batch[index].has_result)
            throw ArgError{ TH_ERR_STATE, "no batched result at this index" };
        HullSlot& s = ctx->batch[index];
        auto st = static_cast<cudaStream_t>(stream);
        if (s.info.num_faces > 0)
        {
            if (!verts || !faces)
                throw ArgError{ TH_ERR_INVALID_ARGUMENT, "verts or faces pointer is NULL" };
            launch_export(s.plan, verts, faces, st);
        }
        TH_CUDA(cudaEventRecord(s.done, st));
    });
}

th_status th_visual_hull_batch_export_all(th_context* ctx, int32_t n, float* const* verts, int64_t* const* faces,
                                          void* stream)
{
    return guarded(ctx, [&] {
        if (n < 0 || n > static_cast<int32_t>(ctx->batch.size()))
            throw ArgError{ TH_ERR_STATE, "no batched result for that many requests" };
        if (n > 0 && (!verts || !faces))
            throw ArgError{ TH_ERR_INVALID_ARGUMENT, "verts or faces array is NULL" };
        for (int32_t i = 0; i < n; ++i)
        {
            if (!ctx->batch[i].has_result)
                throw ArgError{ TH_ERR_STATE, "no batched result at this index" };
            if (ctx->batch[i].info.num_faces > 0 && (!verts[i] || !faces[i]))
                throw ArgError{ TH_ERR_INVALID_ARGUMENT, "verts or faces pointer is NULL" };
        }
        auto st = static_cast<cudaStream_t>(stream);
        BatchState& bs = ctx->bstate;
        const int ns = std::min<int>(n, static_cast<int>(bs.streams.size()));
        if (ns > 1)
        {
            // the exports side by side on the batch's streams, joined back into st
            TH_CUDA(cudaEventRecord(bs.fork, st));
            for (int i = 0; i < ns; ++i)
                TH_CUDA(cudaStreamWaitEvent(bs.streams[i], bs.fork, 0));
        }
        for (int32_t i = 0; i < n; ++i)
        {
            HullSlot& s = ctx->batch[i];
            if (s.info.num_faces > 0)
                launch_export(s.plan, verts[i], faces[i], ns > 1 ? bs.streams[i % ns] : st);
        }
        if (ns > 1)
        {
            for (int i = 0; i < ns; ++i)
            {
                TH_CUDA(cudaEventRecord(bs.joins[i], bs.streams[i]));
                TH_CUDA(cudaStreamWaitEvent(st, bs.joins[i], 0));
            }
        }
        for (int32_t i = 0; i < n; ++i)
            TH_CUDA(cudaEventRecord(ctx->batch[i].done, st));
    });
}

} // extern "C"
