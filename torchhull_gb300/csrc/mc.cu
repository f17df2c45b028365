// Public marching cubes over a dense volume or a coalesced sparse COO volume
// (torchhull marching_cubes: marching_cubes_cuda.cu:376-533 for dense
// volumes, :535-831 for sparse ones).
//
// The reference builds a triangle soup (one vertex per table entry of every
// active cell, cells ascending, table order inside a cell), keys each soup
// vertex by its edge id (ravel(lower end point) << 3 | direction, :99-112,
// direction 1 / 2 / 4 for x / y / z) and sorts the keys with unique_dim; the
// faces are the soup's inverse indices.  The unique vertices therefore come
// in edge-id order: by the ravel index of the lower end point, then by axis.
// Here that order is produced directly: every grid point carries three bits
// (its +x, +y, +z edge holds a vertex), a scan over the points numbers the
// set bits, and a face looks up its vertex as the number of set bits before
// its edge.  The soup order comes from a scan of the per-cell vertex counts,
// so no sort runs.
//
// Which edges hold vertices: every cell's triangulation uses exactly the cell
// edges whose end points lie on different sides of the isolevel (a property
// of the table, checked by the tests).  In a dense volume with all sizes >= 2
// every edge belongs to some cell, so the bits follow from the values alone.
// In a sparse volume an edge counts only when a complete cell (all 8 corners
// present) holds it, so each active cell marks its edges on the entries of
// their lower end points.
//
// Axes: x runs along the last volume dimension (W), y along H, z along the
// first (D).  The reference mixes D and W in its index arithmetic; for
// volumes with D == W (all of its tests) that mixing is invisible and the
// results here are identical.

#include <cuda_fp16.h>

#include "mc_tables.h"
#include "th_internal.h"
#include "th_mc.cuh"

namespace th
{
namespace
{

__device__ const uint8_t mc_count[256] = TH_MC_TRI_COUNT_INIT;
__device__ const uint8_t mc_edges[256][15] = TH_MC_TRI_EDGES_INIT;

constexpr unsigned long long kEmptyKey = ~0ull;

// value < isolevel, compared in the value's own type (:166-171, :210-213).
template <int DT>
__device__ __forceinline__ bool below(const void* v, int64_t i, float iso)
{
    if constexpr (DT == TH_FLOAT64)
        return static_cast<const double*>(v)[i] < static_cast<double>(iso);
    else
        return load_f32<DT>(v, i) < iso;
}

// interpolate_vertex (:72-97) on the edge from point (x, y, z) along axis,
// then the optional map to local coordinates: v * 2 / (size - 1) - 1 as two
// rounded torch operations (:524-531).
__device__ __forceinline__ void mc_vertex(const McPlan& p, int64_t x, int64_t y, int64_t z, int axis, float v1, float v2, float* out)
{
    const float eps = 1e-5f;
    const int64_t c1[3] = { x, y, z };
    float q[3];
    // the reference's check order: snap to p1, to p2, then to p1 again
    int snap = 0;
    if (fabsf(__fsub_rn(p.iso, v1)) < eps)
        snap = 1;
    else if (fabsf(__fsub_rn(p.iso, v2)) < eps)
        snap = 2;
    else if (fabsf(__fsub_rn(v1, v2)) < eps)
        snap = 1;
    const float t = snap ? 0.f : __fdiv_rn(__fsub_rn(p.iso, v1), __fsub_rn(v2, v1));
#pragma unroll
    for (int a = 0; a < 3; ++a)
    {
        // exact float conversions by adds below 2^23 (the 64-bit integer
        // conversions run on GB300's FP64 pipe)
        const int64_t i1 = c1[a], i2 = c1[a] + (a == axis ? 1 : 0);
        const float f1 = i1 < 8388608 ? small_i2f(static_cast<int32_t>(i1)) : static_cast<float>(i1);
        const float f2 = i2 < 8388608 ? small_i2f(static_cast<int32_t>(i2)) : static_cast<float>(i2);
        q[a] = snap == 1 ? f1 : (snap == 2 ? f2 : lerp(f1, f2, t));
        out[a] = p.local ? __fsub_rn(__fmul_rn(q[a], p.scale[a]), 1.f) : q[a];
    }
}

// ---------------------------------------------------------------------------
// dense volumes

template <bool WIDE>
__device__ __forceinline__ void decode(const McPlan& p, int64_t q, int64_t& x, int64_t& y, int64_t& z)
{
    if (WIDE)
    {
        const int64_t r = q / p.W;
        x = q - r * p.W;
        z = r / p.H;
        y = r - z * p.H;
    }
    else
    {
        const uint32_t qq = static_cast<uint32_t>(q);
        const uint32_t r = fast_div(p.div_w, qq);
        x = qq - r * p.div_w.d;
        const uint32_t zz = fast_div(p.div_h, r);
        z = zz;
        y = r - zz * p.div_h.d;
    }
}

struct GroupCount
{
    const McGroup* groups;
    __device__ unsigned long long operator()(int64_t i) const
    {
        const McGroup& e = groups[i];
        return static_cast<unsigned long long>(__popc(e.x) + __popc(e.y) + __popc(e.z));
    }
};

struct GroupEmit
{
    McGroup* groups;
    __device__ void operator()(int64_t i, unsigned long long off, unsigned long long) const
    {
        groups[i].base = off;
    }
};

struct SoupTotal
{
    McCounters* ctr;
    __device__ void operator()(unsigned long long t) const
    {
        ctr->soup = t;
    }
};

// (soup << 32) | active cells of a dense volume
struct PackedTotal
{
    McCounters* ctr;
    __device__ void operator()(unsigned long long t) const
    {
        ctr->soup = t >> 32;
        ctr->active = t & 0xffffffffull;
    }
};

struct VertTotal
{
    McCounters* ctr;
    __device__ void operator()(unsigned long long t) const
    {
        ctr->verts = t;
    }
};

// Vertex index of the edge from point q along axis: the set edge bits before it.
__device__ __forceinline__ unsigned long long dense_vertex(const McGroup* groups, int64_t q, int axis)
{
    const McGroup e = groups[q >> 5];
    const int l = static_cast<int>(q & 31);
    const uint32_t lt = (1u << l) - 1u;
    unsigned long long r = e.base + __popc(e.x & lt) + __popc(e.y & lt) + __popc(e.z & lt);
    if (axis >= 1)
        r += (e.x >> l) & 1u;
    if (axis == 2)
        r += (e.y >> l) & 1u;
    return r;
}

// Soup of the active cell with base point q and code (generate_faces_dense
// :242-306): faces into the unique vertex list, or soup vertices with
// faces = arange.  off: the cell's first soup vertex.
template <int DT, bool WIDE>
__device__ __forceinline__ void dense_emit_cell(const McPlan& p, int64_t q, int code, unsigned long long off, int cnt, float* verts, int64_t* faces)
{
    int64_t x, y, z;
    decode<WIDE>(p, q, x, y, z);
    const int64_t WH = p.W * p.H;
    for (int j = 0; j < cnt; ++j)
    {
        const uint32_t e = mc_edges[code][j];
        const int lo = static_cast<int>(e & 7u), axis = static_cast<int>(e >> 3);
        const int64_t q1 = q + (lo & 1) + ((lo >> 1) & 1) * p.W + ((lo >> 2) & 1) * WH;
        const int64_t k = static_cast<int64_t>(off) + j;
        if (p.unique)
        {
            faces[k] = static_cast<int64_t>(dense_vertex(p.groups, q1, axis));
        }
        else
        {
            const int64_t q2 = q1 + (axis == 0 ? 1 : (axis == 1 ? p.W : WH));
            mc_vertex(p, x + (lo & 1), y + ((lo >> 1) & 1), z + ((lo >> 2) & 1), axis, load_f32<DT>(p.volume, q1),
                      load_f32<DT>(p.volume, q2), verts + 3 * k);
            faces[k] = k;
        }
    }
}

// One pass over a dense volume that loads each value once: a block covers
// 32 x 8 columns (x, y) and marches kMarchZ planes in z, exchanging the
// below-isolevel bits of each plane (with a one-point halo in +x and +y)
// through shared memory, double-buffered.  For every point it writes the cell
// code (0 where no cell starts), ORs its three vertex-edge bits into the
// group words (unique vertices), and adds (soup vertices << 32 | active cell)
// to the sum of its 2048-point tile (one atomic per warp and tile).  groups
// and tiles_soup are zero when it starts.
constexpr int kMarchX = 32, kMarchY = 8, kMarchZ = 16;

template <int DT>
__device__ __forceinline__ uint8_t below_at(const McPlan& p, int64_t x, int64_t y, int64_t z)
{
    return (x < p.W && y < p.H && z < p.D) ? (below<DT>(p.volume, x + p.W * (y + p.H * z), p.iso) ? 1 : 0) : 0;
}

template <int DT>
__global__ void __launch_bounds__(kMarchX * kMarchY) mc_dense_march_kernel(McPlan p)
{
    __shared__ uint8_t plane[2][kMarchY + 1][kMarchX + 1];
    const int tx = threadIdx.x, ty = threadIdx.y, lane = tx;
    const int64_t x = static_cast<int64_t>(blockIdx.x) * kMarchX + tx;
    const int64_t y = static_cast<int64_t>(blockIdx.y) * kMarchY + ty;
    const int64_t z0 = static_cast<int64_t>(blockIdx.z) * kMarchZ;
    const int64_t z1 = z0 + kMarchZ < p.D ? z0 + kMarchZ : p.D;
    const bool in = x < p.W && y < p.H;

    // plane z into buffer k: own bit, and the +x / +y halo
    auto fill = [&](int k, int64_t z) {
        plane[k][ty][tx] = below_at<DT>(p, x, y, z);
        if (tx == kMarchX - 1)
            plane[k][ty][kMarchX] = below_at<DT>(p, x + 1, y, z);
        if (ty == kMarchY - 1)
        {
            plane[k][kMarchY][tx] = below_at<DT>(p, x, y + 1, z);
            if (tx == kMarchX - 1)
                plane[k][kMarchY][kMarchX] = below_at<DT>(p, x + 1, y + 1, z);
        }
    };
    fill(0, z0);
    __syncthreads();
    int cur = 0;
    for (int64_t z = z0; z < z1; ++z)
    {
        const int nxt = cur ^ 1;
        if (z + 1 < p.D)
            fill(nxt, z + 1);
        else
        {
            plane[nxt][ty][tx] = 0;
            if (tx == kMarchX - 1)
                plane[nxt][ty][kMarchX] = 0;
            if (ty == kMarchY - 1)
            {
                plane[nxt][kMarchY][tx] = 0;
                if (tx == kMarchX - 1)
                    plane[nxt][kMarchY][kMarchX] = 0;
            }
        }
        __syncthreads();
        const uint32_t b0 = plane[cur][ty][tx], bx = plane[cur][ty][tx + 1];
        const uint32_t by = plane[cur][ty + 1][tx], bxy = plane[cur][ty + 1][tx + 1];
        const uint32_t c0 = plane[nxt][ty][tx], cx = plane[nxt][ty][tx + 1];
        const uint32_t cy = plane[nxt][ty + 1][tx], cxy = plane[nxt][ty + 1][tx + 1];
        const int64_t q = x + p.W * (y + p.H * z);
        // corner i = (i & 1, i >> 1 & 1, i >> 2 & 1)
        const int code = static_cast<int>(b0 | (bx << 1) | (by << 2) | (bxy << 3) | (c0 << 4) | (cx << 5) | (cy << 6) |
                                          (cxy << 7));
        const bool cell = in && x + 1 < p.W && y + 1 < p.H && z + 1 < p.D;
        const unsigned cnt = cell ? mc_count[code] : 0u;
        if (in)
            p.codes[q] = static_cast<uint8_t>(cell ? code : 0);
        // the warp's 32 points are consecutive in ravel order (or end at the row's end)
        const int64_t q0 = __shfl_sync(0xffffffffu, q, 0);
        // per warp: soup vertices (<= 480) << 16 | active cells (<= 32), for
        // the (at most two) 2048-point tiles the warp's points fall into
        const unsigned packed = (cnt << 16) | (cnt ? 1u : 0u);
        const int64_t t0 = q0 >> 11;
        const bool second = in && (q >> 11) != t0;
        const unsigned a0 = __reduce_add_sync(0xffffffffu, second ? 0u : packed);
        const unsigned a1 = __reduce_add_sync(0xffffffffu, second ? packed : 0u);
        if (lane == 0)
        {
            if (a0)
                atomicAdd(&p.tiles_soup[t0], (static_cast<unsigned long long>(a0 >> 16) << 32) | (a0 & 0xffffu));
            if (a1)
                atomicAdd(&p.tiles_soup[t0 + 1], (static_cast<unsigned long long>(a1 >> 16) << 32) | (a1 & 0xffffu));
        }
        if (p.unique)
        {
            const bool ex = in && x + 1 < p.W && bx != b0;
            const bool ey = in && y + 1 < p.H && by != b0;
            const bool ez = in && z + 1 < p.D && c0 != b0;
            const uint32_t X = __ballot_sync(0xffffffffu, ex), Y = __ballot_sync(0xffffffffu, ey),
                           Z = __ballot_sync(0xffffffffu, ez);
            if (lane == 0)
            {
                const int64_t g0 = q0 >> 5;
                const int sh = static_cast<int>(q0 & 31);
                McGroup& G0 = p.groups[g0];
                if (X << sh)
                    atomicOr(&G0.x, X << sh);
                if (Y << sh)
                    atomicOr(&G0.y, Y << sh);
                if (Z << sh)
                    atomicOr(&G0.z, Z << sh);
                if (sh)
                {
                    McGroup& G1 = p.groups[g0 + 1];
                    if (X >> (32 - sh))
                        atomicOr(&G1.x, X >> (32 - sh));
                    if (Y >> (32 - sh))
                        atomicOr(&G1.y, Y >> (32 - sh));
                    if (Z >> (32 - sh))
                        atomicOr(&G1.z, Z >> (32 - sh));
                }
            }
        }
        cur = nxt;
        __syncthreads(); // plane[cur ^ 1] is refilled next
    }
}

// The tile sums of the march into exclusive offsets, in place (a scan reads
// all counts of a thread before it writes any offset).
struct TileCount
{
    const unsigned long long* tiles;
    __device__ unsigned long long operator()(int64_t i) const
    {
        return tiles[i];
    }
};

struct TileEmit
{
    unsigned long long* tiles;
    __device__ void operator()(int64_t i, unsigned long long off, unsigned long long) const
    {
        tiles[i] = off;
    }
};

// Pass 2, over the same tiles with kScanItems consecutive points per thread
// (one 8-byte read of codes, one block scan per tile): every active cell and
// its first soup vertex into the active list, in cell order.
__global__ void __launch_bounds__(kScanThreads) mc_dense_compact_kernel(McPlan p)
{
    static_assert(kScanItems == 8, "one 8-byte read of codes per thread");
    const int64_t ntiles = (p.points + kScanTile - 1) / kScanTile;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x)
    {
        // tiles without an active cell (most of a volume) have equal offsets
        const unsigned long long next =
                tile + 1 < ntiles ? p.tiles_soup[tile + 1] : ((p.ctr->soup << 32) | p.ctr->active);
        if ((next & 0xffffffffull) == (p.tiles_soup[tile] & 0xffffffffull))
            continue;
        const int64_t base = tile * kScanTile + static_cast<int64_t>(threadIdx.x) * kScanItems;
        uint32_t lo = 0, hi = 0;
        if (base + kScanItems <= p.points)
        {
            const uint2 w = *reinterpret_cast<const uint2*>(p.codes + base);
            lo = w.x;
            hi = w.y;
        }
        else
        {
            for (int k = 0; k < kScanItems && base + k < p.points; ++k)
                (k < 4 ? lo : hi) |= static_cast<uint32_t>(p.codes[base + k]) << (8 * (k & 3));
        }
        unsigned long long s = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k)
        {
            const unsigned cnt = mc_count[((k < 4 ? lo : hi) >> (8 * (k & 3))) & 0xffu];
            s += (static_cast<unsigned long long>(cnt) << 32) | (cnt ? 1ull : 0ull);
        }
        unsigned long long tot;
        unsigned long long off = block_exclusive_scan(s, &tot) + p.tiles_soup[tile];
        if (s == 0)
            continue;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k)
        {
            const unsigned cnt = mc_count[((k < 4 ? lo : hi) >> (8 * (k & 3))) & 0xffu];
            if (cnt)
            {
                const unsigned long long a = off & 0xffffffffull;
                p.active[a] = base + k;
                p.active_soup[a] = off >> 32;
                off += (static_cast<unsigned long long>(cnt) << 32) | 1ull;
            }
        }
    }
}

// The soup of every active cell, one thread per cell.
template <int DT, bool WIDE>
__global__ void __launch_bounds__(256) mc_dense_faces_kernel(McPlan p, float* __restrict__ verts, int64_t* __restrict__ faces)
{
    const int64_t n = static_cast<int64_t>(p.ctr->active);
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        const int64_t q = p.active[i];
        const int code = p.codes[q];
        dense_emit_cell<DT, WIDE>(p, q, code, p.active_soup[i], mc_count[code], verts, faces);
    }
}

// The unique vertices, in edge-id order.  Each lane of a warp reads one
// group; the warp then handles its groups with vertex edges one after the
// other, a lane per point (most groups of a volume have none).
template <int DT, bool WIDE>
__global__ void __launch_bounds__(256) mc_dense_verts_kernel(McPlan p, float* __restrict__ verts)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const int64_t WH = p.W * p.H;
    const uint32_t bit = 1u << lane, lt = bit - 1u;
    for (int64_t g0 = warp * 32; g0 < p.ngroups; g0 += nwarps * 32)
    {
        const int64_t gl = g0 + lane;
        const McGroup mine_group = gl < p.ngroups ? p.groups[gl] : McGroup{ 0u, 0u, 0u, 0u, 0ull };
        uint32_t todo = __ballot_sync(0xffffffffu, (mine_group.x | mine_group.y | mine_group.z) != 0u);
        while (todo)
        {
            const int j = __ffs(todo) - 1;
            todo &= todo - 1;
            const uint32_t ex = __shfl_sync(0xffffffffu, mine_group.x, j);
            const uint32_t ey = __shfl_sync(0xffffffffu, mine_group.y, j);
            const uint32_t ez = __shfl_sync(0xffffffffu, mine_group.z, j);
            const unsigned long long base = __shfl_sync(0xffffffffu, mine_group.base, j);
            const uint32_t mine = ((ex & bit) ? 1u : 0u) | ((ey & bit) ? 2u : 0u) | ((ez & bit) ? 4u : 0u);
            if (!mine)
                continue;
            unsigned long long r = base + __popc(ex & lt) + __popc(ey & lt) + __popc(ez & lt);
            const int64_t q = (g0 + j) * 32 + lane;
            int64_t x, y, z;
            decode<WIDE>(p, q, x, y, z);
            const float v1 = load_f32<DT>(p.volume, q);
#pragma unroll
            for (int a = 0; a < 3; ++a)
            {
                if (!((mine >> a) & 1u))
                    continue;
                const int64_t q2 = q + (a == 0 ? 1 : (a == 1 ? p.W : WH));
                mc_vertex(p, x, y, z, a, v1, load_f32<DT>(p.volume, q2), verts + 3 * r);
                ++r;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// sparse volumes: an open-addressing table from ravel id to entry index
// (the reference uses a stdgpu unordered_map, :729-751)

// MurmurHash3's 64-bit finalizer (fmix64).
__device__ __forceinline__ uint64_t mix64(uint64_t k)
{
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

// Entry t's coordinates, or false when it lies outside the volume.
__device__ __forceinline__ bool entry_point(const McPlan& p, int64_t t, int64_t& x, int64_t& y, int64_t& z)
{
    const int64_t b = p.indices[t];
    z = p.indices[p.nnz + t];
    y = p.indices[2 * p.nnz + t];
    x = p.indices[3 * p.nnz + t];
    return b == 0 && 0 <= x && x < p.W && 0 <= y && y < p.H && 0 <= z && z < p.D;
}

__device__ __forceinline__ int32_t mc_find(const McPlan& p, unsigned long long key)
{
    uint64_t slot = mix64(key) & p.hmask;
    for (uint64_t k = 0; k <= p.hmask; ++k)
    {
        const unsigned long long kk = p.keys[slot];
        if (kk == key)
            return p.slots[slot];
        if (kk == kEmptyKey)
            return -1;
        slot = (slot + 1) & p.hmask;
    }
    return -1;
}

// hash_volume (:114-131): every entry's ravel id into the table; flags
// entries outside the volume and indices that are not strictly ascending.
__global__ void __launch_bounds__(256) mc_sparse_insert_kernel(McPlan p)
{
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < p.nnz; t += stride)
    {
        int64_t x, y, z;
        if (!entry_point(p, t, x, y, z))
        {
            atomicOr(&p.ctr->flags, static_cast<unsigned int>(kMcBadIndex));
            continue;
        }
        const unsigned long long key = static_cast<unsigned long long>(x + p.W * (y + p.H * z));
        if (t > 0)
        {
            int64_t px, py, pz;
            if (entry_point(p, t - 1, px, py, pz) &&
                static_cast<unsigned long long>(px + p.W * (py + p.H * pz)) >= key)
                atomicOr(&p.ctr->flags, static_cast<unsigned int>(kMcUnsorted));
        }
        uint64_t slot = mix64(key) & p.hmask;
        for (uint64_t k = 0; k <= p.hmask; ++k)
        {
            const unsigned long long prev = atomicCAS(&p.keys[slot], kEmptyKey, key);
            if (prev == kEmptyKey || prev == key)
            {
                p.slots[slot] = static_cast<int32_t>(t);
                break;
            }
            slot = (slot + 1) & p.hmask;
        }
    }
}

// Entry indices of the 8 corners of the cell with base entry t at (x, y, z)
// (corner i = base + (i & 1, i >> 1 & 1, i >> 2 & 1)); false if one is absent.
__device__ __forceinline__ bool cell_entries(const McPlan& p, int64_t t, int64_t x, int64_t y, int64_t z, int32_t c[8])
{
    if (!(x + 1 < p.W && y + 1 < p.H && z + 1 < p.D))
        return false;
    const unsigned long long key = static_cast<unsigned long long>(x + p.W * (y + p.H * z));
    const unsigned long long WH = static_cast<unsigned long long>(p.W * p.H);
    c[0] = static_cast<int32_t>(t);
#pragma unroll
    for (int i = 1; i < 8; ++i)
    {
        c[i] = mc_find(p, key + (i & 1) + ((i >> 1) & 1) * static_cast<unsigned long long>(p.W) + ((i >> 2) & 1) * WH);
        if (c[i] < 0)
            return false;
    }
    return true;
}

// classify_voxels_sparse (:180-223) plus, with unique vertices, the marking of
// the cell's vertex edges on the entries of their lower end points.
template <int DT>
__global__ void __launch_bounds__(256) mc_sparse_classify_kernel(McPlan p)
{
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < p.nnz; t += stride)
    {
        int64_t x, y, z;
        int32_t c[8];
        int code = 0;
        if (entry_point(p, t, x, y, z) && cell_entries(p, t, x, y, z, c))
        {
#pragma unroll
            for (int i = 0; i < 8; ++i)
                if (below<DT>(p.values, c[i], p.iso))
                    code |= 1 << i;
            if (p.unique && mc_count[code] != 0)
            {
                // corner lo owns the edges along the axes where its bit is 0;
                // an edge is a vertex edge when its two ends differ in the code
#pragma unroll
                for (int lo = 0; lo < 8; ++lo)
                {
                    uint32_t bits = 0;
#pragma unroll
                    for (int a = 0; a < 3; ++a)
                        if (!((lo >> a) & 1) && (((code >> lo) ^ (code >> (lo | (1 << a)))) & 1))
                            bits |= 1u << a;
                    if (bits)
                        atomicOr(&p.used[c[lo]], bits);
                }
            }
        }
        p.codes[t] = static_cast<uint8_t>(code);
    }
}

struct SparseSoupCount
{
    const uint8_t* codes;
    __device__ unsigned long long operator()(int64_t t) const
    {
        return static_cast<unsigned long long>(mc_count[codes[t]]);
    }
};

struct SparseVertCount
{
    const uint32_t* used;
    __device__ unsigned long long operator()(int64_t t) const
    {
        return static_cast<unsigned long long>(__popc(used[t]));
    }
};

struct SparseVertEmit
{
    unsigned long long* vbase;
    __device__ void operator()(int64_t t, unsigned long long off, unsigned long long) const
    {
        vbase[t] = off;
    }
};

// The unique vertices, in edge-id order (entries are in ravel order).
template <int DT>
__global__ void __launch_bounds__(256) mc_sparse_verts_kernel(McPlan p, float* __restrict__ verts)
{
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    const unsigned long long step[3] = { 1ull, static_cast<unsigned long long>(p.W),
                                         static_cast<unsigned long long>(p.W * p.H) };
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < p.nnz; t += stride)
    {
        const uint32_t bits = p.used[t];
        if (!bits)
            continue;
        int64_t x, y, z;
        entry_point(p, t, x, y, z);
        const unsigned long long key = static_cast<unsigned long long>(x + p.W * (y + p.H * z));
        const float v1 = load_f32<DT>(p.values, t);
        unsigned long long r = p.vbase[t];
#pragma unroll
        for (int a = 0; a < 3; ++a)
        {
            if (!((bits >> a) & 1u))
                continue;
            // present: a complete cell holds this edge
            const int32_t t2 = mc_find(p, key + step[a]);
            const float v2 = t2 >= 0 ? load_f32<DT>(p.values, t2) : __int_as_float(0x7fffffff);
            mc_vertex(p, x, y, z, a, v1, v2, verts + 3 * r);
            ++r;
        }
    }
}

// Soup of one active entry (generate_faces_sparse :308-374).
template <int DT>
struct SparseCellEmit
{
    McPlan p;
    float* verts;
    int64_t* faces;
    __device__ void operator()(int64_t t, unsigned long long off, unsigned long long cnt) const
    {
        if (cnt == 0)
            return;
        int64_t x, y, z;
        int32_t c[8];
        entry_point(p, t, x, y, z);
        if (!cell_entries(p, t, x, y, z, c))
            return; // not reached: an entry with a count has all its corners
        const int code = p.codes[t];
        for (int j = 0; j < static_cast<int>(cnt); ++j)
        {
            const uint32_t e = mc_edges[code][j];
            const int lo = static_cast<int>(e & 7u), axis = static_cast<int>(e >> 3);
            const int64_t k = static_cast<int64_t>(off) + j;
            const int32_t c1 = c[lo];
            if (p.unique)
            {
                faces[k] = static_cast<int64_t>(p.vbase[c1] + __popc(p.used[c1] & ((1u << axis) - 1u)));
            }
            else
            {
                const int32_t c2 = c[lo | (1 << axis)];
                mc_vertex(p, x + (lo & 1), y + ((lo >> 1) & 1), z + ((lo >> 2) & 1), axis, load_f32<DT>(p.values, c1),
                          load_f32<DT>(p.values, c2), verts + 3 * k);
                faces[k] = k;
            }
        }
    }
};

// Blocks of the two point passes: up to 8 per SM.
int dense_grid(const McPlan& p)
{
    const int64_t tiles = (p.points + kScanTile - 1) / kScanTile;
    const int64_t cap = 8LL * sm_count();
    return static_cast<int>(tiles < cap ? tiles : cap);
}

template <int DT, bool WIDE>
void dense_count(const McPlan& p, cudaStream_t s)
{
    const int64_t ntiles = (p.points + kScanTile - 1) / kScanTile;
    TH_CUDA(cudaMemsetAsync(p.tiles_soup, 0, sizeof(unsigned long long) * ntiles, s));
    if (p.unique)
        TH_CUDA(cudaMemsetAsync(p.groups, 0, sizeof(McGroup) * p.ngroups, s));
    const dim3 grid(static_cast<unsigned>((p.W + kMarchX - 1) / kMarchX),
                    static_cast<unsigned>((p.H + kMarchY - 1) / kMarchY),
                    static_cast<unsigned>((p.D + kMarchZ - 1) / kMarchZ));
    mc_dense_march_kernel<DT><<<grid, dim3(kMarchX, kMarchY), 0, s>>>(p);
    TH_LAUNCH_CHECK();
    run_scan(TileCount{ p.tiles_soup }, TileEmit{ p.tiles_soup }, PackedTotal{ p.ctr }, Count{ nullptr, ntiles }, ntiles,
             p.tiles_scan, &p.ctr->scan_soup, s);
    if (p.unique)
        run_scan(GroupCount{ p.groups }, GroupEmit{ p.groups }, VertTotal{ p.ctr }, Count{ nullptr, p.ngroups },
                 p.ngroups, p.tiles_verts, &p.ctr->scan_verts, s);
}

template <int DT, bool WIDE>
void dense_emit(const McPlan& p, float* verts, int64_t* faces, cudaStream_t s)
{
    if (p.unique)
    {
        mc_dense_verts_kernel<DT, WIDE><<<grid_for(p.ngroups * 32, 256), 256, 0, s>>>(p, verts);
        TH_LAUNCH_CHECK();
    }
    mc_dense_compact_kernel<<<dense_grid(p), kScanThreads, 0, s>>>(p);
    TH_LAUNCH_CHECK();
    mc_dense_faces_kernel<DT, WIDE><<<grid_for(p.nactive, 256), 256, 0, s>>>(p, verts, faces);
    TH_LAUNCH_CHECK();
}

template <int DT>
void sparse_count(const McPlan& p, cudaStream_t s)
{
    const int grid = grid_for(p.nnz, 256);
    mc_sparse_insert_kernel<<<grid, 256, 0, s>>>(p);
    TH_LAUNCH_CHECK();
    mc_sparse_classify_kernel<DT><<<grid, 256, 0, s>>>(p);
    TH_LAUNCH_CHECK();
    run_scan_reduce(SparseSoupCount{ p.codes }, SoupTotal{ p.ctr }, Count{ nullptr, p.nnz }, p.nnz, p.tiles_soup,
                    &p.ctr->scan_soup, s);
    if (p.unique)
        run_scan(SparseVertCount{ p.used }, SparseVertEmit{ p.vbase }, VertTotal{ p.ctr }, Count{ nullptr, p.nnz },
                 p.nnz, p.tiles_verts, &p.ctr->scan_verts, s);
}

template <int DT>
void sparse_emit(const McPlan& p, float* verts, int64_t* faces, cudaStream_t s)
{
    if (p.unique)
    {
        mc_sparse_verts_kernel<DT><<<grid_for(p.nnz, 256), 256, 0, s>>>(p, verts);
        TH_LAUNCH_CHECK();
    }
    run_scan_apply(SparseSoupCount{ p.codes }, SparseCellEmit<DT>{ p, verts, faces }, Count{ nullptr, p.nnz }, p.nnz,
                   p.tiles_soup, s);
}

template <class F>
void dispatch_value_dtype(int dt, F&& f)
{
    switch (dt)
    {
    case TH_FLOAT16:
        f.template operator()<TH_FLOAT16>();
        break;
    case TH_FLOAT32:
        f.template operator()<TH_FLOAT32>();
        break;
    default:
        f.template operator()<TH_FLOAT64>();
        break;
    }
}

} // namespace

void launch_mc_count(const McPlan& p, cudaStream_t s)
{
    TH_CUDA(cudaMemsetAsync(p.ctr, 0, sizeof(McCounters), s));
    if (p.sparse)
    {
        if (p.nnz == 0)
            return;
        TH_CUDA(cudaMemsetAsync(p.keys, 0xff, sizeof(unsigned long long) * (p.hmask + 1), s));
        if (p.unique)
            TH_CUDA(cudaMemsetAsync(p.used, 0, sizeof(uint32_t) * p.nnz, s));
        dispatch_value_dtype(p.dtype, [&]<int DT>() { sparse_count<DT>(p, s); });
        return;
    }
    if (p.points == 0)
        return;
    dispatch_value_dtype(p.dtype, [&]<int DT>() {
        if (p.wide)
            dense_count<DT, true>(p, s);
        else
            dense_count<DT, false>(p, s);
    });
}

void launch_mc_emit(const McPlan& p, float* verts, int64_t* faces, cudaStream_t s)
{
    if (p.sparse)
    {
        if (p.nnz == 0)
            return;
        dispatch_value_dtype(p.dtype, [&]<int DT>() { sparse_emit<DT>(p, verts, faces, s); });
        return;
    }
    if (p.points == 0)
        return;
    dispatch_value_dtype(p.dtype, [&]<int DT>() {
        if (p.wide)
            dense_emit<DT, true>(p, verts, faces, s);
        else
            dense_emit<DT, false>(p, verts, faces, s);
    });
}

} // namespace th
