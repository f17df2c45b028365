// Device-side plan of one public marching-cubes request and the launch entry
// points of its two phases (mc.cu).
#pragma once

#include <cstdint>

#include "th_common.cuh"

namespace th
{

enum McFlags : unsigned int
{
    kMcBadIndex = 1, // a sparse index outside the volume (or a batch index other than 0)
    kMcUnsorted = 2, // sparse indices not strictly ascending (not a coalesced tensor)
};

struct McCounters
{
    unsigned long long soup;   // soup vertices, 3 per face
    unsigned long long verts;  // unique vertices
    unsigned long long active; // active cells (dense volumes)
    unsigned int flags;       // McFlags
    unsigned int pad;
    ScanState scan_soup;
    ScanState scan_verts;
};

// Edge bits of 32 consecutive grid points of a dense volume: bit l of x / y /
// z is set when the +x / +y / +z edge of point 32 g + l is a mesh vertex.
struct McGroup
{
    uint32_t x, y, z, pad;
    unsigned long long base; // vertices of all points before the group
};

struct McPlan
{
    int dtype; // TH_FLOAT16, TH_FLOAT32 or TH_FLOAT64
    bool sparse, unique, local;
    bool wide;             // points >= 2^32: 64-bit index decoding
    int64_t D, H, W;       // volume sizes along z, y, x
    int64_t points;        // D * H * W
    FastDiv div_w, div_h;  // by W and by H (points < 2^32)
    float iso;
    float scale[3];        // 2 / (size - 1) along x, y, z
    const void* volume;    // dense: [D, H, W], x fastest
    const int64_t* indices; // sparse: [4, nnz] rows (0, z, y, x)
    const void* values;     // sparse: [nnz]
    int64_t nnz;
    // pools
    McGroup* groups;          // dense, unique: ceil(points / 32)
    int64_t ngroups;
    unsigned long long* keys; // sparse: open-addressing table of ravel ids
    int32_t* slots;           // sparse: entry index of each key
    uint64_t hmask;           // table capacity - 1 (a power of two minus one)
    uint8_t* codes;           // cell code of each point (dense) or entry (sparse); 0: no cell
    uint32_t* used;           // sparse, unique: vertex edge bits of each entry
    unsigned long long* vbase; // sparse, unique: first vertex of each entry
    unsigned long long* tiles_soup;
    unsigned long long* tiles_verts;
    unsigned long long* tiles_scan; // dense: tile sums of the scan over tiles_soup
    int64_t* active;                 // dense: active cells (base points), ascending
    unsigned long long* active_soup; // dense: their first soup vertex
    int64_t nactive;                 // dense: active cells (known after phase 1)
    McCounters* ctr;
};

// Scan tiles a scan over n items needs.
inline int64_t mc_scan_tiles(int64_t n)
{
    return (n + kScanTile - 1) / kScanTile;
}

// Phase 1: the soup and vertex counts (ctr) and the vertex numbering.
void launch_mc_count(const McPlan& p, cudaStream_t s);
// Phase 2: vertices [verts, 3] and faces [soup / 3, 3] into caller buffers.
void launch_mc_emit(const McPlan& p, float* verts, int64_t* faces, cudaStream_t s);

} // namespace th
