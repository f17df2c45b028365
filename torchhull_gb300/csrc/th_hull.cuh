// Device-side state of one visual-hull request and the launch entry points of
// its stages (carve.cu, mesh.cu).  Every count lives in device memory, so the
// stages chain on one stream with no host round trip; kernels are grid-stride
// loops sized from the SM count that read their item count on the device.
#pragma once

#include <cstdint>

#include "th_common.cuh"

namespace th
{

enum OverflowBits : int64_t
{
    kOverflowNodes = 1,
    kOverflowCorners = 2,
    kOverflowSoup = 4,
    kOverflowParents = 8,
};

struct DevCounters
{
    int64_t level_count[kMaxLevel + 2]; // cells of level i (level 0: the root)
    int64_t level_off[kMaxLevel + 3];   // start of level i in the node pool
    int64_t rows;                       // bitmap rows holding at least one corner
    int64_t corners;                    // unique leaf corners (the sparse field)
    int64_t soup;                       // soup vertices, 3 per face
    int64_t verts;                      // unique mesh vertices
    int64_t overflow;                   // OverflowBits
    int64_t row_words;                  // words of the row-occupancy bitmap
    unsigned long long items[kMaxLevel];  // (parent, view) items the carve evaluated per parent level
    unsigned long long field_items;       // (corner, view) pairs the field evaluated
    ScanState scan;
};

// The inputs that differ between requests of one shape, read by the carve
// and field kernels from device memory (written before each run), so that a
// captured graph of the pipeline serves every request of that shape.
struct ReqConsts
{
    float corner[3];
    float length;
    const void* masks;
};

// Per-request constants and buffers, passed to kernels by value.
struct HullPlan
{
    // inputs
    const void* masks;
    int masks_dtype;
    int64_t B, H, W;
    const float* tf;  // [B,16] float32
    const float* sat; // [B,H,W]
    bool opengl, partial, unique;
    float corner[3];
    float length;
    int level;
    // octree node pool: all levels back to back
    int64_t* nodes;
    int64_t node_cap;
    uint8_t* child_masks; // one byte per parent of the current level
    unsigned long long* tile_sums;
    // View skipping (binary masks only).  node_skip[k] has bit b (b < 32) set
    // when view b need not be evaluated for any descendant of node k: the
    // box of node k or of one of its ancestors, grown by two pixels, lies
    // inside the image and holds only ones, so every descendant is "object"
    // there (and, in partial mode, fully inside the frame).  child_skip holds
    // the same masks for the 8 children of each parent of the current level.
    uint32_t* node_skip;  // [node_cap]
    uint32_t* child_skip; // [parent_cap * 8]
    // Out-of-frame views (partial mode): node_out[k] has bit b when node k's
    // box in view b lies more than 2 pixels outside the image (box_out); no
    // descendant's item in view b can change anything, so the item kernel
    // skips it and the children inherit the bit.  child_out: the same for
    // the 8 children of each parent of the current level.
    uint32_t* node_out;   // [node_cap]
    uint32_t* child_out;  // [parent_cap * 8]
    int64_t parent_cap;
    // carve kernel per parent level: 0 = views over lanes, 1 = (parent, view) items
    uint8_t carve_variant[kMaxLevel];
    const unsigned int* nonbinary; // set by the SAT pass when a mask value is not 0/1
    bool skip_ok;                  // exact integer SAT sums (H * W < 2^24)
    // All-ones footprints: bit x of word (b*H + y)*WW + x/32 is set when the
    // mask values of view b at (x, y), (x+1, y), (x, y+1) and (x+1, y+1) are
    // all exactly 1 (as floats).  A bilinear sample whose footprint is such a
    // 2x2 block is exactly 1 (lerp(1, 1, t) == 1 for every t in [0, 1.25],
    // checked exhaustively), so the field skips the four mask reads.
    bool field_ones;
    uint32_t* ones; // [B*H*WW]
    int64_t WW;
    // Field masks: the skip and out-of-frame views of the cells of the last
    // carve level (the parents of the leaves) hold for all their descendants,
    // so for every mesh corner that is one of their lattice points the field
    // factor of those views is exactly 1 (a footprint of four ones with
    // weights in [0, 1], or a point out of the frame).  cell_masks is a dense
    // table over the cells of level L-1, scattered before the field and
    // cleared after it (nullptr: no table, every pair is evaluated).
    uint32_t* cell_masks; // [8^(L-1)]
    bool own_cell_masks;  // launch_field scatters and clears the table (the batched form does it itself)
    // corner grid: R^3 points, one bit each, rows of WR 64-bit words (x fastest)
    int64_t R, WR;
    uint64_t* bitmap;     // [R*R*WR]
    uint32_t* word_rank;  // [R*R*WR] rank of the word's first bit (valid for touched rows)
    uint32_t* rowbits;    // [ceil(R*R/32)] touched-row flags
    uint32_t* rows;       // [R*R] touched rows, ascending
    // sparse field and marching cubes, indexed by corner rank
    int64_t* corners;
    float* values;
    uint8_t* codes;
    uint8_t* emask; // bit a: the edge from this corner along axis a carries a vertex
    uint32_t* soup_off;
    uint32_t* vbase;
    int64_t corner_cap;
    DevCounters* ctr;
    const ReqConsts* rq; // corner, length and masks of the running request (device)
};

// Corner ids inside the pipeline: x | y << 21 | z << 42 (grid points < 2^21
// per axis).  Ascending packed ids are ascending ravelled ids x + y*R + z*R*R,
// and decoding needs shifts instead of 64-bit divisions by R.
__device__ __forceinline__ int64_t pack_corner(int64_t x, int64_t y, int64_t z)
{
    return x | (y << 21) | (z << 42);
}

__device__ __forceinline__ void unpack_corner(int64_t v, int64_t& x, int64_t& y, int64_t& z)
{
    x = v & 0x1FFFFF;
    y = (v >> 21) & 0x1FFFFF;
    z = v >> 42;
}

void launch_hull_init(const HullPlan& p, cudaStream_t s);
// Sparse field export: ravelled ids (x + y*R + z*R*R) and values.
void launch_export_field(const HullPlan& p, int64_t n, int64_t* indices, float* values, cudaStream_t s);
void launch_carve_level(const HullPlan& p, int level_index, cudaStream_t s);
// The leaf list (level L) from the last level's child masks; the carve itself
// only counts the leaves.
void launch_emit_leaves(const HullPlan& p, cudaStream_t s);
void launch_corners(const HullPlan& p, cudaStream_t s);
// The part of launch_corners after the bitmap is set: touched rows, sorted
// unique corners and per-word ranks.
void launch_rank_corners(const HullPlan& p, cudaStream_t s);

// Sets the 8 corner bits of a leaf cell (x, y, z) at resolution 2^L in a
// corner bitmap of R points per axis and WR words per row.
__device__ __forceinline__ void mark_cell_corners(uint64_t* bitmap, uint32_t* rowbits, int64_t R, int64_t WR,
                                                  int64_t x, int64_t y, int64_t z)
{
    const int b = static_cast<int>(x & 63);
#pragma unroll
    for (int q = 0; q < 4; ++q)
    {
        const int64_t row = (y + (q & 1)) + (z + (q >> 1)) * R;
        const int64_t w = row * WR + (x >> 6);
        const uint64_t bits0 = (b < 63) ? (3ull << b) : (1ull << 63);
        if ((bitmap[w] & bits0) != bits0)
            atomicOr(reinterpret_cast<unsigned long long*>(bitmap + w), static_cast<unsigned long long>(bits0));
        if (b == 63 && !(bitmap[w + 1] & 1ull))
            atomicOr(reinterpret_cast<unsigned long long*>(bitmap + w + 1), 1ull);
        const uint32_t rb = 1u << (row & 31);
        if (!(rowbits[row >> 5] & rb))
            atomicOr(rowbits + (row >> 5), rb);
    }
}
// Sets the corner bits of the refined children (child mask m) of a cell whose
// lattice starts at (x, y, z) at resolution 2^L: per lattice row (y + dy,
// z + dz) one OR of the x bits its children cover, instead of four words per
// child (neighbouring children share 27 of their 64 corners).
__device__ __forceinline__ void mark_children_corners(uint64_t* bitmap, uint32_t* rowbits, int64_t R, int64_t WR,
                                                      int64_t x, int64_t y, int64_t z, uint32_t m)
{
#pragma unroll
    for (int dz = 0; dz < 3; ++dz)
    {
#pragma unroll
        for (int dy = 0; dy < 3; ++dy)
        {
            uint32_t xb = 0; // lattice x bits 0..2 of this row
#pragma unroll
            for (int c = 0; c < 8; ++c)
            {
                const int cx = c & 1, cy = (c >> 1) & 1, cz = c >> 2;
                if (((m >> c) & 1u) && (dy == cy || dy == cy + 1) && (dz == cz || dz == cz + 1))
                    xb |= 3u << cx;
            }
            if (!xb)
                continue;
            const int64_t row = (y + dy) + (z + dz) * R;
            const int64_t w = row * WR + (x >> 6);
            const int b = static_cast<int>(x & 63);
            const uint64_t lo = static_cast<uint64_t>(xb) << b;
            if (lo && (bitmap[w] & lo) != lo)
                atomicOr(reinterpret_cast<unsigned long long*>(bitmap + w), static_cast<unsigned long long>(lo));
            if (b > 61)
            {
                const uint64_t hi = static_cast<uint64_t>(xb) >> (64 - b);
                if (hi && (bitmap[w + 1] & hi) != hi)
                    atomicOr(reinterpret_cast<unsigned long long*>(bitmap + w + 1), static_cast<unsigned long long>(hi));
            }
            const uint32_t rb = 1u << (row & 31);
            if (!(rowbits[row >> 5] & rb))
                atomicOr(rowbits + (row >> 5), rb);
        }
    }
}

void launch_field(const HullPlan& p, cudaStream_t s);
void launch_marching_cubes(const HullPlan& p, cudaStream_t s);
void launch_export(const HullPlan& p, float* verts, int64_t* faces, cudaStream_t s);
void launch_cleanup(const HullPlan& p, cudaStream_t s);

} // namespace th
