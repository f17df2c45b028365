// Batched form: many hull requests carved by one persistent launch.
#pragma once

#include <cstdint>

#include "th_common.cuh"

namespace th
{

// Device descriptor of one request of a batch.
struct BatchReq
{
    const float* tf;  // [B,16]
    const float* sat; // [B,H,W]
    int64_t H, W;
    int32_t B, level;
    int32_t partial, opengl;
    int32_t skip_ok;  // exact integer SAT sums (size); binary masks are checked on the device
    int32_t no_carve; // no views or an empty image: the root is refined no further
    const unsigned int* nonbinary;
    float corner[3];
    float length;
    // corner bitmap of this request (R points per axis, WR words per row)
    uint64_t* bitmap;
    uint32_t* rowbits;
    int64_t R, WR;
    uint32_t* cell_masks; // the field's cell-mask table (HullPlan::cell_masks) or nullptr
};

struct BatchCounters
{
    int64_t count[kMaxLevel + 2];            // entries of level i (all requests)
    unsigned long long head[kMaxLevel + 2];  // dequeue position of level i
    unsigned long long overflow;
};

// Entries: request index in bits 40.., the cell (ravelled at resolution 2^i,
// i the level of the list holding it) in bits 0..39.
constexpr int kTagShift = 40;

struct BatchPlan
{
    const BatchReq* reqs;
    int32_t nreq;
    int32_t max_level;
    int64_t* nodes; // level lists back to back (level i starts after levels < i)
    uint32_t* node_skip;
    uint32_t* node_out; // out-of-frame views (HullPlan::node_out)
    int64_t node_cap;
    BatchCounters* ctr;
    // (partial << 1) | opengl when every request shares it, -1 otherwise
    int32_t variant;
    // per cell of the level being carved: refined children, and the
    // children's view-skip masks for the first skip_cap cells
    uint8_t* child_masks;  // [node_cap]
    uint32_t* child_skip;  // [skip_cap * 8]
    uint32_t* child_out;   // [skip_cap * 8]
    int64_t skip_cap;
    unsigned long long* block_sums; // [grid size] children per block
    uint32_t leaf_levels; // bit i: some request ends at level i
    uint32_t mask_levels; // bit i: some request with a cell-mask table has level i + 1
};

void launch_batch_init(const BatchPlan& bp, cudaStream_t s);
// The whole octree of every request, in one cooperative launch.
void launch_batch_carve(const BatchPlan& bp, cudaStream_t s);
// Corner bits of every request's leaves, in one launch.
void launch_batch_mark(const BatchPlan& bp, cudaStream_t s);
// The field's cell-mask tables of every request from its level L-1 cells:
// set before the fields, cleared after them.
void launch_batch_cell_masks(const BatchPlan& bp, bool set, cudaStream_t s);

} // namespace th
