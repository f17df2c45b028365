/*
 * torchhull_gb300: C ABI of the GB300 (sm_103a) visual-hull and Gaussian-blur path.
 *
 * Plain C types only: device pointers, sizes, dtype codes and a CUDA stream
 * passed as void* (a cudaStream_t; NULL is the legacy default stream).  All
 * device work is enqueued on that stream.  Inputs are borrowed; outputs are
 * written into buffers the caller allocates once the sizes are known, so the
 * caller's allocator (for example torch's caching allocator) owns them.
 *
 * Each entry point names the reference interface it replaces
 * (vc-bonn/torchhull v0.3.0, paths relative to that project).
 *
 * Threading: a th_context serves one request at a time.  Use one context per
 * host thread (or guard it with a lock).  A context keeps its device pools
 * between calls, so repeated requests do not allocate.
 */
#ifndef TORCHHULL_GB300_H
#define TORCHHULL_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TH_MAX_LEVEL 12

typedef enum th_status
{
    TH_OK = 0,
    TH_ERR_INVALID_ARGUMENT = 1, /* a TORCH_CHECK of the reference would fail */
    TH_ERR_UNSUPPORTED_DTYPE = 2, /* the reference's AT_DISPATCH has no case for it */
    TH_ERR_CUDA = 3,              /* a CUDA runtime call failed; see th_context_error */
    TH_ERR_OUT_OF_MEMORY = 4,
    TH_ERR_STATE = 5,    /* call order violated (export before a successful run) */
    TH_ERR_NO_DEVICE = 6 /* no usable CUDA device */
} th_status;

/* Element types (same meaning as torch dtypes). */
typedef enum th_dtype
{
    TH_BOOL = 0,
    TH_UINT8 = 1,
    TH_INT8 = 2,
    TH_INT16 = 3,
    TH_INT32 = 4,
    TH_INT64 = 5,
    TH_FLOAT16 = 6,
    TH_FLOAT32 = 7,
    TH_FLOAT64 = 8,
    TH_BFLOAT16 = 9
} th_dtype;

typedef struct th_context th_context;

/* Context holding the device pools for one CUDA device. */
th_status th_context_create(int32_t device, th_context** out);
void th_context_destroy(th_context* ctx);
/* Message of the last failed call on ctx ("" if none); valid until the next call. */
const char* th_context_error(const th_context* ctx);
const char* th_status_string(th_status status);
/* Bytes of device memory the context currently holds in its pools. */
int64_t th_context_device_bytes(const th_context* ctx);

/* Arguments of one visual-hull request.  masks: [B,H,W,1] contiguous device
 * tensor; transforms: [B,4,4] contiguous device tensor (K*T per view). */
typedef struct th_hull_args
{
    const void* masks;
    int32_t masks_dtype; /* uint8, int8, int16, int32, int64, float16, float32, float64 */
    int64_t batch;
    int64_t height;
    int64_t width;
    const void* transforms;
    int32_t transforms_dtype; /* float16, float32, float64 */
    int32_t level;            /* 0 .. TH_MAX_LEVEL */
    float cube_corner_bfl[3];
    float cube_length;
    int32_t masks_partial;
    int32_t transforms_opengl; /* 1: "opengl", 0: "opencv" */
    int32_t unique_verts;
} th_hull_args;

typedef struct th_hull_info
{
    int64_t num_verts;
    int64_t num_faces;
    int64_t num_corners; /* size of the sparse hull field */
    int32_t num_levels;  /* entries of the candidate list, torchhull's candidates_octree */
    int32_t reserved;
    int64_t level_sizes[TH_MAX_LEVEL + 1];
} th_hull_info;

/*
 * Runs the whole visual-hull path for one request on `stream` and returns the
 * mesh sizes (one device->host read of a few counters; nothing else waits).
 * The mesh and the per-level candidates stay in the context until the next
 * th_visual_hull call; fetch them with the export calls below.
 *
 * Replaces torchhull::visual_hull (src/torchhull/_C/include/torchhull/visual_hull.h:11-19,
 * src/torchhull/_C/src/visual_hull.cpp:34-83) and the host/device stages it
 * chains (visual_hull_cuda.cu:582-894, marching_cubes_cuda.cu:535-754,
 * visual_hull_cuda.cu:958-1020).
 */
th_status th_visual_hull(th_context* ctx, const th_hull_args* args, void* stream, th_hull_info* info);

/*
 * Fused blur -> hull request: the visual hull of gaussian_blur(masks,
 * kernel_size, sigma, sparse=True) (blurred in the masks' own float type),
 * with the blurred masks kept in a context pool instead of a tensor the caller
 * allocates and passes back.  Results (and the export calls) are identical to
 * th_gaussian_blur followed by th_visual_hull on its output.  No reference
 * counterpart as one call; it chains gaussian_blur.cpp:15-28 and
 * visual_hull.cpp:34-83.
 */
th_status th_visual_hull_blurred(th_context* ctx,
                                 const th_hull_args* args,
                                 int32_t kernel_size,
                                 float sigma,
                                 void* stream,
                                 th_hull_info* info);

/* Writes the mesh of the last th_visual_hull call: verts [V,3] float32 in world
 * coordinates, faces [F,3] int64 with torchhull's winding (columns 1 and 2
 * swapped, visual_hull_cuda.cu:941-956).  Either pointer may be NULL when its
 * count is 0. */
th_status th_visual_hull_export(th_context* ctx, float* verts, int64_t* faces, void* stream);

/* Candidate cells of level i of the last run (ravelled x-fastest at resolution
 * 2^i, in torchhull's order), the list visual_hull_with_candidate_voxels
 * returns (src/torchhull/_C/src/visual_hull.cpp:85-135). */
th_status th_visual_hull_export_candidates(th_context* ctx, int32_t level, int64_t* dst, void* stream);

/* Sparse hull field of the last run: ravelled grid indices (ascending, grid
 * (2^level+1)^3) and values (visual_hull_cuda.cu:582-894, RavelledSparseTensor). */
th_status th_visual_hull_export_field(th_context* ctx, int64_t* indices, float* values, void* stream);

/*
 * gaussian_blur(images, kernel_size, sigma, sparse, dtype) for images
 * [B,H,W,1] contiguous on the device; out is [B,H,W,1] contiguous of
 * out_dtype (float16/32/64).
 * Replaces torchhull::gaussian_blur (src/torchhull/_C/include/torchhull/gaussian_blur.h:10-15,
 * src/torchhull/_C/src/gaussian_blur.cpp:15-28, gaussian_blur_cuda.cu:73-518).
 */
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
                           void* stream);

/*
 * th_gaussian_blur without any device allocation, for callers that cannot
 * call cudaMalloc: a process whose device memory another framework has already
 * reserved, a per-frame loop that must not risk the device-wide synchronisation
 * cudaMalloc/cudaFree can cause, or a caller with a fixed device-memory budget.
 * No counterpart in the reference.  Same arguments and results as
 * th_gaussian_blur, but no context: its scratch is one 16 MiB array in the
 * library's device memory, held on every GPU that loads the library.  Requests
 * whose tile flags and weights (B*(H/(k/2)+1)*(W/(k/2)+1) + 8*(k*k+1) + 16
 * bytes) exceed 16 MiB return TH_ERR_INVALID_ARGUMENT.  All calls share that
 * array, so calls whose work overlaps on the GPU race.  The first call on a
 * device looks up the array's device address; make it before any stream capture.
 */
th_status th_gaussian_blur_noalloc(const void* images,
                                   int32_t images_dtype,
                                   int64_t batch,
                                   int64_t height,
                                   int64_t width,
                                   int32_t kernel_size,
                                   float sigma,
                                   int32_t sparse,
                                   void* out,
                                   int32_t out_dtype,
                                   void* stream);

/* The float32 integral image of masks [B,H,W,1] into out [B,H,W], with the
 * exact rounding of torch::cumsum(dim 1) then (dim 2) that the reference uses
 * (visual_hull_cuda.cu:76-90). */
th_status th_integral_image(th_context* ctx,
                            const void* masks,
                            int32_t masks_dtype,
                            int64_t batch,
                            int64_t height,
                            int64_t width,
                            float* out,
                            void* stream);

/*
 * Marching cubes over a dense volume or a coalesced sparse COO volume.
 * Replaces torchhull::marching_cubes (src/torchhull/_C/include/torchhull/
 * marching_cubes.h:11-15; marching_cubes_cuda.cu:376-533 dense, :754-831
 * sparse).  Two calls, as for th_visual_hull: th_marching_cubes computes the
 * mesh sizes (one device->host read), th_marching_cubes_export writes the
 * mesh into caller buffers (verts [num_verts,3] float32, faces [num_faces,3]
 * int64).  Axes: x along the volume's last dimension (width), z along its
 * first (depth).
 */
typedef struct th_mc_args
{
    int32_t sparse;         /* 0: dense volume, 1: sparse COO volume */
    int32_t dtype;          /* float16, float32, float64: the volume's or the values' type */
    int64_t depth;          /* sizes of the [1, D, H, W] volume */
    int64_t height;
    int64_t width;
    const void* volume;     /* dense: D*H*W contiguous elements, width fastest */
    const int64_t* indices; /* sparse: [4, nnz] row-major, rows (0, z, y, x), strictly ascending in (z, y, x) */
    const void* values;     /* sparse: [nnz] contiguous */
    int64_t nnz;
    float isolevel;         /* >= 0 */
    int32_t return_local_coords; /* 1: [-1, 1]^3, 0: voxel coordinates */
    int32_t unique_verts;        /* 1: shared vertices, 0: triangle soup */
} th_mc_args;

typedef struct th_mc_info
{
    int64_t num_verts;
    int64_t num_faces;
} th_mc_info;

th_status th_marching_cubes(th_context* ctx, const th_mc_args* args, void* stream, th_mc_info* info);
th_status th_marching_cubes_export(th_context* ctx, float* verts, int64_t* faces, void* stream);

/*
 * Wireframe of one candidate level: torchhull::candidate_voxels_to_wireframes
 * (visual_hull.h, visual_hull.cpp:141-155; visual_hull_cuda.cu:1024-1111),
 * called once per entry of the candidate list.  candidates: [n] int64 device
 * ids ravelled at resolution 2^level_index (x fastest); verts: [8n,3] float32
 * and edges: [12n,2] int64 device buffers of the caller.
 */
th_status th_candidate_wireframe(th_context* ctx,
                                 const int64_t* candidates,
                                 int64_t n,
                                 int32_t level_index,
                                 const float cube_corner_bfl[3],
                                 float cube_length,
                                 float* verts,
                                 int64_t* edges,
                                 void* stream);

/*
 * torchhull::store_curve_network (io.h; io.cpp:11-127): writes a curve network
 * (host arrays verts [nv,3] float32, edges [ne,2] int64) as ".obj" text or
 * ".ply" binary little endian, chosen by the file extension.  Host only (no
 * device needed); ctx may be NULL, else it receives the error message.
 */
th_status th_store_curve_network(th_context* ctx,
                                 const char* filename,
                                 const float* verts,
                                 int64_t nv,
                                 const int64_t* edges,
                                 int64_t ne,
                                 int32_t verbose);

/*
 * Batched form: n independent requests processed together (shared launches,
 * one device->host read for all).  infos[n] receives the sizes; results stay
 * in the context until the next batched call.  No counterpart in the
 * reference, which serves one request per call; each result equals what
 * th_visual_hull returns for that request alone.
 */
th_status th_visual_hull_batch(th_context* ctx, const th_hull_args* args, int32_t n, void* stream, th_hull_info* infos);
th_status th_visual_hull_batch_export(th_context* ctx, int32_t index, float* verts, int64_t* faces, void* stream);
/* The meshes of requests 0..n-1 of the last batch at once (verts[i], faces[i]
 * sized from infos[i]); the exports run side by side and are joined into
 * stream before the call's work on it completes. */
th_status th_visual_hull_batch_export_all(th_context* ctx, int32_t n, float* const* verts, int64_t* const* faces,
                                          void* stream);

/* Stage timing (no reference counterpart).  With profiling on, th_visual_hull
 * records CUDA events between its stages on the request's stream; the times
 * of the last request, in milliseconds, are read back with
 * th_context_stage_times.  Off by default (no events recorded). */
typedef struct th_stage_times
{
    float integral_image_ms; /* transforms conversion + SAT */
    float carve_ms[TH_MAX_LEVEL]; /* classify + compact, per parent level */
    float corners_ms;             /* corner bitmap, row scan, corner ranks */
    float field_ms;
    float marching_cubes_ms; /* cell codes, edge marks, vertex numbering */
    float total_ms;
    int32_t levels;
    /* (parent, view) items the carve evaluated per parent level: views skipped
     * as inherited "object" or out of the frame are not counted */
    int64_t carve_items[TH_MAX_LEVEL];
    /* (corner, view) pairs the field evaluated (pairs whose factor the carve
     * proved to be 1 are not counted) */
    int64_t field_items;
} th_stage_times;

th_status th_context_set_profiling(th_context* ctx, int32_t enable);

/* Tuning options (no reference counterpart). */
typedef enum th_option
{
    /* Carve kernel per octree level: 0 = autotune (default: the first request of
     * each size/level/mode signature is run with both kernels and the faster
     * choice is kept), 1 = views over lanes everywhere, 2 = (parent, view) work
     * items from level 4 on. */
    TH_OPTION_CARVE_KERNEL = 1,
    /* 1 (default): th_visual_hull replays the octree, corner, field and
     * marching-cubes stages of a request as a CUDA graph captured once per
     * request shape (sizes, level, modes, dtype, pools); 0: launches them
     * one by one.  Profiled and autotuning runs always launch directly. */
    TH_OPTION_GRAPHS = 2,
    /* 1: th_visual_hull_batch runs requests that fill the GPU alone (level >= 8
     * and at least 16 M mask pixels) through the per-request pipeline and the
     * others through the shared persistent carve; 0 (default): every request
     * through the shared carve.  Results are identical. */
    TH_OPTION_BATCH_ROUTE = 3,
    /* 1 (default): where the field has no cell masks (below), it first
     * builds a bitmap of the 2x2 pixel footprints whose four mask values are
     * exactly 1 and returns the factor 1 for a sample there without reading
     * the masks (a bilinear sample of four ones is exactly 1); 0: every
     * sample reads its four pixels.  Results are identical. */
    TH_OPTION_FIELD_ONES = 4,
    /* 1 (default): the carve's skip and out-of-frame views of the last
     * level's cells (levels 1 to 10) tell the field which (corner, view)
     * factors are exactly 1, and it skips them; 0: every pair is evaluated.
     * Results are identical. */
    TH_OPTION_FIELD_MASKS = 5,
    /* 1 (default): integral images of 0/1 masks (H*W <= 2^24, W <= 4096) are
     * built in one banded pass (exact integer sums, any order); 0: always the
     * two sequential passes in torch's addition order.  Results are identical. */
    TH_OPTION_SAT_SINGLE_PASS = 6
} th_option;
th_status th_context_set_option(th_context* ctx, int32_t option, int64_t value);
th_status th_context_stage_times(const th_context* ctx, th_stage_times* out);

/* Number of kernels this library has launched in this process (all contexts). */
int64_t th_launch_count(void);

/* Copies `bytes` from src to dst with a kernel on `stream`, a stream of the
 * current device (no reference counterpart).  Each pointer is memory of the
 * current device, managed memory, or pinned host memory (cudaHostAlloc, or
 * cudaHostRegister with a device mapping), which is reached through its device
 * mapping; other host memory and other devices' memory are
 * TH_ERR_INVALID_ARGUMENT.
 * The transfer runs on a few blocks of SMs instead of a DMA copy engine
 * (8 blocks when reading host memory, 6 when writing it, all SMs for device
 * to device), sized to overlap the hull kernels.  On GB300, a loop overlapping
 * hulls with cudaMemcpyAsync copies of their inputs and meshes lost ~70-80 ms
 * in about one run of three (a few consecutive copies at a tenth of their
 * rate); the same loop with this kernel showed no such stall in 40 runs and
 * ran ~5% below the stall-free copy-engine runs. */
th_status th_copy(void* dst, const void* src, int64_t bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TORCHHULL_GB300_H */
