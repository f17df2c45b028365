// CPU oracle for the visual-hull and Gaussian-blur path.
//
// TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
// the smoke check and the CPU baseline leg of the benchmark call it.  The
// product path (the CUDA library and its Python/torch front end) never links,
// loads or falls back to it.
//
// It restates torchhull's CUDA algorithm (vc-bonn/torchhull v0.3.0) on the
// host, step by step and with the same float arithmetic, so that its results
// can be compared bit for bit with the GPU path.  Every function cites the
// reference file:line it follows.  Parity pinning: the reference ships no
// golden vectors, so its own CUDA extension is compiled from its unmodified
// sources (oracle/ref_build.py, with project-written stand-ins for the glm and
// stdgpu surface it uses) and this oracle is held, bit for bit, to that
// build's outputs: live on the GPU (tests/test_gpu_reference.py, up to the
// 32-view 1024^2 level-9 partial scene) and through fixtures the build wrote
// (tests/golden/ref_*.npz, checked on the CPU by tests/test_ref_golden_cpu.py).
#pragma once

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// Element types, same codes as th_dtype in include/torchhull_gb300.h.
enum
{
    ORACLE_BOOL = 0,
    ORACLE_UINT8 = 1,
    ORACLE_INT8 = 2,
    ORACLE_INT16 = 3,
    ORACLE_INT32 = 4,
    ORACLE_INT64 = 5,
    ORACLE_FLOAT16 = 6,
    ORACLE_FLOAT32 = 7,
    ORACLE_FLOAT64 = 8,
    ORACLE_BFLOAT16 = 9,
};

typedef struct oracle_hull oracle_hull;

// Full visual_hull path (visual_hull.cpp:34-58).  masks: [B,H,W,1] contiguous,
// transforms: [B,4,4] contiguous.  Returns NULL and fills err on an argument
// error.  nthreads <= 0 uses all hardware threads.
oracle_hull* oracle_visual_hull(const void* masks,
                                int masks_dtype,
                                int64_t B,
                                int64_t H,
                                int64_t W,
                                const void* transforms,
                                int transforms_dtype,
                                int level,
                                float corner_x,
                                float corner_y,
                                float corner_z,
                                float cube_length,
                                int masks_partial,
                                int transforms_opengl,
                                int unique_verts,
                                int nthreads,
                                char* err,
                                int errlen);

int64_t oracle_hull_num_levels(const oracle_hull* h);
int64_t oracle_hull_level_size(const oracle_hull* h, int64_t i);
void oracle_hull_level_copy(const oracle_hull* h, int64_t i, int64_t* dst);
int64_t oracle_hull_field_size(const oracle_hull* h);
void oracle_hull_field_copy(const oracle_hull* h, int64_t* indices, float* values);
int64_t oracle_hull_num_verts(const oracle_hull* h);
int64_t oracle_hull_num_faces(const oracle_hull* h);
void oracle_hull_mesh_copy(const oracle_hull* h, float* verts, int64_t* faces);
void oracle_hull_free(oracle_hull* h);

// Float32 integral image exactly as torch::cumsum(dim=1) then (dim=2) computes
// it (visual_hull_cuda.cu:76-90).  out: [B,H,W] float32.
int oracle_integral_image(const void* masks, int masks_dtype, int64_t B, int64_t H, int64_t W, float* out, int nthreads);

// Number of float32 weights t, over the bit patterns lo_bits..hi_bits (both
// of one sign), for which bilerp(1, 1, 1, 1, t, t) is not exactly 1 (the
// all-ones footprint shortcut of the GPU field relies on 0 for [0, 1.25]).
int64_t oracle_bilerp_ones_failures(uint32_t lo_bits, uint32_t hi_bits);

// gaussian_blur (gaussian_blur_cuda.cu:73-114 dense, :288-507 sparse).
// out: [B,H,W,1] of out_dtype.  Returns 0 on success.
int oracle_gaussian_blur(const void* images,
                         int images_dtype,
                         int64_t B,
                         int64_t H,
                         int64_t W,
                         int kernel_size,
                         float sigma,
                         int sparse,
                         void* out,
                         int out_dtype,
                         int nthreads,
                         char* err,
                         int errlen);

typedef struct oracle_mesh oracle_mesh;

// marching_cubes (marching_cubes_cuda.cu:146-374 kernels, :376-831 drivers)
// over a list of grid points of a [1, depth, height, width] volume: ids are
// ravel indices x + width (y + height z), strictly ascending (all points for
// a dense volume, the coalesced entries for a sparse one); values: [n] of
// values_dtype (float16, float32, float64).  Returns NULL and fills err on an
// argument error.
oracle_mesh* oracle_marching_cubes(const int64_t* ids,
                                   const void* values,
                                   int values_dtype,
                                   int64_t n,
                                   int64_t depth,
                                   int64_t height,
                                   int64_t width,
                                   float isolevel,
                                   int return_local_coords,
                                   int unique_verts,
                                   int nthreads,
                                   char* err,
                                   int errlen);
int64_t oracle_mesh_num_verts(const oracle_mesh* m);
int64_t oracle_mesh_num_faces(const oracle_mesh* m);
void oracle_mesh_copy(const oracle_mesh* m, float* verts, int64_t* faces);
void oracle_mesh_free(oracle_mesh* m);

// candidate_voxels_to_wireframes for one candidate level (ids ravelled at
// resolution 2^level_index): verts [8n,3], edges [12n,2].
void oracle_candidate_wireframe(const int64_t* candidates,
                                int64_t n,
                                int level_index,
                                float corner_x,
                                float corner_y,
                                float corner_z,
                                float cube_length,
                                float* verts,
                                int64_t* edges);

#ifdef __cplusplus
}
#endif
