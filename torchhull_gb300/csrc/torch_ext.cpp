// Thin torch extension over the C ABI (include/torchhull_gb300.h).
//
// It keeps torchhull's Python-facing signatures, argument names, defaults and
// error behaviour (src/torchhull/_C/python/bindings.cpp:12-251,
// src/torchhull/_C/src/visual_hull.cpp:60-187, gaussian_blur.cpp:15-28):
// tensors in, tensors out, RuntimeError on a failed check.  All computation
// happens in libtorchhull_gb300.so on the current CUDA stream; outputs are
// allocated here through torch's caching allocator once their sizes are known.

#include <torch/extension.h>

#include <ATen/cuda/CUDAContext.h>
#include <c10/cuda/CUDAGuard.h>

#include <array>
#include <map>
#include <mutex>
#include <optional>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/torchhull_gb300.h"

// The reference's TORCH_CHECK_EQ/LE/... checks, with their message
// ("Check failed: a op b (x vs. y). "), raised as RuntimeError on every torch
// version: some versions abort the process on a failed TORCH_CHECK_OP.
#define TH_CHECK_OP(a, b, op) \
    TORCH_CHECK((a)op(b), "Check failed: " #a " " #op " " #b " (", (a), " vs. ", (b), "). ")
#define TH_CHECK_EQ(a, b) TH_CHECK_OP(a, b, ==)
#define TH_CHECK_NE(a, b) TH_CHECK_OP(a, b, !=)
#define TH_CHECK_LE(a, b) TH_CHECK_OP(a, b, <=)
#define TH_CHECK_LT(a, b) TH_CHECK_OP(a, b, <)
#define TH_CHECK_GE(a, b) TH_CHECK_OP(a, b, >=)
#define TH_CHECK_GT(a, b) TH_CHECK_OP(a, b, >)

namespace
{

struct DeviceContext
{
    th_context* ctx = nullptr;
    std::mutex lock;
};

DeviceContext& context_for(int device)
{
    static std::mutex registry_lock;
    static std::map<int, DeviceContext*> registry;
    std::lock_guard<std::mutex> g(registry_lock);
    auto it = registry.find(device);
    if (it != registry.end())
        return *it->second;
    auto* dc = new DeviceContext;
    const th_status st = th_context_create(device, &dc->ctx);
    TORCH_CHECK(st == TH_OK, "torchhull_gb300: cannot create a context on device ", device, ": ", th_status_string(st));
    registry[device] = dc;
    return *dc;
}

// Takes a context lock on a thread that holds the GIL. Waiting happens with the
// GIL released: a thread that holds the lock may itself be waiting for the GIL
// (a batch call re-acquires it on leaving its GIL-free section), so blocking
// on the lock with the GIL held could deadlock the two threads.
std::unique_lock<std::mutex> lock_nogil(std::mutex& m)
{
    std::unique_lock<std::mutex> lk(m, std::defer_lock);
    if (!lk.try_lock())
    {
        pybind11::gil_scoped_release nogil;
        lk.lock();
    }
    return lk;
}

void check(th_status st, th_context* ctx)
{
    if (st == TH_OK)
        return;
    const std::string msg = th_context_error(ctx);
    TORCH_CHECK(false, msg.empty() ? std::string(th_status_string(st)) : msg);
}

int32_t th_dtype_of(at::ScalarType t)
{
    switch (t)
    {
    case at::kBool:
        return TH_BOOL;
    case at::kByte:
        return TH_UINT8;
    case at::kChar:
        return TH_INT8;
    case at::kShort:
        return TH_INT16;
    case at::kInt:
        return TH_INT32;
    case at::kLong:
        return TH_INT64;
    case at::kHalf:
        return TH_FLOAT16;
    case at::kFloat:
        return TH_FLOAT32;
    case at::kDouble:
        return TH_FLOAT64;
    case at::kBFloat16:
        return TH_BFLOAT16;
    default:
        return -1;
    }
}

void* stream_of(const at::Tensor& t)
{
    return static_cast<void*>(at::cuda::getCurrentCUDAStream(t.device().index()).stream());
}

void require_cuda(const at::Tensor& t)
{
    TORCH_CHECK(t.is_cuda(), "No backend implementation available for device \"" + t.device().str() + "\".");
}

th_hull_args hull_args(const at::Tensor& masks,
                       const at::Tensor& transforms,
                       int level,
                       const std::array<float, 3>& cube_corner_bfl,
                       float cube_length,
                       bool masks_partial,
                       const std::string& transforms_convention,
                       bool unique_verts)
{
    // visual_hull_cuda.cu:591-613
    TH_CHECK_EQ(masks.device(), transforms.device());
    TH_CHECK_EQ(masks.dim(), 4);
    TH_CHECK_EQ(transforms.dim(), 3);
    TH_CHECK_EQ(transforms.size(1), 4);
    TH_CHECK_EQ(transforms.size(2), 4);
    TH_CHECK_EQ(masks.size(0), transforms.size(0));
    TH_CHECK_EQ(masks.size(3), 1);
    TH_CHECK_GE(level, 0);
    TH_CHECK_GT(cube_length, 0.f);
    bool opengl = false;
    if (transforms_convention == "opengl")
        opengl = true;
    else if (transforms_convention == "opencv")
        opengl = false;
    else
        TORCH_CHECK(false, "Unsupported transforms_convention \"" + transforms_convention + "\".");

    th_hull_args a{};
    a.masks = masks.data_ptr();
    a.masks_dtype = th_dtype_of(masks.scalar_type());
    a.batch = masks.size(0);
    a.height = masks.size(1);
    a.width = masks.size(2);
    a.transforms = transforms.data_ptr();
    a.transforms_dtype = th_dtype_of(transforms.scalar_type());
    a.level = level;
    a.cube_corner_bfl[0] = cube_corner_bfl[0];
    a.cube_corner_bfl[1] = cube_corner_bfl[1];
    a.cube_corner_bfl[2] = cube_corner_bfl[2];
    a.cube_length = cube_length;
    a.masks_partial = masks_partial ? 1 : 0;
    a.transforms_opengl = opengl ? 1 : 0;
    a.unique_verts = unique_verts ? 1 : 0;
    return a;
}

struct HullOutputs
{
    at::Tensor verts, faces;
    std::vector<at::Tensor> candidates;
    at::Tensor field_indices, field_values;
};

HullOutputs run_visual_hull(const at::Tensor& masks_in,
                            const at::Tensor& transforms_in,
                            int level,
                            const std::array<float, 3>& cube_corner_bfl,
                            float cube_length,
                            bool masks_partial,
                            const std::string& transforms_convention,
                            bool unique_verts,
                            bool want_candidates,
                            bool want_field,
                            int blur_kernel_size = 0,
                            float blur_sigma = 0.f)
{
    require_cuda(masks_in);
    at::cuda::CUDAGuard guard(masks_in.device());
    const at::Tensor masks = masks_in.contiguous();
    const at::Tensor transforms = transforms_in.contiguous();
    th_hull_args a = hull_args(masks, transforms, level, cube_corner_bfl, cube_length, masks_partial,
                               transforms_convention, unique_verts);

    DeviceContext& dc = context_for(masks.device().index());
    auto g = lock_nogil(dc.lock);
    void* stream = stream_of(masks);
    th_hull_info info{};
    if (blur_kernel_size != 0)
        check(th_visual_hull_blurred(dc.ctx, &a, blur_kernel_size, blur_sigma, stream, &info), dc.ctx);
    else
        check(th_visual_hull(dc.ctx, &a, stream, &info), dc.ctx);

    const auto dev = masks.device();
    HullOutputs out;
    out.verts = at::empty({ info.num_verts, 3 }, at::TensorOptions().dtype(at::kFloat).device(dev));
    out.faces = at::empty({ info.num_faces, 3 }, at::TensorOptions().dtype(at::kLong).device(dev));
    check(th_visual_hull_export(dc.ctx, out.verts.data_ptr<float>(), out.faces.data_ptr<int64_t>(), stream), dc.ctx);
    if (want_candidates)
    {
        for (int i = 0; i < info.num_levels; ++i)
        {
            at::Tensor c = at::empty({ info.level_sizes[i] }, at::TensorOptions().dtype(at::kLong).device(dev));
            check(th_visual_hull_export_candidates(dc.ctx, i, c.data_ptr<int64_t>(), stream), dc.ctx);
            out.candidates.push_back(c);
        }
    }
    if (want_field)
    {
        out.field_indices = at::empty({ info.num_corners }, at::TensorOptions().dtype(at::kLong).device(dev));
        out.field_values = at::empty({ info.num_corners }, at::TensorOptions().dtype(at::kFloat).device(dev));
        check(th_visual_hull_export_field(dc.ctx, out.field_indices.data_ptr<int64_t>(),
                                          out.field_values.data_ptr<float>(), stream),
              dc.ctx);
    }
    return out;
}

std::tuple<at::Tensor, at::Tensor> visual_hull(const at::Tensor& masks,
                                               const at::Tensor& transforms,
                                               int level,
                                               const std::array<float, 3>& cube_corner_bfl,
                                               float cube_length,
                                               bool masks_partial,
                                               const std::string& transforms_convention,
                                               bool unique_verts)
{
    auto o = run_visual_hull(masks, transforms, level, cube_corner_bfl, cube_length, masks_partial,
                             transforms_convention, unique_verts, false, false);
    return { o.verts, o.faces };
}

// Fused blur -> hull: visual_hull(gaussian_blur(masks, kernel_size, sigma), ...)
// with the blurred masks kept inside the library (no reference counterpart as
// one call).
std::tuple<at::Tensor, at::Tensor> visual_hull_blurred(const at::Tensor& masks,
                                                       const at::Tensor& transforms,
                                                       int level,
                                                       const std::array<float, 3>& cube_corner_bfl,
                                                       float cube_length,
                                                       bool masks_partial,
                                                       const std::string& transforms_convention,
                                                       int kernel_size,
                                                       float sigma,
                                                       bool unique_verts)
{
    TORCH_CHECK(kernel_size != 0, "Check failed: kernel_size > 0 (0 vs. 0)");
    auto o = run_visual_hull(masks, transforms, level, cube_corner_bfl, cube_length, masks_partial,
                             transforms_convention, unique_verts, false, false, kernel_size, sigma);
    return { o.verts, o.faces };
}

std::tuple<at::Tensor, at::Tensor, std::vector<at::Tensor>> visual_hull_with_candidate_voxels(
        const at::Tensor& masks,
        const at::Tensor& transforms,
        int level,
        const std::array<float, 3>& cube_corner_bfl,
        float cube_length,
        bool masks_partial,
        const std::string& transforms_convention,
        bool unique_verts)
{
    auto o = run_visual_hull(masks, transforms, level, cube_corner_bfl, cube_length, masks_partial,
                             transforms_convention, unique_verts, true, false);
    return { o.verts, o.faces, o.candidates };
}

// The sparse field as (indices, values, grid size R); the Python layer turns
// it into torchhull's coalesced COO tensor (visual_hull_cuda.cu:522-580).
std::tuple<at::Tensor, at::Tensor, int64_t> sparse_visual_hull_field_raw(const at::Tensor& masks,
                                                                         const at::Tensor& transforms,
                                                                         int level,
                                                                         const std::array<float, 3>& cube_corner_bfl,
                                                                         float cube_length,
                                                                         bool masks_partial,
                                                                         const std::string& transforms_convention)
{
    auto o = run_visual_hull(masks, transforms, level, cube_corner_bfl, cube_length, masks_partial,
                             transforms_convention, true, false, true);
    return { o.field_indices, o.field_values, (int64_t{ 1 } << level) + 1 };
}

at::Tensor gaussian_blur(const at::Tensor& images_in,
                         int kernel_size,
                         float sigma,
                         bool sparse,
                         std::optional<at::ScalarType> dtype)
{
    require_cuda(images_in);
    at::cuda::CUDAGuard guard(images_in.device());
    TH_CHECK_EQ(images_in.dim(), 4);
    TH_CHECK_EQ(images_in.size(3), 1);
    const at::Tensor images = images_in.contiguous();
    const at::ScalarType out_type = dtype.value_or(images.scalar_type());
    at::Tensor out = at::empty(images.sizes(), images.options().dtype(out_type));
    DeviceContext& dc = context_for(images.device().index());
    auto g = lock_nogil(dc.lock);
    check(th_gaussian_blur(dc.ctx, images.data_ptr(), th_dtype_of(images.scalar_type()), images.size(0),
                           images.size(1), images.size(2), kernel_size, sigma, sparse ? 1 : 0, out.data_ptr(),
                           th_dtype_of(out_type), stream_of(images)),
          dc.ctx);
    return out;
}

// torchhull::marching_cubes (marching_cubes.cpp:19-31; the tensor checks of
// marching_cubes_cuda.cu:382-385 for dense volumes and :789-795 for sparse
// ones, in the reference's order).
std::tuple<at::Tensor, at::Tensor> marching_cubes(const at::Tensor& volume,
                                                  float isolevel,
                                                  bool return_local_coords,
                                                  bool unique_verts)
{
    require_cuda(volume);
    at::cuda::CUDAGuard guard(volume.device());
    th_mc_args a{};
    at::Tensor dense, indices, values;
    if (volume.is_sparse())
    {
        TH_CHECK_EQ(volume.size(0), 1);
        TH_CHECK_LE(volume.numel(), (static_cast<int64_t>(1) << 60));
        TH_CHECK_EQ(volume.layout(), torch::Layout::Sparse);
        TH_CHECK_EQ(volume.sparse_dim(), 4);
        TH_CHECK_EQ(volume.dense_dim(), 0);
        TH_CHECK_LT(volume.values().numel(), (static_cast<int64_t>(1) << 31)); // stdgpu uses 32-bit indices
        TH_CHECK_GE(isolevel, 0);
        indices = volume.indices().contiguous();
        values = volume.values().contiguous();
        a.sparse = 1;
        a.dtype = th_dtype_of(values.scalar_type());
        a.indices = indices.data_ptr<int64_t>();
        a.values = values.data_ptr();
        a.nnz = values.numel();
    }
    else
    {
        TH_CHECK_EQ(volume.dim(), 4);
        TH_CHECK_EQ(volume.size(0), 1);
        TH_CHECK_LE(volume.numel(), (static_cast<int64_t>(1) << 60));
        TH_CHECK_GE(isolevel, 0);
        dense = volume.contiguous();
        a.sparse = 0;
        a.dtype = th_dtype_of(dense.scalar_type());
        a.volume = dense.data_ptr();
    }
    a.depth = volume.size(1);
    a.height = volume.size(2);
    a.width = volume.size(3);
    a.isolevel = isolevel;
    a.return_local_coords = return_local_coords ? 1 : 0;
    a.unique_verts = unique_verts ? 1 : 0;

    DeviceContext& dc = context_for(volume.device().index());
    auto g = lock_nogil(dc.lock);
    void* stream = stream_of(volume);
    th_mc_info info{};
    check(th_marching_cubes(dc.ctx, &a, stream, &info), dc.ctx);
    const auto dev = volume.device();
    at::Tensor verts = at::empty({ info.num_verts, 3 }, at::TensorOptions().dtype(at::kFloat).device(dev));
    at::Tensor faces = at::empty({ info.num_faces, 3 }, at::TensorOptions().dtype(at::kLong).device(dev));
    check(th_marching_cubes_export(dc.ctx, verts.data_ptr<float>(), faces.data_ptr<int64_t>(), stream), dc.ctx);
    return { verts, faces };
}

// torchhull::candidate_voxels_to_wireframes (visual_hull.cpp:141-155,
// visual_hull_cuda.cu:1060-1111): per candidate level, 8 corners and 12
// edges per voxel.
std::vector<std::tuple<at::Tensor, at::Tensor>> candidate_voxels_to_wireframes(
        const std::vector<at::Tensor>& candidate_voxels,
        const std::array<float, 3>& cube_corner_bfl,
        float cube_length)
{
    TH_CHECK_EQ(candidate_voxels.empty(), false);
    require_cuda(candidate_voxels[0]);
    for (const auto& c : candidate_voxels)
        TH_CHECK_EQ(c.device(), candidate_voxels[0].device());
    at::cuda::CUDAGuard guard(candidate_voxels[0].device());
    const auto dev = candidate_voxels[0].device();
    DeviceContext& dc = context_for(dev.index());
    auto g = lock_nogil(dc.lock);
    void* stream = stream_of(candidate_voxels[0]);
    std::vector<std::tuple<at::Tensor, at::Tensor>> out;
    for (size_t i = 0; i < candidate_voxels.size(); ++i)
    {
        const at::Tensor c = candidate_voxels[i].contiguous();
        TORCH_CHECK(c.scalar_type() == at::kLong, "expected scalar type Long but found ", c.scalar_type());
        const int64_t n = c.numel();
        at::Tensor verts = at::empty({ 8 * n, 3 }, at::TensorOptions().dtype(at::kFloat).device(dev));
        at::Tensor edges = at::empty({ 12 * n, 2 }, at::TensorOptions().dtype(at::kLong).device(dev));
        check(th_candidate_wireframe(dc.ctx, c.data_ptr<int64_t>(), n, static_cast<int32_t>(i), cube_corner_bfl.data(),
                                     cube_length, verts.data_ptr<float>(), edges.data_ptr<int64_t>(), stream),
              dc.ctx);
        out.emplace_back(verts, edges);
    }
    return out;
}

// torchhull::store_curve_network (io.cpp:116-127).
void store_curve_network(const std::string& filename,
                         const std::tuple<at::Tensor, at::Tensor>& curve_network,
                         bool verbose)
{
    const at::Tensor verts = std::get<0>(curve_network).to(at::kCPU).to(at::kFloat).contiguous();
    const at::Tensor edges = std::get<1>(curve_network).to(at::kCPU).to(at::kLong).contiguous();
    TORCH_CHECK(verts.dim() == 2 && verts.size(1) == 3, "curve network vertices must be |V| x 3");
    TORCH_CHECK(edges.dim() == 2 && edges.size(1) == 2, "curve network edges must be |E| x 2");
    const th_status st = th_store_curve_network(nullptr, filename.c_str(), verts.data_ptr<float>(), verts.size(0),
                                                edges.data_ptr<int64_t>(), edges.size(0), verbose ? 1 : 0);
    if (st != TH_OK)
    {
        const size_t dot = filename.find_last_of('.');
        const size_t slash = filename.find_last_of('/');
        const size_t name = slash == std::string::npos ? 0 : slash + 1;
        const std::string ext = (dot == std::string::npos || dot <= name) ? std::string() : filename.substr(dot);
        TORCH_CHECK(false, "No implementation for file extension \"" + ext + "\".");
    }
}

at::Tensor integral_image(const at::Tensor& masks_in)
{
    require_cuda(masks_in);
    at::cuda::CUDAGuard guard(masks_in.device());
    TH_CHECK_EQ(masks_in.dim(), 4);
    const at::Tensor masks = masks_in.contiguous();
    at::Tensor out = at::empty({ masks.size(0), masks.size(1), masks.size(2) }, masks.options().dtype(at::kFloat));
    DeviceContext& dc = context_for(masks.device().index());
    auto g = lock_nogil(dc.lock);
    check(th_integral_image(dc.ctx, masks.data_ptr(), th_dtype_of(masks.scalar_type()), masks.size(0), masks.size(1),
                            masks.size(2) * masks.size(3), out.data_ptr<float>(), stream_of(masks)),
          dc.ctx);
    return out;
}

int64_t device_pool_bytes(int device)
{
    DeviceContext& dc = context_for(device);
    auto g = lock_nogil(dc.lock);
    return th_context_device_bytes(dc.ctx);
}

void set_profiling(int device, bool enable)
{
    DeviceContext& dc = context_for(device);
    auto g = lock_nogil(dc.lock);
    check(th_context_set_profiling(dc.ctx, enable ? 1 : 0), dc.ctx);
}

// Stage times (ms) of the device's last visual_hull call made with profiling on.
pybind11::dict stage_times(int device)
{
    DeviceContext& dc = context_for(device);
    auto g = lock_nogil(dc.lock);
    th_stage_times t{};
    check(th_context_stage_times(dc.ctx, &t), dc.ctx);
    pybind11::dict d;
    d["integral_image"] = t.integral_image_ms;
    pybind11::list carve;
    for (int i = 0; i < t.levels; ++i)
        carve.append(t.carve_ms[i]);
    d["carve"] = carve;
    pybind11::list items;
    for (int i = 0; i < t.levels; ++i)
        items.append(t.carve_items[i]);
    d["carve_items"] = items;
    d["field_items"] = t.field_items;
    d["corners"] = t.corners_ms;
    d["field"] = t.field_ms;
    d["marching_cubes"] = t.marching_cubes_ms;
    d["total"] = t.total_ms;
    return d;
}

int64_t launch_count()
{
    return th_launch_count();
}

// Batched form: a list of requests, each (masks, transforms, level,
// cube_corner_bfl, cube_length, masks_partial, transforms_convention,
// unique_verts), computed together on the device's context; returns the list
// of (verts, faces).  All masks must be on one device.
// Runs a batch on ctx (ctx == nullptr: the device's shared context, taken
// under its lock); lock guards ctx otherwise.
std::vector<std::tuple<at::Tensor, at::Tensor>> run_batch_on(const pybind11::list& requests,
                                                             th_context* own_ctx,
                                                             std::mutex* own_lock,
                                                             int own_device)
{
    const int64_t n = static_cast<int64_t>(requests.size());
    std::vector<std::tuple<at::Tensor, at::Tensor>> out;
    if (n == 0)
        return out;
    std::vector<at::Tensor> keep;
    std::vector<th_hull_args> args;
    keep.reserve(2 * n);
    args.reserve(n);
    int device = -1;
    for (const auto& item : requests)
    {
        auto t = item.cast<pybind11::tuple>();
        TORCH_CHECK(t.size() == 8, "each request is (masks, transforms, level, cube_corner_bfl, cube_length, "
                                   "masks_partial, transforms_convention, unique_verts)");
        at::Tensor masks = t[0].cast<at::Tensor>();
        at::Tensor transforms = t[1].cast<at::Tensor>();
        require_cuda(masks);
        if (device < 0)
            device = masks.device().index();
        TORCH_CHECK(masks.device().index() == device, "all requests of a batch must be on one device");
        masks = masks.contiguous();
        transforms = transforms.contiguous();
        keep.push_back(masks);
        keep.push_back(transforms);
        args.push_back(hull_args(masks, transforms, t[2].cast<int>(), t[3].cast<std::array<float, 3>>(),
                                 t[4].cast<float>(), t[5].cast<bool>(), t[6].cast<std::string>(), t[7].cast<bool>()));
    }
    at::cuda::CUDAGuard guard(keep[0].device());
    TORCH_CHECK(!own_ctx || device == own_device, "masks are not on this context's device");
    th_context* ctx = own_ctx ? own_ctx : context_for(device).ctx;
    auto g = lock_nogil(own_lock ? *own_lock : context_for(device).lock);
    void* stream = stream_of(keep[0]);
    std::vector<th_hull_info> infos(n);
    th_status st;
    {
        pybind11::gil_scoped_release nogil;
        st = th_visual_hull_batch(ctx, args.data(), static_cast<int32_t>(n), stream, infos.data());
    }
    check(st, ctx);
    const auto opts = at::TensorOptions().device(keep[0].device());
    std::vector<float*> vp(n);
    std::vector<int64_t*> fp(n);
    for (int64_t i = 0; i < n; ++i)
    {
        at::Tensor v = at::empty({ infos[i].num_verts, 3 }, opts.dtype(at::kFloat));
        at::Tensor f = at::empty({ infos[i].num_faces, 3 }, opts.dtype(at::kLong));
        vp[i] = v.data_ptr<float>();
        fp[i] = f.data_ptr<int64_t>();
        out.emplace_back(v, f);
    }
    check(th_visual_hull_batch_export_all(ctx, static_cast<int32_t>(n), vp.data(), fp.data(), stream), ctx);
    return out;
}

std::vector<std::tuple<at::Tensor, at::Tensor>> visual_hull_batch(const pybind11::list& requests)
{
    return run_batch_on(requests, nullptr, nullptr, -1);
}

// TH_OPTION_CARVE_KERNEL: 0 autotune, 1 views over lanes, 2 (parent, view) items.
void set_carve_kernel(int device, int mode)
{
    DeviceContext& dc = context_for(device);
    auto g = lock_nogil(dc.lock);
    check(th_context_set_option(dc.ctx, TH_OPTION_CARVE_KERNEL, mode), dc.ctx);
}

void set_graphs(int device, bool enable)
{
    DeviceContext& dc = context_for(device);
    auto g = lock_nogil(dc.lock);
    check(th_context_set_option(dc.ctx, TH_OPTION_GRAPHS, enable ? 1 : 0), dc.ctx);
}

void set_batch_route(int device, bool enable)
{
    DeviceContext& dc = context_for(device);
    auto g = lock_nogil(dc.lock);
    check(th_context_set_option(dc.ctx, TH_OPTION_BATCH_ROUTE, enable ? 1 : 0), dc.ctx);
}

void set_field_ones(int device, bool enable)
{
    DeviceContext& dc = context_for(device);
    auto g = lock_nogil(dc.lock);
    check(th_context_set_option(dc.ctx, TH_OPTION_FIELD_ONES, enable ? 1 : 0), dc.ctx);
}

// Copies src into dst (same byte size, both contiguous, each a CUDA tensor or
// a pinned CPU tensor) with a kernel on the current stream of the CUDA side.
void copy_on_sms(at::Tensor& dst, const at::Tensor& src)
{
    TORCH_CHECK(dst.is_contiguous() && src.is_contiguous(), "copy_on_sms: tensors must be contiguous");
    const int64_t bytes = dst.numel() * static_cast<int64_t>(dst.element_size());
    TORCH_CHECK(bytes == src.numel() * static_cast<int64_t>(src.element_size()), "copy_on_sms: sizes differ");
    TORCH_CHECK(dst.is_cuda() || src.is_cuda(), "copy_on_sms: one side must be a CUDA tensor");
    TORCH_CHECK(dst.is_cuda() || dst.is_pinned(), "copy_on_sms: a CPU destination must be pinned");
    TORCH_CHECK(src.is_cuda() || src.is_pinned(), "copy_on_sms: a CPU source must be pinned");
    TORCH_CHECK(!(dst.is_cuda() && src.is_cuda()) || dst.device() == src.device(),
                "copy_on_sms: both CUDA tensors must be on one device");
    const at::Tensor& dev = dst.is_cuda() ? dst : src;
    at::cuda::CUDAGuard guard(dev.device());
    const th_status st = th_copy(dst.data_ptr(), src.data_ptr(), bytes, stream_of(dev));
    TORCH_CHECK(st == TH_OK, "copy_on_sms: ", th_status_string(st));
}

void set_sat_single_pass(int device, bool enable)
{
    DeviceContext& dc = context_for(device);
    auto g = lock_nogil(dc.lock);
    check(th_context_set_option(dc.ctx, TH_OPTION_SAT_SINGLE_PASS, enable ? 1 : 0), dc.ctx);
}

void set_field_masks(int device, bool enable)
{
    DeviceContext& dc = context_for(device);
    auto g = lock_nogil(dc.lock);
    check(th_context_set_option(dc.ctx, TH_OPTION_FIELD_MASKS, enable ? 1 : 0), dc.ctx);
}

// A context of its own (own pools), for callers that run several requests at
// once on different streams, e.g. a serving loop with one context per slot.
// The call runs on the current stream of the masks' device, with the GIL
// released while the device works.
class HullContext
{
public:
    explicit HullContext(int device) : device_(device)
    {
        const th_status st = th_context_create(device, &ctx_);
        TORCH_CHECK(st == TH_OK, "torchhull_gb300: cannot create a context on device ", device, ": ",
                    th_status_string(st));
    }
    ~HullContext()
    {
        th_context_destroy(ctx_);
    }
    HullContext(const HullContext&) = delete;
    HullContext& operator=(const HullContext&) = delete;

    std::tuple<at::Tensor, at::Tensor> visual_hull(const at::Tensor& masks_in,
                                                   const at::Tensor& transforms_in,
                                                   int level,
                                                   const std::array<float, 3>& cube_corner_bfl,
                                                   float cube_length,
                                                   bool masks_partial,
                                                   const std::string& transforms_convention,
                                                   bool unique_verts)
    {
        require_cuda(masks_in);
        TORCH_CHECK(masks_in.device().index() == device_, "masks are not on this context's device");
        at::cuda::CUDAGuard guard(masks_in.device());
        const at::Tensor masks = masks_in.contiguous();
        const at::Tensor transforms = transforms_in.contiguous();
        th_hull_args a = hull_args(masks, transforms, level, cube_corner_bfl, cube_length, masks_partial,
                                   transforms_convention, unique_verts);
        void* stream = stream_of(masks);
        auto g = lock_nogil(lock_);
        th_hull_info info{};
        th_status st;
        {
            pybind11::gil_scoped_release nogil;
            st = th_visual_hull(ctx_, &a, stream, &info);
        }
        check(st, ctx_);
        const auto dev = masks.device();
        at::Tensor verts = at::empty({ info.num_verts, 3 }, at::TensorOptions().dtype(at::kFloat).device(dev));
        at::Tensor faces = at::empty({ info.num_faces, 3 }, at::TensorOptions().dtype(at::kLong).device(dev));
        check(th_visual_hull_export(ctx_, verts.data_ptr<float>(), faces.data_ptr<int64_t>(), stream), ctx_);
        return { verts, faces };
    }

    // A batch of requests (the tuples of visual_hull_batch) on this context:
    // one persistent carve launch over all of them, on the current stream.
    std::vector<std::tuple<at::Tensor, at::Tensor>> visual_hull_batch(const pybind11::list& requests)
    {
        return run_batch_on(requests, ctx_, &lock_, device_);
    }

    int64_t device_bytes() const
    {
        return th_context_device_bytes(ctx_);
    }

private:
    int device_;
    th_context* ctx_ = nullptr;
    std::mutex lock_;
};

} // namespace

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m)
{
    using namespace pybind11::literals;
    m.def("visual_hull", &visual_hull, "masks"_a, "transforms"_a, "level"_a, "cube_corner_bfl"_a, "cube_length"_a,
          "masks_partial"_a, "transforms_convention"_a, "unique_verts"_a = true,
          "Visual hull of the masks as a mesh (verts [V,3] float32, faces [F,3] int64).");
    m.def("visual_hull_with_candidate_voxels", &visual_hull_with_candidate_voxels, "masks"_a, "transforms"_a, "level"_a,
          "cube_corner_bfl"_a, "cube_length"_a, "masks_partial"_a, "transforms_convention"_a, "unique_verts"_a = true,
          "visual_hull plus the ravelled candidate cells of every octree level.");
    m.def("sparse_visual_hull_field_raw", &sparse_visual_hull_field_raw, "masks"_a, "transforms"_a, "level"_a,
          "cube_corner_bfl"_a, "cube_length"_a, "masks_partial"_a, "transforms_convention"_a,
          "Sparse hull field as (ravelled indices, values, grid size).");
    m.def("gaussian_blur", &gaussian_blur, "images"_a, "kernel_size"_a, "sigma"_a, "sparse"_a = true,
          "dtype"_a = pybind11::none(), "Gaussian blur of [B,H,W,1] images.");
    m.def("visual_hull_blurred", &visual_hull_blurred, "masks"_a, "transforms"_a, "level"_a, "cube_corner_bfl"_a,
          "cube_length"_a, "masks_partial"_a, "transforms_convention"_a, "kernel_size"_a, "sigma"_a,
          "unique_verts"_a = true,
          "visual_hull(gaussian_blur(masks, kernel_size, sigma), ...) in one request; the blurred masks stay in the "
          "library.");
    m.def("marching_cubes", &marching_cubes, "volume"_a, "isolevel"_a, "return_local_coords"_a = true,
          "unique_verts"_a = true,
          "Marching Cubes on a 1 x D x H x W dense or sparse COO volume; returns (verts [V,3] float32, "
          "faces [F,3] int64).");
    m.def("candidate_voxels_to_wireframes", &candidate_voxels_to_wireframes, "candidate_voxels"_a,
          "cube_corner_bfl"_a, "cube_length"_a,
          "Wireframes (verts [8N,3] float32, edges [12N,2] int64) of each candidate level.");
    m.def("store_curve_network", &store_curve_network, "filename"_a, "curve_network"_a, "verbose"_a = false,
          "Stores a curve network (verts, edges) as .obj or .ply.");
    m.def("integral_image", &integral_image, "masks"_a, "Float32 integral image [B,H,W] of masks [B,H,W,1].");
    m.def("device_pool_bytes", &device_pool_bytes, "device"_a, "Bytes held by the device's resident pools.");
    m.def("set_profiling", &set_profiling, "device"_a, "enable"_a, "Record CUDA events between hull stages.");
    m.def("stage_times", &stage_times, "device"_a, "Stage times (ms) of the last profiled visual_hull call.");
    m.def("launch_count", &launch_count, "Kernels launched by the CUDA library in this process.");
    m.def("visual_hull_batch", &visual_hull_batch, "requests"_a,
          "Batched visual hulls: list of (masks, transforms, level, cube_corner_bfl, cube_length, masks_partial, "
          "transforms_convention, unique_verts) -> list of (verts, faces).");
    m.def("set_carve_kernel", &set_carve_kernel, "device"_a, "mode"_a,
          "Carve kernel choice: 0 autotune, 1 views over lanes, 2 (parent, view) items.");
    m.def("set_batch_route", &set_batch_route, "device"_a, "enable"_a,
          "Batched form: run requests that fill the GPU alone through the per-request pipeline (default off).");
    m.def("set_field_ones", &set_field_ones, "device"_a, "enable"_a,
          "Field: skip the mask reads of samples whose 2x2 footprint is all ones (default on).");
    m.def("set_field_masks", &set_field_masks, "device"_a, "enable"_a,
          "Field: skip the (corner, view) pairs whose factor the carve proved to be 1 (default on).");
    m.def("copy_on_sms", &copy_on_sms, "dst"_a, "src"_a,
          "Copy between a CUDA tensor and a pinned CPU (or CUDA) tensor with a kernel on the current stream.");
    m.def("set_sat_single_pass", &set_sat_single_pass, "device"_a, "enable"_a,
          "Integral images of 0/1 masks in one banded pass (default on).");
    m.def("set_graphs", &set_graphs, "device"_a, "enable"_a,
          "Replay each request shape's pipeline as a captured CUDA graph (default on).");
    pybind11::class_<HullContext>(m, "HullContext", "Context with its own device pools (one request at a time).")
            .def(pybind11::init<int>(), "device"_a)
            .def("visual_hull", &HullContext::visual_hull, "masks"_a, "transforms"_a, "level"_a, "cube_corner_bfl"_a,
                 "cube_length"_a, "masks_partial"_a, "transforms_convention"_a, "unique_verts"_a = true)
            .def("visual_hull_batch", &HullContext::visual_hull_batch, "requests"_a,
                 "Batched visual hulls on this context: list of (masks, transforms, level, cube_corner_bfl, "
                 "cube_length, masks_partial, transforms_convention, unique_verts) -> list of (verts, faces).")
            .def("device_bytes", &HullContext::device_bytes);
}
