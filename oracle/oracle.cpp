// CPU oracle for the visual-hull and Gaussian-blur path: TEST INFRASTRUCTURE.
// See oracle.h for what it is, what it is for and how far its parity is pinned.
//
// Build with -ffp-contract=off: only the explicit std::fma calls below may
// fuse, exactly where the reference's device code fuses (explicit fmaf, or an
// a*b+c that nvcc contracts under its default -fmad=true).

#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <limits>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../torchhull_gb300/csrc/mc_tables.h"

namespace
{

const uint8_t MC_COUNT[256] = TH_MC_TRI_COUNT_INIT;
const uint8_t MC_EDGES[256][15] = TH_MC_TRI_EDGES_INIT;

// ---------------------------------------------------------------------------
// element access

float half_to_float(uint16_t h)
{
    _Float16 v;
    std::memcpy(&v, &h, 2);
    return static_cast<float>(v);
}

float round_to_half(float f)
{
    return static_cast<float>(static_cast<_Float16>(f));
}

// Value of element i converted to float the way static_cast<float>(T) does.
float load_as_float(const void* p, int dtype, int64_t i)
{
    switch (dtype)
    {
    case ORACLE_BOOL:
        return static_cast<const uint8_t*>(p)[i] ? 1.f : 0.f;
    case ORACLE_UINT8:
        return static_cast<float>(static_cast<const uint8_t*>(p)[i]);
    case ORACLE_INT8:
        return static_cast<float>(static_cast<const int8_t*>(p)[i]);
    case ORACLE_INT16:
        return static_cast<float>(static_cast<const int16_t*>(p)[i]);
    case ORACLE_INT32:
        return static_cast<float>(static_cast<const int32_t*>(p)[i]);
    case ORACLE_INT64:
        return static_cast<float>(static_cast<const int64_t*>(p)[i]);
    case ORACLE_FLOAT16:
        return half_to_float(static_cast<const uint16_t*>(p)[i]);
    case ORACLE_FLOAT32:
        return static_cast<const float*>(p)[i];
    case ORACLE_FLOAT64:
        return static_cast<float>(static_cast<const double*>(p)[i]);
    default:
        return 0.f;
    }
}

double load_as_double(const void* p, int dtype, int64_t i)
{
    switch (dtype)
    {
    case ORACLE_INT64:
        return static_cast<double>(static_cast<const int64_t*>(p)[i]);
    case ORACLE_FLOAT64:
        return static_cast<const double*>(p)[i];
    default:
        return static_cast<double>(load_as_float(p, dtype, i));
    }
}

bool is_float_dtype(int d)
{
    return d == ORACLE_FLOAT16 || d == ORACLE_FLOAT32 || d == ORACLE_FLOAT64;
}

// ---------------------------------------------------------------------------
// device arithmetic rules

// float -> int64 the way the GPU converts (cvt.rzi.s64.f32): saturate, and
// NaN -> INT64_MIN (measured on GB300 by the arithmetic probe test).
int64_t f2i64(float f)
{
    if (std::isnan(f))
        return std::numeric_limits<int64_t>::min();
    if (f >= 9223372036854775808.0f)
        return std::numeric_limits<int64_t>::max();
    if (f <= -9223372036854775808.0f)
        return std::numeric_limits<int64_t>::min();
    return static_cast<int64_t>(f);
}

int64_t wrap_add(int64_t a, int64_t b)
{
    return static_cast<int64_t>(static_cast<uint64_t>(a) + static_cast<uint64_t>(b));
}
int64_t wrap_sub(int64_t a, int64_t b)
{
    return static_cast<int64_t>(static_cast<uint64_t>(a) - static_cast<uint64_t>(b));
}
int64_t wrap_mul(int64_t a, int64_t b)
{
    return static_cast<int64_t>(static_cast<uint64_t>(a) * static_cast<uint64_t>(b));
}

int64_t clamp64(int64_t v, int64_t lo, int64_t hi)
{
    return std::min(std::max(v, lo), hi);
}

// image_utils.h:56-60
bool in_image(int64_t y, int64_t x, int64_t h, int64_t w, int64_t margin = 0)
{
    return margin <= y && y < h - margin && margin <= x && x < w - margin;
}

// math.h:19-23
float lerp(float v0, float v1, float t)
{
    return std::fma(t, v1, std::fma(-t, v0, v0));
}

// math.h:25-32
float bilerp(float v00, float v10, float v01, float v11, float ty, float tx)
{
    float v0 = lerp(v00, v10, ty);
    float v1 = lerp(v01, v11, ty);
    return lerp(v0, v1, tx);
}

// image_utils.h:67-71
float unnormalize_ndc_false(float c, int64_t size)
{
    return (c + 1.f) * static_cast<float>(size) / 2.f - 0.5f;
}

// image_utils.h:78-82
float align_cv_false(float c)
{
    return c - 0.5f;
}

// visual_hull_cuda.cu:206-213 / :444-448.  nvcc contracts c + v/r*L into
// fma(v/r, L, c); v/r is exact here (r is a power of two).
float world_coordinate(int64_t v, int64_t r, float corner, float length)
{
    return std::fma(static_cast<float>(v) / static_cast<float>(r), length, corner);
}

struct Transform
{
    float a[16];
};

// visual_hull_cuda.cu:142-156 (matrix entries are narrowed to float by fmaf).
void project(const Transform& t, float x, float y, float z, float out[4])
{
    for (int i = 0; i < 4; ++i)
    {
        const float* r = t.a + 4 * i;
        out[i] = std::fma(r[0], x, std::fma(r[1], y, std::fma(r[2], z, r[3])));
    }
}

// visual_hull_cuda.cu:217-228 / :452-462
void to_pixel(const float c[4], bool opengl, int64_t H, int64_t W, float* px, float* py)
{
    if (opengl)
    {
        float nx = c[0] / c[3];
        float ny = c[1] / c[3];
        *px = unnormalize_ndc_false(nx, W);
        *py = unnormalize_ndc_false(ny, H);
    }
    else
    {
        float cx = c[0] / c[2];
        float cy = c[1] / c[2];
        *px = align_cv_false(cx);
        *py = align_cv_false(cy);
    }
}

void parallel_for(int64_t n, int nthreads, const std::function<void(int64_t, int64_t)>& body)
{
    if (n <= 0)
        return;
    int t = nthreads;
    if (t <= 0)
        t = static_cast<int>(std::max(1u, std::thread::hardware_concurrency()));
    int64_t chunks = std::min<int64_t>(t, std::max<int64_t>(1, n / 1024));
    if (chunks <= 1)
    {
        body(0, n);
        return;
    }
    std::vector<std::thread> pool;
    for (int64_t c = 0; c < chunks; ++c)
    {
        int64_t b = n * c / chunks, e = n * (c + 1) / chunks;
        pool.emplace_back([&body, b, e] { body(b, e); });
    }
    for (auto& th : pool)
        th.join();
}

// ---------------------------------------------------------------------------
// integral image: torch::cumsum over H then over W, float32, sequential order
// (visual_hull_cuda.cu:76-90; torch's outer-dimension scan accumulates one
// element at a time starting from 0).

void integral_image(const void* masks, int dt, int64_t B, int64_t H, int64_t W, float* out, int nthreads)
{
    parallel_for(B * W, nthreads, [&](int64_t b0, int64_t b1) {
        for (int64_t bx = b0; bx < b1; ++bx)
        {
            int64_t b = bx / W, x = bx % W;
            float acc = 0.f;
            for (int64_t y = 0; y < H; ++y)
            {
                int64_t i = (b * H + y) * W + x;
                acc = acc + load_as_float(masks, dt, i);
                out[i] = acc;
            }
        }
    });
    parallel_for(B * H, nthreads, [&](int64_t r0, int64_t r1) {
        for (int64_t r = r0; r < r1; ++r)
        {
            float acc = 0.f;
            float* row = out + r * W;
            for (int64_t x = 0; x < W; ++x)
            {
                acc = acc + row[x];
                row[x] = acc;
            }
        }
    });
}

// ---------------------------------------------------------------------------
// octree carving

struct HullSetup
{
    const void* masks;
    int masks_dtype;
    int64_t B, H, W;
    std::vector<Transform> transforms;
    std::vector<float> sat;
    int level;
    float corner[3];
    float length;
    bool partial;
    bool opengl;
};

struct I3
{
    int64_t x, y, z;
};

// image_utils.h:20-36
I3 unravel(int64_t idx, int64_t r)
{
    return I3{ idx % r, idx / r % r, idx / (r * r) };
}

// image_utils.h:38-54
int64_t ravel(const I3& p, int64_t r)
{
    return p.x + p.y * r + p.z * r * r;
}

// marching_cubes_utils.h:41-45
I3 cube_vertex(const I3& g, int i)
{
    return I3{ g.x + (i & 1), g.y + (i >> 1 & 1), g.z + (i >> 2 & 1) };
}

float sat_at(const HullSetup& s, int64_t b, int64_t y, int64_t x)
{
    // sample_zeros_padding, image_utils.h:84-97
    return in_image(y, x, s.H, s.W) ? s.sat[(b * s.H + y) * s.W + x] : 0.f;
}

// classify_children_full (visual_hull_cuda.cu:168-285) and
// classify_children_partial (:287-417) for one child cell gc at resolution rc.
bool classify_child(const HullSetup& s, const I3& gc, int64_t rc, bool last_children)
{
    bool is_empty = false;
    bool should_refine = false;
    bool fully_inside_one_frame = false;
    const float epsilon = 1e-1f;
    const float isolevel = 0.5f;
    const float margin = isolevel - epsilon;

    for (int64_t b = 0; b < s.B; ++b)
    {
        float bmin_x = std::numeric_limits<float>::max(), bmin_y = std::numeric_limits<float>::max();
        float bmax_x = -std::numeric_limits<float>::max(), bmax_y = -std::numeric_limits<float>::max();
        bool fully_inside = true;
        for (int i = 0; i < 8; ++i)
        {
            I3 v = cube_vertex(gc, i);
            float wx = world_coordinate(v.x, rc, s.corner[0], s.length);
            float wy = world_coordinate(v.y, rc, s.corner[1], s.length);
            float wz = world_coordinate(v.z, rc, s.corner[2], s.length);
            float cam[4];
            project(s.transforms[b], wx, wy, wz, cam);
            float px, py;
            to_pixel(cam, s.opengl, s.H, s.W, &px, &py);
            bmin_x = std::fmin(bmin_x, px);
            bmin_y = std::fmin(bmin_y, py);
            bmax_x = std::fmax(bmax_x, px);
            bmax_y = std::fmax(bmax_y, py);
            if (s.partial)
            {
                int64_t rx = f2i64(std::round(px));
                int64_t ry = f2i64(std::round(py));
                if (!in_image(ry, rx, s.H, s.W, 1))
                    fully_inside = false;
            }
        }

        int64_t rmin_x = f2i64(std::round(bmin_x + -0.5f));
        int64_t rmin_y = f2i64(std::round(bmin_y + -0.5f));
        int64_t rmax_x = f2i64(std::round(bmax_x + 0.5f));
        int64_t rmax_y = f2i64(std::round(bmax_y + 0.5f));

        int64_t cmin_x = clamp64(rmin_x, 0, s.W - 1);
        int64_t cmin_y = clamp64(rmin_y, 0, s.H - 1);
        int64_t cmax_x = clamp64(rmax_x, 0, s.W - 1);
        int64_t cmax_y = clamp64(rmax_y, 0, s.H - 1);

        int64_t area = (cmax_y - cmin_y + 1) * (cmax_x - cmin_x + 1);

        float i00 = sat_at(s, b, cmin_y - 1, cmin_x - 1);
        float i10 = sat_at(s, b, cmax_y, cmin_x - 1);
        float i01 = sat_at(s, b, cmin_y - 1, cmax_x);
        float i11 = sat_at(s, b, cmax_y, cmax_x);
        float sum = i11 + i00 - i10 - i01;

        if (!s.partial)
        {
            if (sum <= 0.f + margin)
                is_empty = true;
            else if (sum >= static_cast<float>(area) - margin)
            {
            }
            else
                should_refine = true;
        }
        else
        {
            int64_t full_area = wrap_mul(wrap_add(wrap_sub(rmax_y, rmin_y), 1), wrap_add(wrap_sub(rmax_x, rmin_x), 1));
            if (sum <= 0.f + margin && area == full_area)
                is_empty = true;
            else if (sum >= static_cast<float>(area) - margin && area == full_area)
            {
            }
            else if (cmax_y - cmin_y > 1 && cmax_x - cmin_x > 1)
                should_refine = true;
            fully_inside_one_frame |= fully_inside;
        }
    }
    if (!s.partial)
        return should_refine && !is_empty;
    return should_refine && !is_empty && (!last_children || fully_inside_one_frame);
}

// Level loop with stable compaction (visual_hull_cuda.cu:633-751).
std::vector<std::vector<int64_t>> carve(const HullSetup& s, int nthreads)
{
    std::vector<std::vector<int64_t>> levels;
    levels.push_back({ 0 });
    for (int i = 0; i < s.level; ++i)
    {
        const std::vector<int64_t>& parents = levels.back();
        const int64_t r = int64_t{ 1 } << i;
        const int64_t rc = int64_t{ 1 } << (i + 1);
        const int64_t n = 8 * static_cast<int64_t>(parents.size());
        std::vector<uint8_t> flags(n);
        const bool last = (i == s.level - 1);
        parallel_for(n, nthreads, [&](int64_t t0, int64_t t1) {
            for (int64_t t = t0; t < t1; ++t)
            {
                I3 g = unravel(parents[t / 8], r);
                I3 gc = cube_vertex(I3{ 2 * g.x, 2 * g.y, 2 * g.z }, static_cast<int>(t % 8));
                flags[t] = classify_child(s, gc, rc, last) ? 1 : 0;
            }
        });
        std::vector<int64_t> children;
        for (int64_t t = 0; t < n; ++t)
        {
            if (flags[t])
            {
                I3 g = unravel(parents[t / 8], r);
                I3 gc = cube_vertex(I3{ 2 * g.x, 2 * g.y, 2 * g.z }, static_cast<int>(t % 8));
                children.push_back(ravel(gc, rc));
            }
        }
        levels.push_back(std::move(children));
        if (levels.back().empty())
            break;
    }
    return levels;
}

// ---------------------------------------------------------------------------
// hull field

float mask_at(const HullSetup& s, int64_t b, int64_t y, int64_t x, float pad)
{
    return in_image(y, x, s.H, s.W) ? load_as_float(s.masks, s.masks_dtype, (b * s.H + y) * s.W + x) : pad;
}

// sample_bilinear_mode_{zeros,ones}_padding (image_utils.h:162-214)
float sample_bilinear(const HullSetup& s, int64_t b, float y, float x, float pad)
{
    int64_t yp = f2i64(std::round(y + -0.5f));
    int64_t xp = f2i64(std::round(x + -0.5f));
    float v00 = mask_at(s, b, yp, xp, pad);
    float v10 = mask_at(s, b, wrap_add(yp, 1), xp, pad);
    float v01 = mask_at(s, b, yp, wrap_add(xp, 1), pad);
    float v11 = mask_at(s, b, wrap_add(yp, 1), wrap_add(xp, 1), pad);
    float ty = y - static_cast<float>(yp);
    float tx = x - static_cast<float>(xp);
    return bilerp(v00, v10, v01, v11, ty, tx);
}

// accumulate_hull_counts_{full,partial} (visual_hull_cuda.cu:419-520), views
// applied in ascending order as the host loop :847-886 launches them.
float field_value(const HullSetup& s, int64_t corner_index, int64_t rgrid)
{
    I3 g = unravel(corner_index, rgrid);
    const int64_t rcells = rgrid - 1;
    float wx = world_coordinate(g.x, rcells, s.corner[0], s.length);
    float wy = world_coordinate(g.y, rcells, s.corner[1], s.length);
    float wz = world_coordinate(g.z, rcells, s.corner[2], s.length);
    float value = 1.f;
    for (int64_t b = 0; b < s.B; ++b)
    {
        float cam[4];
        project(s.transforms[b], wx, wy, wz, cam);
        float px, py;
        to_pixel(cam, s.opengl, s.H, s.W, &px, &py);
        if (!s.partial)
        {
            value *= sample_bilinear(s, b, py, px, 0.f);
        }
        else
        {
            int64_t rx = f2i64(std::round(px));
            int64_t ry = f2i64(std::round(py));
            if (in_image(ry, rx, s.H, s.W, 1))
                value *= sample_bilinear(s, b, py, px, 1.f);
        }
    }
    return value;
}

// ---------------------------------------------------------------------------
// sparse marching cubes (marching_cubes_cuda.cu:72-112, :180-223, :308-374,
// :535-707) and the finishing step (visual_hull_cuda.cu:916-1020)

struct F3
{
    float x, y, z;
};

// marching_cubes_cuda.cu:72-97
F3 interpolate_vertex(float iso, const I3& p1, const I3& p2, float v1, float v2)
{
    const float eps = 1e-5f;
    if (std::fabs(iso - v1) < eps)
        return F3{ float(p1.x), float(p1.y), float(p1.z) };
    if (std::fabs(iso - v2) < eps)
        return F3{ float(p2.x), float(p2.y), float(p2.z) };
    if (std::fabs(v1 - v2) < eps)
        return F3{ float(p1.x), float(p1.y), float(p1.z) };
    float t = (iso - v1) / (v2 - v1);
    return F3{ lerp(float(p1.x), float(p2.x), t), lerp(float(p1.y), float(p2.y), t), lerp(float(p1.z), float(p2.z), t) };
}

struct Mesh
{
    std::vector<float> verts;
    std::vector<int64_t> faces;
};

Mesh marching_cubes_sparse(const std::vector<int64_t>& idx,
                           const std::vector<float>& val,
                           int64_t R,
                           bool unique_verts,
                           int nthreads)
{
    Mesh mesh;
    const int64_t N = static_cast<int64_t>(idx.size());
    if (N == 0)
        return mesh;
    const float iso = 0.5f;

    // corner lookup (the role of the stdgpu map, marching_cubes_cuda.cu:133-144)
    auto find = [&](int64_t key) -> int64_t {
        auto it = std::lower_bound(idx.begin(), idx.end(), key);
        return (it != idx.end() && *it == key) ? (it - idx.begin()) : -1;
    };

    // classify_voxels_sparse (:180-223): cell code per corner, 0 if incomplete
    std::vector<uint8_t> code(N, 0);
    std::vector<int64_t> count(N, 0);
    parallel_for(N, nthreads, [&](int64_t t0, int64_t t1) {
        for (int64_t t = t0; t < t1; ++t)
        {
            I3 g = unravel(idx[t], R);
            uint8_t c = 0;
            if (g.x < R - 1 && g.y < R - 1 && g.z < R - 1)
            {
                for (int i = 0; i < 8; ++i)
                {
                    int64_t k = find(ravel(cube_vertex(g, i), R));
                    if (k < 0)
                    {
                        c = 0;
                        break;
                    }
                    if (val[k] < iso)
                        c |= static_cast<uint8_t>(1u << i);
                }
            }
            code[t] = c;
            count[t] = MC_COUNT[c];
        }
    });

    // exclusive scan of soup vertex counts (:626-635)
    std::vector<int64_t> offset(N + 1, 0);
    for (int64_t t = 0; t < N; ++t)
        offset[t + 1] = offset[t] + count[t];
    const int64_t V = offset[N];
    if (V == 0)
        return mesh;

    // generate_faces_sparse (:308-374)
    std::vector<float> soup(3 * V);
    std::vector<int64_t> ids(unique_verts ? V : 0);
    parallel_for(N, nthreads, [&](int64_t t0, int64_t t1) {
        for (int64_t t = t0; t < t1; ++t)
        {
            uint8_t c = code[t];
            if (MC_COUNT[c] == 0)
                continue;
            I3 g = unravel(idx[t], R);
            for (int j = 0; j < MC_COUNT[c]; ++j)
            {
                uint8_t e = MC_EDGES[c][j];
                int lo = e & 7, axis = e >> 3;
                I3 p1 = cube_vertex(g, lo);
                I3 p2 = cube_vertex(g, lo | (1 << axis));
                float v1 = val[find(ravel(p1, R))];
                float v2 = val[find(ravel(p2, R))];
                F3 v = interpolate_vertex(iso, p1, p2, v1, v2);
                int64_t o = offset[t] + j;
                soup[3 * o + 0] = v.x;
                soup[3 * o + 1] = v.y;
                soup[3 * o + 2] = v.z;
                if (unique_verts)
                    ids[o] = (ravel(p1, R) << 3) | (int64_t{ 1 } << axis);
            }
        }
    });

    // torch::unique_dim(sorted, return_inverse) + index_put_ (:674-693)
    if (unique_verts)
    {
        std::vector<int64_t> order(V);
        std::iota(order.begin(), order.end(), 0);
        std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return ids[a] < ids[b]; });
        std::vector<int64_t> inverse(V);
        int64_t u = -1;
        int64_t prev = -1;
        for (int64_t k = 0; k < V; ++k)
        {
            int64_t o = order[k];
            if (k == 0 || ids[o] != prev)
            {
                ++u;
                prev = ids[o];
                mesh.verts.push_back(soup[3 * o + 0]);
                mesh.verts.push_back(soup[3 * o + 1]);
                mesh.verts.push_back(soup[3 * o + 2]);
            }
            inverse[o] = u;
        }
        mesh.faces = std::move(inverse);
    }
    else
    {
        mesh.verts = std::move(soup);
        mesh.faces.resize(V);
        std::iota(mesh.faces.begin(), mesh.faces.end(), 0);
    }
    return mesh;
}

// to_global_coordinates + flip_faces (visual_hull_cuda.cu:916-956)
void finish(Mesh& m, const float corner[3], float length, int level)
{
    const float scale = length / static_cast<float>(int64_t{ 1 } << level);
    for (size_t i = 0; i < m.verts.size(); i += 3)
        for (int a = 0; a < 3; ++a)
            m.verts[i + a] = std::fma(scale, m.verts[i + a], corner[a]);
    for (size_t f = 0; f + 2 < m.faces.size(); f += 3)
        std::swap(m.faces[f + 1], m.faces[f + 2]);
}

void set_err(char* err, int errlen, const std::string& msg)
{
    if (err && errlen > 0)
        std::snprintf(err, static_cast<size_t>(errlen), "%s", msg.c_str());
}

const char* dtype_name(int d)
{
    static const char* names[] = { "Bool", "Byte", "Char", "Short", "Int", "Long", "Half", "Float", "Double", "BFloat16" };
    return (d >= 0 && d <= 9) ? names[d] : "Unknown";
}

} // namespace

struct oracle_hull
{
    std::vector<std::vector<int64_t>> levels;
    std::vector<int64_t> field_idx;
    std::vector<float> field_val;
    Mesh mesh;
};

extern "C" {

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
                                int errlen)
{
    // argument checks, visual_hull_cuda.cu:591-613 and the dtype dispatches :646, :832-845
    if (level < 0)
    {
        set_err(err, errlen, "level must be >= 0");
        return nullptr;
    }
    if (!(cube_length > 0.f))
    {
        set_err(err, errlen, "cube_length must be > 0");
        return nullptr;
    }
    if (!(transforms_dtype == ORACLE_FLOAT16 || transforms_dtype == ORACLE_FLOAT32 || transforms_dtype == ORACLE_FLOAT64))
    {
        set_err(err, errlen, std::string("\"classify_children\" not implemented for '") + dtype_name(transforms_dtype) + "'");
        return nullptr;
    }
    if (masks_dtype == ORACLE_BOOL || masks_dtype == ORACLE_BFLOAT16 || masks_dtype < 0 || masks_dtype > 9)
    {
        set_err(err, errlen, std::string("\"accumulate_hull_counts\" not implemented for '") + dtype_name(masks_dtype) + "'");
        return nullptr;
    }

    HullSetup s;
    s.masks = masks;
    s.masks_dtype = masks_dtype;
    s.B = B;
    s.H = H;
    s.W = W;
    s.level = level;
    s.corner[0] = corner_x;
    s.corner[1] = corner_y;
    s.corner[2] = corner_z;
    s.length = cube_length;
    s.partial = masks_partial != 0;
    s.opengl = transforms_opengl != 0;
    s.transforms.resize(B);
    for (int64_t b = 0; b < B; ++b)
        for (int k = 0; k < 16; ++k)
            s.transforms[b].a[k] = load_as_float(transforms, transforms_dtype, b * 16 + k);
    s.sat.resize(B * H * W);
    integral_image(masks, masks_dtype, B, H, W, s.sat.data(), nthreads);

    auto* out = new oracle_hull;
    out->levels = carve(s, nthreads);
    const std::vector<int64_t>& leaves = out->levels.back();
    if (leaves.empty())
        return out;

    // corners of the leaf cells, sorted and unique (visual_hull_cuda.cu:770-825)
    const int64_t rcells = int64_t{ 1 } << level;
    const int64_t rgrid = rcells + 1;
    std::vector<int64_t> corners(8 * leaves.size());
    for (size_t t = 0; t < corners.size(); ++t)
    {
        I3 g = unravel(leaves[t / 8], rcells);
        corners[t] = ravel(cube_vertex(g, static_cast<int>(t % 8)), rgrid);
    }
    std::sort(corners.begin(), corners.end());
    corners.erase(std::unique(corners.begin(), corners.end()), corners.end());

    const int64_t C = static_cast<int64_t>(corners.size());
    std::vector<float> values(C);
    parallel_for(C, nthreads, [&](int64_t c0, int64_t c1) {
        for (int64_t c = c0; c < c1; ++c)
            values[c] = field_value(s, corners[c], rgrid);
    });

    out->mesh = marching_cubes_sparse(corners, values, rgrid, unique_verts != 0, nthreads);
    finish(out->mesh, s.corner, cube_length, level);
    out->field_idx = std::move(corners);
    out->field_val = std::move(values);
    return out;
}

int64_t oracle_hull_num_levels(const oracle_hull* h)
{
    return static_cast<int64_t>(h->levels.size());
}
int64_t oracle_hull_level_size(const oracle_hull* h, int64_t i)
{
    return static_cast<int64_t>(h->levels[i].size());
}
void oracle_hull_level_copy(const oracle_hull* h, int64_t i, int64_t* dst)
{
    std::copy(h->levels[i].begin(), h->levels[i].end(), dst);
}
int64_t oracle_hull_field_size(const oracle_hull* h)
{
    return static_cast<int64_t>(h->field_idx.size());
}
void oracle_hull_field_copy(const oracle_hull* h, int64_t* indices, float* values)
{
    std::copy(h->field_idx.begin(), h->field_idx.end(), indices);
    std::copy(h->field_val.begin(), h->field_val.end(), values);
}
int64_t oracle_hull_num_verts(const oracle_hull* h)
{
    return static_cast<int64_t>(h->mesh.verts.size() / 3);
}
int64_t oracle_hull_num_faces(const oracle_hull* h)
{
    return static_cast<int64_t>(h->mesh.faces.size() / 3);
}
void oracle_hull_mesh_copy(const oracle_hull* h, float* verts, int64_t* faces)
{
    std::copy(h->mesh.verts.begin(), h->mesh.verts.end(), verts);
    std::copy(h->mesh.faces.begin(), h->mesh.faces.end(), faces);
}
void oracle_hull_free(oracle_hull* h)
{
    delete h;
}

int oracle_integral_image(const void* masks, int masks_dtype, int64_t B, int64_t H, int64_t W, float* out, int nthreads)
{
    integral_image(masks, masks_dtype, B, H, W, out, nthreads);
    return 0;
}

int64_t oracle_bilerp_ones_failures(uint32_t lo_bits, uint32_t hi_bits)
{
    int64_t bad = 0;
    for (uint64_t u = lo_bits; u <= hi_bits; ++u)
    {
        float t;
        const uint32_t b = static_cast<uint32_t>(u);
        std::memcpy(&t, &b, sizeof(float));
        if (bilerp(1.f, 1.f, 1.f, 1.f, t, t) != 1.f)
            ++bad;
    }
    return bad;
}

} // extern "C"

// ---------------------------------------------------------------------------
// Gaussian blur

namespace
{

// image_utils.h:129-160 (reflection without repeating the border sample)
int64_t reflect_index(int64_t y, int64_t n)
{
    if (n == 1)
        return 0;
    int64_t flips = y / (n - 1) + (y < 0 ? 1 : 0);
    int64_t rem = y % (n - 1);
    if (rem < 0)
        rem += n - 1;
    return (flips % 2 == 0) ? rem : (n - 1) - rem;
}

void store_value(void* out, int dtype, int64_t i, double v)
{
    switch (dtype)
    {
    case ORACLE_FLOAT16:
    {
        _Float16 h = static_cast<_Float16>(static_cast<float>(v));
        std::memcpy(static_cast<uint16_t*>(out) + i, &h, 2);
        break;
    }
    case ORACLE_FLOAT32:
        static_cast<float*>(out)[i] = static_cast<float>(v);
        break;
    case ORACLE_FLOAT64:
        static_cast<double*>(out)[i] = v;
        break;
    default:
        break;
    }
}

// images.clone().to(dtype) for one element
void store_converted(const void* in, int idt, void* out, int odt, int64_t i)
{
    if (odt == ORACLE_FLOAT64)
        static_cast<double*>(out)[i] = load_as_double(in, idt, i);
    else if (odt == ORACLE_FLOAT32)
        static_cast<float*>(out)[i] = load_as_float(in, idt, i);
    else
    {
        // c10::Half from double goes through float; from integers through float.
        float f = (idt == ORACLE_FLOAT64) ? static_cast<float>(static_cast<const double*>(in)[i]) : load_as_float(in, idt, i);
        store_value(out, odt, i, f);
    }
}

// Value of input element i as the accumulation type of the output.
double image_value(const void* in, int idt, int odt, int64_t i)
{
    if (odt == ORACLE_FLOAT64)
        return load_as_double(in, idt, i);
    if (odt == ORACLE_FLOAT32)
        return static_cast<double>(load_as_float(in, idt, i));
    float f = (idt == ORACLE_FLOAT64) ? static_cast<float>(static_cast<const double*>(in)[i]) : load_as_float(in, idt, i);
    return round_to_half(f);
}

bool values_differ(const void* in, int idt, int64_t a, int64_t b)
{
    if (idt == ORACLE_INT64)
        return static_cast<const int64_t*>(in)[a] != static_cast<const int64_t*>(in)[b];
    if (idt == ORACLE_FLOAT64)
        return static_cast<const double*>(in)[a] != static_cast<const double*>(in)[b];
    return load_as_float(in, idt, a) != load_as_float(in, idt, b);
}

// tile_convolution_kernel (gaussian_blur_cuda.cu:234-286): 2-D taps, x offset
// outer, y offset inner, one expf per tap, per-pixel normalisation.
double blur_pixel(const void* in, int idt, int odt, int64_t H, int64_t W, int64_t b, int64_t y, int64_t x, int k, float sigma)
{
    const int r = k / 2;
    const float den = 2.f * sigma * sigma;
    if (odt == ORACLE_FLOAT32)
    {
        float acc = 0.f, norm = 0.f;
        for (int i = -r; i <= r; ++i)
            for (int j = -r; j <= r; ++j)
            {
                int64_t yy = reflect_index(y + j, H), xx = reflect_index(x + i, W);
                float iv = static_cast<float>(image_value(in, idt, odt, (b * H + yy) * W + xx));
                float kv = std::exp(-static_cast<float>(i * i + j * j) / den);
                acc = std::fma(kv, iv, acc);
                norm = norm + kv;
            }
        return acc / norm;
    }
    if (odt == ORACLE_FLOAT64)
    {
        double acc = 0.0, norm = 0.0;
        for (int i = -r; i <= r; ++i)
            for (int j = -r; j <= r; ++j)
            {
                int64_t yy = reflect_index(y + j, H), xx = reflect_index(x + i, W);
                double iv = image_value(in, idt, odt, (b * H + yy) * W + xx);
                double kv = static_cast<double>(std::exp(-static_cast<float>(i * i + j * j) / den));
                acc = std::fma(kv, iv, acc);
                norm = norm + kv;
            }
        return acc / norm;
    }
    // c10::Half: every operation rounds back to half
    float acc = 0.f, norm = 0.f;
    for (int i = -r; i <= r; ++i)
        for (int j = -r; j <= r; ++j)
        {
            int64_t yy = reflect_index(y + j, H), xx = reflect_index(x + i, W);
            float iv = static_cast<float>(image_value(in, idt, odt, (b * H + yy) * W + xx));
            float kv = round_to_half(std::exp(-static_cast<float>(i * i + j * j) / den));
            acc = round_to_half(acc + round_to_half(kv * iv));
            norm = round_to_half(norm + kv);
        }
    return round_to_half(acc / norm);
}

} // namespace

extern "C" int oracle_gaussian_blur(const void* images,
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
                                    int errlen)
{
    // gaussian_blur_cuda.cu:294-305, :79-81
    if (kernel_size <= 0)
    {
        set_err(err, errlen, "kernel_size must be > 0");
        return 1;
    }
    if (kernel_size % 2 != 1)
    {
        set_err(err, errlen, "kernel_size must be odd");
        return 1;
    }
    if (!(sigma > 0.f))
    {
        set_err(err, errlen, "sigma must be > 0");
        return 1;
    }
    if (!is_float_dtype(out_dtype))
    {
        set_err(err, errlen, "dtype must be a floating point type");
        return 1;
    }
    if (images_dtype == ORACLE_BOOL || images_dtype == ORACLE_BFLOAT16)
    {
        set_err(err, errlen, std::string("\"edge_kernel\" not implemented for '") + dtype_name(images_dtype) + "'");
        return 1;
    }
    const int64_t N = B * H * W;
    for (int64_t i = 0; i < N; ++i)
        store_converted(images, images_dtype, out, out_dtype, i);
    if (kernel_size == 1)
        return 0;

    const int r = kernel_size / 2;
    if (!sparse)
    {
        // gaussian_blur_cuda.cu:20-114: normalised kernel, reflect pad, conv2d.
        // The reference's conv2d accumulation order belongs to cuDNN; this
        // computes the same sum in double, which is within its tolerance.
        const int k = kernel_size;
        std::vector<double> wk(k * k);
        double sum = 0.0;
        for (int y = 0; y < k; ++y)
            for (int x = 0; x < k; ++x)
            {
                float e = std::exp(-static_cast<float>((y - r) * (y - r) + (x - r) * (x - r)) / (2.f * sigma * sigma));
                double v = (out_dtype == ORACLE_FLOAT16) ? round_to_half(e) : static_cast<double>(e);
                wk[y * k + x] = v;
                sum += v;
            }
        for (auto& v : wk)
            v /= sum;
        parallel_for(B * H, nthreads, [&](int64_t r0, int64_t r1) {
            for (int64_t row = r0; row < r1; ++row)
            {
                int64_t b = row / H, y = row % H;
                for (int64_t x = 0; x < W; ++x)
                {
                    double acc = 0.0;
                    for (int ky = 0; ky < k; ++ky)
                        for (int kx = 0; kx < k; ++kx)
                        {
                            int64_t yy = reflect_index(y + ky - r, H), xx = reflect_index(x + kx - r, W);
                            acc += wk[ky * k + kx] * image_value(images, images_dtype, out_dtype, (b * H + yy) * W + xx);
                        }
                    store_value(out, out_dtype, (b * H + y) * W + x, acc);
                }
            }
        });
        return 0;
    }

    // sparse: edge pixels (gaussian_blur_cuda.cu:116-142)
    const int64_t ts = kernel_size / 2;
    const int64_t TW = W / ts + 1, TH = H / ts + 1;
    std::vector<uint8_t> active(B * TW * TH, 0);
    bool any_edge = false;
    for (int64_t b = 0; b < B; ++b)
        for (int64_t y = 0; y < H; ++y)
            for (int64_t x = 0; x < W; ++x)
            {
                int64_t i = (b * H + y) * W + x;
                bool edge = (x + 1 < W && values_differ(images, images_dtype, i, i + 1)) ||
                            (y + 1 < H && values_differ(images, images_dtype, i, i + W));
                if (!edge)
                    continue;
                any_edge = true;
                // all_tile_indices_kernel (:144-178): 3x3 tile window, clamped
                for (int di = -1; di <= 1; ++di)
                    for (int dj = -1; dj <= 1; ++dj)
                    {
                        int64_t tx = clamp64(x / ts + di, 0, W / ts);
                        int64_t ty = clamp64(y / ts + dj, 0, H / ts);
                        active[(b * TH + ty) * TW + tx] = 1;
                    }
            }
    if (!any_edge)
        return 0;
    parallel_for(B * TH * TW, nthreads, [&](int64_t t0, int64_t t1) {
        for (int64_t t = t0; t < t1; ++t)
        {
            if (!active[t])
                continue;
            int64_t b = t / (TH * TW), ty = t / TW % TH, tx = t % TW;
            for (int64_t ly = 0; ly < ts; ++ly)
                for (int64_t lx = 0; lx < ts; ++lx)
                {
                    int64_t y = ty * ts + ly, x = tx * ts + lx;
                    if (!in_image(y, x, H, W))
                        continue;
                    double v = blur_pixel(images, images_dtype, out_dtype, H, W, b, y, x, kernel_size, sigma);
                    store_value(out, out_dtype, (b * H + y) * W + x, v);
                }
        }
    });
    return 0;
}

// ---------------------------------------------------------------------------
// public marching cubes (marching_cubes_cuda.cu:146-374 kernels, :376-533
// dense driver, :535-831 sparse driver), over a list of grid points

namespace
{

struct McGrid
{
    int64_t W, H, D; // sizes along x, y, z
};

int64_t mc_ravel(const I3& p, const McGrid& g)
{
    return p.x + g.W * (p.y + g.H * p.z);
}

I3 mc_unravel(int64_t id, const McGrid& g)
{
    I3 p;
    p.x = id % g.W;
    p.y = (id / g.W) % g.H;
    p.z = id / (g.W * g.H);
    return p;
}

// points: strictly ascending ravel ids; values: each point's value as a double
// (exact for half, float and double volumes).  A dense volume is the list of
// all its points, which turns the dense driver's cell loop (:146-178) into the
// sparse driver's entry loop (:180-223) over the same cells in the same order.
Mesh marching_cubes_points(const std::vector<int64_t>& ids,
                           const std::vector<double>& vals,
                           const McGrid& grid,
                           float iso,
                           bool unique_verts,
                           bool local,
                           int nthreads)
{
    Mesh mesh;
    const int64_t N = static_cast<int64_t>(ids.size());
    if (N == 0)
        return mesh;
    auto find = [&](int64_t key) -> int64_t {
        auto it = std::lower_bound(ids.begin(), ids.end(), key);
        return (it != ids.end() && *it == key) ? (it - ids.begin()) : -1;
    };
    // value < isolevel in the value's type (:166-171); val[] holds floats (:338-343)
    auto below = [&](int64_t k) { return vals[k] < static_cast<double>(iso); };

    std::vector<uint8_t> code(N, 0);
    std::vector<int64_t> count(N, 0);
    parallel_for(N, nthreads, [&](int64_t t0, int64_t t1) {
        for (int64_t t = t0; t < t1; ++t)
        {
            I3 g = mc_unravel(ids[t], grid);
            uint8_t c = 0;
            if (g.x < grid.W - 1 && g.y < grid.H - 1 && g.z < grid.D - 1)
            {
                for (int i = 0; i < 8; ++i)
                {
                    int64_t k = find(mc_ravel(cube_vertex(g, i), grid));
                    if (k < 0)
                    {
                        c = 0;
                        break;
                    }
                    if (below(k))
                        c |= static_cast<uint8_t>(1u << i);
                }
            }
            code[t] = c;
            count[t] = MC_COUNT[c];
        }
    });

    std::vector<int64_t> offset(N + 1, 0);
    for (int64_t t = 0; t < N; ++t)
        offset[t + 1] = offset[t] + count[t];
    const int64_t V = offset[N];
    if (V == 0)
        return mesh;

    // generate_faces_{dense,sparse} (:242-374)
    std::vector<float> soup(3 * V);
    std::vector<int64_t> edge_ids(unique_verts ? V : 0);
    parallel_for(N, nthreads, [&](int64_t t0, int64_t t1) {
        for (int64_t t = t0; t < t1; ++t)
        {
            uint8_t c = code[t];
            if (MC_COUNT[c] == 0)
                continue;
            I3 g = mc_unravel(ids[t], grid);
            for (int j = 0; j < MC_COUNT[c]; ++j)
            {
                uint8_t e = MC_EDGES[c][j];
                int lo = e & 7, axis = e >> 3;
                I3 p1 = cube_vertex(g, lo);
                I3 p2 = cube_vertex(g, lo | (1 << axis));
                float v1 = static_cast<float>(vals[find(mc_ravel(p1, grid))]);
                float v2 = static_cast<float>(vals[find(mc_ravel(p2, grid))]);
                F3 v = interpolate_vertex(iso, p1, p2, v1, v2);
                int64_t o = offset[t] + j;
                soup[3 * o + 0] = v.x;
                soup[3 * o + 1] = v.y;
                soup[3 * o + 2] = v.z;
                if (unique_verts)
                    edge_ids[o] = (mc_ravel(p1, grid) << 3) | (int64_t{ 1 } << axis); // hash_edge (:99-112)
            }
        }
    });

    // unique_dim(sorted, return_inverse) + index_put_ (:500-511)
    if (unique_verts)
    {
        std::vector<int64_t> order(V);
        std::iota(order.begin(), order.end(), 0);
        std::sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return edge_ids[a] < edge_ids[b]; });
        std::vector<int64_t> inverse(V);
        int64_t u = -1;
        int64_t prev = -1;
        for (int64_t k = 0; k < V; ++k)
        {
            int64_t o = order[k];
            if (k == 0 || edge_ids[o] != prev)
            {
                ++u;
                prev = edge_ids[o];
                mesh.verts.push_back(soup[3 * o + 0]);
                mesh.verts.push_back(soup[3 * o + 1]);
                mesh.verts.push_back(soup[3 * o + 2]);
            }
            inverse[o] = u;
        }
        mesh.faces = std::move(inverse);
    }
    else
    {
        mesh.verts = std::move(soup);
        mesh.faces.resize(V);
        std::iota(mesh.faces.begin(), mesh.faces.end(), 0);
    }

    // local coordinates: verts * (2 / (size - 1)) - 1, two rounded operations (:513-520)
    if (local)
    {
        const float scale[3] = { 2.f / static_cast<float>(grid.W - 1), 2.f / static_cast<float>(grid.H - 1),
                                 2.f / static_cast<float>(grid.D - 1) };
        for (size_t i = 0; i < mesh.verts.size(); i += 3)
            for (int a = 0; a < 3; ++a)
            {
                const float m = mesh.verts[i + a] * scale[a];
                mesh.verts[i + a] = m - 1.f;
            }
    }
    return mesh;
}

} // namespace

struct oracle_mesh
{
    Mesh mesh;
};

extern "C" {

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
                                   int errlen)
{
    if (!(values_dtype == ORACLE_FLOAT16 || values_dtype == ORACLE_FLOAT32 || values_dtype == ORACLE_FLOAT64))
    {
        set_err(err, errlen, std::string("marching cubes not implemented for '") + dtype_name(values_dtype) + "'");
        return nullptr;
    }
    if (depth < 2 || height < 2 || width < 2)
    {
        set_err(err, errlen, "volume sizes must be at least 2");
        return nullptr;
    }
    std::vector<int64_t> pts(ids, ids + n);
    for (int64_t i = 1; i < n; ++i)
        if (pts[i] <= pts[i - 1])
        {
            set_err(err, errlen, "point ids must be strictly ascending");
            return nullptr;
        }
    std::vector<double> vals(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i)
        vals[i] = load_as_double(values, values_dtype, i);
    auto* out = new oracle_mesh;
    out->mesh = marching_cubes_points(pts, vals, McGrid{ width, height, depth }, isolevel, unique_verts != 0,
                                      return_local_coords != 0, nthreads);
    return out;
}

int64_t oracle_mesh_num_verts(const oracle_mesh* m)
{
    return static_cast<int64_t>(m->mesh.verts.size() / 3);
}

int64_t oracle_mesh_num_faces(const oracle_mesh* m)
{
    return static_cast<int64_t>(m->mesh.faces.size() / 3);
}

void oracle_mesh_copy(const oracle_mesh* m, float* verts, int64_t* faces)
{
    std::copy(m->mesh.verts.begin(), m->mesh.verts.end(), verts);
    std::copy(m->mesh.faces.begin(), m->mesh.faces.end(), faces);
}

void oracle_mesh_free(oracle_mesh* m)
{
    delete m;
}

} // extern "C"

// ---------------------------------------------------------------------------
// candidate_voxels_to_wireframes (visual_hull_cuda.cu:1024-1111), one level

extern "C" void oracle_candidate_wireframe(const int64_t* candidates,
                                           int64_t n,
                                           int level_index,
                                           float corner_x,
                                           float corner_y,
                                           float corner_z,
                                           float cube_length,
                                           float* verts,
                                           int64_t* edges)
{
    // edge_to_vertex_table (marching_cubes_table.h:335-338)
    static const int e2v[12][2] = { { 0, 1 }, { 1, 5 }, { 4, 5 }, { 0, 4 }, { 2, 3 }, { 3, 7 },
                                    { 6, 7 }, { 2, 6 }, { 0, 2 }, { 1, 3 }, { 5, 7 }, { 4, 6 } };
    const int64_t r = int64_t{ 1 } << level_index;
    const float step = cube_length / static_cast<float>(r);
    const float c[3] = { corner_x, corner_y, corner_z };
    for (int64_t t = 0; t < n; ++t)
    {
        const int64_t id = candidates[t];
        const int64_t g[3] = { id % r, (id / r) % r, id / (r * r) };
        for (int i = 0; i < 8; ++i)
            for (int a = 0; a < 3; ++a)
                verts[3 * (8 * t + i) + a] = std::fma(step, static_cast<float>(g[a] + ((i >> a) & 1)), c[a]);
        for (int i = 0; i < 12; ++i)
        {
            edges[2 * (12 * t + i) + 0] = 8 * t + e2v[i][0];
            edges[2 * (12 * t + i) + 1] = 8 * t + e2v[i][1];
        }
    }
}
