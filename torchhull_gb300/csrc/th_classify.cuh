// Per-(parent, view) carve routine shared by the plain and the batched
// carve kernels: the 3x3x3 lattice of a parent projected into one view and
// the classification of its eight children (see carve.cu for the design).
#pragma once

#include <cfloat>

#include "th_common.cuh"

namespace th
{

struct Box
{
    float minx, miny, maxx, maxy;
};

__device__ __forceinline__ Box merge(const Box& a, const Box& b)
{
    return Box{ fminf(a.minx, b.minx), fminf(a.miny, b.miny), fmaxf(a.maxx, b.maxx), fmaxf(a.maxy, b.maxy) };
}

// Saturating float -> int32 (NaN to a value outside every image).
__device__ __forceinline__ int32_t f2i32(float f)
{
    return __float2int_rz(f);
}

__device__ __forceinline__ bool fits_i32(float f)
{
    return f > -2147483648.0f && f < 2147483648.0f;
}

__device__ __forceinline__ float box_sum(const float* __restrict__ sat_b, int32_t W, int32_t x0, int32_t y0, int32_t x1, int32_t y1)
{
    // sample_zeros_padding at the four corners (image_utils.h:84-97); inputs are
    // clamped to the image, so only the -1 row/column can leave it.
    const float* row_hi = sat_b + static_cast<int64_t>(y1) * W;
    const float* row_lo = sat_b + static_cast<int64_t>(y0 - 1) * W;
    const float i11 = row_hi[x1];
    const float i10 = x0 > 0 ? row_hi[x0 - 1] : 0.f;
    const float i01 = y0 > 0 ? row_lo[x1] : 0.f;
    const float i00 = (x0 > 0 && y0 > 0) ? row_lo[x0 - 1] : 0.f;
    return __fsub_rn(__fsub_rn(__fadd_rn(i11, i00), i10), i01);
}

enum ViewClass : uint32_t
{
    kNone = 0,
    kEmpty = 1,
    kRefine = 2,
    kObject = 3,
};

struct ViewResult
{
    uint32_t cls;
    bool skip; // the child's children may skip this view
};

// One child in one view from its pixel box (visual_hull_cuda.cu:236-285 and
// :365-410).  The box starts the reference's min/max from +-FLT_MAX.
// want_skip: evaluate the skip rule (the caller checked corners in front and,
// if needed, two pixels inside).  1 <= H, W < 2^23; Hf, Wf the same as floats.
template <bool PARTIAL>
__device__ __forceinline__ ViewResult classify_view(const float* __restrict__ sat_b, int32_t H, int32_t W, float Hf, float Wf, Box bb, bool want_skip, int grow = 2)
{
    const float margin = 0.5f - 0.1f; // isolevel - epsilon (visual_hull_cuda.cu:259-267)
    bb.minx = fminf(FLT_MAX, bb.minx);
    bb.miny = fminf(FLT_MAX, bb.miny);
    bb.maxx = fmaxf(-FLT_MAX, bb.maxx);
    bb.maxy = fmaxf(-FLT_MAX, bb.maxy);
    const float vminx = __fadd_rn(bb.minx, -0.5f);
    const float vminy = __fadd_rn(bb.miny, -0.5f);
    const float vmaxx = __fadd_rn(bb.maxx, 0.5f);
    const float vmaxy = __fadd_rn(bb.maxy, 0.5f);
    // the rounded corners clamped to the image
    const Snapped x0 = round_clamp(vminx, __fsub_rn(Wf, 1.f));
    const Snapped y0 = round_clamp(vminy, __fsub_rn(Hf, 1.f));
    const Snapped x1 = round_clamp(vmaxx, __fsub_rn(Wf, 1.f));
    const Snapped y1 = round_clamp(vmaxy, __fsub_rn(Hf, 1.f));
    // every rounded corner inside the image (the clamps were no-ops): round(v)
    // is in [0, size - 1] exactly when v is in (-0.5, size - 0.5)
    const float hx = __fsub_rn(Wf, 0.5f), hy = __fsub_rn(Hf, 0.5f);
    const bool framed = vminx > -0.5f && vminx < hx && vmaxx > -0.5f && vmaxx < hx && vminy > -0.5f &&
                        vminy < hy && vmaxy > -0.5f && vmaxy < hy;
    if (PARTIAL && !framed && fabsf(vminx) < 4194304.f && fabsf(vmaxx) < 4194304.f && fabsf(vminy) < 4194304.f &&
        fabsf(vmaxy) < 4194304.f)
    {
        // Not "whole": with |v| < 2^22 the rounded box spans at least 2
        // pixels per axis (v_max - v_min >= 1 and round(v + 1) >= round(v) + 1),
        // so on an axis that leaves the image the clamp shortens it and the
        // clamped area is below the unclamped one.  Neither empty nor object
        // then, and the sum is not needed.
        ViewResult res{ kNone, false };
        if (y1.i - y0.i > 1 && x1.i - x0.i > 1)
            res.cls = kRefine;
        return res;
    }
    const float sum = box_sum(sat_b, W, x0.i, y0.i, x1.i, y1.i);
    // float(area) of the int64 area: a product of two exact integers, rounded once
    const float area_f = __fmul_rn(__fadd_rn(__fsub_rn(y1.f, y0.f), 1.f), __fadd_rn(__fsub_rn(x1.f, x0.f), 1.f));
    bool whole = true;
    if (PARTIAL && !framed)
    {
        // full_area_bb (:377) from the unclamped rounded box, int64 arithmetic
        // wrapping like the device's; exact int64 values when int32 cannot hold them.
        const float fminx = roundf(vminx), fminy = roundf(vminy);
        const float fmaxx = roundf(vmaxx), fmaxy = roundf(vmaxy);
        int64_t rminx, rminy, rmaxx, rmaxy;
        if (fits_i32(fminx) && fits_i32(fminy) && fits_i32(fmaxx) && fits_i32(fmaxy))
        {
            rminx = f2i32(fminx);
            rminy = f2i32(fminy);
            rmaxx = f2i32(fmaxx);
            rmaxy = f2i32(fmaxy);
        }
        else
        {
            rminx = f2i64(fminx);
            rminy = f2i64(fminy);
            rmaxx = f2i64(fmaxx);
            rmaxy = f2i64(fmaxy);
        }
        const int64_t area = static_cast<int64_t>(y1.i - y0.i + 1) * static_cast<int64_t>(x1.i - x0.i + 1);
        const uint64_t fy = static_cast<uint64_t>(rmaxy) - static_cast<uint64_t>(rminy) + 1u;
        const uint64_t fx = static_cast<uint64_t>(rmaxx) - static_cast<uint64_t>(rminx) + 1u;
        whole = (static_cast<uint64_t>(area) == fy * fx);
    }
    ViewResult res{ kNone, false };
    if (sum <= 0.f + margin && whole)
        res.cls = kEmpty;
    else if (sum >= __fsub_rn(area_f, margin) && whole)
        res.cls = kObject;
    else if (!PARTIAL || (y1.i - y0.i > 1 && x1.i - x0.i > 1))
        res.cls = kRefine;
    if (want_skip && res.cls == kObject && framed && x0.i >= grow && y0.i >= grow && x1.i <= W - 1 - grow &&
        y1.i <= H - 1 - grow && x0.i <= x1.i && y0.i <= y1.i)
    {
        // the box grown by `grow` pixels is inside the image: all ones there?
        const int32_t gx0 = x0.i - grow, gy0 = y0.i - grow, gx1 = x1.i + grow, gy1 = y1.i + grow;
        const float grown = box_sum(sat_b, W, gx0, gy0, gx1, gy1);
        const float g2 = grow == 1 ? 3.f : 5.f; // 2 * grow + 1
        res.skip = grown == __fmul_rn(__fadd_rn(__fsub_rn(y1.f, y0.f), g2), __fadd_rn(__fsub_rn(x1.f, x0.f), g2));
    }
    return res;
}

#ifndef TH_CARVE_ROLL_Z
#define TH_CARVE_ROLL_Z 1
#endif

struct ItemResult
{
    uint32_t empty, refine, inside, skip; // 8-bit child masks
    uint32_t out;                         // children out of the frame for good (partial mode, want_out)
};

// Partial mode: a child box (from corners all in front of the camera) more
// than 2 pixels outside the image on one side, with every coordinate below
// 2^21 in magnitude.  Every descendant's corners project into this box up to
// rounding errors far below a pixel, so every descendant's box leaves the
// frame on that side too: never whole, a clamped extent of one pixel there
// (not refined), no corner in frame (not inside).  Such a view contributes
// nothing to any descendant and is skipped below.
__device__ __forceinline__ bool box_out(const Box& bb, float Hf, float Wf)
{
    const float lim = 2097152.f;
    return (bb.maxx < -2.f || bb.minx > __fadd_rn(Wf, 1.f) || bb.maxy < -2.f || bb.miny > __fadd_rn(Hf, 1.f)) &&
           fabsf(bb.minx) < lim && fabsf(bb.maxx) < lim && fabsf(bb.miny) < lim && fabsf(bb.maxy) < lim;
}

// Shared-memory accumulators of one warp's chunk of parents (one slot each).
struct WarpSlots
{
    uint32_t empty[32], refine[32], inside[32];
    uint32_t cskip[32][8];
    // out-of-frame view masks of the children: per child, and for all 8
    uint32_t cout[32][8], cout_all[32];
};

// Position of the j-th set bit of m (j < popc(m)).
__device__ __forceinline__ int select_bit(uint32_t m, int j)
{
    for (int t = 0; t < j; ++t)
        m &= m - 1;
    return __ffs(m) - 1;
}

// World coordinates of the lattice of the cell idx (ravelled at resolution
// 2^li): c + v/r * L with the product fused (visual_hull_cuda.cu:206-213);
// v/r == v * (1/r) exactly (r = 2^k).
__device__ __forceinline__ void lattice_world(const float corner[3],
                                              float length,
                                              int64_t idx,
                                              int li,
                                              float inv_rc,
                                              float wx[3],
                                              float wy[3],
                                              float wz[3])
{
    const int64_t mask = (int64_t{ 1 } << li) - 1;
    const int32_t gx = static_cast<int32_t>(idx & mask), gy = static_cast<int32_t>((idx >> li) & mask),
                  gz = static_cast<int32_t>(idx >> (2 * li));
#pragma unroll
    for (int d = 0; d < 3; ++d)
    {
        // lattice coordinates below 2^(li + 1) <= 2^14
        wx[d] = __fmaf_rn(__fmul_rn(small_i2f(2 * gx + d), inv_rc), length, corner[0]);
        wy[d] = __fmaf_rn(__fmul_rn(small_i2f(2 * gy + d), inv_rc), length, corner[1]);
        wz[d] = __fmaf_rn(__fmul_rn(small_i2f(2 * gz + d), inv_rc), length, corner[2]);
    }
}

// The per-view data an item reads.
struct ViewSource
{
    const float* tf;  // [B,16] float32 transforms
    const float* sat; // [B,H,W] integral images
    int64_t H, W;     // below 2^23
    float Hf, Wf;     // H, W as floats
};

__device__ __forceinline__ ViewSource make_view_source(const float* tf, const float* sat, int64_t H, int64_t W)
{
    return ViewSource{ tf, sat, H, W, small_i2f(static_cast<int32_t>(H)), small_i2f(static_cast<int32_t>(W)) };
}

// One (parent, view) item: the parent's lattice projected into view b.
// want_skip: compute the children's skip bits; skip_inside: the skip rule also
// needs the child's corners two pixels inside the frame; want_out (partial
// mode): compute the children's out-of-frame bits (box_out); grow: the skip
// rule's margin in pixels, 2 for masks inherited by all descendants, 1 for the
// children whose own children are leaves (one level below them, and the
// field's bilinear footprints of the leaves' corners, stay within one pixel);
// want_inside (partial mode): compute the children's "fully inside" bits (only
// the last level uses them).
//
// "Every corner rounds into the frame" (a pixel coordinate q passes when
// 0.5 <= q < size - 1.5, NaN fails) is tested on the child's box: for corners
// without NaN it holds for all eight exactly when it holds for the box's
// minimum and maximum, so the box test plus a NaN bit per lattice point gives
// the per-corner answer (fminf/fmaxf leave NaN out of the box).
template <bool PARTIAL, bool OPENGL>
__device__ __forceinline__ ItemResult classify_item(const ViewSource& p,
                                                    int64_t b,
                                                    const float wx[3],
                                                    const float wy[3],
                                                    const float wz[3],
                                                    bool want_skip,
                                                    bool skip_inside,
                                                    bool want_out = false,
                                                    int grow = 2,
                                                    bool want_inside = true)
{
    const int32_t H = static_cast<int32_t>(p.H), W = static_cast<int32_t>(p.W);
    const float Hf = p.Hf, Wf = p.Wf;
    const float* m = p.tf + 16 * b;
    // rows x, y and the divisor row (w for OpenGL, z for OpenCV)
    const float4 rx = *reinterpret_cast<const float4*>(m);
    const float4 ry = *reinterpret_cast<const float4*>(m + 4);
    const float4 rd = *reinterpret_cast<const float4*>(m + (OPENGL ? 12 : 8));
    const float* sat_b = p.sat + b * p.H * p.W;
    const float in_hx = __fsub_rn(Wf, 1.5f), in_hy = __fsub_rn(Hf, 1.5f);
    const float in2_hx = __fsub_rn(Wf, 2.5f), in2_hy = __fsub_rn(Hf, 2.5f);
    ItemResult out{ 0, 0, 0, 0, 0 };
    want_out = PARTIAL && want_out;
    want_inside = PARTIAL && want_inside;
    const bool want_in2 = PARTIAL && want_skip && skip_inside;
    const bool want_nan = want_inside || want_in2;
    Box prev[4];
    uint32_t prev_nan = 0, prev_front = 0;
    // Rolled (the default), the plane loop keeps one copy of the plane's code,
    // a third of the unrolled footprint: 9-11 % faster carve levels on GB300
    // (fewer instruction-fetch stalls); unrolled, it schedules across planes.
#if TH_CARVE_ROLL_Z
#pragma unroll 1
#else
#pragma unroll
#endif
    for (int z = 0; z < 3; ++z)
    {
        const float wzz = z == 0 ? wz[0] : (z == 1 ? wz[1] : wz[2]);
        const float tzx = __fmaf_rn(rx.z, wzz, rx.w);
        const float tzy = __fmaf_rn(ry.z, wzz, ry.w);
        const float tzd = __fmaf_rn(rd.z, wzz, rd.w);
        float px[9], py[9];
        uint32_t nan9 = 0, front9 = 0;
#pragma unroll
        for (int y = 0; y < 3; ++y)
        {
            const float tyx = __fmaf_rn(rx.y, wy[y], tzx);
            const float tyy = __fmaf_rn(ry.y, wy[y], tzy);
            const float tyd = __fmaf_rn(rd.y, wy[y], tzd);
#pragma unroll
            for (int x = 0; x < 3; ++x)
            {
                const int k = x + 3 * y;
                const float cx = __fmaf_rn(rx.x, wx[x], tyx);
                const float cy = __fmaf_rn(ry.x, wx[x], tyy);
                const float cd = __fmaf_rn(rd.x, wx[x], tyd);
                const float nx = __fdiv_rn(cx, cd);
                const float ny = __fdiv_rn(cy, cd);
                if (OPENGL)
                {
                    // (n + 1) * size / 2 - 0.5 (image_utils.h:67-71); /2 == *0.5 exactly
                    px[k] = __fsub_rn(__fmul_rn(__fmul_rn(__fadd_rn(nx, 1.f), Wf), 0.5f), 0.5f);
                    py[k] = __fsub_rn(__fmul_rn(__fmul_rn(__fadd_rn(ny, 1.f), Hf), 0.5f), 0.5f);
                }
                else
                {
                    px[k] = __fsub_rn(nx, 0.5f);
                    py[k] = __fsub_rn(ny, 0.5f);
                }
                if ((want_skip || want_out) && cd > 0.f)
                    front9 |= 1u << k;
                if (want_nan && !(px[k] == px[k] && py[k] == py[k]))
                    nan9 |= 1u << k;
            }
        }
        Box cur[4];
        uint32_t cur_nan = 0, cur_front = 0;
#pragma unroll
        for (int c = 0; c < 4; ++c)
        {
            const int cx = c & 1, cy = c >> 1;
            const int k0 = cx + 3 * cy, k1 = k0 + 1, k2 = k0 + 3, k3 = k0 + 4;
            cur[c] = Box{ fminf(fminf(px[k0], px[k1]), fminf(px[k2], px[k3])),
                          fminf(fminf(py[k0], py[k1]), fminf(py[k2], py[k3])),
                          fmaxf(fmaxf(px[k0], px[k1]), fmaxf(px[k2], px[k3])),
                          fmaxf(fmaxf(py[k0], py[k1]), fmaxf(py[k2], py[k3])) };
            const uint32_t need = (1u << k0) | (1u << k1) | (1u << k2) | (1u << k3);
            if (nan9 & need)
                cur_nan |= 1u << c;
            if ((front9 & need) == need)
                cur_front |= 1u << c;
        }
        if (z > 0)
        {
#pragma unroll
            for (int c = 0; c < 4; ++c)
            {
                const uint32_t cbit = 1u << c;
                const uint32_t bit = 1u << (c + 4 * (z - 1));
                const bool front = (prev_front & cur_front & cbit) != 0;
                const bool nan = ((prev_nan | cur_nan) & cbit) != 0;
                const Box cb = merge(prev[c], cur[c]);
                // 1 <= round(q) < size - 1 (round half away from zero) exactly
                // when 0.5 <= q < size - 1.5; two pixels in: 1.5 <= q < size - 2.5
                const bool in2 = want_in2 && !nan && cb.minx >= 1.5f && cb.maxx < in2_hx && cb.miny >= 1.5f &&
                                 cb.maxy < in2_hy;
                const ViewResult r = classify_view<PARTIAL>(sat_b, H, W, Hf, Wf, cb,
                                                            want_skip && front && (!skip_inside || in2), grow);
                if (want_out && front && box_out(cb, Hf, Wf))
                    out.out |= bit;
                if (r.cls == kEmpty)
                    out.empty |= bit;
                else if (r.cls == kRefine)
                    out.refine |= bit;
                if (r.skip)
                    out.skip |= bit;
                if (want_inside && !nan && cb.minx >= 0.5f && cb.maxx < in_hx && cb.miny >= 0.5f &&
                    cb.maxy < in_hy)
                    out.inside |= bit;
            }
        }
#pragma unroll
        for (int c = 0; c < 4; ++c)
            prev[c] = cur[c];
        prev_nan = cur_nan;
        prev_front = cur_front;
    }
    return out;
}


} // namespace th
