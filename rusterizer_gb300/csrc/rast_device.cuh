// rast_device.cuh - per-vertex, per-triangle and per-fragment math of the raster pipeline.
//
// Every function restates one step of the reference renderer (NiklasJonsson/rusterizer,
// file:line cited) with the same binary32 operation order. The translation units that
// include this file are compiled with --fmad=false and IEEE division/sqrt, so each
// expression below rounds once per operation, like the reference's release build.
#pragma once

#include <cstdint>
#include <cfloat>
#include <cuda_runtime.h>

#include "rast_types.h"

namespace rast {

// ------------------------------------------------------------------ scalar rules

// Rust `f as u32` (truncate, saturate, NaN -> 0): cvt.rzi.u32.f32 saturates by definition.
__device__ __forceinline__ uint32_t sat_u32(float f) { return __float2uint_rz(f); }
// Rust `f as usize` on a 64-bit target.
__device__ __forceinline__ uint64_t sat_u64(float f) { return __float2ull_rz(f); }

// f32::clamp(0.0, 1.0) as used by clamp_bary (src/rasterizer/mod.rs:102-106):
// NaN and -0.0 pass through unchanged.
__device__ __forceinline__ float clamp01(float x) {
    if (x < 0.0f) x = 0.0f;
    if (x > 1.0f) x = 1.0f;
    return x;
}

// ------------------------------------------------------------------ vertex stage

// Vector::dot (src/math/vector.rs:17-23): sum from 0.0, in order.
__device__ __forceinline__ float dot4(const float* r, float x, float y, float z, float w) {
    float s = 0.0f;
    s = s + r[0] * x;
    s = s + r[1] * y;
    s = s + r[2] * z;
    s = s + r[3] * w;
    return s;
}

// Rasterizer::perspective_divide (src/rasterizer/mod.rs:284-313): (x/w, y/w, z/w, w)
__device__ __forceinline__ float4 persp_divide(float4 c) {
    return make_float4(c.x / c.w, c.y / c.w, c.z / c.w, c.w);
}

// viewport_transform's per-vertex closure (src/rasterizer/mod.rs:318-331) on an NDC vertex;
// w passes through as depths_camera_space (mod.rs:338-342). Returns (sx, sy, sz, w).
__device__ __forceinline__ float4 viewport(float4 n, float fw, float fh) {
    const float zmin = 0.0f, zmax = 1.0f;
    float sx = fw * (n.x + 1.0f) / 2.0f;
    float sy = fh * (1.0f - (n.y + 1.0f) / 2.0f);
    float sz = (n.z + 1.0f) * 0.5f * (zmax - zmin) + zmin;
    return make_float4(sx, sy, sz, n.w);
}

__device__ __forceinline__ float4 to_screen(float4 c, float fw, float fh) {
    return viewport(persp_divide(c), fw, fh);
}

// Clip-plane predicates of try_clip's fast checks (src/rasterizer/clipping.rs:86-104):
// bits 0..5 "inside" (x >= -w, x <= w, y >= -w, y <= w, z >= -w, z <= w),
// bits 6..11 "outside" (x < -w, x > w, ...). NaN sets neither.
__device__ __forceinline__ uint32_t clip_code(float4 c) {
    uint32_t code = 0;
    const float v[3] = {c.x, c.y, c.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        code |= (uint32_t)(v[a] >= -c.w) << (2 * a);
        code |= (uint32_t)(v[a] <= c.w) << (2 * a + 1);
        code |= (uint32_t)(v[a] < -c.w) << (6 + 2 * a);
        code |= (uint32_t)(v[a] > c.w) << (6 + 2 * a + 1);
    }
    return code;
}
constexpr uint32_t kInsideAll = 0x3Fu;

// triangle_2x_area (src/rasterizer/mod.rs:15-21) with Vec2::cross (src/math/vector.rs:183-185)
__device__ __forceinline__ float tri2x_area(float x0, float y0, float x1, float y1, float x2,
                                            float y2) {
    float v10x = x1 - x0, v10y = y1 - y0;
    float v20x = x2 - x0, v20y = y2 - y0;
    return v10x * v20y - v20x * v10y;
}

// ------------------------------------------------------------------ clipping

struct ClipVert {
    float p[4];  // clip-space x, y, z, w
    float a[6];  // VertexAttribute colour r,g,b,a then uv (src/graphics_primitives.rs:9-13)
};

// distance_measure (src/rasterizer/clipping.rs:29-38), planes in CLIP_PLANES order (:53-60)
__device__ __forceinline__ float distance_measure(int plane, const float* p) {
    switch (plane) {
        case 0: return p[3] + p[0];
        case 1: return p[3] - p[0];
        case 2: return p[3] + p[1];
        case 3: return p[3] - p[1];
        case 4: return p[3] + p[2];
        default: return p[3] - p[2];
    }
}

// compute_intersection (clipping.rs:43-51) + the attribute lerp (clipping.rs:149, :161)
__device__ __forceinline__ void clip_intersect(const ClipVert& pv, float dp, const ClipVert& cv,
                                               float dc, ClipVert& out) {
    float alpha = dp / (dp - dc);
    float om = 1.0f - alpha;
#pragma unroll
    for (int k = 0; k < 4; ++k) out.p[k] = pv.p[k] * om + cv.p[k] * alpha;
#pragma unroll
    for (int k = 0; k < 6; ++k) out.a[k] = (cv.a[k] - pv.a[k]) * alpha + pv.a[k];
}

// Classification part of try_clip (src/rasterizer/clipping.rs:62-112): 0 Outside, 1 Inside,
// 2 needs Sutherland-Hodgman. area is triangle_2x_area of the clip-space xy.
__device__ __forceinline__ int clip_classify(float area, uint32_t c0, uint32_t c1, uint32_t c2) {
    if (fabsf(area) < kCullEps) return 0;
    uint32_t all = c0 & c1 & c2;
    if (all & 0xFC0u) return 0;
    if ((all & kInsideAll) == kInsideAll) return 1;
    return 2;
}

// ------------------------------------------------------------------ triangle setup

// RasterizerTriangle (src/rasterizer/mod.rs:177-222): edge points, inward normals, screen
// depths, camera-space w, 1 / (2 * area), attributes.
struct TriSetup {
    float px[3], py[3];
    float nx[3], ny[3];
    float z[3], w[3];
    float inv_area;
};

// RasterizerTriangle::new (src/rasterizer/mod.rs:186-222)
__device__ __forceinline__ void tri_setup(TriSetup& t, const float4 s[3]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        t.px[k] = s[k].x;
        t.py[k] = s[k].y;
        t.z[k] = s[k].z;
        t.w[k] = s[k].w;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        int n = (k + 1) % 3;
        float vx = s[n].x - s[k].x, vy = s[n].y - s[k].y;
        t.nx[k] = -vy;
        t.ny[k] = vx;
    }
    t.inv_area = 1.0f / tri2x_area(s[0].x, s[0].y, s[1].x, s[1].y, s[2].x, s[2].y);
}

// PixelBoundingBox::from (src/rasterizer/bounding_box.rs:13-41) clamped to the viewport
// (Rasterizer::bounding_box, src/rasterizer/mod.rs:347-361). Half-open [x0,x1) x [y0,y1).
// The reference converts with `as usize` (64-bit saturation) and then clamps to the viewport;
// converting with 32-bit saturation gives the same clamped result for any viewport below 2^32:
// both conversions agree below 2^32, and at or above it both results exceed the viewport and
// are clamped to it (NaN and negatives give 0 either way).
__device__ __forceinline__ void pixel_bbox(const float4 s[3], uint32_t width, uint32_t height,
                                           uint32_t& x0, uint32_t& x1, uint32_t& y0,
                                           uint32_t& y1) {
    float mnx = FLT_MAX, mxx = -FLT_MAX, mny = FLT_MAX, mxy = -FLT_MAX;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        mnx = fminf(mnx, s[k].x);
        mxx = fmaxf(mxx, s[k].x);
        mny = fminf(mny, s[k].y);
        mxy = fmaxf(mxy, s[k].y);
    }
    x0 = min(sat_u32(floorf(mnx)), width);
    x1 = min(sat_u32(ceilf(mxx)), width);
    y0 = min(sat_u32(floorf(mny)), height);
    y1 = min(sat_u32(ceilf(mxy)), height);
}

// EdgeFunctions::eval_single (src/rasterizer/mod.rs:125-132): normal . (p - point), dot
// accumulated from 0.0.
__device__ __forceinline__ float edge_eval(float nx, float ny, float px, float py, float x,
                                           float y) {
    float dx = x - px, dy = y - py;
    float s = 0.0f;
    s = s + nx * dx;
    s = s + ny * dy;
    return s;
}

// edge_eval without the leading 0.0 + : the same value except that an exact zero can come out
// as -0.0 instead of +0.0, which no edge test (e > 0, e < 0, tie rule) can tell apart, nor the
// sample depth computed from it (interp_depth_fast). The coverage loop's form.
__device__ __forceinline__ float edge_eval_test(float nx, float ny, float px, float py, float x, float y) {
    const float dx = x - px, dy = y - py;
    return nx * dx + ny * dy;
}

// EdgeFunctions::inside for one edge (src/rasterizer/mod.rs:148-170) without branches: pass
// when the value is positive, or when it is zero (or NaN) and the tie rule holds; the tie rule
// keys off the normal: x > 0, or x not negative and y < 0 (edge_tie, once per triangle edge).
__device__ __forceinline__ bool edge_tie(float nx, float ny) { return (nx > 0.0f) | (!(nx < 0.0f) & (ny < 0.0f)); }
__device__ __forceinline__ bool edge_pass_t(float e, bool tie) { return (e > 0.0f) | (!(e < 0.0f) & tie); }

// clamp01 that returns a NaN as a NaN of unspecified payload and may return +0.0 for -0.0
// (max.NaN / min.NaN: two instructions).
__device__ __forceinline__ float clamp01_nan(float x) {
    float r;
    asm("max.NaN.f32 %0, %1, 0f00000000;" : "=f"(r) : "f"(x));
    asm("min.NaN.f32 %0, %1, 0f3F800000;" : "=f"(r) : "f"(r));
    return r;
}

// RasterizerTriangle::fragment's interpolate_depth (src/rasterizer/mod.rs:226-236):
// b0 = clamp(e1 inv), b1 = clamp(e2 inv), b2 = clamp((1 - b0) - b1), z = (b0 z0 + b1 z1) +
// b2 z2 with inv = 1 / triangle_2x_area, here over edge values that may carry either sign of
// zero (edge_eval_test) and with clamp01_nan. The depth comes out bit for bit as the
// reference's (edge values with the
// leading 0 +, clamp01), except for the payload of a NaN (a NaN depth never passes the depth
// test, and a shader that reads it saturates it to 0): flipping the sign of a zero b0 or b1
// flips only the sign of a zero product b * z, and the sum can then only change from +0 to
// -0 when another product is -0 too, which needs a corner depth of -0 -- the viewport's final
// + zmin makes every screen depth +0 rather than -0; b2 = clamp01((1 - b0) - b1) is never -0.
__device__ __forceinline__ float interp_depth_fast(float e1, float e2, float inv, float z0, float z1,
                                                   float z2) {
    const float b0 = clamp01_nan(e1 * inv);
    const float b1 = clamp01_nan(e2 * inv);
    const float b2 = clamp01_nan(1.0f - b0 - b1);
    return b0 * z0 + b1 * z1 + b2 * z2;
}

// RGSS_SAMPLE_PATTERN (src/rasterizer/mod.rs:109-114); 1 sample = pixel centre (extension).
template <int S>
__device__ __forceinline__ float sample_dx(int i) {
    if (S == 1) return 0.5f;
    return i == 0 ? 5.0f / 8.0f : i == 1 ? 7.0f / 8.0f : i == 2 ? 3.0f / 8.0f : 1.0f / 8.0f;
}
template <int S>
__device__ __forceinline__ float sample_dy(int i) {
    if (S == 1) return 0.5f;
    return i == 0 ? 1.0f / 8.0f : i == 1 ? 5.0f / 8.0f : i == 2 ? 7.0f / 8.0f : 3.0f / 8.0f;
}

// Fragment::interpolate's sample-point choice (src/rasterizer/mod.rs:70-83): pixel centre
// when every sample passed the depth test, else the first passed sample.
template <int S>
__device__ __forceinline__ void interp_point(uint32_t x, uint32_t y, uint32_t dm, float& xs,
                                             float& ys) {
    // offsets of the first passed sample, selected without branches
    const int i = __ffs(dm) - 1;
    float dx = 0.5f, dy = 0.5f;
#pragma unroll
    for (int k = 0; k < S; ++k) {
        dx = i == k ? sample_dx<S>(k) : dx;
        dy = i == k ? sample_dy<S>(k) : dy;
    }
    const bool all = dm == (1u << S) - 1u;
    xs = (float)x + (all ? 0.5f : dx);
    ys = (float)y + (all ? 0.5f : dy);
}

// Perspective-correct barycentrics of Fragment::interpolate (src/rasterizer/mod.rs:85-94).
__device__ __forceinline__ void persp_bary(float e0, float e1, float e2, float w0, float w1,
                                           float w2, float& u, float& v, float& w) {
    float fu = e1 / w0;
    float fv = e2 / w1;
    float fw = e0 / w2;
    float sum = fu + fv + fw;
    u = clamp01(fu / sum);
    v = clamp01(fv / sum);
    w = clamp01(1.0f - u - v);
}

// ------------------------------------------------------------------ texture / colour

// Texture::read_texel (src/texture.rs:47-63) on a u32-per-texel RGBA8 image. The flat byte
// index wraps like a release build; a start past the buffer (where the reference panics)
// flags *oob and reads texel 0. Returns the texel word (byte 0 = red).
__device__ __forceinline__ uint32_t read_texel(const uint32_t* __restrict__ tex, uint32_t tw,
                                               uint32_t th, uint64_t x, uint64_t y, bool& oob) {
    uint64_t start = x * 4u + y * 4u * (uint64_t)tw;
    uint64_t len = (uint64_t)tw * (uint64_t)th * 4u;
    if (start >= len) {
        oob = true;
        start = 0;
    }
    return __ldg(tex + (start >> 2));
}

// Texture::sample (src/texture.rs:65-83): manual f32 bilinear filter. inv255[b] holds
// (b as f32) / 255.0 (Color::from_rgba, src/color.rs:22-29), correctly rounded.
__device__ __forceinline__ void tex_sample(const uint32_t* __restrict__ tex, uint32_t tw,
                                           uint32_t th, float u, float v,
                                           const float* inv255, float out[4], bool& oob) {
    float x = u * (float)(uint64_t)(tw - 1);
    float y = v * (float)(uint64_t)(th - 1);
    uint32_t tl, tr, bl, br;
    if (x >= 0.0f && y >= 0.0f && x <= (float)(tw - 1) && y <= (float)(th - 1) && tw < 65536u && th < 65536u) {
        // inside the texture (every in-range uv): floor/ceil stay below the size, so there is no
        // row wrap or read past the end, and the flat index x + y * w fits 32 bits
        const uint32_t xf = (uint32_t)floorf(x), xc = (uint32_t)ceilf(x);
        const uint32_t yf = (uint32_t)floorf(y), yc = (uint32_t)ceilf(y);
        tl = __ldg(tex + xf + yf * tw);
        tr = __ldg(tex + xc + yf * tw);
        bl = __ldg(tex + xf + yc * tw);
        br = __ldg(tex + xc + yc * tw);
    } else {
        uint64_t xf = sat_u64(floorf(x)), xc = sat_u64(ceilf(x));
        uint64_t yf = sat_u64(floorf(y)), yc = sat_u64(ceilf(y));
        tl = read_texel(tex, tw, th, xf, yf, oob);
        tr = read_texel(tex, tw, th, xc, yf, oob);
        bl = read_texel(tex, tw, th, xf, yc, oob);
        br = read_texel(tex, tw, th, xc, yc, oob);
    }
    float x_f = x - truncf(x);
    float y_f = y - truncf(y);
    float omx = 1.0f - x_f, omy = 1.0f - y_f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float ctl = inv255[(tl >> (8 * k)) & 0xFFu];
        float ctr = inv255[(tr >> (8 * k)) & 0xFFu];
        float cbl = inv255[(bl >> (8 * k)) & 0xFFu];
        float cbr = inv255[(br >> (8 * k)) & 0xFFu];
        float y0 = ctl * omx + ctr * x_f;
        float y1 = cbl * omx + cbr * x_f;
        out[k] = y0 * omy + y1 * y_f;
    }
}

// Color::to_argb (src/color.rs:15-20): saturating casts, OR-combined u32 shifts.
__device__ __forceinline__ uint32_t to_argb(float r, float g, float b, float a) {
    return (sat_u32(a * 255.0f) << 24) | (sat_u32(r * 255.0f) << 16) |
           (sat_u32(g * 255.0f) << 8) | sat_u32(b * 255.0f);
}

// ColorBuffer::box_filter_color (src/rasterizer/buffers.rs:111-125)
template <int S>
__device__ __forceinline__ uint32_t box_filter(const uint32_t* c) {
    uint32_t rs = 0, gs = 0, bs = 0;
#pragma unroll
    for (int i = 0; i < S; ++i) {
        rs += (c[i] & 0x00FF0000u) >> 16;
        gs += (c[i] & 0x0000FF00u) >> 8;
        bs += c[i] & 0x000000FFu;
    }
    return (0xFFu << 24) | (rs / (uint32_t)S) << 16 | (gs / (uint32_t)S) << 8 | (bs / (uint32_t)S);
}

}  // namespace rast
