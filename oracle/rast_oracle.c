/*
 * rast_oracle.c - CPU oracle for the rusterizer per-frame raster pipeline.
 *
 * TEST INFRASTRUCTURE ONLY (see rast_oracle.h). A plain-C restatement of the reference's
 * CPU renderer; each function cites the reference file:line it follows. Build with
 * -O2 -ffp-contract=off (no -ffast-math): every float operation below must round once,
 * in the order written, exactly like the reference's release build (Rust never contracts
 * a*b+c into an FMA).
 *
 * The reference panics on two inputs that this restatement turns into status bits instead:
 * a texel read past the end of the texture buffer (ORACLE_TEXTURE_OOB; the read then uses
 * texel 0) and an index >= nverts (ORACLE_INVALID_ARG; the draw is refused).
 */
#define _POSIX_C_SOURCE 200809L /* pthread barriers under -std=c11 */
#include "rast_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <sched.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ constants */

/* src/rasterizer/buffers.rs:5-8 */
#define CLEAR_COLOR 0xFF191919u
#define TILE_SIZE 64u
/* src/rasterizer/clipping.rs:12 */
#define CULL_DEGENERATE_TRIANGLE_AREA_EPS 0.000001f

/* RGSS_SAMPLE_PATTERN, src/rasterizer/mod.rs:109-114. The 1-sample entry (pixel centre)
 * is this project's MSAA-1 extension; the reference is 4x only (mod.rs:23). */
static const float RGSS4[4][2] = {
    {5.0f / 8.0f, 1.0f / 8.0f},
    {7.0f / 8.0f, 5.0f / 8.0f},
    {3.0f / 8.0f, 7.0f / 8.0f},
    {1.0f / 8.0f, 3.0f / 8.0f},
};
static const float CENTRE1[1][2] = {{0.5f, 0.5f}};

/* ------------------------------------------------------------------ scalar rules */

/* Rust `f as u32`: truncate toward zero, saturate, NaN -> 0 */
static uint32_t sat_u32(float f) {
    if (f != f) return 0u;
    if (f <= 0.0f) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}
/* Rust `f as usize` on a 64-bit target */
static uint64_t sat_u64(float f) {
    if (f != f) return 0u;
    if (f <= 0.0f) return 0u;
    if (f >= 18446744073709551616.0f) return UINT64_MAX;
    return (uint64_t)f;
}
/* f32::clamp (NaN and -0.0 pass through), used by clamp_bary src/rasterizer/mod.rs:102-106 */
static float clamp01(float x) {
    if (x < 0.0f) x = 0.0f;
    if (x > 1.0f) x = 1.0f;
    return x;
}

/* ------------------------------------------------------------------ math */

/* Vector::dot, src/math/vector.rs:17-23: sum starts at 0.0 and accumulates in order */
static float dot4(const float* a, const float* b) {
    float s = 0.0f;
    for (int k = 0; k < 4; ++k) s = s + a[k] * b[k];
    return s;
}

/* Mat4 * Mat4, src/math/matrix.rs:56-79 (row i of self dot column j of other) */
void oracle_kat_mat4_mul(const float a[16], const float b[16], float out[16]) {
    float r[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            float col[4] = {b[0 * 4 + j], b[1 * 4 + j], b[2 * 4 + j], b[3 * 4 + j]};
            r[i * 4 + j] = dot4(&a[i * 4], col);
        }
    memcpy(out, r, sizeof(r));
}

/* Mat4 * Vec4, src/math/vector.rs:219-240 */
void oracle_kat_mat4_vec(const float m[16], const float v[4], float out[4]) {
    float r[4];
    for (int i = 0; i < 4; ++i) r[i] = dot4(&m[i * 4], v);
    memcpy(out, r, sizeof(r));
}

/* Vector::len, src/math/vector.rs:38-40: fold(0.0, acc + e*e).sqrt() */
float oracle_kat_vec3_len(const float v[3]) {
    float acc = 0.0f;
    for (int k = 0; k < 3; ++k) acc = acc + v[k] * v[k];
    return sqrtf(acc);
}
/* Vector::normalized, src/math/vector.rs:42-44: self / self.len() per component */
void oracle_kat_vec3_normalized(const float v[3], float out[3]) {
    float l = oracle_kat_vec3_len(v);
    for (int k = 0; k < 3; ++k) out[k] = v[k] / l;
}

static void mat_set(float o[16], float a00, float a01, float a02, float a03, float a10, float a11,
                    float a12, float a13, float a20, float a21, float a22, float a23, float a30,
                    float a31, float a32, float a33) {
    float t[16] = {a00, a01, a02, a03, a10, a11, a12, a13, a20, a21, a22, a23, a30, a31, a32, a33};
    memcpy(o, t, sizeof(t));
}
/* src/math/transform.rs:19-41 */
void oracle_kat_rotate_x(float rad, float o[16]) {
    mat_set(o, 1, 0, 0, 0, 0, cosf(rad), -sinf(rad), 0, 0, sinf(rad), cosf(rad), 0, 0, 0, 0, 1);
}
/* src/math/transform.rs:43-65 */
void oracle_kat_rotate_y(float rad, float o[16]) {
    mat_set(o, cosf(rad), 0, sinf(rad), 0, 0, 1, 0, 0, -sinf(rad), 0, cosf(rad), 0, 0, 0, 0, 1);
}
/* src/math/transform.rs:67-89 */
void oracle_kat_rotate_z(float rad, float o[16]) {
    mat_set(o, cosf(rad), -sinf(rad), 0, 0, sinf(rad), cosf(rad), 0, 0, 0, 0, 1, 0, 0, 0, 0, 1);
}
/* src/math/transform.rs:10-17 */
void oracle_kat_translate(float x, float y, float z, float o[16]) {
    mat_set(o, 1, 0, 0, x, 0, 1, 0, y, 0, 0, 1, z, 0, 0, 0, 1);
}
/* src/math/mod.rs:92-122 */
void oracle_kat_project(float near_, float far_, float aspect, float fov, float o[16]) {
    float half_width = tanf(fov / 2.0f) * near_;
    float half_height = aspect * half_width;
    mat_set(o, near_ / half_width, 0, 0, 0, 0, near_ / half_height, 0, 0, 0, 0,
            -(far_ + near_) / (far_ - near_), -2.0f * far_ * near_ / (far_ - near_), 0, 0, -1.0f,
            0);
}

/* ------------------------------------------------------------------ clipping */

typedef struct {
    float p[4]; /* clip-space x, y, z, w */
    float a[6]; /* VertexAttribute: colour r,g,b,a then uv (src/graphics_primitives.rs:9-13) */
} cvert;

/* triangle_2x_area, src/rasterizer/mod.rs:15-21 with Vec2::cross src/math/vector.rs:183-185 */
static float tri2x_area(float x0, float y0, float x1, float y1, float x2, float y2) {
    float v10x = x1 - x0, v10y = y1 - y0;
    float v20x = x2 - x0, v20y = y2 - y0;
    return v10x * v20y - v20x * v10y;
}

/* distance_measure, src/rasterizer/clipping.rs:29-38; planes in CLIP_PLANES order :53-60 */
static float distance_measure(int plane, const float* p) {
    switch (plane) {
    case 0: return p[3] + p[0]; /* LEFT */
    case 1: return p[3] - p[0]; /* RIGHT */
    case 2: return p[3] + p[1]; /* BOTTOM */
    case 3: return p[3] - p[1]; /* TOP */
    case 4: return p[3] + p[2]; /* NEAR */
    default: return p[3] - p[2]; /* FAR */
    }
}

/* compute_intersection (clipping.rs:43-51) plus the attribute lerp of :149 / :161 */
static cvert intersect(const cvert* prev, float dprev, const cvert* cur, float dcur) {
    cvert r;
    float alpha = dprev / (dprev - dcur);
    float om = 1.0f - alpha;
    for (int k = 0; k < 4; ++k) r.p[k] = prev->p[k] * om + cur->p[k] * alpha;
    for (int k = 0; k < 6; ++k) r.a[k] = (cur->a[k] - prev->a[k]) * alpha + prev->a[k];
    return r;
}

/* clipping::try_clip, src/rasterizer/clipping.rs:62-195.
 * Returns 0 Outside, 1 Inside, 2 Clipped (poly holds *n vertices; fan them from vertex 0). */
static int try_clip(const cvert in[3], cvert* poly, int* n, uint32_t* status) {
    if (fabsf(tri2x_area(in[0].p[0], in[0].p[1], in[1].p[0], in[1].p[1], in[2].p[0], in[2].p[1])) <
        CULL_DEGENERATE_TRIANGLE_AREA_EPS)
        return 0;
    int inside[3][2] = {{1, 1}, {1, 1}, {1, 1}};
    int outside[3][2] = {{1, 1}, {1, 1}, {1, 1}};
    for (int v = 0; v < 3; ++v) {
        const float* p = in[v].p;
        for (int a = 0; a < 3; ++a) {
            inside[a][0] &= p[a] >= -p[3];
            inside[a][1] &= p[a] <= p[3];
            outside[a][0] &= p[a] < -p[3];
            outside[a][1] &= p[a] > p[3];
        }
    }
    for (int a = 0; a < 3; ++a)
        if (outside[a][0] || outside[a][1]) return 0;
    int all_in = 1;
    for (int a = 0; a < 3; ++a) all_in &= inside[a][0] & inside[a][1];
    if (all_in) return 1;

    cvert bufA[ORACLE_MAX_POLY], bufB[ORACLE_MAX_POLY];
    cvert* cur_poly = bufA;
    cvert* nxt = bufB;
    int cn = 3;
    memcpy(cur_poly, in, 3 * sizeof(cvert));
    for (int plane = 0; plane < 6; ++plane) {
        int on = 0;
        for (int i = 0; i < cn; ++i) {
            int pi = (i + cn - 1) % cn;
            const cvert* pv = &cur_poly[pi];
            const cvert* cv = &cur_poly[i];
            float dp = distance_measure(plane, pv->p);
            float dc = distance_measure(plane, cv->p);
            int pin = dp >= 0.0f, cin = dc >= 0.0f;
            int need = (pin && cin) ? 1 : (pin && !cin) ? 1 : (!pin && cin) ? 2 : 0;
            if (on + need > ORACLE_MAX_POLY) {
                *status |= ORACLE_CLIP_OVERFLOW;
                return 0;
            }
            if (pin && cin) {
                nxt[on++] = *cv;
            } else if (pin && !cin) {
                nxt[on++] = intersect(pv, dp, cv, dc);
            } else if (!pin && cin) {
                nxt[on++] = intersect(pv, dp, cv, dc);
                nxt[on++] = *cv;
            }
        }
        cvert* t = cur_poly;
        cur_poly = nxt;
        nxt = t;
        cn = on;
    }
    if (cn == 0) return 0;
    if (cur_poly != poly) memcpy(poly, cur_poly, (size_t)cn * sizeof(cvert));
    *n = cn;
    return 2;
}

/* ------------------------------------------------------------------ setup */

typedef struct {
    float px[3], py[3]; /* EdgeFunctions.points */
    float nx[3], ny[3]; /* EdgeFunctions.normals */
    float z[3];         /* RasterizerTriangle.depths (screen z) */
    float w[3];         /* depths_camera_space */
    float inv_area;
    float a[3][6];
    uint64_t bx0, bx1, by0, by1; /* viewport-clamped pixel box, half-open */
    uint32_t tri, sub;
} rec;

/* perspective_divide (mod.rs:284-313) + viewport_transform (mod.rs:315-345) of one vertex */
static void to_screen(const float* p, int width, int height, float* sx, float* sy, float* sz,
                      float* w) {
    float nx = p[0] / p[3], ny = p[1] / p[3], nz = p[2] / p[3];
    const float zmin = 0.0f, zmax = 1.0f;
    *sx = (float)width * (nx + 1.0f) / 2.0f;
    *sy = (float)height * (1.0f - (ny + 1.0f) / 2.0f);
    *sz = (nz + 1.0f) * 0.5f * (zmax - zmin) + zmin;
    *w = p[3];
}

/* RasterizerTriangle::new (mod.rs:186-222) + Rasterizer::bounding_box (mod.rs:347-361,
 * bounding_box.rs:13-41) */
static void setup_rec(rec* r, const float sx[3], const float sy[3], const float sz[3],
                      const float w[3], const float a[3][6], int width, int height) {
    for (int k = 0; k < 3; ++k) {
        r->px[k] = sx[k];
        r->py[k] = sy[k];
        r->z[k] = sz[k];
        r->w[k] = w[k];
        memcpy(r->a[k], a[k], 6 * sizeof(float));
    }
    for (int k = 0; k < 3; ++k) {
        int n = (k + 1) % 3;
        float vx = sx[n] - sx[k], vy = sy[n] - sy[k];
        r->nx[k] = -vy;
        r->ny[k] = vx;
    }
    r->inv_area = 1.0f / tri2x_area(sx[0], sy[0], sx[1], sy[1], sx[2], sy[2]);
    float mnx = FLT_MAX, mxx = -FLT_MAX, mny = FLT_MAX, mxy = -FLT_MAX;
    for (int k = 0; k < 3; ++k) {
        mnx = fminf(mnx, sx[k]);
        mxx = fmaxf(mxx, sx[k]);
        mny = fminf(mny, sy[k]);
        mxy = fmaxf(mxy, sy[k]);
    }
    uint64_t x0 = sat_u64(floorf(mnx)), x1 = sat_u64(ceilf(mxx));
    uint64_t y0 = sat_u64(floorf(mny)), y1 = sat_u64(ceilf(mxy));
    if (x1 > (uint64_t)width) x1 = (uint64_t)width;
    if (y1 > (uint64_t)height) y1 = (uint64_t)height;
    r->bx0 = x0;
    r->bx1 = x1;
    r->by0 = y0;
    r->by1 = y1;
}

/* EdgeFunctions::eval_single, mod.rs:125-132: normal.dot(p - point), dot from 0.0 */
static void eval_single(const rec* r, float x, float y, float e[3]) {
    for (int k = 0; k < 3; ++k) {
        float dx = x - r->px[k], dy = y - r->py[k];
        float s = 0.0f;
        s = s + r->nx[k] * dx;
        s = s + r->ny[k] * dy;
        e[k] = s;
    }
}

/* EdgeFunctions::inside, mod.rs:148-170 (tie rule for exact-zero or NaN edge values) */
static int inside3(const rec* r, const float e[3]) {
    for (int k = 0; k < 3; ++k) {
        float v = e[k];
        if (v > 0.0f) continue;
        if (v < 0.0f) return 0;
        if (r->nx[k] > 0.0f) continue;
        if (r->nx[k] < 0.0f) return 0;
        if (r->ny[k] < 0.0f) continue;
        return 0;
    }
    return 1;
}

/* RasterizerTriangle::fragment's interpolate_depth closure, mod.rs:226-236 */
static float interp_depth(const rec* r, const float e[3]) {
    float b0 = clamp01(e[1] * r->inv_area);
    float b1 = clamp01(e[2] * r->inv_area);
    float b2 = clamp01(1.0f - b0 - b1);
    return b0 * r->z[0] + b1 * r->z[1] + b2 * r->z[2];
}

/* Fragment::interpolate, mod.rs:69-100 */
static void interpolate(const rec* r, uint64_t x, uint64_t y, unsigned mask, int nsamp,
                        const float (*pat)[2], float out[6]) {
    float xs = (float)x + 0.5f, ys = (float)y + 0.5f;
    unsigned all = (1u << nsamp) - 1u;
    if (mask != all) {
        for (int i = 0; i < nsamp; ++i)
            if (mask & (1u << i)) {
                xs = (float)x + pat[i][0];
                ys = (float)y + pat[i][1];
                break;
            }
    }
    float e[3];
    eval_single(r, xs, ys, e);
    float fu = e[1] / r->w[0];
    float fv = e[2] / r->w[1];
    float fw = e[0] / r->w[2];
    float sum = fu + fv + fw;
    float u = clamp01(fu / sum);
    float v = clamp01(fv / sum);
    float w = clamp01(1.0f - u - v);
    for (int k = 0; k < 6; ++k) out[k] = r->a[0][k] * u + r->a[1][k] * v + r->a[2][k] * w;
}

/* ------------------------------------------------------------------ texture / colour */

typedef struct {
    uint8_t* data;
    int w, h;
} otex;

/* Texture::read_texel, src/texture.rs:47-63 with Color::from_rgba src/color.rs:22-29.
 * Index arithmetic wraps like a release build; a start past the buffer (the reference's
 * slice-index panic) sets *oob and reads texel 0 instead. */
static void read_texel(const otex* t, uint64_t x, uint64_t y, float c[4], int* oob) {
    uint64_t start = x * 4u + y * 4u * (uint64_t)t->w;
    uint64_t len = (uint64_t)t->w * (uint64_t)t->h * 4u;
    if (start >= len) {
        *oob = 1;
        start = 0;
    }
    for (int k = 0; k < 4; ++k) c[k] = (float)t->data[start + (uint64_t)k] / 255.0f;
}

/* Texture::sample, src/texture.rs:65-83 (manual bilinear filter in f32) */
static void tex_sample(const otex* t, float u, float v, float out[4], int* oob) {
    float x = u * (float)(uint64_t)(t->w - 1);
    float y = v * (float)(uint64_t)(t->h - 1);
    uint64_t xf = sat_u64(floorf(x)), xc = sat_u64(ceilf(x));
    uint64_t yf = sat_u64(floorf(y)), yc = sat_u64(ceilf(y));
    float tl[4], tr[4], bl[4], br[4];
    read_texel(t, xf, yf, tl, oob);
    read_texel(t, xc, yf, tr, oob);
    read_texel(t, xf, yc, bl, oob);
    read_texel(t, xc, yc, br, oob);
    float x_f = x - truncf(x);
    float y_f = y - truncf(y);
    for (int k = 0; k < 4; ++k) {
        float y0 = tl[k] * (1.0f - x_f) + tr[k] * x_f;
        float y1 = bl[k] * (1.0f - x_f) + br[k] * x_f;
        out[k] = y0 * (1.0f - y_f) + y1 * y_f;
    }
}

/* Color::to_argb, src/color.rs:15-20 (saturating casts, OR-combined) */
static uint32_t to_argb(const float c[4] /* r,g,b,a */) {
    return (sat_u32(c[3] * 255.0f) << 24) | (sat_u32(c[0] * 255.0f) << 16) |
           (sat_u32(c[1] * 255.0f) << 8) | sat_u32(c[2] * 255.0f);
}

/* ColorBuffer::box_filter_color, src/rasterizer/buffers.rs:111-125 */
static uint32_t box_filter(const uint32_t* c, int n) {
    uint32_t rs = 0, gs = 0, bs = 0;
    for (int i = 0; i < n; ++i) {
        rs += (c[i] & 0x00FF0000u) >> 16;
        gs += (c[i] & 0x0000FF00u) >> 8;
        bs += c[i] & 0x000000FFu;
    }
    return (0xFFu << 24) | (rs / (uint32_t)n) << 16 | (gs / (uint32_t)n) << 8 | (bs / (uint32_t)n);
}

/* ------------------------------------------------------------------ buffer tiles */

struct oracle_tiles {
    int n;
    uint64_t n_horizontal;
    uint64_t* rect; /* min_x, max_x, min_y, max_y */
    uint8_t* mask[2];
    int mask_idx;
};

/* BufferTiles::new, src/rasterizer/buffers.rs:19-47 */
oracle_tiles* oracle_tiles_create(int width, int height) {
    oracle_tiles* t = (oracle_tiles*)calloc(1, sizeof(*t));
    uint64_t w = (uint64_t)width, h = (uint64_t)height;
    uint64_t nh = w / TILE_SIZE + ((w % TILE_SIZE == 0) ? 0 : 1);
    uint64_t nv = h / TILE_SIZE + ((h % TILE_SIZE == 0) ? 0 : 1);
    t->n = (int)(nh * nv);
    t->n_horizontal = nh;
    t->rect = (uint64_t*)malloc(sizeof(uint64_t) * 4 * (size_t)(t->n ? t->n : 1));
    int i = 0;
    for (uint64_t j = 0; j < nv; ++j)
        for (uint64_t k = 0; k < nh; ++k, ++i) {
            uint64_t mx = (k + 1) * TILE_SIZE, my = (j + 1) * TILE_SIZE;
            t->rect[4 * i + 0] = k * TILE_SIZE;
            t->rect[4 * i + 1] = mx < w ? mx : w;
            t->rect[4 * i + 2] = j * TILE_SIZE;
            t->rect[4 * i + 3] = my < h ? my : h;
        }
    t->mask[0] = (uint8_t*)calloc((size_t)(t->n ? t->n : 1), 1);
    t->mask[1] = (uint8_t*)calloc((size_t)(t->n ? t->n : 1), 1);
    return t;
}
void oracle_tiles_destroy(oracle_tiles* t) {
    if (!t) return;
    free(t->rect);
    free(t->mask[0]);
    free(t->mask[1]);
    free(t);
}
int oracle_tiles_len(const oracle_tiles* t) { return t->n; }
void oracle_tiles_get(const oracle_tiles* t, int i, uint64_t out[4]) {
    memcpy(out, &t->rect[4 * i], 4 * sizeof(uint64_t));
}
/* BufferTiles::tile_idx + mark, buffers.rs:49-56 (an index past the end, which would panic,
 * is ignored) */
void oracle_tiles_mark(oracle_tiles* t, uint64_t row, uint64_t col) {
    uint64_t idx = (row / TILE_SIZE) * t->n_horizontal + (col / TILE_SIZE);
    /* written once per tile and frame: band threads that share a cache line of the mask then
     * only read it */
    if (idx < (uint64_t)t->n && !t->mask[t->mask_idx][idx]) t->mask[t->mask_idx][idx] = 1;
}
/* BufferTiles::next, buffers.rs:58-63 */
void oracle_tiles_next(oracle_tiles* t) {
    t->mask_idx = (t->mask_idx + 1) % 2;
    memset(t->mask[t->mask_idx], 0, (size_t)t->n);
}
static int count_mask(const oracle_tiles* t, int which) {
    int c = 0;
    for (int i = 0; i < t->n; ++i) c += t->mask[which][i] != 0;
    return c;
}
/* marked / prev_marked, buffers.rs:65-79 */
int oracle_tiles_marked_count(const oracle_tiles* t) { return count_mask(t, t->mask_idx); }
int oracle_tiles_prev_marked_count(const oracle_tiles* t) {
    return count_mask(t, (t->mask_idx + 1) % 2);
}
int oracle_tiles_mask(const oracle_tiles* t, int which, int i) { return t->mask[which][i]; }

/* ------------------------------------------------------------------ context */

struct oracle_ctx {
    int w, h, msaa;
    float clear_depth;
    uint32_t* cbuf; /* [w*h*msaa] */
    float* dbuf;    /* [w*h*msaa] */
    uint32_t* resolve;
    oracle_tiles* tiles;
    otex tex[16];
    int ntex;
    uint32_t status;
    uint64_t shaded, fsinv, oob;
    uint64_t tri_base; /* running triangle index over draws, for the fragment log */
    uint32_t* log;
    uint64_t log_cap, log_n;
    int nthreads; /* threads of the last draw, reused by the resolve */
};

/* ------------------------------------------------------------------ threads */

/* Runs fn(arg, part, nparts) for part = 0 .. nparts-1 on nparts threads (the caller's thread
 * runs part 0). The reference is single-threaded; this only spreads independent work. */
typedef void (*part_fn)(void* arg, int part, int nparts);
typedef struct {
    part_fn fn;
    void* arg;
    int part, nparts;
} part_job;
static void* part_main(void* p) {
    part_job* j = (part_job*)p;
    j->fn(j->arg, j->part, j->nparts);
    return NULL;
}
static void run_parts(part_fn fn, void* arg, int nparts) {
    if (nparts <= 1) {
        fn(arg, 0, 1);
        return;
    }
    part_job* jobs = (part_job*)calloc((size_t)nparts, sizeof(part_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nparts, sizeof(pthread_t));
    for (int k = 0; k < nparts; ++k) {
        jobs[k].fn = fn;
        jobs[k].arg = arg;
        jobs[k].part = k;
        jobs[k].nparts = nparts;
        if (k) pthread_create(&th[k], NULL, part_main, &jobs[k]);
    }
    fn(arg, 0, nparts);
    for (int k = 1; k < nparts; ++k) pthread_join(th[k], NULL);
    free(jobs);
    free(th);
}
static size_t part_lo(size_t n, int part, int nparts) { return n * (size_t)part / (size_t)nparts; }

oracle_ctx* oracle_create(int width, int height, int msaa, float clear_depth) {
    if (width <= 0 || height <= 0 || width > 65535 || height > 65535) return NULL;
    if (msaa != 1 && msaa != 4) return NULL;
    oracle_ctx* c = (oracle_ctx*)calloc(1, sizeof(*c));
    size_t np = (size_t)width * (size_t)height;
    c->w = width;
    c->h = height;
    c->msaa = msaa;
    c->clear_depth = clear_depth;
    c->cbuf = (uint32_t*)malloc(np * (size_t)msaa * sizeof(uint32_t));
    c->dbuf = (float*)malloc(np * (size_t)msaa * sizeof(float));
    c->resolve = (uint32_t*)malloc(np * sizeof(uint32_t));
    for (size_t i = 0; i < np * (size_t)msaa; ++i) {
        c->cbuf[i] = CLEAR_COLOR;
        c->dbuf[i] = clear_depth;
    }
    for (size_t i = 0; i < np; ++i) c->resolve[i] = CLEAR_COLOR;
    c->tiles = oracle_tiles_create(width, height);
    return c;
}

void oracle_destroy(oracle_ctx* c) {
    if (!c) return;
    free(c->cbuf);
    free(c->dbuf);
    free(c->resolve);
    oracle_tiles_destroy(c->tiles);
    for (int i = 0; i < c->ntex; ++i) free(c->tex[i].data);
    free(c->log);
    free(c);
}

uint32_t oracle_bind_texture(oracle_ctx* c, int slot, const uint8_t* rgba8, int w, int h) {
    if (!c || slot != c->ntex || slot >= 16 || w <= 0 || h <= 0 || !rgba8)
        return ORACLE_INVALID_ARG;
    size_t n = (size_t)w * (size_t)h * 4;
    c->tex[slot].data = (uint8_t*)malloc(n);
    memcpy(c->tex[slot].data, rgba8, n);
    c->tex[slot].w = w;
    c->tex[slot].h = h;
    c->ntex++;
    return ORACLE_OK;
}

void oracle_log_enable(oracle_ctx* c, uint64_t capacity) {
    free(c->log);
    c->log = (uint32_t*)malloc((size_t)capacity * 4 * sizeof(uint32_t));
    c->log_cap = capacity;
    c->log_n = 0;
}
uint64_t oracle_log_count(const oracle_ctx* c) { return c->log_n; }
void oracle_log_copy(const oracle_ctx* c, uint32_t* out) {
    memcpy(out, c->log, (size_t)c->log_n * 4 * sizeof(uint32_t));
}

/* per-thread accumulation for the row-band parallel pixel loop */
typedef struct {
    oracle_ctx* c;
    const rec* const* part_recs; /* the block's records, in submission order, in nparts parts */
    const size_t* part_n;
    /* with several bands: per part, the indices of its records whose rows meet each band
     * (band b's at band_idx[part][band_off[part][b] .. band_off[part][b + 1])), in order */
    uint32_t* const* band_idx;
    size_t* const* band_off;
    int nparts;
    int fs_id;
    uint64_t band, nbands;
    uint64_t shaded, fsinv, oob;
} band_job;

static void shade_and_write(oracle_ctx* c, const rec* r, int fs_id, uint64_t x, uint64_t y,
                            unsigned cov, const float sd[4], unsigned dm, uint64_t* shaded,
                            uint64_t* fsinv, uint64_t* oobc) {
    const int S = c->msaa;
    const float(*pat)[2] = S == 4 ? RGSS4 : CENTRE1;
    float attr[6];
    interpolate(r, x, y, dm, S, pat, attr);
    float col[4];
    if (fs_id == ORACLE_FS_TEXTURE) {
        /* FS::Texture, upstream src/main.rs:214-216 */
        int oob = 0;
        tex_sample(&c->tex[0], attr[4], attr[5], col, &oob);
        if (oob) (*oobc)++;
    } else if (fs_id == ORACLE_FS_COLOR) {
        /* FS::Color, upstream src/main.rs:217 */
        col[0] = attr[0];
        col[1] = attr[1];
        col[2] = attr[2];
        col[3] = attr[3];
    } else {
        /* FS::Debug, upstream src/main.rs:218-220: grayscale(frag_coords.depths[0]) */
        col[0] = sd[0];
        col[1] = sd[0];
        col[2] = sd[0];
        col[3] = 1.0f;
    }
    (void)cov;
    uint32_t argb = to_argb(col);
    /* write_pixel, mod.rs:380-397 */
    oracle_tiles_mark(c->tiles, y, x);
    size_t base = ((size_t)y * (size_t)c->w + (size_t)x) * (size_t)S;
    for (int i = 0; i < S; ++i)
        if (dm & (1u << i)) {
            c->cbuf[base + (size_t)i] = argb;
            c->dbuf[base + (size_t)i] = sd[i];
            (*shaded)++;
        }
    (*fsinv)++;
}

/* Per-triangle pixel loop of Rasterizer::rasterize, mod.rs:443-473, over the pixels of band
 * `band` of `nbands`: the 64x64 tiles (tile row tr, tile column tc) with (tr + tc) modulo
 * nbands equal to band (every pixel when nbands is 1). The diagonal interleave spreads a strip
 * of the screen, rows or columns, over every band. Bands share no tile, so they run on separate
 * threads; each visits the pixels of a box in the reference's row-major order. */
static void raster_rec(oracle_ctx* c, const rec* r, int fs_id, uint64_t band, uint64_t nbands,
                       uint64_t* shaded, uint64_t* fsinv, uint64_t* oobc) {
    const int S = c->msaa;
    const float(*pat)[2] = S == 4 ? RGSS4 : CENTRE1;
    for (uint64_t y = r->by0; y < r->by1; ++y) {
        const uint64_t tr = y / TILE_SIZE;
        for (uint64_t x = r->bx0; x < r->bx1; ++x) {
            if (nbands > 1 && (tr + x / TILE_SIZE) % nbands != band) {
                x = (x / TILE_SIZE + 1) * TILE_SIZE - 1;  /* to the next tile column */
                continue;
            }
            float e[4][3];
            unsigned cov = 0;
            for (int i = 0; i < S; ++i) {
                eval_single(r, (float)x + pat[i][0], (float)y + pat[i][1], e[i]);
                if (inside3(r, e[i])) cov |= 1u << i;
            }
            if (!cov) continue;
            float sd[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            for (int i = 0; i < S; ++i)
                if (cov & (1u << i)) sd[i] = interp_depth(r, e[i]);
            /* depth_coverage, mod.rs:363-378: strict less-than */
            size_t base = ((size_t)y * (size_t)c->w + (size_t)x) * (size_t)S;
            unsigned dm = 0;
            for (int i = 0; i < S; ++i)
                if ((cov & (1u << i)) && sd[i] < c->dbuf[base + (size_t)i]) dm |= 1u << i;
            if (c->log && c->log_n < c->log_cap) {
                uint32_t* L = &c->log[4 * c->log_n++];
                L[0] = r->tri;
                L[1] = r->sub;
                L[2] = (uint32_t)((y << 16) | x);
                L[3] = (dm << 8) | cov;
            }
            if (!dm) continue;
            shade_and_write(c, r, fs_id, x, y, cov, sd, dm, shaded, fsinv, oobc);
        }
    }
}

static void* band_main(void* arg) {
    band_job* j = (band_job*)arg;
    /* counted in locals: the jobs of neighbouring bands share cache lines */
    uint64_t shaded = 0, fsinv = 0, oob = 0;
    for (int p = 0; p < j->nparts; ++p) {
        if (j->nbands > 1) {
            const uint32_t* L = j->band_idx[p];
            for (size_t i = j->band_off[p][j->band]; i < j->band_off[p][j->band + 1]; ++i)
                raster_rec(j->c, &j->part_recs[p][L[i]], j->fs_id, j->band, j->nbands, &shaded, &fsinv, &oob);
        } else {
            for (size_t i = 0; i < j->part_n[p]; ++i)
                raster_rec(j->c, &j->part_recs[p][i], j->fs_id, j->band, j->nbands, &shaded, &fsinv, &oob);
        }
    }
    j->shaded = shaded;
    j->fsinv = fsinv;
    j->oob = oob;
    return NULL;
}

/* Clip + divide + viewport + setup of one assembled triangle (mod.rs:425-441). Appends 0..n-2
 * records. */
static size_t triangle_records(const oracle_ctx* c, const cvert tri[3], uint32_t tri_index, rec* out,
                               uint32_t* status) {
    cvert poly[ORACLE_MAX_POLY];
    int n = 0;
    int res = try_clip(tri, poly, &n, status);
    if (res == 0) return 0;
    const cvert* src = tri;
    if (res == 1) {
        n = 3;
    } else {
        src = poly;
    }
    size_t k = 0;
    for (int f = 0; f + 2 < n; ++f) {
        /* fan [v0, v(f+1), v(f+2)], clipping.rs:185-190 */
        const cvert* v[3] = {&src[0], &src[f + 1], &src[f + 2]};
        float sx[3], sy[3], sz[3], w[3], a[3][6];
        for (int q = 0; q < 3; ++q) {
            to_screen(v[q]->p, c->w, c->h, &sx[q], &sy[q], &sz[q], &w[q]);
            memcpy(a[q], v[q]->a, sizeof(a[q]));
        }
        setup_rec(&out[k], sx, sy, sz, w, (const float(*)[6])a, c->w, c->h);
        out[k].tri = tri_index;
        out[k].sub = (uint32_t)f;
        ++k;
    }
    return k;
}

/* vertex shader P*V*W*v over a range of vertices (upstream src/main.rs:147-152) */
typedef struct {
    const float* pos;
    const float* mvp;
    float* clip;
    uint32_t nverts;
} vs_job;
static void vs_part(void* a, int part, int nparts) {
    vs_job* j = (vs_job*)a;
    size_t v0 = part_lo(j->nverts, part, nparts), v1 = part_lo(j->nverts, part + 1, nparts);
    for (size_t v = v0; v < v1; ++v) {
        float p4[4] = {j->pos[3 * v], j->pos[3 * v + 1], j->pos[3 * v + 2], 1.0f};
        oracle_kat_mat4_vec(j->mvp, p4, &j->clip[4 * v]);
    }
}

/* primitive assembly + clip/setup (render.rs:75-96, mod.rs:425-441) of a range of triangles
 * into that range's own record area, in submission order */
typedef struct {
    const oracle_ctx* c;
    const float* clip;
    const float* uv;
    const float* rgba;
    const uint32_t* idx;
    size_t t0, t1;
    rec* recs;       /* record area of triangle t0 + k starts at recs + k * maxper */
    size_t maxper;
    rec** part_recs;
    size_t* part_n;
    uint32_t* part_status;
    int nbands;            /* > 1: also list each part's records by band (band_main) */
    uint32_t** band_idx;   /* per part, grown as needed (band_cap entries) */
    size_t* band_cap;
    size_t** band_off;     /* per part, nbands + 1 offsets */
} setup_job;

/* The bands ((tile row + tile column) modulo nbands) whose tiles a record's box meets: the
 * diagonals from (tr0 + tc0) to (tr1 + tc1); calls add(b) once per band. Records with an empty
 * box meet none. */
static void rec_bands(const rec* r, int nbands, void (*add)(void*, int), void* arg) {
    if (r->by0 >= r->by1 || r->bx0 >= r->bx1) return;
    const uint64_t d0 = r->by0 / TILE_SIZE + r->bx0 / TILE_SIZE;
    const uint64_t d1 = (r->by1 - 1) / TILE_SIZE + (r->bx1 - 1) / TILE_SIZE;
    if (d1 - d0 + 1 >= (uint64_t)nbands) {
        for (int b = 0; b < nbands; ++b) add(arg, b);
        return;
    }
    for (uint64_t d = d0; d <= d1; ++d) add(arg, (int)(d % (uint64_t)nbands));
}
typedef struct {
    size_t* off;
    uint32_t* idx;
    uint32_t rec;
} band_fill;
static void band_count_add(void* a, int b) { ((band_fill*)a)->off[b + 1]++; }
static void band_fill_add(void* a, int b) {
    band_fill* f = (band_fill*)a;
    f->idx[f->off[b]++] = f->rec;
}
static void setup_part(void* a, int part, int nparts) {
    setup_job* j = (setup_job*)a;
    size_t n = j->t1 - j->t0;
    size_t lo = part_lo(n, part, nparts), hi = part_lo(n, part + 1, nparts);
    rec* out = j->recs + lo * j->maxper;
    size_t k = 0;
    uint32_t status = 0;
    for (size_t t = j->t0 + lo; t < j->t0 + hi; ++t) {
        cvert tri[3];
        for (int q = 0; q < 3; ++q) {
            uint32_t vi = j->idx[3 * t + (size_t)q];
            memcpy(tri[q].p, &j->clip[4 * (size_t)vi], 4 * sizeof(float));
            if (j->rgba)
                memcpy(tri[q].a, &j->rgba[4 * (size_t)vi], 4 * sizeof(float));
            else
                tri[q].a[0] = tri[q].a[1] = tri[q].a[2] = tri[q].a[3] = 0.0f;
            tri[q].a[4] = j->uv[2 * (size_t)vi];
            tri[q].a[5] = j->uv[2 * (size_t)vi + 1];
        }
        k += triangle_records(j->c, tri, (uint32_t)(j->c->tri_base + t), &out[k], &status);
    }
    j->part_recs[part] = out;
    j->part_n[part] = k;
    j->part_status[part] = status;
    if (j->nbands > 1) {
        /* counting sort of the part's record indices by band, keeping their order */
        const int nb = j->nbands;
        size_t* off = j->band_off[part];
        for (int b = 0; b <= nb; ++b) off[b] = 0;
        band_fill f = {off, NULL, 0};
        for (size_t i = 0; i < k; ++i) rec_bands(&out[i], nb, band_count_add, &f);
        for (int b = 0; b < nb; ++b) off[b + 1] += off[b];
        if (off[nb] > j->band_cap[part]) {
            free(j->band_idx[part]);
            j->band_cap[part] = off[nb] + off[nb] / 2;
            j->band_idx[part] = (uint32_t*)malloc(sizeof(uint32_t) * j->band_cap[part]);
        }
        f.idx = j->band_idx[part];
        for (size_t i = 0; i < k; ++i) {
            f.rec = (uint32_t)i;
            rec_bands(&out[i], nb, band_fill_add, &f);
        }
        /* the fill advanced each band's start to its end: shift back */
        for (int b = nb; b > 0; --b) off[b] = off[b - 1];
        off[0] = 0;
    }
}

/* One draw's pixel work on a pool of threads created once per draw: per block of triangles,
 * every thread clips and sets up its part of the block, then (after a barrier) rasterizes its
 * band of rows over all the block's records in submission order. */
/* Sense-reversing barrier that spins (yielding now and then): the pool's threads meet twice
 * per block, and a sleeping barrier's wake-up latency would dominate small blocks. */
typedef struct {
    atomic_int count;
    atomic_int sense;
    int n;
} spin_barrier;
static void spin_barrier_wait(spin_barrier* b, int* local_sense) {
    const int s = !*local_sense;
    *local_sense = s;
    if (atomic_fetch_add(&b->count, 1) == b->n - 1) {
        atomic_store(&b->count, 0);
        atomic_store(&b->sense, s);
    } else {
        for (unsigned spins = 0; atomic_load(&b->sense) != s; ++spins)
            if ((spins & 1023u) == 1023u) sched_yield();
    }
}

typedef struct {
    oracle_ctx* c;
    setup_job* sj;       /* the block's setup (t0, t1 set per block) */
    size_t ntris, block;
    int nthreads, nbands, fs_id;
    spin_barrier bar;
} draw_pool;
typedef struct {
    draw_pool* pool;
    int k;
    uint64_t shaded, fsinv, oob;
} draw_worker;
static void* draw_worker_main(void* arg) {
    draw_worker* w = (draw_worker*)arg;
    draw_pool* P = w->pool;
    int sense = 0;
    for (size_t t0 = 0; t0 < P->ntris; t0 += P->block) {
        const size_t t1 = t0 + P->block < P->ntris ? t0 + P->block : P->ntris;
        const int nparts = (t1 - t0) >= 4096u ? P->nthreads : 1;
        if (w->k < nparts) {
            setup_job j = *P->sj;
            j.t0 = t0;
            j.t1 = t1;
            setup_part(&j, w->k, nparts);
        }
        spin_barrier_wait(&P->bar, &sense);
        if (w->k < P->nbands) {
            band_job b = {P->c, (const rec* const*)P->sj->part_recs, P->sj->part_n, P->sj->band_idx,
                          P->sj->band_off, nparts, P->fs_id, (uint64_t)w->k, (uint64_t)P->nbands, 0, 0, 0};
            band_main(&b);
            w->shaded += b.shaded;
            w->fsinv += b.fsinv;
            w->oob += b.oob;
        }
        if (w->k == 0)
            for (int p = 0; p < nparts; ++p) P->c->status |= P->sj->part_status[p];
        spin_barrier_wait(&P->bar, &sense);
    }
    return NULL;
}

uint32_t oracle_draw(oracle_ctx* c, const float* pos, const float* uv, const float* rgba,
                     uint32_t nverts, const uint32_t* idx, uint32_t ntris, const float world[16],
                     const float view[16], const float proj[16], int fs_id, int nthreads) {
    if (!c || (nverts && (!pos || !uv)) || (ntris && !idx)) return ORACLE_INVALID_ARG;
    if (fs_id < 0 || fs_id > 2) return ORACLE_INVALID_ARG;
    if (fs_id == ORACLE_FS_TEXTURE && c->ntex == 0) return ORACLE_INVALID_ARG;
    /* primitive_assembly (src/render.rs:75-96) would panic on an out-of-range index */
    for (uint64_t i = 0; i < (uint64_t)ntris * 3; ++i)
        if (idx[i] >= nverts) return ORACLE_INVALID_ARG;
    if (c->log) nthreads = 1;
    if (nthreads < 1) nthreads = 1;
    c->nthreads = nthreads;

    /* vertex shader P*V*W*v, left-associative (upstream src/main.rs:147-152) */
    float pv[16], mvp[16];
    oracle_kat_mat4_mul(proj, view, pv);
    oracle_kat_mat4_mul(pv, world, mvp);
    float* clip = (float*)malloc(sizeof(float) * 4 * (size_t)(nverts ? nverts : 1));
    {
        vs_job vj = {pos, mvp, clip, nverts};
        run_parts(vs_part, &vj, nverts >= 65536u ? nthreads : 1);
    }

    const size_t BLOCK = 1u << 16;
    const size_t maxper = ORACLE_MAX_POLY - 2;
    rec* recs = (rec*)malloc(sizeof(rec) * BLOCK * maxper);
    rec** part_recs = (rec**)calloc((size_t)nthreads, sizeof(rec*));
    size_t* part_n = (size_t*)calloc((size_t)nthreads, sizeof(size_t));
    uint32_t* part_status = (uint32_t*)calloc((size_t)nthreads, sizeof(uint32_t));
    setup_job sj = {c, clip, uv, rgba, idx, 0, 0, recs, maxper, part_recs, part_n, part_status, 1, NULL, NULL, NULL};
    uint64_t shaded = 0, fsinv = 0, oob = 0;
    if (nthreads == 1) {
        for (size_t t0 = 0; t0 < ntris; t0 += BLOCK) {
            sj.t0 = t0;
            sj.t1 = t0 + BLOCK < ntris ? t0 + BLOCK : ntris;
            setup_part(&sj, 0, 1);
            c->status |= part_status[0];
            for (size_t i = 0; i < part_n[0]; ++i)
                raster_rec(c, &part_recs[0][i], fs_id, 0, 1, &shaded, &fsinv, &oob);
        }
    } else {
        /* bands of 64x64 tiles interleaved along the diagonals ((tile row + tile column) % nb):
         * no two threads mark one tile, and a block of triangles that covers a strip of the
         * screen still spreads over every band */
        const uint64_t rows_tiles = ((uint64_t)c->h + TILE_SIZE - 1) / TILE_SIZE +
                                    ((uint64_t)c->w + TILE_SIZE - 1) / TILE_SIZE - 1;
        draw_pool P;
        P.c = c;
        P.sj = &sj;
        P.ntris = ntris;
        P.block = BLOCK;
        P.nthreads = nthreads;
        P.nbands = (uint64_t)nthreads > rows_tiles ? (int)rows_tiles : nthreads;
        sj.nbands = P.nbands;
        sj.band_idx = (uint32_t**)calloc((size_t)nthreads, sizeof(uint32_t*));
        sj.band_cap = (size_t*)calloc((size_t)nthreads, sizeof(size_t));
        sj.band_off = (size_t**)calloc((size_t)nthreads, sizeof(size_t*));
        for (int k = 0; k < nthreads; ++k) sj.band_off[k] = (size_t*)calloc((size_t)P.nbands + 1, sizeof(size_t));
        P.fs_id = fs_id;
        atomic_init(&P.bar.count, 0);
        atomic_init(&P.bar.sense, 0);
        P.bar.n = nthreads;
        draw_worker* ws = (draw_worker*)calloc((size_t)nthreads, sizeof(draw_worker));
        pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
        for (int k = 0; k < nthreads; ++k) {
            ws[k].pool = &P;
            ws[k].k = k;
            if (k) pthread_create(&th[k], NULL, draw_worker_main, &ws[k]);
        }
        draw_worker_main(&ws[0]);
        for (int k = 1; k < nthreads; ++k) pthread_join(th[k], NULL);
        for (int k = 0; k < nthreads; ++k) {
            shaded += ws[k].shaded;
            fsinv += ws[k].fsinv;
            oob += ws[k].oob;
        }
        free(ws);
        free(th);
        for (int k = 0; k < nthreads; ++k) {
            free(sj.band_idx[k]);
            free(sj.band_off[k]);
        }
        free(sj.band_idx);
        free(sj.band_cap);
        free(sj.band_off);
    }
    free(part_recs);
    free(part_n);
    free(part_status);
    free(recs);
    free(clip);
    c->tri_base += ntris;
    c->shaded += shaded;
    c->fsinv += fsinv;
    c->oob += oob;
    if (oob) c->status |= ORACLE_TEXTURE_OOB;
    return ORACLE_OK;
}

/* Rasterizer::resolve_and_clear, src/rasterizer/mod.rs:478-518, over a range of tiles (the
 * tiles are disjoint, so ranges run on separate threads) */
typedef struct {
    oracle_ctx* c;
    int prev;
} resolve_job;
static void resolve_part(void* a, int part, int nparts) {
    resolve_job* j = (resolve_job*)a;
    oracle_ctx* c = j->c;
    const int S = c->msaa;
    oracle_tiles* t = c->tiles;
    int i0 = (int)part_lo((size_t)t->n, part, nparts), i1 = (int)part_lo((size_t)t->n, part + 1, nparts);
    for (int i = i0; i < i1; ++i) {
        if (!t->mask[j->prev][i]) continue;
        for (uint64_t y = t->rect[4 * i + 2]; y < t->rect[4 * i + 3]; ++y)
            for (uint64_t x = t->rect[4 * i]; x < t->rect[4 * i + 1]; ++x)
                c->resolve[y * (uint64_t)c->w + x] = CLEAR_COLOR;
    }
    for (int i = i0; i < i1; ++i) {
        if (!t->mask[t->mask_idx][i]) continue;
        for (uint64_t y = t->rect[4 * i + 2]; y < t->rect[4 * i + 3]; ++y)
            for (uint64_t x = t->rect[4 * i]; x < t->rect[4 * i + 1]; ++x) {
                size_t p = (size_t)(y * (uint64_t)c->w + x);
                c->resolve[p] = box_filter(&c->cbuf[p * (size_t)S], S);
                for (int s = 0; s < S; ++s) {
                    c->cbuf[p * (size_t)S + (size_t)s] = CLEAR_COLOR;
                    c->dbuf[p * (size_t)S + (size_t)s] = c->clear_depth;
                }
            }
    }
}

uint32_t oracle_framebuffer(oracle_ctx* c, uint32_t* argb_out) {
    oracle_tiles* t = c->tiles;
    resolve_job rj = {c, (t->mask_idx + 1) % 2};
    run_parts(resolve_part, &rj, c->nthreads > 1 && t->n >= 64 ? c->nthreads : 1);
    oracle_tiles_next(t);
    if (argb_out) memcpy(argb_out, c->resolve, (size_t)c->w * (size_t)c->h * sizeof(uint32_t));
    uint32_t st = c->status;
    c->status = 0;
    c->tri_base = 0;
    return st;
}

void oracle_read_samples(const oracle_ctx* c, float* depth_out, uint32_t* color_out) {
    size_t n = (size_t)c->w * (size_t)c->h * (size_t)c->msaa;
    if (depth_out) memcpy(depth_out, c->dbuf, n * sizeof(float));
    if (color_out) memcpy(color_out, c->cbuf, n * sizeof(uint32_t));
}

void oracle_stats(const oracle_ctx* c, uint64_t* shaded, uint64_t* fsinv, uint64_t* oob) {
    if (shaded) *shaded = c->shaded;
    if (fsinv) *fsinv = c->fsinv;
    if (oob) *oob = c->oob;
}

/* ------------------------------------------------------------------ known-answer shims */

void oracle_kat_perspective_divide(const float clip[12], float ndc[12]) {
    for (int v = 0; v < 3; ++v) {
        const float* p = &clip[4 * v];
        ndc[4 * v + 0] = p[0] / p[3];
        ndc[4 * v + 1] = p[1] / p[3];
        ndc[4 * v + 2] = p[2] / p[3];
        ndc[4 * v + 3] = p[3];
    }
}

void oracle_kat_viewport(int width, int height, const float ndc[12], float out_points[6],
                         float out_depths[3], float out_w[3], float* out_inv_area,
                         float out_normals[6]) {
    float sx[3], sy[3], sz[3], w[3], a[3][6] = {{0}};
    const float zmin = 0.0f, zmax = 1.0f;
    for (int v = 0; v < 3; ++v) {
        const float* p = &ndc[4 * v];
        sx[v] = (float)width * (p[0] + 1.0f) / 2.0f;
        sy[v] = (float)height * (1.0f - (p[1] + 1.0f) / 2.0f);
        sz[v] = (p[2] + 1.0f) * 0.5f * (zmax - zmin) + zmin;
        w[v] = p[3];
    }
    rec r;
    setup_rec(&r, sx, sy, sz, w, (const float(*)[6])a, width, height);
    for (int v = 0; v < 3; ++v) {
        out_points[2 * v] = r.px[v];
        out_points[2 * v + 1] = r.py[v];
        out_depths[v] = r.z[v];
        out_w[v] = r.w[v];
        out_normals[2 * v] = r.nx[v];
        out_normals[2 * v + 1] = r.ny[v];
    }
    *out_inv_area = r.inv_area;
}

static void rec_from_screen(rec* r, const float screen[9], const float* w3, const float* attrs) {
    float sx[3], sy[3], sz[3], w[3], a[3][6] = {{0}};
    for (int v = 0; v < 3; ++v) {
        sx[v] = screen[3 * v];
        sy[v] = screen[3 * v + 1];
        sz[v] = screen[3 * v + 2];
        w[v] = w3 ? w3[v] : 1.0f;
        if (attrs) memcpy(a[v], &attrs[6 * v], 6 * sizeof(float));
    }
    setup_rec(r, sx, sy, sz, w, (const float(*)[6])a, 65535, 65535);
}

int oracle_kat_eval_single(const float screen[9], float x, float y, float e_out[3]) {
    rec r;
    rec_from_screen(&r, screen, NULL, NULL);
    eval_single(&r, x, y, e_out);
    return inside3(&r, e_out);
}

int oracle_kat_fragment(const float screen[9], int x, int y, float depths_out[4]) {
    rec r;
    rec_from_screen(&r, screen, NULL, NULL);
    float e[4][3];
    unsigned cov = 0;
    for (int i = 0; i < 4; ++i) {
        eval_single(&r, (float)x + RGSS4[i][0], (float)y + RGSS4[i][1], e[i]);
        if (inside3(&r, e[i])) cov |= 1u << i;
    }
    for (int i = 0; i < 4; ++i) depths_out[i] = (cov & (1u << i)) ? interp_depth(&r, e[i]) : 0.0f;
    return (int)cov;
}

void oracle_kat_interpolate(const float screen[9], const float w[3], const float attrs[18], int x,
                            int y, float out[6]) {
    rec r;
    rec_from_screen(&r, screen, w, attrs);
    unsigned cov = 0;
    for (int i = 0; i < 4; ++i) {
        float e[3];
        eval_single(&r, (float)x + RGSS4[i][0], (float)y + RGSS4[i][1], e);
        if (inside3(&r, e)) cov |= 1u << i;
    }
    interpolate(&r, (uint64_t)x, (uint64_t)y, cov, 4, RGSS4, out);
}

int oracle_kat_clip(const float verts[12], const float attrs[18], int* out_ntris, float* out_verts,
                    float* out_attrs) {
    cvert tri[3], poly[ORACLE_MAX_POLY];
    for (int v = 0; v < 3; ++v) {
        memcpy(tri[v].p, &verts[4 * v], 4 * sizeof(float));
        memcpy(tri[v].a, &attrs[6 * v], 6 * sizeof(float));
    }
    int n = 0;
    uint32_t st = 0;
    int res = try_clip(tri, poly, &n, &st);
    *out_ntris = 0;
    if (res != 2) return res;
    for (int f = 0; f + 2 < n; ++f) {
        const cvert* v[3] = {&poly[0], &poly[f + 1], &poly[f + 2]};
        for (int q = 0; q < 3; ++q) {
            memcpy(&out_verts[(3 * f + q) * 4], v[q]->p, 4 * sizeof(float));
            memcpy(&out_attrs[(3 * f + q) * 6], v[q]->a, 6 * sizeof(float));
        }
    }
    *out_ntris = n - 2;
    return res;
}

void oracle_kat_bbox(const float points[6], uint64_t out[4]) {
    float mnx = FLT_MAX, mxx = -FLT_MAX, mny = FLT_MAX, mxy = -FLT_MAX;
    for (int k = 0; k < 3; ++k) {
        mnx = fminf(mnx, points[2 * k]);
        mxx = fmaxf(mxx, points[2 * k]);
        mny = fminf(mny, points[2 * k + 1]);
        mxy = fmaxf(mxy, points[2 * k + 1]);
    }
    out[0] = sat_u64(floorf(mnx));
    out[1] = sat_u64(ceilf(mxx));
    out[2] = sat_u64(floorf(mny));
    out[3] = sat_u64(ceilf(mxy));
}

uint32_t oracle_kat_box_filter(const uint32_t colors[4]) { return box_filter(colors, 4); }

uint32_t oracle_kat_to_argb(const float rgba[4]) { return to_argb(rgba); }

int oracle_kat_tex_sample(const uint8_t* rgba8, int w, int h, float u, float v, float out[4]) {
    otex t = {(uint8_t*)rgba8, w, h};
    int oob = 0;
    tex_sample(&t, u, v, out, &oob);
    return oob;
}
