/*
 * rast_oracle.h - CPU oracle for the rusterizer per-frame raster pipeline.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference
 * renderer's CPU path (NiklasJonsson/rusterizer, Rust 2021). It exists to check
 * the CUDA implementation; only the test suite, the smoke check and the CPU
 * baseline leg of the benchmark may load it. The product library never links it.
 *
 * Every function names the reference file:line it restates. All float arithmetic
 * is IEEE binary32 with one rounding per operation, in the reference's operation
 * order; the file must be compiled with -ffp-contract=off and without -ffast-math
 * (aarch64 GCC contracts a*b+c into fmadd by default, which would change results).
 *
 * Pinning: the restatement is checked against all 46 unit tests of the reference
 * crate (their inputs and expected f32 values, re-expressed in tests/).
 */
#ifndef RAST_ORACLE_H
#define RAST_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status bits (OR-ed) */
#define ORACLE_OK 0u
#define ORACLE_INVALID_ARG 1u
#define ORACLE_TEXTURE_OOB 2u  /* reference would panic in Texture::read_texel (texture.rs:51-56) */
#define ORACLE_CLIP_OVERFLOW 4u /* clip polygon exceeded ORACLE_MAX_POLY vertices (never seen) */

#define ORACLE_MAX_POLY 32

/* fragment shader ids (src/main.rs:212-222) */
#define ORACLE_FS_TEXTURE 0
#define ORACLE_FS_COLOR 1
#define ORACLE_FS_DEBUG 2

typedef struct oracle_ctx oracle_ctx;

/* Rasterizer::new (src/rasterizer/mod.rs:273-281). msaa is 4 (reference) or 1 (extension:
 * one sample at the pixel centre). clear_depth defaults to FLT_MAX in the reference
 * (src/rasterizer/buffers.rs:6). */
oracle_ctx* oracle_create(int width, int height, int msaa, float clear_depth);
void oracle_destroy(oracle_ctx* ctx);

/* Uniforms::bind_texture (src/uniform.rs:29-33): slot must equal the number bound so far.
 * The texture is RGBA8 row-major; the oracle keeps its own copy. */
uint32_t oracle_bind_texture(oracle_ctx* ctx, int slot, const uint8_t* rgba8, int w, int h);

/* Renderer::render (src/render.rs:98-114) with the demo vertex shader P*V*W*v
 * (src/main.rs:147-152 of the upstream demo) and fragment shader fs_id.
 * pos: nverts*3 f32, uv: nverts*2 f32, rgba: nverts*4 f32 or NULL (colour (0,0,0,0)),
 * idx: ntris*3 u32. Matrices are row-major 4x4 (Matrix.array, src/math/matrix.rs:7-16).
 * nthreads>1 splits the pixel loop into row bands (same per-pixel order, same result). */
uint32_t oracle_draw(oracle_ctx* ctx, const float* pos, const float* uv, const float* rgba,
                     uint32_t nverts, const uint32_t* idx, uint32_t ntris, const float world[16],
                     const float view[16], const float proj[16], int fs_id, int nthreads);

/* Rasterizer::framebuffer -> resolve_and_clear (src/rasterizer/mod.rs:478-522).
 * Writes width*height ARGB u32, row-major, y=0 top. Returns the status bits gathered since
 * the previous framebuffer call and clears them. */
uint32_t oracle_framebuffer(oracle_ctx* ctx, uint32_t* argb_out);

/* Per-sample buffers as they stand now (before framebuffer): depth f32 and colour ARGB u32,
 * laid out [y][x][sample]. Either pointer may be NULL. */
void oracle_read_samples(const oracle_ctx* ctx, float* depth_out, uint32_t* color_out);

/* Statistics since creation: samples written (sum of popcount of depth-passed masks),
 * fragment-shader invocations, and texture reads past the end of the texel buffer. */
void oracle_stats(const oracle_ctx* ctx, uint64_t* shaded_samples, uint64_t* fs_invocations,
                  uint64_t* texture_oob);

/* Optional fragment log: when enabled, every fragment with a non-empty geometric coverage
 * mask is recorded as 4 u32 words {tri, (sub<<8)|cov|(dmask<<4)... } see oracle_log_get. */
void oracle_log_enable(oracle_ctx* ctx, uint64_t capacity);
uint64_t oracle_log_count(const oracle_ctx* ctx);
/* record i: tri index within the draw stream (running over draws), sub-triangle, x, y,
 * geometric coverage mask, depth-passed mask */
void oracle_log_copy(const oracle_ctx* ctx, uint32_t* out /* count*4 */);

/* ---------------- known-answer entry points (one reference function each) ------------- */

/* Vector::dot accumulation (src/math/vector.rs:17-23) and Mat4*Mat4 (src/math/matrix.rs:56-79) */
void oracle_kat_mat4_mul(const float a[16], const float b[16], float out[16]);
/* Mat4*Vec4 (src/math/vector.rs:219-240) */
void oracle_kat_mat4_vec(const float m[16], const float v[4], float out[4]);
/* Vector::len / normalized (src/math/vector.rs:38-44) on a 3-vector */
float oracle_kat_vec3_len(const float v[3]);
void oracle_kat_vec3_normalized(const float v[3], float out[3]);
/* transform::rotate_x/y/z, translate, rotate (src/math/transform.rs:10-96), project (src/math/mod.rs:92-122) */
void oracle_kat_rotate_x(float rad, float out[16]);
void oracle_kat_rotate_y(float rad, float out[16]);
void oracle_kat_rotate_z(float rad, float out[16]);
void oracle_kat_translate(float x, float y, float z, float out[16]);
void oracle_kat_project(float near_, float far_, float aspect, float fov, float out[16]);
/* Rasterizer::perspective_divide (src/rasterizer/mod.rs:284-313): in/out 3 vertices x,y,z,w */
void oracle_kat_perspective_divide(const float clip[12], float ndc[12]);
/* viewport_transform + RasterizerTriangle::new (src/rasterizer/mod.rs:315-345, :186-222):
 * out_points 3x(x,y), out_depths z, out_w w, out_inv_area, out_normals 3x(x,y) */
void oracle_kat_viewport(int width, int height, const float ndc[12], float out_points[6],
                         float out_depths[3], float out_w[3], float* out_inv_area,
                         float out_normals[6]);
/* EdgeFunctions::eval_single + inside (src/rasterizer/mod.rs:125-132, :148-170) for a screen
 * triangle given as 3x(x,y,z). Returns inside (0/1). */
int oracle_kat_eval_single(const float screen[9], float x, float y, float e_out[3]);
/* EdgeFunctions::eval at pixel (x,y) then RasterizerTriangle::fragment (src/rasterizer/mod.rs:
 * 134-146, :225-253). Returns the coverage mask; depths[4] the sampled depths. */
int oracle_kat_fragment(const float screen[9], int x, int y, float depths_out[4]);
/* eval + fragment + Fragment::interpolate with the geometric coverage mask
 * (src/rasterizer/mod.rs:69-100; test helper verify_uvs_at :874-879).
 * attrs: 3 x (r,g,b,a,u,v). out: (r,g,b,a,u,v). */
void oracle_kat_interpolate(const float screen[9], const float w[3], const float attrs[18],
                            int x, int y, float out[6]);
/* clipping::try_clip (src/rasterizer/clipping.rs:62-195). Returns 0 Outside, 1 Inside,
 * 2 Clipped; out_verts receives ntris*3 vertices (x,y,z,w), out_attrs ntris*3*6. */
int oracle_kat_clip(const float verts[12], const float attrs[18], int* out_ntris, float* out_verts,
                    float* out_attrs);
/* PixelBoundingBox::from (src/rasterizer/bounding_box.rs:13-41): min_x,max_x,min_y,max_y */
void oracle_kat_bbox(const float points[6], uint64_t out[4]);
/* ColorBuffer::box_filter_color (src/rasterizer/buffers.rs:111-125) with 4 samples */
uint32_t oracle_kat_box_filter(const uint32_t colors[4]);
/* Color::to_argb (src/color.rs:15-20) */
uint32_t oracle_kat_to_argb(const float rgba[4]);
/* Texture::sample (src/texture.rs:65-83); returns 1 when a texel read ran past the buffer */
int oracle_kat_tex_sample(const uint8_t* rgba8, int w, int h, float u, float v, float out[4]);

/* BufferTiles (src/rasterizer/buffers.rs:10-80) */
typedef struct oracle_tiles oracle_tiles;
oracle_tiles* oracle_tiles_create(int width, int height);
void oracle_tiles_destroy(oracle_tiles* t);
int oracle_tiles_len(const oracle_tiles* t);
void oracle_tiles_get(const oracle_tiles* t, int i, uint64_t out[4]); /* min_x,max_x,min_y,max_y */
void oracle_tiles_mark(oracle_tiles* t, uint64_t row, uint64_t col);
void oracle_tiles_next(oracle_tiles* t);
int oracle_tiles_marked_count(const oracle_tiles* t);
int oracle_tiles_prev_marked_count(const oracle_tiles* t);
int oracle_tiles_mask(const oracle_tiles* t, int which, int i); /* masks[which][i] */

#ifdef __cplusplus
}
#endif
#endif
