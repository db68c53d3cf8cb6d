/*
 * rast.h - C ABI of the GB300 (sm_103a) raster pipeline.
 *
 * Drop-in boundary for the per-frame raster path of the Rust software rasterizer
 * NiklasJonsson/rusterizer. Each entry point names the reference interface it replaces
 * (paths are inside that crate). Plain pointers and sizes only; no exceptions cross the ABI,
 * every call returns a rast_status. A context owns its device memory and CUDA stream; host
 * arrays passed in are only read during the call. One context per host thread (the reference
 * Renderer is `&mut self` everywhere and not Sync).
 *
 * Conventions shared with the reference:
 *   - matrices are row-major float[16] (Matrix.array, src/math/matrix.rs:7-16);
 *   - the vertex shader is P * V * W * v (upstream demo src/main.rs:147-152);
 *   - output is width*height ARGB u32, row-major, y = 0 at the top (src/color.rs:15-20,
 *     src/rasterizer/mod.rs:315-345);
 *   - 4x rotated-grid MSAA (src/rasterizer/mod.rs:23, :109-114); msaa = 1 is an extension
 *     with one sample at the pixel centre.
 */
#ifndef RAST_H
#define RAST_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rast_status {
    RAST_OK = 0,
    RAST_INVALID_ARG = 1,      /* bad handle, size, index >= nverts, slot order, ... */
    RAST_OOM = 2,              /* device allocation failed */
    RAST_ADMISSION_REFUSED = 3,/* server: request does not fit the HBM budget */
    RAST_BIN_OVERFLOW = 4,     /* bin capacity exceeded even after regrowth */
    RAST_TIMEOUT = 5,          /* a bounded wait expired */
    RAST_TEXTURE_OOB = 6,      /* a texel read ran past the texture (the reference panics in
                                  Texture::read_texel, src/texture.rs:51-56); image still
                                  produced, with texel 0 read instead */
    RAST_CLIP_OVERFLOW = 7,    /* a clipped polygon exceeded 32 vertices (never observed) */
    RAST_CUDA_ERROR = 8,
    RAST_NOT_READY = 9         /* server: result not finished yet */
} rast_status;

typedef struct rast_ctx rast_ctx;
typedef uint32_t rast_mesh;

enum { RAST_VS_MVP = 0 };
/* fragment shaders of the upstream demo, selected by id (src/main.rs:67-77) */
enum { RAST_FS_TEXTURE = 0, RAST_FS_COLOR = 1, RAST_FS_DEBUG = 2 };

const char* rast_status_string(rast_status s);

/* Renderer::new / Rasterizer::new (src/render.rs:48-69, src/rasterizer/mod.rs:273-281).
 * width, height in [1, 16384]; msaa 4 (reference) or 1. */
rast_ctx* rast_create(int width, int height, int msaa, rast_status* status);
void rast_destroy(rast_ctx* ctx);

/* Depth clear value; the reference uses f32::MAX (src/rasterizer/buffers.rs:6). */
rast_status rast_set_clear_depth(rast_ctx* ctx, float depth);
/* Screen tile edge in pixels (8, 16 or 32); 0 selects automatically: 32 for frames of 8192
 * triangles or more, else 16 (either one when the other would exceed 16384 tiles, and 32 when
 * both would). Frames of more than 16384 tiles are binned in several counting passes, one per
 * 16384 tiles: any size rast_create accepts renders, large ones at some cost in binning. */
rast_status rast_set_tile_size(rast_ctx* ctx, int tile);

/* How raster tiles are split between the two raster kernels (no counterpart in the reference,
 * whose pixel loop is serial): bins with at least min_entries entries (rounded down to a power
 * of two) are rastered by a whole CTA per tile, the others by one warp per tile. 0 sends every
 * bin to the CTA-wide kernel (the default), 0xFFFFFFFF every bin to the warp kernel. Results
 * are identical either way; only speed changes. */
rast_status rast_set_heavy_tile_entries(rast_ctx* ctx, uint32_t min_entries);

/* Upload a mesh (Mesh{vertices, indices, attributes}, src/mesh.rs:5-12) so that it stays
 * resident. pos: nverts*3 f32; uv: nverts*2 f32; rgba: nverts*4 f32 or NULL (colour
 * (0,0,0,0)); idx: ntris*3 u32, each < nverts (primitive_assembly would panic otherwise,
 * src/render.rs:75-96). */
rast_status rast_mesh_upload(rast_ctx* ctx, const float* pos, const float* uv, const float* rgba,
                             uint32_t nverts, const uint32_t* idx, uint32_t ntris,
                             rast_mesh* out);
rast_status rast_mesh_free(rast_ctx* ctx, rast_mesh mesh);
/* Overwrite a resident mesh with new host data of the same vertex and triangle counts (the
 * reference borrows the mesh afresh on every render call, src/render.rs:98-110); copies only,
 * no allocation. rgba must be given iff the mesh was uploaded with colours. The indices are
 * checked on the device, not here: a triangle with an index >= nverts is skipped and the
 * next rast_framebuffer returns RAST_INVALID_ARG. */
rast_status rast_mesh_update(rast_ctx* ctx, rast_mesh mesh, const float* pos, const float* uv,
                             const float* rgba, const uint32_t* idx);
/* The same copies, enqueued without waiting (no counterpart in the reference): they start
 * once the frames already enqueued on the context have finished, and the next rast_framebuffer
 * or rast_framebuffer_async that draws this mesh waits for them on the device. The host arrays
 * must stay unchanged until that frame has returned (rast_framebuffer) or its stream has been
 * synchronised; page-locked arrays make the copies truly asynchronous. With two meshes used
 * in turn, one host thread streams the next frame's mesh while the current frame renders.
 * Synchronous updates, frees, batches and servers first wait for pending copies. */
rast_status rast_mesh_update_async(rast_ctx* ctx, rast_mesh mesh, const float* pos, const float* uv,
                                   const float* rgba, const uint32_t* idx);

/* Uniforms::bind_texture (src/uniform.rs:29-33): slot must equal the number already bound.
 * rgba8 is w*h*4 bytes, row-major, (0,0) top-left (Texture, src/texture.rs:6-13). */
rast_status rast_texture_upload(rast_ctx* ctx, int slot, const uint8_t* rgba8, int w, int h);

/* Uniforms::write_block().{world, view, projection} (src/uniform.rs:4-45). */
rast_status rast_set_uniforms(rast_ctx* ctx, const float world[16], const float view[16],
                              const float proj[16]);

/* Renderer::render(mesh, vertex_shader, fragment_shader) (src/render.rs:98-114): queues the
 * draw with the current uniforms; draws keep submission order. */
rast_status rast_draw(rast_ctx* ctx, rast_mesh mesh, int vs_id, int fs_id);

/* Rasterizer::framebuffer (src/rasterizer/mod.rs:478-522): renders every queued draw,
 * resolves, clears, and writes width*height ARGB u32 to argb_out (host or device pointer;
 * NULL keeps the result on the device only). */
rast_status rast_framebuffer(rast_ctx* ctx, uint32_t* argb_out);

/* Same frame, enqueued on the context stream without waiting: no overflow re-run and no
 * status readback (capacities come from earlier rast_framebuffer calls). argb_out is a device
 * pointer (the frame writes it), NULL, or host memory: the frame then resolves into one of two
 * staging buffers in turn, and a side stream copies it to argb_out once the frame is done, so
 * that one host thread's next frame renders while this one is copied. Page-locked host memory
 * makes that copy asynchronous. The host image is complete after rast_wait_output(ctx,
 * argb_out) (or any synchronous call of the context). Used by throughput loops; no counterpart
 * in the reference. */
rast_status rast_framebuffer_async(rast_ctx* ctx, uint32_t* argb_out);

/* Waits until the asynchronous copies into host array argb_out (every one when NULL) enqueued
 * by rast_framebuffer_async have landed. */
rast_status rast_wait_output(rast_ctx* ctx, const uint32_t* argb_out);

/* One frame of one mesh that allocates nothing. No counterpart in the reference: it is for
 * callers that cannot allocate device memory when they render (an engine or plugin host that
 * owns all device memory through its own pool, or a loop that must not let cudaMalloc or
 * cudaFree synchronise the device). The caller passes device pointers for the mesh (d_pos
 * nverts*3, d_uv nverts*2, d_rgba nverts*4 or NULL, d_idx ntris*3; a triangle with an index
 * >= nverts is skipped on the device and the call returns RAST_INVALID_ARG),
 * the RGBA8 texture (d_tex, one u32 per texel; needed for fs_id 0) and the width*height ARGB
 * output, plus host row-major world/view/proj matrices. All intermediate buffers live in one
 * 32 MiB array in device memory owned by the library and held on every GPU that loads it
 * until exit; frames that need more, or more than 262144 vertices or triangles, return
 * RAST_INVALID_ARG without launching anything. A frame whose bins or clipped polygons
 * overflow the first estimate is run again with the measured sizes (up to three runs, as
 * rast_framebuffer does) while they still fit the array, else RAST_INVALID_ARG. The first
 * call on a device looks up that array's address (make it before any stream capture). Work
 * runs on `stream` (cudaStream_t, NULL = legacy default) and the call waits for it to finish.
 * Calls share the array: calls whose GPU work overlaps race and must be serialised by the
 * caller. Host stack use is small (the descriptor staging is static, under a lock). Same
 * image, status and bit-exactness as rast_framebuffer for the same inputs. */
rast_status rast_render_noalloc(int width, int height, int msaa, int tile, float clear_depth,
                                const float* d_pos, const float* d_uv, const float* d_rgba,
                                uint32_t nverts, const uint32_t* d_idx, uint32_t ntris,
                                const float world[16], const float view[16], const float proj[16],
                                const uint32_t* d_tex, int tex_w, int tex_h, int fs_id,
                                uint32_t* d_argb, void* stream);

/* ---- batched rendering (no counterpart in the reference: one Renderer draws one scene) ---- */

/* One independent scene of a batch: one resident mesh, one fragment shader, its own target. */
typedef struct rast_scene {
    int width, height, msaa; /* msaa 1 or 4 */
    int tile;                /* 8, 16 or 32; 0 = the context's autotuned choice */
    float clear_depth;
    rast_mesh mesh;
    int texture;             /* texture slot used by RAST_FS_TEXTURE */
    int fs_id;
    float world[16], view[16], proj[16];
    uint32_t* argb_out;      /* width*height ARGB: device pointer, or host pointer (copied back) */
} rast_scene;

/* Renders n scenes with one launch of each pipeline kernel for the whole batch; the raster
 * kernel is persistent and takes tiles of all scenes from one queue, heaviest first. Same
 * per-scene results as rendering each scene alone. Synchronous. */
rast_status rast_render_batch(rast_ctx* ctx, const rast_scene* scenes, uint32_t n);

/* Settings the batch autotuner chooses, per MSAA class ([0] MSAA 1, [1] MSAA 4). */
typedef struct rast_tuning {
    int tile[2];                  /* bin edge in pixels: 8, 16 or 32 */
    uint32_t heavy_entries[2];    /* rast_set_heavy_tile_entries threshold: 0 = every bin CTA-wide,
                                     0xFFFFFFFF = every bin one warp per tile */
    int raster_ctas_per_sm[2];    /* persistent raster CTAs per SM, 0 = as many as fit */
    uint64_t bin_capacity;        /* bin entries reserved for the batch (measured need + 1/8) */
    float batch_ms;               /* batch time with the chosen settings */
} rast_tuning;

/* Times the batch under each candidate setting and keeps the fastest in the context (used by
 * rast_render_batch, rast_batch_create and servers created afterwards, where rast_scene.tile is
 * 0): first the bin edge 8/16/32 of both MSAA classes together, under every bin CTA-wide and
 * under every bin one warp per tile; then, from the best of those, per class the raster
 * kernel split (every bin CTA-wide, bins of 128+, 512+ or 2048+ entries CTA-wide and the rest
 * one warp per tile, every bin one warp per tile) with all the raster CTAs that fit, 4 or 2 per
 * SM; then the bin edge again under the chosen splits; finally one run measures each scene's bins
 * and the batch reserves that plus an eighth. Images are written to scratch, not the scenes'
 * outputs. No counterpart in the reference (its tile size is the constant TILE_SIZE = 64,
 * src/rasterizer/buffers.rs:8). */
rast_status rast_autotune_batch_ex(rast_ctx* ctx, const rast_scene* scenes, uint32_t n, rast_tuning* out);
/* The same, returning the bin edges only: best_tiles[0] = MSAA 1, [1] = MSAA 4. */
rast_status rast_autotune_batch(rast_ctx* ctx, const rast_scene* scenes, uint32_t n,
                                int best_tiles[2]);

/* A batch captured into a CUDA graph once (after one sizing run) and re-rendered by one graph
 * launch per call. argb_out pointers are device pointers or page-locked host memory (the graph
 * then resolves those scenes into the batch's own staging buffer and copies them out at its
 * end; pageable host memory is refused with RAST_INVALID_ARG). Two batches launched in turn
 * without waiting overlap one's copies with the other's kernels. The batch owns its own scratch
 * and stream; the context's meshes and textures must outlive it. */
typedef struct rast_batch rast_batch;
rast_status rast_batch_create(rast_ctx* ctx, const rast_scene* scenes, uint32_t n, rast_batch** out);
rast_status rast_batch_launch(rast_batch* batch, int wait);
void* rast_batch_stream(rast_batch* batch);
rast_status rast_batch_destroy(rast_batch* batch);

/* ---- serving (no counterpart in the reference) --------------------------------------------
 * A dispatcher thread renders submitted scenes with continuous batching: whenever one of
 * `streams` launch slots is free, every queued request that fits the HBM budget (and
 * max_batch) goes into one batched launch, so requests that arrive while others run are
 * admitted as slots and memory free up, and two batches can overlap on the device. Meshes and
 * textures stay resident in the context (upload them before creating the server and do not
 * change them while it runs). one_per_launch = 1 gives the plain server (one request per
 * launch) for comparison. */
typedef struct rast_server rast_server;
typedef struct rast_server_config {
    uint64_t hbm_budget_bytes; /* in-flight scratch + image bytes admitted at once (0 = 40 GB) */
    uint32_t max_batch;        /* scenes per launch (0 = no limit) */
    int streams;               /* batches in flight at once, 1 or 2 (0 = 2; other values are
                                  RAST_INVALID_ARG); the plain server always runs one */
    int one_per_launch;        /* 1: plain server, one request per launch */
} rast_server_config;

rast_status rast_server_create(rast_ctx* ctx, const rast_server_config* cfg, rast_server** out);
/* Queues one scene (argb_out: device or pinned host pointer). RAST_ADMISSION_REFUSED when the
 * scene alone exceeds the budget. Thread-safe. */
rast_status rast_server_submit(rast_server* srv, const rast_scene* scene, uint64_t* request_id);
/* RAST_NOT_READY until the request has finished; then its status, and latency from submit to
 * completion in ms. Returning the final status releases the request's record: a later poll or
 * wait on the same id is RAST_INVALID_ARG. Finished requests nobody collects are kept for the
 * most recent 65536 completions only, so a server that runs indefinitely stays bounded. */
rast_status rast_server_poll(rast_server* srv, uint64_t request_id, double* latency_ms);
/* Waits up to timeout_ms (negative = no limit) for the request; RAST_TIMEOUT when it expires
 * (the request keeps running). Returning the final status releases the record, as for poll. */
rast_status rast_server_wait(rast_server* srv, uint64_t request_id, int timeout_ms, double* latency_ms);
/* Latency percentiles over the most recent 2^20 requests completed since the last reset;
 * completed and requests_per_s count every completion since the reset. */
rast_status rast_server_stats(rast_server* srv, double* p50_ms, double* p99_ms, uint64_t* completed,
                              double* requests_per_s, double* mean_batch);
rast_status rast_server_reset_stats(rast_server* srv);
/* Requests queued, rendering now, and request records held (queued, running, finished and not
 * yet collected). */
rast_status rast_server_info(rast_server* srv, uint64_t* queued, uint64_t* running, uint64_t* tracked);
/* Drains the queue and stops the dispatcher. */
rast_status rast_server_destroy(rast_server* srv);

/* Per-frame statistics of the last framebuffer call: samples written (popcount of
 * depth-passed masks), fragment-shader invocations, texel reads past the texture. */
rast_status rast_stats(rast_ctx* ctx, uint64_t* shaded_samples, uint64_t* fs_invocations,
                       uint64_t* texture_oob);

/* The context's CUDA stream (cudaStream_t) for event timing by the caller. */
void* rast_stream(rast_ctx* ctx);
/* Pipeline kernels this process has launched through the library so far (every context,
 * batch and server; a captured batch counts its kernels once, at capture). For throughput
 * accounting; no counterpart in the reference. */
uint64_t rast_kernel_launches(void);

/* Stage timing with CUDA events on the context stream. When enabled, rast_stage_times
 * fills up to n floats (ms) of the last frame: vertex, bin-count, scan, scatter, raster. */
rast_status rast_set_profiling(rast_ctx* ctx, int enable);
int rast_stage_times(rast_ctx* ctx, float* ms, int n);

/* ---- parity / debug ------------------------------------------------------------------ */

/* Capture the per-sample buffers (depth f32, colour ARGB) of the next frames before resolve;
 * the reference's DepthBuffer / ColorBuffer (src/rasterizer/buffers.rs:82-157). */
rast_status rast_debug_capture_samples(rast_ctx* ctx, int enable);
/* [y][x][sample] arrays of width*height*msaa elements; either pointer may be NULL. */
rast_status rast_read_samples(rast_ctx* ctx, float* depth, uint32_t* color);
/* Fragment log of the next frames: per fragment with a non-empty coverage mask, 4 u32 words
 * {triangle, sub-triangle, (y << 16) | x, (depth-passed mask << 8) | coverage mask}. */
rast_status rast_debug_log_enable(rast_ctx* ctx, uint64_t capacity);
rast_status rast_debug_log_read(rast_ctx* ctx, uint32_t* out, uint64_t capacity,
                                uint64_t* count);
/* Runs one pipeline device function on the GPU for known-answer tests (op codes in
 * rusterizer_gb300/csrc/rast_api.cu). */
rast_status rast_debug_kat(int op, const void* in, size_t in_bytes, void* out, size_t out_bytes);

#ifdef __cplusplus
}
#endif
#endif
