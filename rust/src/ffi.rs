//! Raw bindings of include/rast.h (one `extern "C"` item per entry point used by the façade).
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub type rast_status = c_int;
pub type rast_mesh = u32;

pub const RAST_OK: rast_status = 0;
pub const RAST_INVALID_ARG: rast_status = 1;
pub const RAST_OOM: rast_status = 2;
pub const RAST_ADMISSION_REFUSED: rast_status = 3;
pub const RAST_BIN_OVERFLOW: rast_status = 4;
pub const RAST_TIMEOUT: rast_status = 5;
pub const RAST_TEXTURE_OOB: rast_status = 6;
pub const RAST_CLIP_OVERFLOW: rast_status = 7;
pub const RAST_CUDA_ERROR: rast_status = 8;
pub const RAST_NOT_READY: rast_status = 9;

pub const RAST_VS_MVP: c_int = 0;
pub const RAST_FS_TEXTURE: c_int = 0;
pub const RAST_FS_COLOR: c_int = 1;
pub const RAST_FS_DEBUG: c_int = 2;

#[repr(C)]
pub struct rast_ctx {
    _opaque: [u8; 0],
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct rast_scene {
    pub width: c_int,
    pub height: c_int,
    pub msaa: c_int,
    pub tile: c_int,
    pub clear_depth: f32,
    pub mesh: rast_mesh,
    pub texture: c_int,
    pub fs_id: c_int,
    pub world: [f32; 16],
    pub view: [f32; 16],
    pub proj: [f32; 16],
    pub argb_out: *mut u32,
}

extern "C" {
    pub fn rast_status_string(s: rast_status) -> *const c_char;
    pub fn rast_create(width: c_int, height: c_int, msaa: c_int, status: *mut rast_status) -> *mut rast_ctx;
    pub fn rast_destroy(ctx: *mut rast_ctx);
    pub fn rast_set_clear_depth(ctx: *mut rast_ctx, depth: f32) -> rast_status;
    pub fn rast_set_tile_size(ctx: *mut rast_ctx, tile: c_int) -> rast_status;
    pub fn rast_mesh_upload(
        ctx: *mut rast_ctx,
        pos: *const f32,
        uv: *const f32,
        rgba: *const f32,
        nverts: u32,
        idx: *const u32,
        ntris: u32,
        out: *mut rast_mesh,
    ) -> rast_status;
    pub fn rast_mesh_free(ctx: *mut rast_ctx, mesh: rast_mesh) -> rast_status;
    pub fn rast_mesh_update(
        ctx: *mut rast_ctx,
        mesh: rast_mesh,
        pos: *const f32,
        uv: *const f32,
        rgba: *const f32,
        idx: *const u32,
    ) -> rast_status;
    pub fn rast_texture_upload(ctx: *mut rast_ctx, slot: c_int, rgba8: *const u8, w: c_int, h: c_int) -> rast_status;
    pub fn rast_set_uniforms(ctx: *mut rast_ctx, world: *const f32, view: *const f32, proj: *const f32) -> rast_status;
    pub fn rast_draw(ctx: *mut rast_ctx, mesh: rast_mesh, vs_id: c_int, fs_id: c_int) -> rast_status;
    pub fn rast_mesh_update_async(
        ctx: *mut rast_ctx,
        mesh: rast_mesh,
        pos: *const f32,
        uv: *const f32,
        rgba: *const f32,
        idx: *const u32,
    ) -> rast_status;
    pub fn rast_framebuffer(ctx: *mut rast_ctx, argb_out: *mut u32) -> rast_status;
    pub fn rast_framebuffer_async(ctx: *mut rast_ctx, argb_out: *mut u32) -> rast_status;
    pub fn rast_wait_output(ctx: *mut rast_ctx, argb_out: *const u32) -> rast_status;
    pub fn rast_render_batch(ctx: *mut rast_ctx, scenes: *const rast_scene, n: u32) -> rast_status;
    pub fn rast_stats(
        ctx: *mut rast_ctx,
        shaded_samples: *mut u64,
        fs_invocations: *mut u64,
        texture_oob: *mut u64,
    ) -> rast_status;
    pub fn rast_stream(ctx: *mut rast_ctx) -> *mut c_void;
}
