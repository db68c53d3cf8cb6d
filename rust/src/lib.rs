//! The rusterizer render API (`Renderer`, `Uniforms`, `Mesh`, shaders, framebuffer out) over
//! the GB300 raster pipeline in `include/rast.h`.
//!
//! Same call order as the reference demo (src/main.rs:170-176 of the reference crate):
//! `Renderer::new(w, h)`, `uniforms().bind_texture(0, tex)`, per frame
//! `uniforms().write_block().{world, view, projection} = ..`, `render(&mesh, vs, fs)` for every
//! draw, then `framebuffer()` (or `display()`). The shaders the reference passes as function
//! pointers (`VertexShader`/`FragmentShader`, src/render.rs:33-36) are CUDA device functions
//! here, chosen by the marker types that implement the two traits below. There is no CPU
//! fallback: a context that cannot be created is an error.

pub mod ffi;

use std::collections::HashMap;
use std::ffi::CStr;
use std::fmt;
use std::os::raw::c_int;

/// Row-major 4x4 matrix, the layout of the reference's `Matrix.array` (src/math/matrix.rs:7-16).
pub type Mat4 = [[f32; 4]; 4];

pub fn identity() -> Mat4 {
    let mut m = [[0.0f32; 4]; 4];
    for (i, row) in m.iter_mut().enumerate() {
        row[i] = 1.0;
    }
    m
}

/// Status of a failed call (include/rast.h `rast_status`).
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub struct Error(pub ffi::rast_status);

impl fmt::Display for Error {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        let s = unsafe { CStr::from_ptr(ffi::rast_status_string(self.0)) };
        write!(f, "{} ({})", s.to_string_lossy(), self.0)
    }
}

impl std::error::Error for Error {}

fn check(st: ffi::rast_status) -> Result<(), Error> {
    if st == ffi::RAST_OK {
        Ok(())
    } else {
        Err(Error(st))
    }
}

/// Linear RGBA in [0, 1] (src/color.rs of the reference).
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct Color {
    pub r: f32,
    pub g: f32,
    pub b: f32,
    pub a: f32,
}

impl Color {
    pub fn new(r: f32, g: f32, b: f32, a: f32) -> Self {
        Color { r, g, b, a }
    }
}

/// Per-vertex attributes (src/graphics_primitives.rs:9-13).
#[derive(Clone, Copy, Debug, Default)]
pub struct VertexAttribute {
    pub color: Color,
    pub uvs: [f32; 2],
}

impl From<(Color, [f32; 2])> for VertexAttribute {
    fn from((color, uvs): (Color, [f32; 2])) -> Self {
        VertexAttribute { color, uvs }
    }
}

/// `Mesh<WorldSpace>` (src/mesh.rs:5-12): points, triangle list indices, attributes.
#[derive(Clone, Debug, Default)]
pub struct Mesh {
    pub vertices: Vec<[f32; 3]>,
    pub indices: Vec<usize>,
    pub attributes: Vec<VertexAttribute>,
}

/// RGBA8 texture, (0, 0) at the top-left (src/texture.rs:6-13).
#[derive(Clone)]
pub struct Texture {
    buf: Vec<u8>,
    width: usize,
    height: usize,
}

impl Texture {
    pub fn from_rgba8(buf: Vec<u8>, width: usize, height: usize) -> Self {
        assert_eq!(buf.len(), width * height * 4, "texture must be width*height RGBA8");
        Texture { buf, width, height }
    }

    /// Texture::from_png_file (src/texture.rs:26-45): 8-bit RGBA, non-interlaced.
    #[cfg(feature = "png")]
    pub fn from_png_file(path: impl AsRef<std::path::Path>) -> Self {
        let file = std::fs::File::open(path).expect("Failed to read file");
        let decoder = png::Decoder::new(file);
        let (info, mut reader) = decoder.read_info().expect("Failed to read info");
        assert!(info.color_type == png::ColorType::RGBA && info.bit_depth == png::BitDepth::Eight);
        let mut buf = vec![0; info.buffer_size()];
        reader.next_frame(&mut buf).expect("Failed to decode");
        Texture { buf, width: info.width as usize, height: info.height as usize }
    }

    pub fn width(&self) -> usize {
        self.width
    }

    pub fn height(&self) -> usize {
        self.height
    }
}

/// world / view / projection (src/uniform.rs:4-9).
#[derive(Clone, Copy, Debug)]
pub struct UniformBlock {
    pub world: Mat4,
    pub view: Mat4,
    pub projection: Mat4,
}

/// Uniforms (src/uniform.rs:11-45): bound textures and the uniform block.
pub struct Uniforms {
    textures: Vec<Texture>,
    uniform_block: UniformBlock,
}

impl Uniforms {
    pub fn new() -> Self {
        Uniforms {
            textures: Vec::new(),
            uniform_block: UniformBlock { world: identity(), view: identity(), projection: identity() },
        }
    }

    /// Textures are bound in order: `index` must equal the number already bound.
    pub fn bind_texture(&mut self, index: usize, tex: Texture) {
        assert!(self.textures.len() == index);
        self.textures.push(tex);
    }

    pub fn get_texture(&self, index: usize) -> &Texture {
        &self.textures[index]
    }

    pub fn read_block(&self) -> &UniformBlock {
        &self.uniform_block
    }

    pub fn write_block(&mut self) -> &mut UniformBlock {
        &mut self.uniform_block
    }
}

impl Default for Uniforms {
    fn default() -> Self {
        Self::new()
    }
}

/// A vertex shader that runs on the device, selected by id.
pub trait VertexShader {
    const ID: c_int;
}

/// A fragment shader that runs on the device, selected by id.
pub trait FragmentShader {
    const ID: c_int;
}

/// `P * V * W * v`, the demo's vertex shader (src/main.rs:147-152).
pub struct MvpVertexShader;
impl VertexShader for MvpVertexShader {
    const ID: c_int = ffi::RAST_VS_MVP;
}

/// `FS::Texture`: bilinear sample of texture 0 at the interpolated uv (src/main.rs:67-77).
pub struct TextureShader;
impl FragmentShader for TextureShader {
    const ID: c_int = ffi::RAST_FS_TEXTURE;
}

/// `FS::Color`: the interpolated vertex colour.
pub struct ColorShader;
impl FragmentShader for ColorShader {
    const ID: c_int = ffi::RAST_FS_COLOR;
}

/// `FS::Debug`: grayscale of the first sample's depth.
pub struct DebugShader;
impl FragmentShader for DebugShader {
    const ID: c_int = ffi::RAST_FS_DEBUG;
}

/// Per-frame counters of the last `framebuffer()`.
#[derive(Clone, Copy, Debug, Default)]
pub struct Stats {
    pub shaded_samples: u64,
    pub fs_invocations: u64,
    pub texture_oob: u64,
}

/// A mesh kept on the device between frames (upload once, draw many times).
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub struct ResidentMesh(ffi::rast_mesh);

/// One scene of `Renderer::render_batch`: a resident mesh with its own target and matrices.
pub struct BatchScene<'a> {
    pub width: usize,
    pub height: usize,
    pub msaa: usize,
    pub mesh: ResidentMesh,
    pub texture: usize,
    pub fs_id: c_int,
    pub uniforms: UniformBlock,
    pub out: &'a mut [u32],
}

struct Flat {
    pos: Vec<f32>,
    uv: Vec<f32>,
    rgba: Vec<f32>,
    idx: Vec<u32>,
}

fn flatten(mesh: &Mesh) -> Flat {
    assert_eq!(mesh.vertices.len(), mesh.attributes.len(), "one attribute per vertex");
    assert!(mesh.indices.len() % 3 == 0, "triangle list");
    let mut f = Flat {
        pos: Vec::with_capacity(mesh.vertices.len() * 3),
        uv: Vec::with_capacity(mesh.vertices.len() * 2),
        rgba: Vec::with_capacity(mesh.vertices.len() * 4),
        idx: Vec::with_capacity(mesh.indices.len()),
    };
    for v in &mesh.vertices {
        f.pos.extend_from_slice(v);
    }
    for a in &mesh.attributes {
        f.uv.extend_from_slice(&a.uvs);
        f.rgba.extend_from_slice(&[a.color.r, a.color.g, a.color.b, a.color.a]);
    }
    for &i in &mesh.indices {
        // primitive_assembly panics on an index past the vertex list (src/render.rs:75-96)
        assert!(i < mesh.vertices.len(), "index {} out of range", i);
        f.idx.push(i as u32);
    }
    f
}

fn flat16(m: &Mat4) -> [f32; 16] {
    let mut o = [0.0f32; 16];
    for r in 0..4 {
        o[4 * r..4 * r + 4].copy_from_slice(&m[r]);
    }
    o
}

/// Renderer (src/render.rs:38-145) on one GB300. Not `Sync`, like the reference.
pub struct Renderer {
    ctx: *mut ffi::rast_ctx,
    width: usize,
    height: usize,
    uniforms: Uniforms,
    textures_uploaded: usize,
    meshes: HashMap<(usize, usize, usize), ffi::rast_mesh>,
    fb: Vec<u32>,
    last_status: ffi::rast_status,
}

impl Renderer {
    /// Renderer::new: 4x MSAA like the reference. Panics when no context can be created.
    pub fn new(width: usize, height: usize) -> Renderer {
        Self::with_msaa(width, height, 4).unwrap_or_else(|e| panic!("{}", e))
    }

    /// msaa 4 (the reference's RGSS pattern) or 1 (one sample at the pixel centre).
    pub fn with_msaa(width: usize, height: usize, msaa: usize) -> Result<Renderer, Error> {
        let mut st = 0;
        let ctx = unsafe { ffi::rast_create(width as c_int, height as c_int, msaa as c_int, &mut st) };
        if ctx.is_null() {
            return Err(Error(st));
        }
        Ok(Renderer {
            ctx,
            width,
            height,
            uniforms: Uniforms::new(),
            textures_uploaded: 0,
            meshes: HashMap::new(),
            fb: vec![0; width * height],
            last_status: ffi::RAST_OK,
        })
    }

    pub fn uniforms(&mut self) -> &mut Uniforms {
        &mut self.uniforms
    }

    /// Depth clear value (the reference's is f32::MAX, src/rasterizer/buffers.rs:6).
    pub fn set_clear_depth(&mut self, depth: f32) {
        check(unsafe { ffi::rast_set_clear_depth(self.ctx, depth) }).unwrap();
    }

    fn sync_textures(&mut self) -> Result<(), Error> {
        while self.textures_uploaded < self.uniforms.textures.len() {
            let t = &self.uniforms.textures[self.textures_uploaded];
            check(unsafe {
                ffi::rast_texture_upload(
                    self.ctx,
                    self.textures_uploaded as c_int,
                    t.buf.as_ptr(),
                    t.width as c_int,
                    t.height as c_int,
                )
            })?;
            self.textures_uploaded += 1;
        }
        Ok(())
    }

    /// Keep a mesh on the device; draw it with `render_resident` or in batches.
    pub fn upload(&mut self, mesh: &Mesh) -> Result<ResidentMesh, Error> {
        let f = flatten(mesh);
        let mut h = 0;
        check(unsafe {
            ffi::rast_mesh_upload(
                self.ctx,
                f.pos.as_ptr(),
                f.uv.as_ptr(),
                f.rgba.as_ptr(),
                mesh.vertices.len() as u32,
                f.idx.as_ptr(),
                (f.idx.len() / 3) as u32,
                &mut h,
            )
        })?;
        Ok(ResidentMesh(h))
    }

    /// Renderer::render (src/render.rs:98-114): queue `mesh` with the current uniforms. The
    /// mesh is borrowed for this call only, as in the reference: its data is copied to the
    /// device now (into a buffer reused for the same mesh on later calls).
    pub fn render<V: VertexShader, F: FragmentShader>(&mut self, mesh: &Mesh, _vs: V, _fs: F) {
        self.sync_textures().unwrap_or_else(|e| panic!("{}", e));
        let key = (mesh.vertices.as_ptr() as usize, mesh.vertices.len(), mesh.indices.len());
        let h = match self.meshes.get(&key) {
            Some(&h) => {
                let f = flatten(mesh);
                check(unsafe {
                    ffi::rast_mesh_update(self.ctx, h, f.pos.as_ptr(), f.uv.as_ptr(), f.rgba.as_ptr(), f.idx.as_ptr())
                })
                .unwrap_or_else(|e| panic!("{}", e));
                h
            }
            None => {
                let h = self.upload(mesh).unwrap_or_else(|e| panic!("{}", e)).0;
                self.meshes.insert(key, h);
                h
            }
        };
        self.draw(h, V::ID, F::ID);
    }

    /// Queue a resident mesh with the current uniforms.
    pub fn render_resident<V: VertexShader, F: FragmentShader>(&mut self, mesh: ResidentMesh, _vs: V, _fs: F) {
        self.sync_textures().unwrap_or_else(|e| panic!("{}", e));
        self.draw(mesh.0, V::ID, F::ID);
    }

    fn draw(&mut self, h: ffi::rast_mesh, vs: c_int, fs: c_int) {
        let b = self.uniforms.uniform_block;
        let (w, v, p) = (flat16(&b.world), flat16(&b.view), flat16(&b.projection));
        check(unsafe { ffi::rast_set_uniforms(self.ctx, w.as_ptr(), v.as_ptr(), p.as_ptr()) }).unwrap();
        check(unsafe { ffi::rast_draw(self.ctx, h, vs, fs) }).unwrap_or_else(|e| panic!("{}", e));
    }

    /// Rasterizer::framebuffer (src/rasterizer/mod.rs:478-522): render the queued draws,
    /// resolve, clear, and return width*height ARGB, y = 0 at the top. A texel read past the
    /// texture (where the reference panics) leaves `last_status() == RAST_TEXTURE_OOB`.
    pub fn framebuffer(&mut self) -> &[u32] {
        match self.try_framebuffer() {
            Ok(()) => &self.fb,
            Err(e) => panic!("{}", e),
        }
    }

    pub fn try_framebuffer(&mut self) -> Result<(), Error> {
        let st = unsafe { ffi::rast_framebuffer(self.ctx, self.fb.as_mut_ptr()) };
        self.last_status = st;
        if st == ffi::RAST_OK || st == ffi::RAST_TEXTURE_OOB {
            Ok(())
        } else {
            Err(Error(st))
        }
    }

    /// Headless stand-in for Renderer::display (src/render.rs:116-127): renders the frame.
    pub fn display(&mut self) -> Result<bool, Error> {
        self.try_framebuffer().map(|_| true)
    }

    pub fn last_status(&self) -> ffi::rast_status {
        self.last_status
    }

    pub fn width(&self) -> usize {
        self.width
    }

    pub fn height(&self) -> usize {
        self.height
    }

    pub fn stats(&self) -> Stats {
        let mut s = Stats::default();
        check(unsafe { ffi::rast_stats(self.ctx, &mut s.shaded_samples, &mut s.fs_invocations, &mut s.texture_oob) })
            .unwrap();
        s
    }

    /// Render independent scenes with one launch per pipeline kernel (no reference
    /// counterpart). Each scene's image is what rendering it alone gives.
    pub fn render_batch(&mut self, scenes: &mut [BatchScene<'_>]) -> Result<(), Error> {
        self.sync_textures()?;
        let mut raw = Vec::with_capacity(scenes.len());
        for s in scenes.iter_mut() {
            assert_eq!(s.out.len(), s.width * s.height);
            raw.push(ffi::rast_scene {
                width: s.width as c_int,
                height: s.height as c_int,
                msaa: s.msaa as c_int,
                tile: 0,
                clear_depth: f32::MAX,
                mesh: s.mesh.0,
                texture: s.texture as c_int,
                fs_id: s.fs_id,
                world: flat16(&s.uniforms.world),
                view: flat16(&s.uniforms.view),
                proj: flat16(&s.uniforms.projection),
                argb_out: s.out.as_mut_ptr(),
            });
        }
        let st = unsafe { ffi::rast_render_batch(self.ctx, raw.as_ptr(), raw.len() as u32) };
        if st == ffi::RAST_OK || st == ffi::RAST_TEXTURE_OOB {
            Ok(())
        } else {
            Err(Error(st))
        }
    }
}

impl Drop for Renderer {
    fn drop(&mut self) {
        unsafe { ffi::rast_destroy(self.ctx) }
    }
}
