"""Python mirror of the reference's render API over the C ABI.

Same names, argument meaning and error behaviour as src/render.rs, src/uniform.rs and
src/texture.rs: Renderer(width, height) -> uniforms().write_block().{world, view, projection}
and bind_texture(index, texture) -> render(mesh, vertex_shader, fragment_shader) ->
framebuffer(). The window of the reference (display(), display_frame_time()) is replaced by a
headless framebuffer read-back. Shaders are selected by id (VS_MVP; FS_TEXTURE, FS_COLOR,
FS_DEBUG), the CUDA device functions that stand in for the demo's Rust fn pointers.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import FS_COLOR, FS_DEBUG, FS_TEXTURE, VS_MVP, RastError, check  # noqa: F401
from . import math as rm

_fp = ctypes.POINTER(ctypes.c_float)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_u8p = ctypes.POINTER(ctypes.c_uint8)


def _f32(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if shape is not None:
        a = a.reshape(shape)
    return a


class UniformBlock:
    """UniformBlock{world, view, projection} (src/uniform.rs:4-9)."""

    def __init__(self):
        self.world = rm.identity()
        self.view = rm.identity()
        self.projection = rm.identity()


class Texture:
    """RGBA8 texture, (0, 0) at the top-left (src/texture.rs:6-13)."""

    def __init__(self, rgba8):
        t = np.ascontiguousarray(rgba8, dtype=np.uint8)
        if t.ndim != 3 or t.shape[2] != 4:
            raise ValueError("texture must be (h, w, 4) uint8")
        self.buf = t
        self.height, self.width = t.shape[:2]

    @staticmethod
    def from_rgba8(rgba8):
        return Texture(rgba8)

    @staticmethod
    def from_png_file(path):
        """Texture::from_png_file (src/texture.rs:26-45) for 8-bit RGBA, non-interlaced PNGs."""
        from .png import read_png_rgba8
        return Texture(read_png_rgba8(path))


class Uniforms:
    """Uniforms (src/uniform.rs:11-45)."""

    def __init__(self, renderer):
        self._r = renderer
        self._block = UniformBlock()
        self._textures = []

    def read_block(self):
        return self._block

    def write_block(self):
        return self._block

    def bind_texture(self, index, tex):
        # the reference asserts index == number bound so far (src/uniform.rs:29-33)
        if index != len(self._textures):
            raise ValueError(f"textures must be bound in order: expected index {len(self._textures)}")
        if not isinstance(tex, Texture):
            tex = Texture(tex)
        check(_lib.load().rast_texture_upload(self._r._ctx, index, tex.buf.ctypes.data_as(_u8p),
                                              tex.width, tex.height), "bind_texture")
        self._textures.append(tex)

    def get_texture(self, index):
        return self._textures[index]


class Mesh:
    """Mesh{vertices, indices, attributes} (src/mesh.rs:5-12) as arrays: pos (n,3), uv (n,2),
    rgba (n,4) or None, idx (m,3). Uploaded once per renderer and kept resident."""

    def __init__(self, pos, uv, idx, rgba=None):
        self.pos = _f32(pos, (-1, 3))
        self.uv = _f32(uv, (-1, 2))
        self.rgba = None if rgba is None else _f32(rgba, (-1, 4))
        self.idx = np.ascontiguousarray(np.asarray(idx, dtype=np.uint32).reshape(-1, 3))

    @staticmethod
    def from_dict(d):
        return Mesh(d["pos"], d["uv"], d["idx"], d.get("rgba"))


class Renderer:
    """Renderer (src/render.rs:38-145) on the GPU pipeline. msaa is 4 like the reference, or 1."""

    def __init__(self, width, height, msaa=4, tile=0):
        L = _lib.load()
        st = ctypes.c_int(0)
        self._ctx = L.rast_create(int(width), int(height), int(msaa), ctypes.byref(st))
        if not self._ctx:
            raise RastError(st.value, "Renderer::new")
        self.width, self.height, self.msaa = int(width), int(height), int(msaa)
        self._uniforms = Uniforms(self)
        self._meshes = {}
        self.last_status = _lib.OK
        if tile:
            check(L.rast_set_tile_size(self._ctx, int(tile)), "tile size")

    def close(self):
        if getattr(self, "_ctx", None):
            _lib.load().rast_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def uniforms(self):
        return self._uniforms

    def set_clear_depth(self, depth):
        check(_lib.load().rast_set_clear_depth(self._ctx, float(np.float32(depth))))

    def set_heavy_tile_entries(self, min_entries):
        """Bins with at least min_entries entries are rastered by a whole CTA per tile, the rest
        by one warp per tile (0: all CTA-wide, the default; 0xFFFFFFFF: all by warps)."""
        check(_lib.load().rast_set_heavy_tile_entries(self._ctx, int(min_entries)), "heavy tile entries")

    def upload(self, mesh):
        """Make a mesh resident (once per mesh object); returns its handle."""
        key = id(mesh)
        if key in self._meshes:
            return self._meshes[key][0]
        orig = mesh
        if isinstance(mesh, dict):
            mesh = Mesh.from_dict(mesh)
        h = ctypes.c_uint32()
        rg = None if mesh.rgba is None else mesh.rgba.ctypes.data_as(_fp)
        check(_lib.load().rast_mesh_upload(self._ctx, mesh.pos.ctypes.data_as(_fp),
                                           mesh.uv.ctypes.data_as(_fp), rg, len(mesh.pos),
                                           mesh.idx.ctypes.data_as(_u32p), len(mesh.idx),
                                           ctypes.byref(h)), "mesh upload")
        self._meshes[key] = (h.value, orig)  # keeps the object, and so its id, alive
        return h.value

    def update(self, mesh, pos, uv, idx, rgba=None):
        """Overwrite an uploaded mesh's data in place (same counts). Indices are checked on the
        device: an out-of-range index makes the next framebuffer() raise INVALID_ARG."""
        h = self.upload(mesh)
        pos = np.ascontiguousarray(pos, np.float32)
        uv = np.ascontiguousarray(uv, np.float32)
        idx = np.ascontiguousarray(idx, np.uint32)
        rg = None if rgba is None else np.ascontiguousarray(rgba, np.float32).ctypes.data_as(_fp)
        check(_lib.load().rast_mesh_update(self._ctx, h, pos.ctypes.data_as(_fp), uv.ctypes.data_as(_fp),
                                           rg, idx.ctypes.data_as(_u32p)), "mesh update")

    def update_async(self, mesh, pos, uv, idx, rgba=None):
        """Like update(), with the copies on a side stream after the frames already enqueued; the
        next frame that draws this mesh waits for them on the device. The arrays must stay
        unchanged until that frame is done (page-locked arrays make the copies asynchronous)."""
        h = self.upload(mesh)
        ptr = lambda a: ctypes.cast(_data_ptr(a), _fp)  # noqa: E731
        check(_lib.load().rast_mesh_update_async(self._ctx, h, ptr(pos), ptr(uv),
                                                 None if rgba is None else ptr(rgba),
                                                 ctypes.cast(_data_ptr(idx), _u32p)), "mesh update")

    def render(self, mesh, vertex_shader=VS_MVP, fragment_shader=FS_TEXTURE):
        """Renderer::render (src/render.rs:98-114): queue the mesh with the current uniforms."""
        L = _lib.load()
        h = self.upload(mesh)
        b = self._uniforms.read_block()
        check(L.rast_set_uniforms(self._ctx, _f32(b.world).ctypes.data_as(_fp),
                                  _f32(b.view).ctypes.data_as(_fp),
                                  _f32(b.projection).ctypes.data_as(_fp)), "uniforms")
        check(L.rast_draw(self._ctx, h, int(vertex_shader), int(fragment_shader)), "render")

    def framebuffer(self, out=None):
        """Rasterizer::framebuffer (src/rasterizer/mod.rs:520-522): resolve, clear, and return
        height x width ARGB u32 (y = 0 at the top). A texel read past the texture, where the
        reference panics, leaves last_status == TEXTURE_OOB."""
        if out is None:
            out = np.empty((self.height, self.width), dtype=np.uint32)
        st = _lib.load().rast_framebuffer(self._ctx, out.ctypes.data_as(ctypes.c_void_p))
        self.last_status = st
        if st not in (_lib.OK, _lib.TEXTURE_OOB):
            raise RastError(st, "framebuffer")
        return out

    def framebuffer_async(self, out):
        """Enqueue the frame without waiting (rast_framebuffer_async). `out` is a device pointer,
        a CUDA tensor, or host memory (a numpy array or a page-locked CPU tensor): the image is
        then copied out on a side stream while the next frame renders, and is complete after
        wait_output(out). No overflow re-run: capacities come from earlier framebuffer() calls."""
        st = _lib.load().rast_framebuffer_async(self._ctx, ctypes.c_void_p(_data_ptr(out)))
        if st not in (_lib.OK, _lib.TEXTURE_OOB):
            raise RastError(st, "framebuffer_async")
        return st

    def wait_output(self, out=None):
        """Wait for the asynchronous copies into host array `out` (all of them when None)."""
        check(_lib.load().rast_wait_output(self._ctx, None if out is None else ctypes.c_void_p(_data_ptr(out))),
              "wait_output")

    def display(self):
        """Headless stand-in for Renderer::display (src/render.rs:116-127)."""
        return self.framebuffer()

    def stats(self):
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        check(_lib.load().rast_stats(self._ctx, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"shaded_samples": a.value, "fs_invocations": b.value, "texture_oob": c.value}

    # ---- parity helpers
    def capture_samples(self, enable=True):
        check(_lib.load().rast_debug_capture_samples(self._ctx, int(enable)))

    def read_samples(self):
        d = np.empty((self.height, self.width, self.msaa), np.float32)
        c = np.empty((self.height, self.width, self.msaa), np.uint32)
        check(_lib.load().rast_read_samples(self._ctx, d.ctypes.data_as(_fp), c.ctypes.data_as(_u32p)))
        return d, c

    def log_enable(self, capacity):
        check(_lib.load().rast_debug_log_enable(self._ctx, int(capacity)))

    def log(self):
        L = _lib.load()
        n = ctypes.c_uint64()
        check(L.rast_debug_log_read(self._ctx, None, 0, ctypes.byref(n)))
        out = np.empty((n.value, 4), np.uint32)
        if n.value:
            check(L.rast_debug_log_read(self._ctx, out.ctypes.data_as(_u32p), n.value, ctypes.byref(n)))
        return out

    def stream(self):
        return _lib.load().rast_stream(self._ctx)

    def set_profiling(self, on=True):
        check(_lib.load().rast_set_profiling(self._ctx, int(on)))

    def stage_times(self):
        ms = (ctypes.c_float * 5)()
        n = _lib.load().rast_stage_times(self._ctx, ms, 5)
        return list(ms[:n])


def _data_ptr(a):
    """Address of a numpy array, a torch tensor or a plain integer pointer."""
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return int(a.data_ptr())


def render_scene(scene, tile=0, capture=False, log_capacity=0, renderer=None, heavy_entries=None):
    """Render a scene dict (rusterizer_gb300.scenes) once; returns (argb, status, renderer)."""
    r = renderer or Renderer(scene["width"], scene["height"], scene.get("msaa", 4), tile=tile)
    if heavy_entries is not None:
        r.set_heavy_tile_entries(heavy_entries)
    if renderer is None:
        r.set_clear_depth(scene.get("clear_depth", np.finfo(np.float32).max))
        for i, t in enumerate(scene.get("textures", [])):
            r.uniforms().bind_texture(i, Texture(t))
    if capture:
        r.capture_samples(True)
    if log_capacity:
        r.log_enable(log_capacity)
    blk = r.uniforms().write_block()
    blk.view = scene["view"]
    blk.projection = scene["proj"]
    for d in scene["draws"]:
        blk.world = d["world"]
        r.render(d, VS_MVP, d.get("fs", FS_TEXTURE))
    argb = r.framebuffer()
    return argb, r.last_status, r
