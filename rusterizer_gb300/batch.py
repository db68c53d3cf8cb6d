"""Batched rendering front end over rast_render_batch / rast_batch_* (include/rast.h).

Many independent scenes (each its own mesh, texture, resolution and MSAA) are rendered by one
launch of each pipeline kernel; a fixed batch can be captured into a CUDA graph and replayed.
The reference renders one scene per Renderer and has no batched form.
"""
import ctypes
import json
import os

import numpy as np

from . import _lib
from ._lib import Scene, check
from .renderer import Mesh, Renderer, Texture

_fp = ctypes.POINTER(ctypes.c_float)
TUNE_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")


def _mat16(m):
    a = np.ascontiguousarray(np.asarray(m, np.float32).reshape(16))
    return (ctypes.c_float * 16)(*a.tolist())


class BatchRenderer:
    """Holds resident meshes and textures of many scenes and renders them together."""

    def __init__(self):
        # the context's own framebuffer size is unused by batches
        self.r = Renderer(16, 16, 4)
        self._ctx = self.r._ctx
        self.scenes = []       # rast_scene descriptors
        self.meta = []         # (width, height, msaa) per scene
        self._tex_count = 0
        self._graphs = []

    def close(self):
        for g in self._graphs:
            _lib.load().rast_batch_destroy(g)
        self._graphs = []
        self.r.close()

    def add_scene(self, scene, tile=0):
        """Upload a scene dict (rusterizer_gb300.scenes) with exactly one draw; returns its index."""
        assert len(scene["draws"]) == 1, "batched scenes carry one draw"
        d = scene["draws"][0]
        mesh = self.r.upload(Mesh.from_dict(d))
        tex = -1
        if d.get("fs", 0) == 0:
            t = Texture(scene["textures"][0])
            self.r.uniforms().bind_texture(self._tex_count, t)
            tex = self._tex_count
            self._tex_count += 1
        s = Scene()
        s.width, s.height, s.msaa = scene["width"], scene["height"], scene.get("msaa", 4)
        s.tile = int(tile)
        s.clear_depth = float(np.float32(scene.get("clear_depth", np.finfo(np.float32).max)))
        s.mesh, s.texture, s.fs_id = mesh, tex, int(d.get("fs", 0))
        s.world, s.view, s.proj = _mat16(d["world"]), _mat16(scene["view"]), _mat16(scene["proj"])
        s.argb_out = None
        self.scenes.append(s)
        self.meta.append((s.width, s.height, s.msaa))
        return len(self.scenes) - 1

    def _array(self, outputs, indices):
        arr = (Scene * len(indices))()
        for k, i in enumerate(indices):
            arr[k] = self.scenes[i]
            arr[k].argb_out = outputs[k]
        return arr

    def render(self, outputs, indices=None):
        """Render scenes `indices` (default all) into `outputs` (one device pointer per scene, an
        int, or numpy uint32 arrays of shape (h, w) on the host)."""
        indices = list(range(len(self.scenes))) if indices is None else list(indices)
        ptrs = [o.ctypes.data if isinstance(o, np.ndarray) else int(o) for o in outputs]
        arr = self._array(ptrs, indices)
        st = _lib.load().rast_render_batch(self._ctx, arr, len(indices))
        if st not in (_lib.OK, _lib.TEXTURE_OOB):
            raise _lib.RastError(st, "render_batch")
        return st

    def autotune(self, outputs, indices=None, cache=True):
        """Pick the fastest settings for this batch (rast_autotune_batch_ex): bin edge, raster
        kernel split and raster CTAs per SM for each MSAA class, and the bin capacity; kept in
        the context and cached on disk."""
        indices = list(range(len(self.scenes))) if indices is None else list(indices)
        ptrs = [int(o) for o in outputs]
        arr = self._array(ptrs, indices)
        t = _lib.Tuning()
        check(_lib.load().rast_autotune_batch_ex(self._ctx, arr, len(indices), ctypes.byref(t)), "autotune")
        res = {"msaa1_tile": t.tile[0], "msaa4_tile": t.tile[1],
               "msaa1_heavy_entries": t.heavy_entries[0], "msaa4_heavy_entries": t.heavy_entries[1],
               "msaa1_raster_ctas_per_sm": t.raster_ctas_per_sm[0], "msaa4_raster_ctas_per_sm": t.raster_ctas_per_sm[1],
               "bin_capacity": t.bin_capacity, "batch_ms": t.batch_ms, "scenes": len(indices)}
        if cache:
            try:
                os.makedirs(os.path.dirname(TUNE_CACHE), exist_ok=True)
                with open(TUNE_CACHE, "w") as f:
                    json.dump(res, f)
            except OSError:
                pass
        return res

    def capture(self, outputs, indices=None):
        """CUDA-graph capture of a fixed batch (device outputs); returns a handle for replay()."""
        indices = list(range(len(self.scenes))) if indices is None else list(indices)
        arr = self._array([int(o) for o in outputs], indices)
        h = ctypes.c_void_p()
        check(_lib.load().rast_batch_create(self._ctx, arr, len(indices), ctypes.byref(h)), "batch_create")
        self._graphs.append(h.value)
        return h.value

    @staticmethod
    def replay(handle, wait=True):
        st = _lib.load().rast_batch_launch(handle, int(wait))
        if st not in (_lib.OK, _lib.TEXTURE_OOB):
            raise _lib.RastError(st, "batch_launch")
        return st

    @staticmethod
    def graph_stream(handle):
        return _lib.load().rast_batch_stream(handle)
