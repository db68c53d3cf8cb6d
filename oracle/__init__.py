"""ctypes wrapper around the CPU oracle (oracle/rast_oracle.c).

TEST INFRASTRUCTURE ONLY: a restatement of the reference renderer's CPU path used to check
the CUDA implementation. Only tests/, the smoke check and the benchmark's CPU-baseline leg
may import this module; the product package never does.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

_f = ctypes.c_float
_fp = ctypes.POINTER(ctypes.c_float)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_vp = ctypes.c_void_p

OK = 0
INVALID_ARG = 1
TEXTURE_OOB = 2
CLIP_OVERFLOW = 4

FS_TEXTURE, FS_COLOR, FS_DEBUG = 0, 1, 2


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        sig = {
            "oracle_create": (_vp, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _f]),
            "oracle_destroy": (None, [_vp]),
            "oracle_bind_texture": (ctypes.c_uint32, [_vp, ctypes.c_int, _u8p, ctypes.c_int, ctypes.c_int]),
            "oracle_draw": (ctypes.c_uint32, [_vp, _fp, _fp, _fp, ctypes.c_uint32, _u32p, ctypes.c_uint32,
                                              _fp, _fp, _fp, ctypes.c_int, ctypes.c_int]),
            "oracle_framebuffer": (ctypes.c_uint32, [_vp, _u32p]),
            "oracle_read_samples": (None, [_vp, _fp, _u32p]),
            "oracle_stats": (None, [_vp, _u64p, _u64p, _u64p]),
            "oracle_log_enable": (None, [_vp, ctypes.c_uint64]),
            "oracle_log_count": (ctypes.c_uint64, [_vp]),
            "oracle_log_copy": (None, [_vp, _u32p]),
            "oracle_kat_mat4_mul": (None, [_fp, _fp, _fp]),
            "oracle_kat_mat4_vec": (None, [_fp, _fp, _fp]),
            "oracle_kat_vec3_len": (_f, [_fp]),
            "oracle_kat_vec3_normalized": (None, [_fp, _fp]),
            "oracle_kat_rotate_x": (None, [_f, _fp]),
            "oracle_kat_rotate_y": (None, [_f, _fp]),
            "oracle_kat_rotate_z": (None, [_f, _fp]),
            "oracle_kat_translate": (None, [_f, _f, _f, _fp]),
            "oracle_kat_project": (None, [_f, _f, _f, _f, _fp]),
            "oracle_kat_perspective_divide": (None, [_fp, _fp]),
            "oracle_kat_viewport": (None, [ctypes.c_int, ctypes.c_int, _fp, _fp, _fp, _fp, _fp, _fp]),
            "oracle_kat_eval_single": (ctypes.c_int, [_fp, _f, _f, _fp]),
            "oracle_kat_fragment": (ctypes.c_int, [_fp, ctypes.c_int, ctypes.c_int, _fp]),
            "oracle_kat_interpolate": (None, [_fp, _fp, _fp, ctypes.c_int, ctypes.c_int, _fp]),
            "oracle_kat_clip": (ctypes.c_int, [_fp, _fp, ctypes.POINTER(ctypes.c_int), _fp, _fp]),
            "oracle_kat_bbox": (None, [_fp, _u64p]),
            "oracle_kat_box_filter": (ctypes.c_uint32, [_u32p]),
            "oracle_kat_to_argb": (ctypes.c_uint32, [_fp]),
            "oracle_kat_tex_sample": (ctypes.c_int, [_u8p, ctypes.c_int, ctypes.c_int, _f, _f, _fp]),
            "oracle_tiles_create": (_vp, [ctypes.c_int, ctypes.c_int]),
            "oracle_tiles_destroy": (None, [_vp]),
            "oracle_tiles_len": (ctypes.c_int, [_vp]),
            "oracle_tiles_get": (None, [_vp, ctypes.c_int, _u64p]),
            "oracle_tiles_mark": (None, [_vp, ctypes.c_uint64, ctypes.c_uint64]),
            "oracle_tiles_next": (None, [_vp]),
            "oracle_tiles_marked_count": (ctypes.c_int, [_vp]),
            "oracle_tiles_prev_marked_count": (ctypes.c_int, [_vp]),
            "oracle_tiles_mask": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def fptr(a):
    return a.ctypes.data_as(_fp)


def f32(x, n=None):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    if n is not None:
        assert a.size == n, (a.size, n)
    return a


class Oracle:
    """Stateful oracle renderer mirroring Renderer/Rasterizer of the reference."""

    def __init__(self, width, height, msaa=4, clear_depth=np.finfo(np.float32).max):
        self.w, self.h, self.msaa = int(width), int(height), int(msaa)
        self._ctx = lib().oracle_create(self.w, self.h, self.msaa, float(np.float32(clear_depth)))
        if not self._ctx:
            raise ValueError("invalid oracle configuration")
        self._keep = []

    def close(self):
        if self._ctx:
            lib().oracle_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bind_texture(self, slot, rgba8):
        t = np.ascontiguousarray(rgba8, dtype=np.uint8)
        h, w = t.shape[:2]
        return lib().oracle_bind_texture(self._ctx, slot, t.ctypes.data_as(_u8p), w, h)

    def draw(self, pos, uv, idx, world, view, proj, fs_id=FS_TEXTURE, rgba=None, nthreads=1):
        pos = f32(pos).reshape(-1)
        uv = f32(uv).reshape(-1)
        idx = np.ascontiguousarray(idx, dtype=np.uint32).reshape(-1)
        nverts = pos.size // 3
        ntris = idx.size // 3
        rg = None if rgba is None else f32(rgba).reshape(-1)
        return lib().oracle_draw(self._ctx, fptr(pos), fptr(uv), None if rg is None else fptr(rg),
                                 nverts, idx.ctypes.data_as(_u32p), ntris,
                                 fptr(f32(world, 16)), fptr(f32(view, 16)), fptr(f32(proj, 16)),
                                 int(fs_id), int(nthreads))

    def framebuffer(self):
        out = np.empty((self.h, self.w), dtype=np.uint32)
        st = lib().oracle_framebuffer(self._ctx, out.ctypes.data_as(_u32p))
        return out, st

    def read_samples(self):
        d = np.empty((self.h, self.w, self.msaa), dtype=np.float32)
        c = np.empty((self.h, self.w, self.msaa), dtype=np.uint32)
        lib().oracle_read_samples(self._ctx, fptr(d), c.ctypes.data_as(_u32p))
        return d, c

    def stats(self):
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        lib().oracle_stats(self._ctx, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return {"shaded_samples": a.value, "fs_invocations": b.value, "texture_oob": c.value}

    def log_enable(self, capacity):
        lib().oracle_log_enable(self._ctx, int(capacity))

    def log(self):
        n = lib().oracle_log_count(self._ctx)
        out = np.empty((n, 4), dtype=np.uint32)
        if n:
            lib().oracle_log_copy(self._ctx, out.ctypes.data_as(_u32p))
        return out


def render_scene(scene, nthreads=1, log_capacity=0):
    """Render a scene dict (see rusterizer_gb300.scenes) with the oracle; returns
    (argb[h,w], depth samples, colour samples, stats, status, log)."""
    o = Oracle(scene["width"], scene["height"], scene.get("msaa", 4),
               scene.get("clear_depth", np.finfo(np.float32).max))
    if log_capacity:
        o.log_enable(log_capacity)
    for slot, tex in enumerate(scene.get("textures", [])):
        st = o.bind_texture(slot, tex)
        assert st == OK
    status = 0
    for d in scene["draws"]:
        status |= o.draw(d["pos"], d["uv"], d["idx"], d["world"], scene["view"], scene["proj"],
                         d.get("fs", FS_TEXTURE), d.get("rgba"), nthreads=nthreads)
    depth, color = o.read_samples()
    stats = o.stats()
    log = o.log() if log_capacity else None
    argb, st = o.framebuffer()
    status |= st
    o.close()
    return argb, depth, color, stats, status, log
