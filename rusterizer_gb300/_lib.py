"""ctypes binding of the C ABI in include/rast.h (librast.so, built in-tree for sm_103a).

There is no CPU fallback: if the shared library is missing or fails to load, every entry point
raises RuntimeError.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "librast.so")

OK, INVALID_ARG, OOM, ADMISSION_REFUSED, BIN_OVERFLOW, TIMEOUT, TEXTURE_OOB, CLIP_OVERFLOW, \
    CUDA_ERROR, NOT_READY = range(10)
STATUS_NAMES = ["OK", "INVALID_ARG", "OOM", "ADMISSION_REFUSED", "BIN_OVERFLOW", "TIMEOUT",
                "TEXTURE_OOB", "CLIP_OVERFLOW", "CUDA_ERROR", "NOT_READY"]

VS_MVP = 0
FS_TEXTURE, FS_COLOR, FS_DEBUG = 0, 1, 2

_c = ctypes
_vp = _c.c_void_p
_fp = _c.POINTER(_c.c_float)
_u8p = _c.POINTER(_c.c_uint8)
_u32p = _c.POINTER(_c.c_uint32)
_u64p = _c.POINTER(_c.c_uint64)
_i = _c.c_int
_u32 = _c.c_uint32
_u64 = _c.c_uint64

SIGNATURES = {
    "rast_status_string": (_c.c_char_p, [_i]),
    "rast_create": (_vp, [_i, _i, _i, _c.POINTER(_i)]),
    "rast_destroy": (None, [_vp]),
    "rast_set_clear_depth": (_i, [_vp, _c.c_float]),
    "rast_set_tile_size": (_i, [_vp, _i]),
    "rast_set_heavy_tile_entries": (_i, [_vp, _u32]),
    "rast_mesh_upload": (_i, [_vp, _fp, _fp, _fp, _u32, _u32p, _u32, _u32p]),
    "rast_mesh_free": (_i, [_vp, _u32]),
    "rast_mesh_update": (_i, [_vp, _u32, _fp, _fp, _fp, _u32p]),
    "rast_mesh_update_async": (_i, [_vp, _u32, _fp, _fp, _fp, _u32p]),
    "rast_texture_upload": (_i, [_vp, _i, _u8p, _i, _i]),
    "rast_set_uniforms": (_i, [_vp, _fp, _fp, _fp]),
    "rast_draw": (_i, [_vp, _u32, _i, _i]),
    "rast_framebuffer": (_i, [_vp, _vp]),
    "rast_framebuffer_async": (_i, [_vp, _vp]),
    "rast_wait_output": (_i, [_vp, _vp]),
    "rast_render_noalloc": (_i, [_i, _i, _i, _i, _c.c_float, _vp, _vp, _vp, _u32, _vp, _u32,
                                 _fp, _fp, _fp, _vp, _i, _i, _i, _vp, _vp]),
    "rast_render_batch": (_i, [_vp, _vp, _u32]),
    "rast_autotune_batch": (_i, [_vp, _vp, _u32, _c.POINTER(_i)]),
    "rast_autotune_batch_ex": (_i, [_vp, _vp, _u32, _vp]),
    "rast_kernel_launches": (_u64, []),
    "rast_batch_create": (_i, [_vp, _vp, _u32, _c.POINTER(_vp)]),
    "rast_batch_launch": (_i, [_vp, _i]),
    "rast_batch_stream": (_vp, [_vp]),
    "rast_batch_destroy": (_i, [_vp]),
    "rast_server_create": (_i, [_vp, _vp, _c.POINTER(_vp)]),
    "rast_server_submit": (_i, [_vp, _vp, _u64p]),
    "rast_server_poll": (_i, [_vp, _u64, _c.POINTER(_c.c_double)]),
    "rast_server_wait": (_i, [_vp, _u64, _i, _c.POINTER(_c.c_double)]),
    "rast_server_stats": (_i, [_vp, _c.POINTER(_c.c_double), _c.POINTER(_c.c_double), _u64p,
                               _c.POINTER(_c.c_double), _c.POINTER(_c.c_double)]),
    "rast_server_reset_stats": (_i, [_vp]),
    "rast_server_info": (_i, [_vp, _u64p, _u64p, _u64p]),
    "rast_server_destroy": (_i, [_vp]),
    "rast_stats": (_i, [_vp, _u64p, _u64p, _u64p]),
    "rast_stream": (_vp, [_vp]),
    "rast_set_profiling": (_i, [_vp, _i]),
    "rast_stage_times": (_i, [_vp, _fp, _i]),
    "rast_debug_capture_samples": (_i, [_vp, _i]),
    "rast_read_samples": (_i, [_vp, _fp, _u32p]),
    "rast_debug_log_enable": (_i, [_vp, _u64]),
    "rast_debug_log_read": (_i, [_vp, _u32p, _u64, _u64p]),
    "rast_debug_kat": (_i, [_i, _vp, _c.c_size_t, _vp, _c.c_size_t]),
}

class Scene(ctypes.Structure):
    """struct rast_scene (include/rast.h)."""
    _fields_ = [("width", _c.c_int), ("height", _c.c_int), ("msaa", _c.c_int), ("tile", _c.c_int),
                ("clear_depth", _c.c_float), ("mesh", _c.c_uint32), ("texture", _c.c_int),
                ("fs_id", _c.c_int), ("world", _c.c_float * 16), ("view", _c.c_float * 16),
                ("proj", _c.c_float * 16), ("argb_out", _c.c_void_p)]


class Tuning(ctypes.Structure):
    """struct rast_tuning (include/rast.h)."""
    _fields_ = [("tile", _c.c_int * 2), ("heavy_entries", _c.c_uint32 * 2), ("raster_ctas_per_sm", _c.c_int * 2),
                ("bin_capacity", _c.c_uint64), ("batch_ms", _c.c_float)]


class ServerConfig(ctypes.Structure):
    """struct rast_server_config (include/rast.h)."""
    _fields_ = [("hbm_budget_bytes", _c.c_uint64), ("max_batch", _c.c_uint32), ("streams", _c.c_int),
                ("one_per_launch", _c.c_int)]


_lib = None


def load():
    """Load librast.so once; raises RuntimeError when it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("librast.so is not built (run python rusterizer_gb300/build.py); "
                               "there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class RastError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__(f"{what}: {name}" if what else name)


def check(status, what=""):
    if status != OK:
        raise RastError(status, what)
    return status
