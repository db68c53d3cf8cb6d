"""Continuous-batching render server over rast_server_* (include/rast.h).

Scenes are uploaded once (meshes and textures stay resident); requests then name a scene and
an output buffer. The native dispatcher batches whatever is queued whenever a launch slot is
free and admits requests against an HBM budget; latency is measured from submit to completion.
"""
import ctypes

from . import _lib
from ._lib import ServerConfig, check
from .batch import BatchRenderer


class RenderServer:
    def __init__(self, batch_renderer: BatchRenderer, budget_bytes=40 << 30, max_batch=0, streams=2,
                 one_per_launch=False):
        self.br = batch_renderer
        cfg = ServerConfig(int(budget_bytes), int(max_batch), int(streams), int(bool(one_per_launch)))
        h = ctypes.c_void_p()
        check(_lib.load().rast_server_create(self.br._ctx, ctypes.byref(cfg), ctypes.byref(h)), "server_create")
        self._h = h.value

    def submit(self, scene_index, out_ptr):
        """Queue scene `scene_index` of the batch renderer; its image goes to out_ptr (device)."""
        s = _lib.Scene()
        ctypes.pointer(s)[0] = self.br.scenes[scene_index]
        s.argb_out = int(out_ptr)
        rid = ctypes.c_uint64()
        st = _lib.load().rast_server_submit(self._h, ctypes.byref(s), ctypes.byref(rid))
        if st != _lib.OK:
            raise _lib.RastError(st, "server_submit")
        return rid.value

    def wait(self, rid, timeout_ms=-1):
        lat = ctypes.c_double()
        st = _lib.load().rast_server_wait(self._h, rid, int(timeout_ms), ctypes.byref(lat))
        return st, lat.value

    def poll(self, rid):
        lat = ctypes.c_double()
        st = _lib.load().rast_server_poll(self._h, rid, ctypes.byref(lat))
        return st, lat.value

    def stats(self):
        p50, p99, rps, mb = (ctypes.c_double() for _ in range(4))
        n = ctypes.c_uint64()
        check(_lib.load().rast_server_stats(self._h, ctypes.byref(p50), ctypes.byref(p99), ctypes.byref(n),
                                            ctypes.byref(rps), ctypes.byref(mb)))
        return {"p50_ms": p50.value, "p99_ms": p99.value, "completed": n.value, "req_per_s": rps.value,
                "mean_batch": mb.value}

    def info(self):
        """Requests queued, rendering now, and request records the server holds."""
        q, r, t = (ctypes.c_uint64() for _ in range(3))
        check(_lib.load().rast_server_info(self._h, ctypes.byref(q), ctypes.byref(r), ctypes.byref(t)))
        return {"queued": q.value, "running": r.value, "tracked": t.value}

    def reset_stats(self):
        check(_lib.load().rast_server_reset_stats(self._h))

    def close(self):
        if self._h:
            _lib.load().rast_server_destroy(self._h)
            self._h = None
