"""Shared helpers for the GPU-vs-oracle parity tests."""
import numpy as np

import oracle
from rusterizer_gb300 import renderer, scenes


def gpu_render(scene, tile=0, log_capacity=0, heavy_entries=None):
    argb, st, r = renderer.render_scene(scene, tile=tile, capture=True, log_capacity=log_capacity,
                                        heavy_entries=heavy_entries)
    depth, color = r.read_samples()
    stats = r.stats()
    log = r.log() if log_capacity else None
    r.close()
    return argb, depth, color, stats, st, log


def sort_log(log):
    if log is None or len(log) == 0:
        return np.zeros((0, 4), np.uint32)
    keys = (log[:, 2], log[:, 1], log[:, 0])
    return log[np.lexsort(keys)]


def channel_diff(a, b):
    d = 0
    for sh in (0, 8, 16, 24):
        d = max(d, int(np.abs(((a >> sh) & 0xFF).astype(np.int32) - ((b >> sh) & 0xFF).astype(np.int32)).max()))
    return d


def assert_parity(scene, tile=0, log=True, nthreads=1, colour_lsb=0, log_capacity=0, heavy_entries=None):
    """Coverage (fragment log), depth-passed masks, per-sample depth and colour bit-exact;
    resolved ARGB within colour_lsb per channel (0 = bit-exact, the expected result).
    A log that reaches its capacity fails the test: both sides drop the rows past it, and the
    GPU's rows arrive in no fixed order, so a full log compares different subsets."""
    cap = 0
    if log:
        cap = log_capacity or 4 * scenes.scene_triangles(scene) + 4 * scene["width"] * scene["height"]
    ga, gd, gc, gs, gst, glog = gpu_render(scene, tile=tile, log_capacity=cap, heavy_entries=heavy_entries)
    oa, od, oc, os_, ost, olog = oracle.render_scene(scene, nthreads=nthreads if not log else 1,
                                                     log_capacity=cap)
    if log:
        assert len(olog) < cap and len(glog) < cap, f"fragment log full at {cap} rows: raise log_capacity"
        gl, ol = sort_log(glog), sort_log(olog)
        assert gl.shape == ol.shape, (gl.shape, ol.shape)
        bad = np.nonzero((gl != ol).any(1))[0]
        assert len(bad) == 0, f"fragment log differs at {len(bad)} rows, first {gl[bad[0]]} vs {ol[bad[0]]}"
    dbad = np.nonzero(gd.view(np.uint32) != od.view(np.uint32))
    assert len(dbad[0]) == 0, f"{len(dbad[0])} depth samples differ, first at {tuple(x[0] for x in dbad)}"
    cbad = np.nonzero(gc != oc)
    assert len(cbad[0]) == 0, f"{len(cbad[0])} colour samples differ, first at {tuple(x[0] for x in cbad)}"
    assert channel_diff(ga, oa) <= colour_lsb
    if colour_lsb == 0:
        assert (ga == oa).all()
    assert gs["shaded_samples"] == os_["shaded_samples"]
    assert gs["fs_invocations"] == os_["fs_invocations"]
    assert gs["texture_oob"] == os_["texture_oob"]
    assert (gst == 6) == bool(ost & oracle.TEXTURE_OOB)
    return ga, gs
