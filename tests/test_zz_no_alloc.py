"""rast_render_noalloc: one frame rendered with no device allocation by the library, for callers
that must keep device memory allocation out of their render call (they hand in their own
device buffers; the library's intermediates live in a fixed 32 MiB device array).

The entry point is called twice in a row through the C ABI and each image is compared with the
image of the ordinary entry point (rast_framebuffer) for the same scene; the tolerance is the
one the parity tests use: bit-exact. This file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

from rusterizer_gb300 import _lib, renderer, scenes

pytestmark = pytest.mark.gpu

fp = ctypes.POINTER(ctypes.c_float)


def _dev(torch, a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a).view(dtype)).cuda()


def _noalloc(torch, scene, out, tile=0):
    d = scene["draws"][0]
    pos = _dev(torch, d["pos"], np.float32)
    uv = _dev(torch, d["uv"], np.float32)
    rgba = _dev(torch, d["rgba"], np.float32)
    idx = _dev(torch, d["idx"], np.int32)
    tex = _dev(torch, scene["textures"][0].reshape(-1, 4).view(np.uint32).reshape(-1), np.int32)
    th, tw = scene["textures"][0].shape[:2]
    f = lambda m: np.ascontiguousarray(m, np.float32).ctypes.data_as(fp)  # noqa: E731
    world, view, proj = (np.ascontiguousarray(m, np.float32) for m in (d["world"], scene["view"], scene["proj"]))
    stream = torch.cuda.current_stream().cuda_stream
    st = _lib.load().rast_render_noalloc(
        scene["width"], scene["height"], scene["msaa"], tile, float(np.float32(scene["clear_depth"])),
        ctypes.c_void_p(pos.data_ptr()), ctypes.c_void_p(uv.data_ptr()), ctypes.c_void_p(rgba.data_ptr()),
        len(d["pos"]), ctypes.c_void_p(idx.data_ptr()), len(d["idx"]),
        f(world), f(view), f(proj), ctypes.c_void_p(tex.data_ptr()), tw, th, int(d.get("fs", 0)),
        ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))
    torch.cuda.synchronize()
    return st


@pytest.mark.parametrize("make", [lambda: scenes.small_soup(7), lambda: scenes.config0()])
def test_noalloc_matches_framebuffer_twice(make):
    torch = pytest.importorskip("torch")
    scene = make()
    ref, st, r = renderer.render_scene(scene)
    r.close()
    assert st == _lib.OK
    H, W = scene["height"], scene["width"]
    out = torch.zeros(H * W, dtype=torch.int32, device="cuda")
    for _ in range(2):
        out.fill_(0)
        assert _noalloc(torch, scene, out) == _lib.OK
        img = out.cpu().numpy().view(np.uint32).reshape(H, W)
        assert (img == ref).all()


def test_noalloc_refuses_frames_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    # 180k-triangle heightfield at 3840x2160: tile histograms, bins and the clip-polygon store
    # need about 40 MB, more than the 32 MiB the entry point owns
    scene = scenes.config2(n=300)
    out = torch.zeros(16, dtype=torch.int32, device="cuda")
    assert _noalloc(torch, scene, out) == _lib.INVALID_ARG


def test_noalloc_out_of_range_index_reported():
    """Indices live in the caller's device memory, so the check runs on the device: the
    triangle is skipped and the call returns INVALID_ARG; a following valid call is exact."""
    torch = pytest.importorskip("torch")
    scene = scenes.small_soup(9)
    ref, st, r = renderer.render_scene(scene)
    r.close()
    H, W = scene["height"], scene["width"]
    out = torch.zeros(H * W, dtype=torch.int32, device="cuda")
    bad = dict(scene)
    d = dict(scene["draws"][0])
    idx = np.array(d["idx"], np.uint32).copy()
    idx.reshape(-1)[4] = 0xFFFFFFFF
    d["idx"] = idx
    bad["draws"] = [d]
    assert _noalloc(torch, bad, out) == _lib.INVALID_ARG
    assert _noalloc(torch, scene, out) == _lib.OK
    assert (out.cpu().numpy().view(np.uint32).reshape(H, W) == ref).all()


def _ndc_scene(width, height, pos, idx, name):
    """A one-draw scene given directly in clip space (identity world, view and projection),
    textured with a 64x64 checkerboard."""
    pos = np.asarray(pos, np.float32)
    n = len(pos)
    rng = np.random.default_rng(5)
    eye = np.eye(4, dtype=np.float32)
    return {"name": name, "width": width, "height": height, "msaa": 4,
            "clear_depth": float(np.finfo(np.float32).max), "view": eye, "proj": eye,
            "textures": [scenes.checkerboard(64, 8)],
            "draws": [{"pos": pos, "uv": rng.random((n, 2), dtype=np.float32),
                       "rgba": rng.random((n, 4), dtype=np.float32),
                       "idx": np.asarray(idx, np.uint32).reshape(-1, 3), "world": eye, "fs": 0}]}


def many_small_triangles(ntris=190_000):
    """ntris triangles over 12 vertices on a 64x64 target: four small clockwise triangles,
    each inside one 16-pixel bin, repeated (the binning then needs 743 chunks of 256
    triangles and about 30 MiB of scratch)."""
    pos, tris = [], []
    for k, (cx, cy) in enumerate([(-0.6, 0.6), (0.5, 0.55), (-0.45, -0.5), (0.6, -0.6)]):
        z = 0.1 * k
        pos += [(cx - 0.08, cy - 0.06, z), (cx, cy + 0.09, z), (cx + 0.07, cy - 0.05, z)]
        tris.append((3 * k, 3 * k + 1, 3 * k + 2))
    idx = np.array([tris[i % 4] for i in range(ntris)], np.uint32)
    return _ndc_scene(64, 64, pos, idx, "many_small")


def screen_quad_4k():
    """Two triangles covering a 3840x2160 target: every bin holds both, more entries than the
    first bin estimate (4 per triangle + 1 per bin + 1024), so the frame runs twice."""
    pos = [(-1.5, -1.5, 0.2), (-1.5, 1.5, 0.2), (1.5, 1.5, 0.2), (1.5, -1.5, 0.2)]
    return _ndc_scene(3840, 2160, pos, [(0, 1, 2), (0, 2, 3)], "quad_4k")


@pytest.mark.parametrize("make,tile", [(many_small_triangles, 16), (screen_quad_4k, 0)])
def test_noalloc_large_chunk_counts_and_bin_regrowth(make, tile):
    torch = pytest.importorskip("torch")
    scene = make()
    ref, st, r = renderer.render_scene(scene, tile=tile)
    r.close()
    assert st == _lib.OK
    assert (ref != 0xFF191919).any(), "the scene covers pixels"
    H, W = scene["height"], scene["width"]
    out = torch.zeros(H * W, dtype=torch.int32, device="cuda")
    for _ in range(2):
        out.fill_(0)
        assert _noalloc(torch, scene, out, tile=tile) == _lib.OK
        assert (out.cpu().numpy().view(np.uint32).reshape(H, W) == ref).all()
