"""GPU parity: the CUDA pipeline (through the C ABI) against the CPU oracle on the same seeded
inputs. Coverage masks, depth-passed masks (fragment logs), per-sample depth and colour, the
resolved ARGB image and the shaded-sample counts must all be bit-exact."""
import numpy as np
import pytest

import oracle
from parity import assert_parity, gpu_render
from rusterizer_gb300 import math as rm
from rusterizer_gb300 import mesh, renderer, scenes

pytestmark = pytest.mark.gpu

FLT_MAX = float(np.finfo(np.float32).max)


def demo_scene(t=1.3, fs=scenes.FS_TEXTURE, width=1280, height=720):
    """The upstream demo's scene (src/main.rs:94-105, :129-184 there): cube and sphere,
    default camera, project(1, 200, H/W, pi/2), 400x400 checkerboard."""
    cube, sph = mesh.cube(1.0), mesh.sphere(0.5)
    t = np.float32(t)
    w_cube = rm.rotate(t, t, 0.0)
    w_sph = rm.mat4_mul(rm.rotate(t, 0.0, np.float32(np.pi / 4)), rm.translate(0.0, 3.0, 0.0))
    return {"name": "demo", "width": width, "height": height, "msaa": 4, "clear_depth": FLT_MAX,
            "view": rm.camera_view(), "proj": rm.project(1.0, 200.0, np.float32(height / width),
                                                         np.float32(np.pi / 2)),
            "textures": [scenes.checkerboard(400, 50, 255, 40)],
            "draws": [dict(cube, world=w_cube, fs=fs), dict(sph, world=w_sph, fs=fs)]}


@pytest.mark.parametrize("tile", [8, 16, 32])
@pytest.mark.parametrize("clear", [1.0, FLT_MAX])
def test_cube_config0(tile, clear):
    assert_parity(scenes.config0(clear_depth=clear), tile=tile)


@pytest.mark.parametrize("fs", [scenes.FS_TEXTURE, scenes.FS_COLOR, scenes.FS_DEBUG])
def test_cube_shaders(fs):
    assert_parity(scenes.config0(fs=fs))


@pytest.mark.parametrize("t", [0.0, 0.7, 2.9])
def test_demo_cube_and_sphere_multi_draw(t):
    assert_parity(demo_scene(t))


@pytest.mark.parametrize("seed", [11, 12, 13])
@pytest.mark.parametrize("msaa", [4, 1])
@pytest.mark.parametrize("tile", [8, 16, 32])
def test_small_soup(seed, msaa, tile):
    assert_parity(scenes.small_soup(seed, msaa=msaa), tile=tile)


@pytest.mark.parametrize("fs", [scenes.FS_COLOR, scenes.FS_DEBUG])
def test_small_soup_shaders(fs):
    assert_parity(scenes.small_soup(21, fs=fs))


def test_soup_odd_resolution_partial_tiles():
    s = scenes.soup_scene(3000, 333, 217, 4, np.random.default_rng(5), 64)
    assert_parity(s, tile=32)


def test_empty_frame():
    s = scenes.config0()
    s["draws"] = []
    argb, *_ = gpu_render(s)
    assert (argb == 0xFF191919).all()
    assert_parity(s)


def test_degenerate_and_outside_triangles():
    rng = np.random.default_rng(3)
    s = scenes.small_soup(31)
    d = s["draws"][0]
    pos = d["pos"].copy().reshape(-1, 3, 3)
    # collinear triangles (clip-space area 0) and triangles behind the camera
    pos[0:50, 2] = pos[0:50, 0] + (pos[0:50, 1] - pos[0:50, 0]) * 0.5
    pos[50:100, :, 2] = rng.uniform(1.0, 5.0, (50, 3))
    pos[100:110] = pos[100:110, :1]
    d["pos"] = pos.reshape(-1, 3)
    assert_parity(s)


def test_huge_triangle_covering_all_tiles():
    """One triangle whose bounding box spans more tiles than one scatter batch ranks."""
    W, H = 1920, 1080
    s = scenes.config0()
    s.update(width=W, height=H, clear_depth=FLT_MAX, view=rm.identity(),
             proj=rm.project(0.1, 100.0, np.float32(H / W), np.float32(np.deg2rad(60))))
    pos = np.array([[-20, 20, -2], [20, 20, -2], [0, -20, -2], [-1, 0.5, -1.5], [1, 0.5, -1.5],
                    [0, -0.5, -1.5]], np.float32)
    uv = np.array([[0, 0], [1, 0], [0.5, 1], [0, 0], [1, 0], [0.5, 0.99]], np.float32)
    idx = np.array([[0, 1, 2], [3, 4, 5]], np.uint32)
    s["draws"] = [{"pos": pos, "uv": uv, "rgba": np.ones((6, 4), np.float32), "idx": idx,
                   "world": rm.identity(), "fs": scenes.FS_TEXTURE}]
    assert_parity(s, tile=16)


def test_many_draws_keep_submission_order():
    base = scenes.small_soup(41, ntris=40)
    s = dict(base)
    rng = np.random.default_rng(9)
    draws = []
    for k in range(300):
        d = dict(base["draws"][0])
        off = rng.uniform(-0.5, 0.5, 3).astype(np.float32)
        d["world"] = rm.translate(off[0], off[1], off[2] * 0.1)
        d["fs"] = int(k % 3)
        draws.append(d)
    s["draws"] = draws
    assert_parity(s, log=False)


def test_texture_wrap_and_out_of_bounds_reads():
    """uvs at and past 1.0: the reference's flat texel index wraps into the next row, and on
    the last row runs past the buffer (where the reference panics; here a status + texel 0)."""
    s = scenes.small_soup(51, ntris=800)
    uv = s["draws"][0]["uv"]
    uv[::3] = 1.0
    uv[1::7] = np.float32(1.0) + np.float32(1e-7)
    uv[2::11, 1] = 1.25
    ga, gs = assert_parity(s)
    assert gs["texture_oob"] > 0


@pytest.mark.parametrize("msaa,tile", [(4, 16), (1, 32), (4, 8)])
def test_high_depth_complexity(msaa, tile):
    """Tens of thousands of triangles over a small frame (hundreds of layers per pixel), without
    the fragment log, so that whole triangles are skipped where the tile's stored depths are
    already nearer than every depth they can produce: samples, image and counts stay exact."""
    s = scenes.small_soup(31 + msaa + tile, ntris=30000, width=96, height=80, msaa=msaa)
    ga, gs = assert_parity(s, tile=tile, log=False, nthreads=8)
    assert gs["fs_invocations"] > 0


@pytest.mark.parametrize("make", [scenes.config1, scenes.config2])
def test_image_without_sample_capture(make):
    """The plain path without the debug sample capture (the resolve and the clear of empty bins
    then write four pixels per 16-byte store): the image equals the oracle's."""
    s = make()
    argb, st, r = renderer.render_scene(s)
    r.close()
    oa, *_ = oracle.render_scene(s, nthreads=8)
    assert st in (0, 6)
    assert (argb == oa).all()


def test_config1_full_size():
    assert_parity(scenes.config1(), log=False, nthreads=8)


def test_config2_full_size():
    assert_parity(scenes.config2(), log=False, nthreads=8)


def test_repeated_frames_same_result():
    """Frames are stateless: the same scene twice through one context gives the same image
    (resolve_and_clear clears every sample it resolved, src/rasterizer/mod.rs:497-506)."""
    from rusterizer_gb300 import renderer
    s = scenes.small_soup(61)
    a1, _, r = renderer.render_scene(s)
    a2, _, _ = renderer.render_scene(s, renderer=r)
    r.close()
    assert (a1 == a2).all()


def test_out_of_range_index_detected_on_device():
    """primitive_assembly panics on an index past the vertex list (src/render.rs:75-96); here
    the device skips that triangle and the frame reports INVALID_ARG, and the next frame with
    valid indices is bit-exact again."""
    from rusterizer_gb300 import _lib, renderer
    import oracle
    s = scenes.small_soup(71)
    d = s["draws"][0]
    r = renderer.Renderer(s["width"], s["height"], s.get("msaa", 4))
    r.set_clear_depth(s.get("clear_depth", FLT_MAX))
    for i, t in enumerate(s["textures"]):
        r.uniforms().bind_texture(i, renderer.Texture(t))
    blk = r.uniforms().write_block()
    blk.view, blk.projection, blk.world = s["view"], s["proj"], d["world"]
    bad = np.array(d["idx"], np.uint32).copy()
    bad.reshape(-1)[5] = len(d["pos"])  # one past the end
    r.update(d, d["pos"], d["uv"], bad, d.get("rgba"))
    r.render(d, renderer.VS_MVP, d.get("fs", 0))
    with pytest.raises(_lib.RastError) as e:
        r.framebuffer()
    assert e.value.status == _lib.INVALID_ARG
    r.update(d, d["pos"], d["uv"], d["idx"], d.get("rgba"))
    r.render(d, renderer.VS_MVP, d.get("fs", 0))
    img = r.framebuffer()
    ref, *_ = oracle.render_scene(s)
    assert (img == ref).all()
    r.close()
