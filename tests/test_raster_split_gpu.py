"""Parity of the two raster kernels: every bin rastered by one warp per tile (k_raster_warp),
every bin by a whole CTA (k_raster), and the split between them by bin entry count
(rast_set_heavy_tile_entries). The reference has one serial pixel loop (src/rasterizer/
mod.rs:330-395); whichever kernel rasters a tile, coverage, depth-passed masks, samples, image
and counts must equal the oracle's bit for bit.

The warp kernel stages 32 items per batch, one per lane; scenes with hundreds of entries per
bin run many batches and drain its fragment and shade rings many times over.
"""
import numpy as np
import pytest

from parity import assert_parity
from rusterizer_gb300 import scenes
from test_edge_cases_gpu import W, H, grid_scene, shared_edge_fan

pytestmark = pytest.mark.gpu

ALL_WARP = 0xFFFFFFFF
SPLITS = [ALL_WARP, 16]


@pytest.mark.parametrize("heavy", SPLITS)
@pytest.mark.parametrize("tile", [8, 16, 32])
def test_cube(heavy, tile):
    assert_parity(scenes.config0(), tile=tile, heavy_entries=heavy)


@pytest.mark.parametrize("fs", [scenes.FS_TEXTURE, scenes.FS_COLOR, scenes.FS_DEBUG])
def test_cube_shaders_warp_kernel(fs):
    assert_parity(scenes.config0(fs=fs, clear_depth=float(np.finfo(np.float32).max)),
                  heavy_entries=ALL_WARP)


@pytest.mark.parametrize("heavy", SPLITS + [64])
@pytest.mark.parametrize("msaa", [4, 1])
@pytest.mark.parametrize("tile", [8, 16, 32])
def test_small_soup(heavy, msaa, tile):
    assert_parity(scenes.small_soup(11 + tile, msaa=msaa), tile=tile, heavy_entries=heavy)


@pytest.mark.parametrize("heavy", SPLITS)
@pytest.mark.parametrize("msaa,tile", [(4, 16), (1, 32), (4, 8)])
def test_high_depth_complexity(heavy, msaa, tile):
    """Hundreds of entries per bin: many item batches per tile, depth culling between them."""
    s = scenes.small_soup(37 + msaa + tile, ntris=30000, width=96, height=80, msaa=msaa)
    ga, gs = assert_parity(s, tile=tile, log=False, nthreads=8, heavy_entries=heavy)
    assert gs["fs_invocations"] > 0


@pytest.mark.parametrize("heavy", SPLITS)
def test_deep_bins_with_fragment_log(heavy):
    """A few thousand triangles over a small frame with the fragment log on (no depth culling):
    every covered sample of every batch, in order."""
    s = scenes.small_soup(43, ntris=3000, width=64, height=48)
    assert_parity(s, tile=16, heavy_entries=heavy, log_capacity=4_000_000)


@pytest.mark.parametrize("fs,tile", [(scenes.FS_TEXTURE, 32), (scenes.FS_COLOR, 16), (scenes.FS_DEBUG, 8)])
def test_clipped_fans_warp_kernel(fs, tile):
    """Clipped polygons (fans of up to 7 triangles per bin entry) mixed with grid triangles:
    entries whose fans straddle the end of a 32-item batch."""
    rng = np.random.default_rng(13)
    tris = shared_edge_fan(rng, 10)
    z = list(rng.uniform(-0.9, 0.9, len(tris)).astype(np.float32))
    for _ in range(60):
        pts = [(int(v[0]), int(v[1])) for v in rng.integers(-8 * 600, 8 * 850, (3, 2))]
        tris.append(pts)
        z.append(np.float32(rng.choice([-1.5, 1.5, 0.0, -0.999, 0.999])))
    s = grid_scene(tris, fs=fs, z=np.array(z, np.float32), seed=7)
    assert_parity(s, tile=tile, log_capacity=len(tris) * W * H, heavy_entries=ALL_WARP)


def test_depth_ties_warp_kernel():
    rng = np.random.default_rng(23)
    base = shared_edge_fan(rng, 20)
    tris = base + base + base
    z = np.full(len(tris), np.float32(0.25), np.float32)
    assert_parity(grid_scene(tris, fs=scenes.FS_COLOR, z=z, seed=9), tile=16, heavy_entries=ALL_WARP)


def test_texture_out_of_bounds_warp_kernel():
    s = scenes.small_soup(53, ntris=800)
    uv = s["draws"][0]["uv"]
    uv[::3] = 1.0
    uv[2::11, 1] = 1.25
    ga, gs = assert_parity(s, heavy_entries=ALL_WARP)
    assert gs["texture_oob"] > 0


@pytest.mark.parametrize("heavy", SPLITS)
def test_config1_full_size(heavy):
    assert_parity(scenes.config1(), log=False, nthreads=8, heavy_entries=heavy)


@pytest.mark.parametrize("heavy", [0, ALL_WARP])
@pytest.mark.parametrize("msaa", [4, 1])
@pytest.mark.parametrize("tile", [8, 16, 32])
@pytest.mark.parametrize("wh", [(1000, 300), (260, 70), (36, 20), (333, 217)])
def test_tile_store_partial_tiles(heavy, msaa, tile, wh):
    """Edge tiles that stick out of the frame on the right and at the bottom, with each raster
    kernel: the warp kernel writes full tile rows with 16-byte stores when the frame's rows are
    a multiple of 16 bytes (widths that are multiples of 4) and pixel by pixel otherwise (333
    wide, and tiles past the right edge). Without the sample capture, which always takes the
    pixel path, the image must equal the oracle's."""
    import oracle
    from rusterizer_gb300 import renderer
    W, H = wh
    s = scenes.soup_scene(1500, W, H, msaa, np.random.default_rng(W * 7 + H + tile), 64)
    argb, st, r = renderer.render_scene(s, tile=tile, heavy_entries=heavy)
    r.close()
    oa, *_ = oracle.render_scene(s, nthreads=4)
    assert st in (0, 6)
    assert (argb == oa).all()
