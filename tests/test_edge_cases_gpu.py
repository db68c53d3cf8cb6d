"""GPU parity on adversarial geometry: edges through sample points (exact zero edge values, so
the tie rule decides), shared edges in both windings, axis-aligned edges, slivers, huge and
clipped triangles, depth at the clip range ends. Vertices are placed on the 1/8-pixel grid
through an identity camera, so the screen positions (and the zero edge values) are exact.
Every case compares fragment logs, sample buffers, image and counts with the oracle."""
import numpy as np
import pytest

from parity import assert_parity
from rusterizer_gb300 import math as rm
from rusterizer_gb300 import scenes

pytestmark = pytest.mark.gpu

W, H = 256, 256


def ndc(sx, sy):
    """Screen position (multiples of 1/8 pixel) -> NDC x, y that map back to it exactly."""
    return np.float32(sx / 128.0 - 1.0), np.float32(1.0 - sy / 128.0)


def grid_scene(tris, msaa=4, fs=scenes.FS_TEXTURE, z=None, seed=0):
    """tris: (n, 3, 2) screen positions in eighths of a pixel."""
    rng = np.random.default_rng(seed)
    n = len(tris)
    pos = np.zeros((n * 3, 3), np.float32)
    for i, t in enumerate(tris):
        for k in range(3):
            x, y = ndc(t[k][0] / 8.0, t[k][1] / 8.0)
            pos[3 * i + k] = (x, y, z[i] if z is not None else np.float32(rng.uniform(-0.9, 0.9)))
    uv = rng.uniform(0, 1, (n * 3, 2)).astype(np.float32)
    rgba = rng.uniform(0, 1, (n * 3, 4)).astype(np.float32)
    idx = np.arange(n * 3, dtype=np.uint32).reshape(-1, 3)
    return {"name": "grid", "width": W, "height": H, "msaa": msaa, "clear_depth": np.float32(np.finfo(np.float32).max),
            "view": rm.identity(), "proj": rm.identity(), "textures": [scenes.noise_texture(32, rng)],
            "draws": [{"pos": pos, "uv": uv, "rgba": rgba, "idx": idx, "world": rm.identity(), "fs": fs}]}


def shared_edge_fan(rng, n):
    """Fans of triangles around a centre, every pair sharing an edge, vertices on the grid."""
    tris = []
    for _ in range(n):
        cx, cy = rng.integers(8 * 8, 8 * 248, 2)
        r = int(rng.integers(8, 8 * 24))
        k = int(rng.integers(3, 9))
        ang = np.sort(rng.uniform(0, 2 * np.pi, k))
        ring = [(int(cx + r * np.cos(a)), int(cy + r * np.sin(a))) for a in ang]
        for j in range(k):
            a, b = ring[j], ring[(j + 1) % k]
            tri = [(int(cx), int(cy)), a, b]
            if rng.uniform() < 0.5:
                tri = [tri[0], tri[2], tri[1]]  # the other winding covers nothing
            tris.append(tri)
    return tris


@pytest.mark.parametrize("msaa", [4, 1])
@pytest.mark.parametrize("tile", [8, 16, 32])
def test_edges_through_sample_points(msaa, tile):
    rng = np.random.default_rng(100 + msaa + tile)
    tris = shared_edge_fan(rng, 40)
    # axis-aligned right triangles with corners on pixel corners and sample offsets
    for _ in range(80):
        x, y = (int(v) for v in rng.integers(0, 8 * 240, 2))
        w, h = (int(v) for v in rng.integers(1, 8 * 16, 2))
        tris.append([(x, y), (x + w, y), (x, y + h)])
        tris.append([(x + w, y), (x + w, y + h), (x, y + h)])
    assert_parity(grid_scene(tris, msaa=msaa, seed=msaa * 7 + tile), tile=tile)


def test_slivers_and_tiny_triangles():
    rng = np.random.default_rng(7)
    tris = []
    for _ in range(300):
        x, y = (int(v) for v in rng.integers(0, 8 * 250, 2))
        dx, dy = (int(v) for v in rng.integers(-8 * 120, 8 * 120, 2))
        e = int(rng.integers(1, 4))  # one to three eighths of a pixel wide
        tris.append([(x, y), (x + dx, y + dy), (x + dx + e, y + dy + (e if rng.uniform() < 0.5 else -e))])
    for _ in range(300):
        x, y = (int(v) for v in rng.integers(8, 8 * 250, 2))
        tris.append([(x, y), (x + int(rng.integers(1, 9)), y), (x, y + int(rng.integers(1, 9)))])
    assert_parity(grid_scene(tris, seed=3), tile=16)


@pytest.mark.parametrize("fs,tile", [(scenes.FS_TEXTURE, 32), (scenes.FS_COLOR, 16), (scenes.FS_DEBUG, 8)])
def test_clipped_and_huge_triangles(fs, tile):
    """Vertices far outside the viewport (clipped on the side planes) and depths beyond the
    near and far planes (clipped in z), mixed with grid triangles."""
    rng = np.random.default_rng(11)
    tris = shared_edge_fan(rng, 10)
    z = list(rng.uniform(-0.9, 0.9, len(tris)).astype(np.float32))
    for _ in range(60):
        pts = [(int(v[0]), int(v[1])) for v in rng.integers(-8 * 600, 8 * 850, (3, 2))]
        tris.append(pts)
        z.append(np.float32(rng.choice([-1.5, 1.5, 0.0, -0.999, 0.999])))
    s = grid_scene(tris, fs=fs, z=np.array(z, np.float32), seed=5)
    # each huge triangle can log every pixel of the viewport
    assert_parity(s, tile=tile, log_capacity=len(tris) * W * H)


def test_depth_ties_keep_first_writer():
    """Coplanar duplicates: equal depths, the strict depth test keeps the first triangle's
    colour (src/rasterizer/mod.rs:363-378)."""
    rng = np.random.default_rng(21)
    base = shared_edge_fan(rng, 20)
    tris = base + base + base
    z = np.full(len(tris), np.float32(0.25), np.float32)
    s = grid_scene(tris, fs=scenes.FS_COLOR, z=z, seed=9)
    assert_parity(s, tile=16)


@pytest.mark.parametrize("W,H,msaa,ntris,tile", [
    (8192, 4320, 4, 20000, 0),     # 256 x 135 = 34 560 bins of 32 pixels: three counting bands
    (16384, 16384, 1, 3000, 0),    # the largest frame: 262 144 bins, sixteen bands
    (4100, 4100, 4, 6000, 16),     # 16-pixel bins asked for: 66 049 bins, five bands
])
def test_frames_beyond_one_counting_band(W, H, msaa, ntris, tile):
    """Frames with more bins than one counting pass covers are counted band by band; the image
    must equal the oracle's like any other frame (no sample capture at these sizes)."""
    import oracle
    from rusterizer_gb300 import renderer
    s = scenes.soup_scene(ntris, W, H, msaa, np.random.default_rng(W + H + msaa), 64)
    argb, st, r = renderer.render_scene(s, tile=tile)
    r.close()
    assert st in (0, 6), st
    oa, *_ = oracle.render_scene(s, nthreads=8)
    assert (argb == oa).all()


def nonfinite_scene(fs, seed=3):
    """A soup with NaN, +-inf and +-1e30 (infinite after the transform) in vertex positions,
    texture coordinates and vertex colours."""
    s = scenes.small_soup(61 + fs, ntris=1500, fs=fs)
    d = s["draws"][0]
    pos, uv, rgba = d["pos"].copy(), d["uv"].copy(), d["rgba"].copy()
    rng = np.random.default_rng(seed)
    n = len(pos)
    for val in (np.nan, np.inf, -np.inf, 1e30, -1e30):
        i = rng.choice(n, 12, replace=False)
        pos[i, rng.integers(0, 3, 12)] = val
    for val in (np.nan, np.inf, -np.inf, 1e30):
        i = rng.choice(n, 20, replace=False)
        uv[i, rng.integers(0, 2, 20)] = val
        i = rng.choice(n, 20, replace=False)
        rgba[i, rng.integers(0, 4, 20)] = val
    d.update(pos=pos.astype(np.float32), uv=uv.astype(np.float32), rgba=rgba.astype(np.float32))
    return s


@pytest.mark.parametrize("heavy", [None, 0xFFFFFFFF])
@pytest.mark.parametrize("tile", [16, 32])
@pytest.mark.parametrize("fs", [scenes.FS_TEXTURE, scenes.FS_COLOR, scenes.FS_DEBUG])
def test_nonfinite_inputs(fs, tile, heavy):
    """Non-finite inputs take the reference's paths: f32::min/max skip NaN in the box,
    saturating casts send NaN to 0 and infinities to the ends, comparisons with NaN fail (the
    edge tie rule, the clip tests, the depth test), clamp passes NaN, and texels past the
    texture are reported. Coverage, depth, samples, image and counts equal the oracle's."""
    assert_parity(nonfinite_scene(fs), tile=tile, log_capacity=4_000_000, heavy_entries=heavy)


@pytest.mark.parametrize("heavy", [None, 0xFFFFFFFF])
@pytest.mark.parametrize("msaa", [4, 1])
@pytest.mark.parametrize("wh", [(1, 1), (1, 300), (300, 1), (17, 9), (33, 65)])
def test_degenerate_frame_shapes(wh, msaa, heavy):
    """Frames of one pixel, one row, one column and sizes below one bin: partial tiles on
    every side, bins that hold a single pixel."""
    W, H = wh
    s = scenes.soup_scene(400, W, H, msaa, np.random.default_rng(W * 31 + H), 16)
    assert_parity(s, log_capacity=4_000_000, heavy_entries=heavy)


def test_empty_meshes_between_draws():
    """Meshes with no triangles (and no vertices) drawn between other draws: they add nothing
    and the draws around them keep their submission order."""
    base = scenes.small_soup(71, ntris=600)
    d = base["draws"][0]
    empty = {"pos": np.zeros((0, 3), np.float32), "uv": np.zeros((0, 2), np.float32),
             "rgba": np.zeros((0, 4), np.float32), "idx": np.zeros((0, 3), np.uint32),
             "world": d["world"], "fs": scenes.FS_TEXTURE}
    shifted = dict(d, world=rm.mat4_mul(rm.translate(0.1, 0.0, 0.0), d["world"]), fs=scenes.FS_COLOR)
    s = dict(base, draws=[empty, d, empty, shifted, empty])
    assert_parity(s)
