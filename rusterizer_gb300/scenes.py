"""Seeded synthetic scenes for the five benchmark configurations.

The reference ships no benchmark scenes (its demo animates a cube and a sphere in a window),
so these generators stand in for them with the shapes, sizes and value distributions the
configurations specify. Every scene is a plain dict:

    {"name", "width", "height", "msaa", "clear_depth", "view" (4x4), "proj" (4x4),
     "textures": [RGBA8 (h, w, 4) uint8, ...],
     "draws": [{"pos" (n,3) f32, "uv" (n,2) f32, "rgba" (n,4) f32, "idx" (m,3) u32,
                "world" (4x4), "fs": 0 textured | 1 vertex colour | 2 depth debug}, ...]}

Triangles are emitted clockwise in screen space, the winding the reference's edge functions
cover (src/rasterizer/mod.rs:192-197); with the reference's camera conventions a triangle
(v0, v1, v2) given in camera space projects clockwise iff v0 . (v1 x v2) > 0.
"""
import numpy as np

from . import math as rm
from . import mesh

FLT_MAX = float(np.finfo(np.float32).max)
FS_TEXTURE, FS_COLOR, FS_DEBUG = 0, 1, 2


def checkerboard(n, square, hi=255, lo=128):
    """n x n RGBA8 checkerboard of `square`-texel squares, grey levels hi/lo, alpha 255."""
    yy, xx = np.mgrid[0:n, 0:n]
    v = np.where(((xx // square) + (yy // square)) % 2 == 0, hi, lo).astype(np.uint8)
    t = np.empty((n, n, 4), np.uint8)
    t[..., 0] = t[..., 1] = t[..., 2] = v
    t[..., 3] = 255
    return t


def noise_texture(n, rng):
    return rng.integers(0, 256, size=(n, n, 4), dtype=np.uint8)


def scene_bytes(scene):
    """Algorithmic bytes of one frame: 20 per vertex (xyz + uv), 12 per triangle (indices),
    every bound texture once, 4 per output pixel."""
    b = 4 * scene["width"] * scene["height"]
    for t in scene.get("textures", []):
        b += t.nbytes
    for d in scene["draws"]:
        b += 20 * len(d["pos"]) + 12 * len(d["idx"])
    return int(b)


def scene_triangles(scene):
    return int(sum(len(d["idx"]) for d in scene["draws"]))


# ---------------------------------------------------------------- config 0: the cube

def config0(clear_depth=1.0, fs=FS_TEXTURE):
    """Unit cube (src/mesh.rs:67-149), rotated 30 deg about Y and 20 deg about X, 3 units in
    front of the reference's default camera (src/camera.rs:46-53), fov 60, near 0.1, far 100,
    64x64 checkerboard of 8-texel squares, 800x600, 4x MSAA, depth cleared to 1.0."""
    W, H = 800, 600
    cube = mesh.cube(1.0)
    world = rm.mat4_mul(rm.translate(0.0, 0.0, -2.0),
                        rm.rotate(np.float32(np.deg2rad(20.0)), np.float32(np.deg2rad(30.0)), 0.0))
    return {"name": "cube", "width": W, "height": H, "msaa": 4, "clear_depth": clear_depth,
            "view": rm.camera_view(), "proj": rm.project(0.1, 100.0, np.float32(H / W),
                                                         np.float32(np.deg2rad(60.0))),
            "textures": [checkerboard(64, 8)],
            "draws": [dict(cube, world=world, fs=fs)]}


# ---------------------------------------------------------------- config 1: triangle soup

def _random_rotations(rng, n):
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], 1)


def _equilateral(rng, centroid, edge):
    n = len(centroid)
    ang = np.array([0.0, 2 * np.pi / 3, 4 * np.pi / 3])
    canon = np.stack([np.cos(ang), np.sin(ang), np.zeros(3)], -1)  # (3, 3), edge sqrt(3)
    R = _random_rotations(rng, n)
    v = np.einsum("nij,kj->nki", R, canon) * (edge / np.sqrt(3.0))[:, None, None]
    return v + centroid[:, None, :]


def _make_clockwise(v):
    t = np.einsum("ni,ni->n", v[:, 0], np.cross(v[:, 1], v[:, 2]))
    flip = t < 0
    v[flip, 1], v[flip, 2] = v[flip, 2].copy(), v[flip, 1].copy()
    return v


def soup(ntris, width, height, rng, near=0.1, far=100.0, fov_deg=60.0, straddle=0.1,
         min_px=1.0, max_px=64.0):
    """Independent triangles in view space: centroids uniform in x,y in [-4,4], z in [-20,-1];
    equilateral, edge length log-uniform so the projected size is min_px..max_px; random
    orientation; a `straddle` fraction placed across the near plane (z = -near)."""
    fov = np.deg2rad(fov_deg)
    focal_px = width / (2.0 * np.tan(fov / 2.0))
    ns = int(round(straddle * ntris))
    nr = ntris - ns
    size_px = np.exp(rng.uniform(np.log(min_px), np.log(max_px), size=ntris))
    c = np.empty((ntris, 3))
    c[:nr, 0] = rng.uniform(-4, 4, nr)
    c[:nr, 1] = rng.uniform(-4, 4, nr)
    c[:nr, 2] = rng.uniform(-20, -1, nr)
    edge = np.empty(ntris)
    edge[:nr] = size_px[:nr] * (-c[:nr, 2]) / focal_px
    # near-plane straddlers, sized for the same screen-space range at z = -near
    hw = near * np.tan(fov / 2.0)
    hh = hw * height / width
    c[nr:, 0] = rng.uniform(-0.9 * hw, 0.9 * hw, ns)
    c[nr:, 1] = rng.uniform(-0.9 * hh, 0.9 * hh, ns)
    edge[nr:] = size_px[nr:] * near / focal_px
    c[nr:, 2] = -near + rng.uniform(-0.2, 0.2, ns) * edge[nr:]
    v = _equilateral(rng, c, edge)
    for _ in range(64):
        zs = v[nr:, :, 2]
        bad = ~((zs.min(1) < -near) & (zs.max(1) > -near))
        if not bad.any():
            break
        ib = np.nonzero(bad)[0] + nr
        v[ib] = _equilateral(rng, c[ib], edge[ib])
    v = _make_clockwise(v)
    pos = v.reshape(-1, 3).astype(np.float32)
    uv = rng.random((3 * ntris, 2), dtype=np.float32)  # [0, 1): keeps u*(w-1) inside the texture
    rgba = rng.random((3 * ntris, 4), dtype=np.float32)
    idx = np.arange(3 * ntris, dtype=np.uint32).reshape(-1, 3)
    return {"pos": pos, "uv": uv, "rgba": rgba, "idx": idx}


def soup_scene(ntris, width, height, msaa, rng, tex_size, name="soup", fs=FS_TEXTURE):
    m = soup(ntris, width, height, rng)
    return {"name": name, "width": width, "height": height, "msaa": msaa,
            "clear_depth": FLT_MAX, "view": rm.identity(),
            "proj": rm.project(0.1, 100.0, np.float32(height / width),
                               np.float32(np.deg2rad(60.0))),
            "textures": [noise_texture(tex_size, rng)],
            "draws": [dict(m, world=rm.identity(), fs=fs)]}


def config1(seed=1, ntris=100_000, width=1920, height=1080):
    """100k-triangle soup, 1920x1080, 4x MSAA, 1024x1024 uniform-noise texture."""
    return soup_scene(ntris, width, height, 4, np.random.default_rng(seed), 1024, name="soup100k")


# ---------------------------------------------------------------- config 2: heightfield

HEIGHTFIELD_CAMERA_DISTANCE = 22.75  # mean projected triangle area 0.50 px (mean_screen_area)


def heightfield(n=1000, size=8.0, rng=None, amplitude=0.2, octaves=8):
    """(n+1)^2 vertex grid over x,z in [-size/2, size/2]; height = sum of `octaves` seeded
    sinusoids whose amplitudes sum to `amplitude`; uv = grid / n; 2 n^2 triangles."""
    rng = rng or np.random.default_rng(2)
    g = np.linspace(-size / 2, size / 2, n + 1)
    X, Z = np.meshgrid(g, g)  # row j = z index, column i = x index
    amps = rng.uniform(0.5, 1.0, octaves)
    amps *= amplitude / amps.sum()
    ang = rng.uniform(0, 2 * np.pi, octaves)
    mag = 2 * np.pi / size * rng.uniform(2.0, 24.0, octaves)
    ph = rng.uniform(0, 2 * np.pi, octaves)
    Y = np.zeros_like(X)
    for a, t, k, p in zip(amps, ang, mag, ph):
        Y += a * np.sin(k * (np.cos(t) * X + np.sin(t) * Z) + p)
    pos = np.stack([X, Y, Z], -1).reshape(-1, 3).astype(np.float32)
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1))
    uv = np.stack([ii / n, jj / n], -1).reshape(-1, 2).astype(np.float32)
    q = np.arange(n)
    qi, qj = np.meshgrid(q, q)
    v00 = (qj * (n + 1) + qi).reshape(-1)
    v10 = v00 + 1
    v01 = v00 + (n + 1)
    v11 = v01 + 1
    # quads split along the v00-v11 diagonal, consecutive triangles adjacent on screen
    tri = np.stack([np.stack([v00, v01, v11], -1), np.stack([v00, v11, v10], -1)], 1)
    idx = tri.reshape(-1, 3).astype(np.uint32)
    rgba = np.concatenate([uv, np.full((len(uv), 1), 0.5, np.float32),
                           np.ones((len(uv), 1), np.float32)], 1)
    return {"pos": pos, "uv": uv, "rgba": rgba.astype(np.float32), "idx": idx}


def config2(seed=2, n=1000, width=3840, height=2160, distance=HEIGHTFIELD_CAMERA_DISTANCE):
    """2M-triangle heightfield (1000x1000 quads), viewed from 45 degrees above, 3840x2160,
    4x MSAA, 2048x2048 checkerboard; mean projected triangle area about 0.5 px."""
    rng = np.random.default_rng(seed)
    m = heightfield(n=n, rng=rng)
    d = np.array([0.0, -1.0, 1.0]) / np.sqrt(2.0)
    cam = -distance * d
    view = rm.camera_view(pos=cam, up=(0.0, 1.0, 0.0), direction=d)
    proj = rm.project(0.1, 100.0, np.float32(height / width), np.float32(np.deg2rad(60.0)))
    m["idx"] = _orient_indexed(m["pos"], m["idx"], view)
    return {"name": "heightfield2M", "width": width, "height": height, "msaa": 4,
            "clear_depth": FLT_MAX, "view": view, "proj": proj,
            "textures": [checkerboard(2048, 128)],
            "draws": [dict(m, world=rm.identity(), fs=FS_TEXTURE)]}


def _orient_indexed(pos, idx, view):
    """Flip the index order of an indexed mesh if its first triangle is counter-clockwise
    (the heightfield faces the camera everywhere it is seen from above)."""
    v = pos[idx[0]].astype(np.float64)
    V = np.asarray(view, np.float64)
    cam = (V[:3, :3] @ v.T).T + V[:3, 3]
    t = np.dot(cam[0], np.cross(cam[1], cam[2]))
    if t < 0:
        idx = idx[:, [0, 2, 1]].copy()
    return np.ascontiguousarray(idx)


def mean_screen_area(scene):
    """Mean projected area in pixels of all triangles (float64, for tuning generators)."""
    tot, cnt = 0.0, 0
    P = np.asarray(scene["proj"], np.float64)
    V = np.asarray(scene["view"], np.float64)
    W, H = scene["width"], scene["height"]
    for d in scene["draws"]:
        M = P @ V @ np.asarray(d["world"], np.float64)
        p = np.concatenate([d["pos"].astype(np.float64), np.ones((len(d["pos"]), 1))], 1) @ M.T
        sx = W * (p[:, 0] / p[:, 3] + 1) / 2
        sy = H * (1 - (p[:, 1] / p[:, 3] + 1) / 2)
        i = d["idx"].astype(np.int64)
        a = 0.5 * np.abs((sx[i[:, 1]] - sx[i[:, 0]]) * (sy[i[:, 2]] - sy[i[:, 0]]) -
                         (sx[i[:, 2]] - sx[i[:, 0]]) * (sy[i[:, 1]] - sy[i[:, 0]]))
        tot += a.sum()
        cnt += len(a)
    return tot / max(cnt, 1)


# ---------------------------------------------------------------- configs 3 and 4: batches

RESOLUTIONS = [(256, 256), (512, 512), (1024, 768), (1920, 1080)]


def batch_scene_specs(nscenes=256, seed=3, min_tris=100, max_tris=200_000):
    """Per-scene (ntris, width, height, msaa, seed) for the batched configuration."""
    rng = np.random.default_rng(seed)
    specs = []
    for s in range(nscenes):
        ntris = int(round(np.exp(rng.uniform(np.log(min_tris), np.log(max_tris)))))
        w, h = RESOLUTIONS[rng.integers(0, len(RESOLUTIONS))]
        msaa = int((1, 4)[rng.integers(0, 2)])
        specs.append((ntris, w, h, msaa, int(rng.integers(0, 2**31 - 1))))
    return specs


def batch_scene(spec):
    ntris, w, h, msaa, sseed = spec
    return soup_scene(ntris, w, h, msaa, np.random.default_rng(sseed), 512,
                      name=f"soup{ntris}_{w}x{h}_msaa{msaa}")


def config3(seed=3, nscenes=256):
    """256 independent scenes: ntris log-uniform in [100, 200k] from the soup generator,
    resolution uniform over four sizes, MSAA uniform over {1, 4}, own 512x512 noise texture."""
    return [batch_scene(s) for s in batch_scene_specs(nscenes, seed)]


def config4_specs(seed=4, nscenes=256):
    """Scene pool of the serving configuration (drawn like config 3)."""
    return batch_scene_specs(nscenes, seed)


def small_soup(seed, ntris=2000, width=256, height=192, msaa=4, fs=FS_TEXTURE):
    """Small soup used by parity tests (oracle finishes in well under a second)."""
    return soup_scene(ntris, width, height, msaa, np.random.default_rng(seed), 64,
                      name=f"small{seed}", fs=fs)
