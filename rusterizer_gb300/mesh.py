"""Mesh generators mirroring the reference's src/mesh.rs.

A mesh is a dict with 'pos' (n,3) f32, 'uv' (n,2) f32, 'rgba' (n,4) f32 and 'idx' (m,3) u32;
the reference keeps the same data as Mesh{vertices, indices, attributes} with
VertexAttribute{color, uvs} per vertex (src/graphics_primitives.rs:9-13).
"""
import numpy as np

from . import math as rm

f32 = np.float32
RED = (1.0, 0.0, 0.0, 1.0)
GREEN = (0.0, 1.0, 0.0, 1.0)
BLUE = (0.0, 0.0, 1.0, 1.0)
WHITE = (1.0, 1.0, 1.0, 1.0)


def _mesh(pos, uv, rgba, idx):
    return {"pos": np.asarray(pos, np.float32).reshape(-1, 3),
            "uv": np.asarray(uv, np.float32).reshape(-1, 2),
            "rgba": np.asarray(rgba, np.float32).reshape(-1, 4),
            "idx": np.asarray(idx, np.uint32).reshape(-1, 3)}


def centered_quad(width):
    """mesh::centered_quad (src/mesh.rs:14-40)."""
    h = f32(width) / f32(2.0)
    pos = [(-h, h, 2.0), (h, h, 2.0), (h, -h, 2.0), (-h, -h, 2.0)]
    return _mesh(pos, [(0, 0), (1, 0), (1, 1), (0, 1)], [RED, BLUE, GREEN, WHITE],
                 [0, 1, 2, 0, 2, 3])


def triangle():
    """mesh::triangle (src/mesh.rs:42-65)."""
    return _mesh([(-1, -1, 2), (0, 1, 2), (1, -1, 2)], [(0, 1), (1, 0), (1, 1)],
                 [RED, BLUE, GREEN], [0, 1, 2])


def cube(width=1.0):
    """mesh::cube (src/mesh.rs:67-149): 24 vertices, 12 triangles, per-face uvs."""
    w = f32(width)
    corners = [
        (-0.5, 0.5, -0.5), (0.5, 0.5, -0.5), (0.5, -0.5, -0.5), (-0.5, -0.5, -0.5),  # front
        (0.5, 0.5, 0.5), (-0.5, 0.5, 0.5), (-0.5, -0.5, 0.5), (0.5, -0.5, 0.5),      # back
        (-0.5, 0.5, 0.5), (-0.5, 0.5, -0.5), (-0.5, -0.5, -0.5), (-0.5, -0.5, 0.5),  # left
        (0.5, 0.5, -0.5), (0.5, 0.5, 0.5), (0.5, -0.5, 0.5), (0.5, -0.5, -0.5),      # right
        (-0.5, 0.5, -0.5), (-0.5, 0.5, 0.5), (0.5, 0.5, 0.5), (0.5, 0.5, -0.5),      # top
        (-0.5, -0.5, 0.5), (-0.5, -0.5, -0.5), (0.5, -0.5, -0.5), (0.5, -0.5, 0.5),  # bottom
    ]
    pos = np.array([[f32(c) * w for c in p] for p in corners], dtype=np.float32)
    idx = []
    for i in range(6):
        o = i * 4
        idx += [o + 0, o + 1, o + 2, o + 0, o + 2, o + 3]
    rgba = [(RED, BLUE, GREEN)[i % 3] for i in range(24)]
    uv = [(0, 0), (1, 0), (1, 1), (0, 1)] * 6
    return _mesh(pos, uv, rgba, idx)


def sphere(radius=0.5):
    """mesh::sphere (src/mesh.rs:151-207): 17 x 9 samples, ISO spherical coordinates."""
    n_phi, n_theta = 17, 9
    r = f32(radius)
    pi = f32(np.pi)
    pos, uv, rgba, idx = [], [], [], []
    for i in range(n_theta):
        for j in range(n_phi):
            theta_ratio = f32(f32(i) / f32(n_theta - 1))
            phi_ratio = f32(f32(j) / f32(n_phi - 1))
            phi = f32(f32(pi * f32(2.0)) * phi_ratio)
            theta = f32(pi * theta_ratio)
            st = rm.sinf(theta)
            x = f32(f32(r * st) * rm.cosf(phi))
            y = f32(r * rm.cosf(theta))
            z = f32(f32(r * st) * rm.sinf(phi))
            pos.append((x, y, z))
            if i < n_theta - 1 and j < n_phi - 1:
                idx += [n_phi * i + j, n_phi * i + (j + 1), n_phi * (i + 1) + (j + 1),
                        n_phi * i + j, n_phi * (i + 1) + (j + 1), n_phi * (i + 1) + j]
            rgba.append((abs(x), abs(y), abs(z), 1.0))
            uv.append((phi_ratio, theta_ratio))
    return _mesh(pos, uv, rgba, idx)
