"""Host-side linear algebra with the reference's exact f32 operation order.

Mirrors the reference crate's math module (src/math/{vector,matrix,transform,mod}.rs and
src/camera.rs). Matrices are 4x4 row-major float32 numpy arrays, the layout of
Matrix.array (src/math/matrix.rs:7-16). Every scalar operation rounds to f32 once, in the
reference's order (Vector::dot accumulates from 0.0, src/math/vector.rs:17-23), and
sin/cos/tan come from the C library's sinf/cosf/tanf, which is what Rust's f32 methods call
on Linux. The results feed rast_set_uniforms; the GPU then only evaluates MVP * v.
"""
import ctypes
import ctypes.util

import numpy as np

f32 = np.float32

_libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
for _n in ("sinf", "cosf", "tanf", "sqrtf"):
    getattr(_libm, _n).restype = ctypes.c_float
    getattr(_libm, _n).argtypes = [ctypes.c_float]


def sinf(x):
    return f32(_libm.sinf(f32(x)))


def cosf(x):
    return f32(_libm.cosf(f32(x)))


def tanf(x):
    return f32(_libm.tanf(f32(x)))


def sqrtf(x):
    return f32(_libm.sqrtf(f32(x)))


def dot(a, b):
    """Vector::dot (src/math/vector.rs:17-23): sum = 0.0; sum += a[k]*b[k] in order."""
    s = f32(0.0)
    for x, y in zip(a, b):
        s = f32(s + f32(f32(x) * f32(y)))
    return s


def mat4(*vals):
    """mat4(x00, x01, ..., x33), src/math/matrix.rs:20-54 (row-major)."""
    assert len(vals) == 16
    return np.array(vals, dtype=np.float32).reshape(4, 4)


def identity():
    return np.eye(4, dtype=np.float32)


def mat4_mul(a, b):
    """Mat4 * Mat4 (src/math/matrix.rs:56-79): out[i][j] = row_i(a) . col_j(b)."""
    a = np.asarray(a, dtype=np.float32)
    b = np.asarray(b, dtype=np.float32)
    out = np.empty((4, 4), dtype=np.float32)
    for i in range(4):
        for j in range(4):
            out[i, j] = dot(a[i, :], b[:, j])
    return out


def mat4_vec(m, v):
    """Mat4 * Vec4 / Point4 (src/math/vector.rs:219-240, src/math/point.rs:161-170)."""
    m = np.asarray(m, dtype=np.float32)
    return np.array([dot(m[i, :], v) for i in range(4)], dtype=np.float32)


def transpose(m):
    return np.ascontiguousarray(np.asarray(m, dtype=np.float32).T)


def vec_len(v):
    """Vector::len (src/math/vector.rs:38-40): fold(0.0, acc + e*e).sqrt()."""
    acc = f32(0.0)
    for e in v:
        acc = f32(acc + f32(f32(e) * f32(e)))
    return sqrtf(acc)


def normalized(v):
    """Vector::normalized (src/math/vector.rs:42-44)."""
    n = vec_len(v)
    return np.array([f32(f32(e) / n) for e in v], dtype=np.float32)


def cross3(a, b):
    """Vec3::cross (src/math/vector.rs:197-204)."""
    a = [f32(x) for x in a]
    b = [f32(x) for x in b]
    return np.array([f32(a[1] * b[2] - a[2] * b[1]),
                     f32(a[2] * b[0] - a[0] * b[2]),
                     f32(a[0] * b[1] - a[1] * b[0])], dtype=np.float32)


def translate(x, y, z):
    """transform::translate (src/math/transform.rs:10-17)."""
    return mat4(1, 0, 0, x, 0, 1, 0, y, 0, 0, 1, z, 0, 0, 0, 1)


def rotate_x(rad):
    """transform::rotate_x (src/math/transform.rs:19-41)."""
    c, s = cosf(rad), sinf(rad)
    return mat4(1, 0, 0, 0, 0, c, -s, 0, 0, s, c, 0, 0, 0, 0, 1)


def rotate_y(rad):
    """transform::rotate_y (src/math/transform.rs:43-65)."""
    c, s = cosf(rad), sinf(rad)
    return mat4(c, 0, s, 0, 0, 1, 0, 0, -s, 0, c, 0, 0, 0, 0, 1)


def rotate_z(rad):
    """transform::rotate_z (src/math/transform.rs:67-89)."""
    c, s = cosf(rad), sinf(rad)
    return mat4(c, -s, 0, 0, s, c, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1)


def rotate(x, y, z):
    """transform::rotate (src/math/transform.rs:91-96): Rz * Ry * Rx, left-associative."""
    return mat4_mul(mat4_mul(rotate_z(z), rotate_y(y)), rotate_x(x))


def project(near, far, aspect_ratio, vert_fov):
    """math::project (src/math/mod.rs:92-122)."""
    near, far, aspect_ratio, vert_fov = f32(near), f32(far), f32(aspect_ratio), f32(vert_fov)
    assert near > 0
    half_width = f32(tanf(f32(vert_fov / f32(2.0))) * near)
    half_height = f32(aspect_ratio * half_width)
    return mat4(f32(near / half_width), 0, 0, 0,
                0, f32(near / half_height), 0, 0,
                0, 0, f32(f32(-f32(far + near)) / f32(far - near)),
                f32(f32(f32(f32(-2.0) * far) * near) / f32(far - near)),
                0, 0, -1, 0)


def camera_view(pos=(0.0, 0.0, -5.0), up=(0.0, 1.0, 0.0), direction=(0.0, 0.0, 1.0)):
    """Camera::get_view_matrix (src/camera.rs:10-43); defaults are Camera::default (:46-53)."""
    up = normalized(np.asarray(up, dtype=np.float32))
    direction = normalized(np.asarray(direction, dtype=np.float32))
    cam_z = np.array([f32(-1.0) * d for d in direction], dtype=np.float32)
    cam_x = normalized(cross3(cam_z, up))
    cam_y = normalized(cross3(cam_x, cam_z))
    rotation_inv = transpose(mat4(cam_x[0], cam_y[0], cam_z[0], 0,
                                  cam_x[1], cam_y[1], cam_z[1], 0,
                                  cam_x[2], cam_y[2], cam_z[2], 0,
                                  0, 0, 0, 1))
    p = np.asarray(pos, dtype=np.float32)
    translation_inv = translate(f32(-1.0) * p[0], f32(-1.0) * p[1], f32(-1.0) * p[2])
    return mat4_mul(rotation_inv, translation_inv)


def mvp(proj, view, world):
    """P * V * W as the demo vertex shader evaluates it (left-associative)."""
    return mat4_mul(mat4_mul(proj, view), world)
