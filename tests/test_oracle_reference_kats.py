"""Pins the CPU oracle (and the host math mirror) to the reference crate's 46 unit tests.

Each test re-expresses one reference test (file:line in tests/golden/reference_unit_tests.json)
with the same inputs and bit-exact expected f32 values.
"""
import ctypes

import numpy as np
import pytest

import oracle
from f32lit import arr, f32lit
from rusterizer_gb300 import math as rm

L = oracle.lib()
fp = oracle.fptr


def bits(a):
    return np.asarray(a, dtype=np.float32).view(np.uint32)


def assert_f32_eq(got, exp):
    got = np.asarray(got, dtype=np.float32)
    exp = np.asarray(exp, dtype=np.float32)
    # assert_eq! on f32 compares with ==, so 0.0 == -0.0; everything else bit for bit
    ok = (got == exp) | (bits(got) == bits(exp))
    assert ok.all(), f"\n got {got!r}\n exp {exp!r}"


# ------------------------------------------------------------------ src/rasterizer/mod.rs

def test_perspective_divide(ref_tests):
    t = ref_tests["mod_rs"]["perspective_divide"]
    clip = arr(t["clip"]).reshape(-1)
    out = np.zeros(12, np.float32)
    L.oracle_kat_perspective_divide(fp(clip), fp(out))
    assert_f32_eq(out, arr(t["expected"]).reshape(-1))


@pytest.mark.parametrize("name", ["viewport_transform_1", "viewport_transform_2"])
def test_viewport_transform(ref_tests, name):
    t = ref_tests["mod_rs"][name]
    ndc = arr(t["ndc"]).reshape(-1)
    pts, dep, w, nrm = (np.zeros(6, np.float32), np.zeros(3, np.float32), np.zeros(3, np.float32),
                        np.zeros(6, np.float32))
    inv = ctypes.c_float()
    L.oracle_kat_viewport(t["width"], t["height"], fp(ndc), fp(pts), fp(dep), fp(w),
                          ctypes.byref(inv), fp(nrm))
    assert_f32_eq(w, arr(t["ndc"])[:, 3])
    assert_f32_eq(dep, arr(t["depths"]))
    assert_f32_eq(np.float32(inv.value), f32lit(t["inv_2x_area"]))
    assert_f32_eq(pts, arr(t["points"]).reshape(-1))


def test_coverage_mask(ref_tests):
    # CoverageMask (mod.rs:25-60) is a u8 bit set; kernels and oracle use the same bit ops
    m = 0
    assert m == 0
    for _op, i, v, expect in ref_tests["mod_rs"]["coverage_mask"]["ops"]:
        m = (m & ~(1 << i)) | (int(v) << i)
        assert [(m >> k) & 1 == 1 for k in range(4)] == expect
        assert (m != 0) == any(expect)


def _edge_tri(ref_tests):
    return arr(ref_tests["mod_rs"]["edge_triangle"]["screen"]).reshape(-1)


@pytest.mark.parametrize("name", ["edge_functions_basic", "edge_functions_partial"])
def test_edge_functions(ref_tests, name):
    scr = _edge_tri(ref_tests)
    for x, y, mask in ref_tests["mod_rs"][name]["evals"]:
        d = np.zeros(4, np.float32)
        assert L.oracle_kat_fragment(fp(scr), x, y, fp(d)) == mask, (x, y)


def test_edge_functions_tie_breaker(ref_tests):
    scr = _edge_tri(ref_tests)
    # normals from the viewport shim: identity viewport of the already-screen triangle
    pts = scr.reshape(3, 3)
    nrm = []
    for k in range(3):
        n = (k + 1) % 3
        vx = np.float32(pts[n, 0] - pts[k, 0])
        vy = np.float32(pts[n, 1] - pts[k, 1])
        nrm.append((-vy, vx))
    for c in ref_tests["mod_rs"]["edge_functions_tie_breaker"]["cases"]:
        e = np.zeros(3, np.float32)
        inside = L.oracle_kat_eval_single(fp(scr), f32lit(c["p"][0]), f32lit(c["p"][1]), fp(e))
        assert bool(inside) == c["inside"]
        k = c["zero_edge"]
        assert e[k] == 0.0
        nx = nrm[k][0]
        assert {"positive": nx > 0, "negative": nx < 0, "zero": nx == 0}[c["normal_x"]]
        if "normal_y" in c:
            assert nrm[k][1] < 0


@pytest.mark.parametrize("name", ["fragment_creation_same_depth",
                                  "fragment_creation_same_depth_partial_coverage"])
def test_fragment_creation_same_depth(ref_tests, name):
    t = ref_tests["mod_rs"][name]
    d = np.zeros(4, np.float32)
    L.oracle_kat_fragment(fp(_edge_tri(ref_tests)), t["pixel"][0], t["pixel"][1], fp(d))
    assert_f32_eq(d, arr(t["depths"]))


def test_fragment_creation_interp_depth(ref_tests):
    t = ref_tests["mod_rs"]["fragment_creation_interp_depth"]
    scr = arr(t["screen"]).reshape(-1)
    for c in t["cases"]:
        d = np.zeros(4, np.float32)
        L.oracle_kat_fragment(fp(scr), c["pixel"][0], c["pixel"][1], fp(d))
        assert_f32_eq(d, arr(c["depths"]))


def test_fragment_creation_interp_attr_same_depth(ref_tests):
    t = ref_tests["mod_rs"]["fragment_creation_interp_attr_same_depth"]
    scr = arr(t["screen"]).reshape(-1)
    w = arr(t["w"])
    attrs = np.zeros((3, 6), np.float32)
    attrs[:, 0] = 1.0  # Color::red()
    attrs[:, 3] = 1.0
    attrs[:, 4:6] = arr(t["uvs"])
    for c in t["cases"]:
        out = np.zeros(6, np.float32)
        L.oracle_kat_interpolate(fp(scr), fp(w), fp(attrs.reshape(-1)), c["pixel"][0],
                                 c["pixel"][1], fp(out))
        assert_f32_eq(out[4:6], arr(c["uv"]))


# ------------------------------------------------------------------ src/rasterizer/clipping.rs

CLIP_RESULT = {0: "Outside", 1: "Inside", 2: "Clipped"}


def clip(verts):
    v = np.asarray(verts, np.float32).reshape(-1)
    a = np.zeros(18, np.float32)
    a.reshape(3, 6)[:, 0] = 1.0
    a.reshape(3, 6)[:, 3] = 1.0
    n = ctypes.c_int()
    ov = np.zeros(30 * 3 * 4, np.float32)
    oa = np.zeros(30 * 3 * 6, np.float32)
    r = L.oracle_kat_clip(fp(v), fp(a), ctypes.byref(n), fp(ov), fp(oa))
    return CLIP_RESULT[r], ov[: n.value * 12].reshape(n.value, 3, 4)


@pytest.mark.parametrize("name", ["fully_inside", "cull_degenerate", "outside",
                                  "partial_right_side_overlap", "two_side_overlap",
                                  "partial_right_side_overlap_single", "on_right_edge",
                                  "late_outside", "complete_coverage", "small_triangle",
                                  "test_clipped_tris_are_inside"])
def test_clipping(ref_tests, name):
    t = ref_tests["clipping_rs"][name]
    res, tris = clip(arr(t["v"]))
    assert res == t["result"]
    if "tris" in t:
        exp = arr(t["tris"])
        assert tris.shape == exp.shape
        assert_f32_eq(tris, exp)
    if "ntris" in t:
        assert tris.shape[0] == t["ntris"]
    if "reclip" in t:
        for tri in tris:
            assert clip(tri)[0] == t["reclip"]


# ------------------------------------------------------------------ src/rasterizer/buffers.rs

def test_box_filter(ref_tests):
    b = ref_tests["buffers_rs"]
    col = b["colors"]

    def avg(cs):
        a = np.array([col[c] if isinstance(c, str) else c for c in cs], dtype=np.uint32)
        return L.oracle_kat_box_filter(a.ctypes.data_as(oracle._u32p))

    for (c,) in b["average_same_color"]["cases"]:
        assert avg([c] * 4) == col[c]
    for name in ("average_two_colors", "average_three_colors", "average_colors"):
        for cs, exp in b[name]["cases"]:
            assert avg(cs) == exp, name


def _tiles(w, h):
    t = L.oracle_tiles_create(w, h)
    return t


def _tile(t, i):
    o = np.zeros(4, np.uint64)
    L.oracle_tiles_get(t, i, o.ctypes.data_as(oracle._u64p))
    return [int(v) for v in o]  # min_x, max_x, min_y, max_y


def test_buffer_tiles_pow_2_square(ref_tests):
    TS = 64
    t = _tiles(128, 128)
    n = L.oracle_tiles_len(t)
    assert n == 128 // TS * 128 // TS
    assert all(L.oracle_tiles_mask(t, 0, i) == 0 for i in range(n))
    assert _tile(t, 0) == [0, TS, 0, TS]
    assert _tile(t, 128 // TS - 1) == [128 - TS, 128, 0, TS]
    assert _tile(t, n - 1) == [128 - TS, 128, 128 - TS, 128]
    L.oracle_tiles_mark(t, 0, 0)
    assert L.oracle_tiles_mask(t, 0, 0)
    L.oracle_tiles_mark(t, TS - 1, TS - 1)
    assert L.oracle_tiles_marked_count(t) == 1
    L.oracle_tiles_mark(t, 127, 127)
    assert L.oracle_tiles_marked_count(t) == 2
    assert L.oracle_tiles_mask(t, 0, n - 1)
    L.oracle_tiles_mark(t, 64, 64)
    assert L.oracle_tiles_marked_count(t) == 2
    assert L.oracle_tiles_mask(t, 0, 64 // TS * (128 // TS) + 64 // TS)
    L.oracle_tiles_destroy(t)


def test_buffer_tiles_uneven_rect(ref_tests):
    TS = 64
    t = _tiles(442, 711)
    nh, nv = 7, 12
    n = L.oracle_tiles_len(t)
    assert n == nh * nv
    assert _tile(t, 0) == [0, TS, 0, TS]
    assert _tile(t, n - 1) == [442 - 442 % TS, 442, 711 - 711 % TS, 711]
    assert _tile(t, 442 // TS) == [442 - 442 % TS, 442, 0, TS]
    assert _tile(t, nh * (nv - 1)) == [0, TS, 711 - 711 % TS, 711]
    L.oracle_tiles_mark(t, 0, 0)
    assert L.oracle_tiles_mask(t, 0, 0)
    L.oracle_tiles_mark(t, TS - 1, TS - 1)
    assert L.oracle_tiles_marked_count(t) == 1
    L.oracle_tiles_mark(t, 711, 442)
    assert L.oracle_tiles_marked_count(t) == 2
    assert L.oracle_tiles_mask(t, 0, n - 1)
    L.oracle_tiles_mark(t, 64, 64)
    assert L.oracle_tiles_marked_count(t) == 3
    k = 64 // TS * (442 // TS + 1) + 64 // TS
    assert L.oracle_tiles_mask(t, 0, k)
    L.oracle_tiles_next(t)
    assert L.oracle_tiles_marked_count(t) == 0
    assert L.oracle_tiles_prev_marked_count(t) == 3
    assert L.oracle_tiles_mask(t, 0, k)
    assert L.oracle_tiles_mask(t, 0, n - 1)
    L.oracle_tiles_next(t)
    assert L.oracle_tiles_marked_count(t) == 0
    assert L.oracle_tiles_prev_marked_count(t) == 0
    L.oracle_tiles_destroy(t)


# ------------------------------------------------------------------ bounding_box.rs, color.rs

def test_bounding_box(ref_tests):
    for c in ref_tests["bounding_box_rs"]["cases"]:
        o = np.zeros(4, np.uint64)
        L.oracle_kat_bbox(fp(arr(c["points"]).reshape(-1)), o.ctypes.data_as(oracle._u64p))
        assert [int(v) for v in o] == c["bbox"]


def test_argb(ref_tests):
    for rgba, exp in ref_tests["color_rs"]["cases"]:
        assert L.oracle_kat_to_argb(fp(arr(rgba))) == exp


# ------------------------------------------------------------------ src/math/matrix.rs

def _M(ref_tests):
    return arr(ref_tests["matrix_rs"]["M"]).reshape(4, 4)


def oracle_mul(a, b):
    out = np.zeros(16, np.float32)
    L.oracle_kat_mat4_mul(fp(np.ascontiguousarray(a, np.float32).reshape(-1)),
                          fp(np.ascontiguousarray(b, np.float32).reshape(-1)), fp(out))
    return out.reshape(4, 4)


def test_matrix_eq_operator(ref_tests):
    M = _M(ref_tests)
    I0, I1 = rm.identity(), rm.identity()
    assert (I0 == I1).all() and (M == M).all()
    assert not (M == I0).all() and not (I1 == M).all()


def test_matrix_mul_identity(ref_tests):
    I = rm.identity()
    assert_f32_eq(oracle_mul(I, I), I)
    assert_f32_eq(rm.mat4_mul(I, I), I)


def test_matrix_rows_columns_transpose(ref_tests):
    M = _M(ref_tests)
    assert M[0].tolist() == [1, 2, 3, 4] and M[3].tolist() == [13, 14, 15, 16]
    assert M[:, 0].tolist() == [1, 5, 9, 13] and M[:, 3].tolist() == [4, 8, 12, 16]
    Mt = rm.transpose(M)
    assert Mt.reshape(-1).tolist() == [1, 5, 9, 13, 2, 6, 10, 14, 3, 7, 11, 15, 4, 8, 12, 16]
    assert (rm.transpose(Mt) == M).all()


def test_matrix_mul(ref_tests):
    M = _M(ref_tests)
    t = ref_tests["matrix_rs"]["mul"]
    for got in (oracle_mul(M, M), rm.mat4_mul(M, M)):
        assert_f32_eq(got, np.array(t["M_M"], np.float32))
    for got in (oracle_mul(M, rm.transpose(M)), rm.mat4_mul(M, rm.transpose(M))):
        assert_f32_eq(got, np.array(t["M_Mt"], np.float32))


# ------------------------------------------------------------------ src/math/vector.rs

def oracle_len(v):
    return np.float32(L.oracle_kat_vec3_len(fp(np.asarray(v, np.float32))))


def oracle_normalized(v):
    o = np.zeros(3, np.float32)
    L.oracle_kat_vec3_normalized(fp(np.asarray(v, np.float32)), fp(o))
    return o


def test_vector_equality(ref_tests):
    v, v1, v2, v3 = (oracle_len(arr(x)) for x in (["0", "0", "0"], ["1", "2", "3"], ["1", "2", "3"],
                                                  ["3", "2", "3"]))
    assert v1 == v2 and v != v1 and v3 != v1 and v3 != v


def test_vector_length(ref_tests):
    for vec, exp in ref_tests["vector_rs"]["length"]["cases"]:
        assert_f32_eq(oracle_len(arr(vec)), f32lit(exp))
        assert_f32_eq(rm.vec_len(arr(vec)), f32lit(exp))


def test_vector_normalized(ref_tests):
    for vec in ref_tests["vector_rs"]["normalized"]["cases"]:
        assert oracle_len(oracle_normalized(arr(vec))) == np.float32(1.0)
        assert rm.vec_len(rm.normalized(arr(vec))) == np.float32(1.0)


def test_vector_neg(ref_tests):
    for vec in ref_tests["vector_rs"]["neg"]["cases"]:
        v = arr(vec)
        assert_f32_eq(np.float32(-1.0) * v, arr(["-" + s if not s.startswith("-") else s[1:]
                                                  for s in vec]))


def test_vector_mul_div(ref_tests):
    for vec, s, exp in ref_tests["vector_rs"]["mul"]["cases"]:
        assert_f32_eq(arr(vec) * f32lit(s), arr(exp))
    for vec, s, exp in ref_tests["vector_rs"]["div"]["cases"]:
        assert_f32_eq(arr(vec) / f32lit(s), arr(exp))


def test_vector_add(ref_tests):
    t = ref_tests["vector_rs"]["add"]
    v = arr(t["v"])
    exp = arr(t["expected"])
    for i in range(3):
        for j in range(3):
            assert_f32_eq(v[i] + v[j], exp[i * 3 + j])


def oracle_mv(m, v):
    o = np.zeros(4, np.float32)
    L.oracle_kat_mat4_vec(fp(np.ascontiguousarray(m, np.float32).reshape(-1)),
                          fp(np.asarray(v, np.float32)), fp(o))
    return o


def test_mat4_mul_identity(ref_tests):
    for vec in arr(ref_tests["vector_rs"]["mat4_mul_identity"]["v"]):
        assert_f32_eq(oracle_mv(rm.identity(), vec), vec)
        assert_f32_eq(rm.mat4_vec(rm.identity(), vec), vec)


def test_mat4_mul_translate(ref_tests):
    t = ref_tests["vector_rs"]["mat4_mul_translate"]
    tx, ty, tz = (f32lit(s) for s in t["t"])
    To = np.zeros(16, np.float32)
    L.oracle_kat_translate(tx, ty, tz, fp(To))
    Tp = rm.translate(tx, ty, tz)
    assert_f32_eq(To.reshape(4, 4), Tp)
    for vec, exp in zip(arr(t["v"]), arr(t["expected"])):
        assert_f32_eq(oracle_mv(Tp, vec), exp)
        assert_f32_eq(rm.mat4_vec(Tp, vec), exp)


def test_mat4_mul_rotate_lh(ref_tests):
    t = ref_tests["vector_rs"]["mat4_mul_rotate_lh"]
    half_pi = np.float32(np.pi / 2)  # std::f32::consts::FRAC_PI_2
    mats = []
    for fn_o, fn_p in ((L.oracle_kat_rotate_x, rm.rotate_x), (L.oracle_kat_rotate_y, rm.rotate_y),
                       (L.oracle_kat_rotate_z, rm.rotate_z)):
        o = np.zeros(16, np.float32)
        fn_o(half_pi, fp(o))
        assert_f32_eq(o.reshape(4, 4), fn_p(half_pi))
        mats.append(fn_p(half_pi))
    v = arr(t["v"])
    exp = arr(t["expected"])
    for i, m in enumerate(mats):
        for j in range(3):
            for w in (0.0, 1.0):
                got = oracle_mv(m, np.append(v[j], np.float32(w)))
                assert_f32_eq(got, np.append(exp[i * 3 + j], np.float32(w)))
                assert_f32_eq(rm.mat4_vec(m, np.append(v[j], np.float32(w))), got)


def test_project_matches_host_math():
    o = np.zeros(16, np.float32)
    L.oracle_kat_project(np.float32(0.1), np.float32(100.0), np.float32(600 / 800),
                         np.float32(np.pi / 3), fp(o))
    assert_f32_eq(o.reshape(4, 4), rm.project(0.1, 100.0, np.float32(600 / 800), np.pi / 3))
