"""The reference's unit-test vectors run through the CUDA device functions themselves
(rast_debug_kat runs one pipeline function in a one-thread kernel)."""
import ctypes

import numpy as np
import pytest

from f32lit import arr, f32lit
from rusterizer_gb300 import _lib

pytestmark = pytest.mark.gpu


def kat(op, inp, out_bytes):
    inp = np.ascontiguousarray(inp)
    out = np.zeros(out_bytes, np.uint8)
    st = _lib.load().rast_debug_kat(op, inp.ctypes.data_as(ctypes.c_void_p), inp.nbytes,
                                    out.ctypes.data_as(ctypes.c_void_p), out.nbytes)
    assert st == 0
    return out


def as_f32(b):
    return b.view(np.float32)


def eq(got, exp):
    got = np.asarray(got, np.float32)
    exp = np.asarray(exp, np.float32)
    assert ((got == exp) | (got.view(np.uint32) == exp.view(np.uint32))).all(), (got, exp)


def test_perspective_divide(ref_tests):
    t = ref_tests["mod_rs"]["perspective_divide"]
    out = as_f32(kat(0, arr(t["clip"]).reshape(-1), 48))
    eq(out, arr(t["expected"]).reshape(-1))


@pytest.mark.parametrize("name", ["viewport_transform_1", "viewport_transform_2"])
def test_viewport(ref_tests, name):
    t = ref_tests["mod_rs"][name]
    inp = np.concatenate([np.array([t["width"], t["height"]], np.int32).view(np.float32),
                          arr(t["ndc"]).reshape(-1)])
    out = as_f32(kat(1, inp, 19 * 4))
    eq(out[0:6], arr(t["points"]).reshape(-1))
    eq(out[6:9], arr(t["depths"]))
    eq(out[9:12], arr(t["ndc"])[:, 3])
    eq(out[12], f32lit(t["inv_2x_area"]))


def frag_in(screen, x, y):
    return np.concatenate([np.asarray(screen, np.float32).reshape(-1),
                           np.array([x, y], np.int32).view(np.float32)])


@pytest.mark.parametrize("name", ["edge_functions_basic", "edge_functions_partial"])
def test_edge_functions(ref_tests, name):
    scr = arr(ref_tests["mod_rs"]["edge_triangle"]["screen"])
    for x, y, mask in ref_tests["mod_rs"][name]["evals"]:
        out = kat(2, frag_in(scr, x, y), 20)
        assert out[:4].view(np.uint32)[0] == mask, (x, y)


def test_tie_breaker(ref_tests):
    scr = arr(ref_tests["mod_rs"]["edge_triangle"]["screen"]).reshape(-1)
    for c in ref_tests["mod_rs"]["edge_functions_tie_breaker"]["cases"]:
        out = kat(3, np.concatenate([scr, arr(c["p"])]), 16)
        assert bool(out[12:16].view(np.uint32)[0]) == c["inside"]
        assert as_f32(out[:12])[c["zero_edge"]] == 0.0


def test_fragment_depths(ref_tests):
    m = ref_tests["mod_rs"]
    scr = arr(m["edge_triangle"]["screen"])
    for name in ("fragment_creation_same_depth", "fragment_creation_same_depth_partial_coverage"):
        t = m[name]
        out = kat(2, frag_in(scr, *t["pixel"]), 20)
        eq(as_f32(out[4:20]), arr(t["depths"]))
    t = m["fragment_creation_interp_depth"]
    for c in t["cases"]:
        out = kat(2, frag_in(arr(t["screen"]), *c["pixel"]), 20)
        eq(as_f32(out[4:20]), arr(c["depths"]))


def test_interpolated_uvs(ref_tests):
    t = ref_tests["mod_rs"]["fragment_creation_interp_attr_same_depth"]
    attrs = np.zeros((3, 6), np.float32)
    attrs[:, 0] = 1.0
    attrs[:, 3] = 1.0
    attrs[:, 4:6] = arr(t["uvs"])
    for c in t["cases"]:
        inp = np.concatenate([frag_in(arr(t["screen"]), *c["pixel"]), arr(t["w"]), attrs.reshape(-1)])
        out = as_f32(kat(4, inp, 24))
        eq(out[4:6], arr(c["uv"]))


@pytest.mark.parametrize("name", ["fully_inside", "cull_degenerate", "outside",
                                  "partial_right_side_overlap", "two_side_overlap",
                                  "partial_right_side_overlap_single", "on_right_edge",
                                  "late_outside", "complete_coverage", "small_triangle",
                                  "test_clipped_tris_are_inside"])
def test_clipping(ref_tests, name):
    t = ref_tests["clipping_rs"][name]
    res_names = {0: "Outside", 1: "Inside", 2: "Clipped"}

    def clip(v):
        inp = np.concatenate([np.asarray(v, np.float32).reshape(-1), np.zeros(18, np.float32)])
        out = kat(5, inp, 8 + 30 * 48)
        res, n = out[:8].view(np.int32)
        return res_names[int(res)], as_f32(out[8:8 + n * 48]).reshape(n, 3, 4)

    res, tris = clip(arr(t["v"]))
    assert res == t["result"]
    if "tris" in t:
        eq(tris, arr(t["tris"]))
    if "ntris" in t:
        assert len(tris) == t["ntris"]
    if "reclip" in t:
        for tri in tris:
            assert clip(tri)[0] == t["reclip"]


def test_bbox(ref_tests):
    for c in ref_tests["bounding_box_rs"]["cases"]:
        out = kat(6, arr(c["points"]).reshape(-1), 32).view(np.uint64)
        assert [int(v) for v in out] == c["bbox"]


def test_box_filter_and_argb(ref_tests):
    b = ref_tests["buffers_rs"]
    col = b["colors"]
    cases = [([col[c]] * 4, col[c]) for (c,) in b["average_same_color"]["cases"]]
    for name in ("average_two_colors", "average_three_colors", "average_colors"):
        cases += [([col[c] if isinstance(c, str) else c for c in cs], e) for cs, e in b[name]["cases"]]
    for cs, e in cases:
        assert kat(7, np.array(cs, np.uint32), 4).view(np.uint32)[0] == e
    for rgba, e in ref_tests["color_rs"]["cases"]:
        assert kat(8, arr(rgba), 4).view(np.uint32)[0] == e


def test_mat4_vec(ref_tests):
    from rusterizer_gb300 import math as rm
    t = ref_tests["vector_rs"]["mat4_mul_translate"]
    T = rm.translate(*[f32lit(x) for x in t["t"]])
    for v, e in zip(arr(t["v"]), arr(t["expected"])):
        eq(as_f32(kat(10, np.concatenate([T.reshape(-1), v]), 16)), e)


def test_texture_sample_matches_oracle():
    import oracle
    rng = np.random.default_rng(0)
    tex = rng.integers(0, 256, (7, 5, 4), dtype=np.uint8)
    words = tex.reshape(-1, 4).copy().view(np.uint32).reshape(-1)
    for u, v in [(0.0, 0.0), (1.0, 1.0), (0.3, 0.7), (1.0000001, 0.5), (0.5, 1.0000001), (2.0, 2.0)]:
        inp = np.concatenate([np.array([5, 7], np.int32).view(np.float32),
                              np.array([u, v], np.float32), words.view(np.float32)])
        out = kat(9, inp, 20)
        o = np.zeros(4, np.float32)
        oob = oracle.lib().oracle_kat_tex_sample(tex.ctypes.data_as(oracle._u8p), 5, 7, np.float32(u),
                                                 np.float32(v), oracle.fptr(o))
        eq(as_f32(out[:16]), o)
        assert bool(out[16:20].view(np.uint32)[0]) == bool(oob)
