"""Streaming mesh data into resident meshes: rast_mesh_update_async with two meshes used in
turn (the next frame's mesh is copied while the current frame renders) gives every frame the
image of the data it was given, the same as the synchronous rast_mesh_update and the oracle.
The reference borrows the mesh afresh on every render call (src/render.rs:98-114)."""
import ctypes

import numpy as np
import pytest

import oracle
from rusterizer_gb300 import _lib, renderer, scenes

pytestmark = pytest.mark.gpu

fp = ctypes.POINTER(ctypes.c_float)
u32p = ctypes.POINTER(ctypes.c_uint32)


def _scenes():
    a, b = scenes.small_soup(3), scenes.small_soup(4)
    assert a["draws"][0]["pos"].shape == b["draws"][0]["pos"].shape
    assert (a["view"] == b["view"]).all() and (a["proj"] == b["proj"]).all()
    b = dict(b, textures=a["textures"])  # one bound texture for both
    return [a, b]


def _arrays(torch, d):
    pin = lambda x, t: torch.from_numpy(np.ascontiguousarray(x).view(t)).pin_memory()  # noqa: E731
    return pin(d["pos"], np.float32), pin(d["uv"], np.float32), pin(np.asarray(d["idx"], np.uint32), np.int32)


def test_async_updates_of_two_meshes_in_turn():
    torch = pytest.importorskip("torch")
    sc = _scenes()
    refs = [oracle.render_scene(s)[0] for s in sc]
    s0 = sc[0]
    H, W = s0["height"], s0["width"]
    L = _lib.load()
    r = renderer.Renderer(W, H, s0["msaa"])
    r.uniforms().bind_texture(0, renderer.Texture(s0["textures"][0]))
    blk = r.uniforms().write_block()
    blk.view, blk.projection, blk.world = s0["view"], s0["proj"], s0["draws"][0]["world"]
    # two resident meshes used in turn; their upload data is overwritten before any frame
    slots = [renderer.Mesh.from_dict(dict(s["draws"][0], rgba=None)) for s in sc]
    handles = [r.upload(m) for m in slots]
    assert handles[0] != handles[1]
    data = [_arrays(torch, s["draws"][0]) for s in sc]
    out = torch.zeros(W * H, dtype=torch.int32).pin_memory()
    order = [0, 1, 1, 0, 1, 0, 0, 1]  # the scene whose data frame k renders

    def send(update, k):
        p, u, i = data[order[k]]
        assert update(r._ctx, handles[k % 2], ctypes.cast(p.data_ptr(), fp), ctypes.cast(u.data_ptr(), fp),
                      None, ctypes.cast(i.data_ptr(), u32p)) == _lib.OK

    send(L.rast_mesh_update, 0)
    for k in range(len(order)):
        # the next frame's data goes to the other mesh while this frame renders
        if k + 1 < len(order):
            send(L.rast_mesh_update_async, k + 1)
        r.render(slots[k % 2], renderer.VS_MVP, 0)
        st = L.rast_framebuffer(r._ctx, ctypes.c_void_p(out.data_ptr()))
        assert st == _lib.OK, st
        img = out.numpy().view(np.uint32).reshape(H, W)
        assert (img == refs[order[k]]).all(), (k, order[k])
    r.close()
