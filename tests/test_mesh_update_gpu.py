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
            if k % 2:  # through the Python mirror
                p, u, i = data[order[k + 1]]
                r.update_async(slots[(k + 1) % 2], p, u, i)
            else:
                send(L.rast_mesh_update_async, k + 1)
        r.render(slots[k % 2], renderer.VS_MVP, 0)
        st = L.rast_framebuffer(r._ctx, ctypes.c_void_p(out.data_ptr()))
        assert st == _lib.OK, st
        img = out.numpy().view(np.uint32).reshape(H, W)
        assert (img == refs[order[k]]).all(), (k, order[k])
    r.close()


def test_async_frames_into_host_memory():
    """rast_framebuffer_async into host arrays: each frame resolves into one of two staging
    buffers and is copied on a side stream while the next frame renders. Every image must equal
    the synchronous frame of the same view once rast_wait_output returns, in pinned and pageable
    memory, and a synchronous frame into the same array afterwards must not be overwritten by
    an earlier frame's late copy."""
    torch = pytest.importorskip("torch")
    from rusterizer_gb300 import math as rm
    s = scenes.small_soup(5, ntris=3000)
    H, W = s["height"], s["width"]
    L = _lib.load()
    r = renderer.Renderer(W, H, s["msaa"])
    r.uniforms().bind_texture(0, renderer.Texture(s["textures"][0]))
    blk = r.uniforms().write_block()
    blk.view, blk.projection = s["view"], s["proj"]
    d = s["draws"][0]
    worlds = [rm.mat4_mul(rm.translate(np.float32(0.05 * k), 0.0, 0.0), d["world"]) for k in range(7)]

    def frame(k):
        blk.world = worlds[k]
        r.render(d, renderer.VS_MVP, d.get("fs", 0))

    want = []
    for k in range(len(worlds)):
        frame(k)
        want.append(r.framebuffer().copy())  # synchronous: also sizes the context's capacities
    assert len({w.tobytes() for w in want}) == len(want)  # the views differ
    pinned = [torch.zeros(W * H, dtype=torch.int32).pin_memory() for _ in range(2)]
    pageable = [np.zeros(W * H, np.uint32) for _ in range(2)]
    for outs, ptr in ((pinned, lambda o: o.data_ptr()), (pageable, lambda o: o.ctypes.data)):
        for k in range(len(worlds)):
            frame(k)
            if outs is pinned:  # through the C ABI
                assert L.rast_framebuffer_async(r._ctx, ctypes.c_void_p(ptr(outs[k % 2]))) == _lib.OK
            else:  # through the Python mirror
                r.framebuffer_async(outs[k % 2])
            if k:
                prev = outs[(k - 1) % 2]
                if outs is pinned:
                    assert L.rast_wait_output(r._ctx, ctypes.c_void_p(ptr(prev))) == _lib.OK
                else:
                    r.wait_output(prev)
                got = prev.numpy() if hasattr(prev, "numpy") else prev
                assert (got.view(np.uint32).reshape(H, W) == want[k - 1]).all(), k - 1
        r.wait_output()
        last = outs[(len(worlds) - 1) % 2]
        got = last.numpy() if hasattr(last, "numpy") else last
        assert (got.view(np.uint32).reshape(H, W) == want[-1]).all()
    # an asynchronous frame, then a synchronous one into the same host array
    frame(0)
    assert L.rast_framebuffer_async(r._ctx, ctypes.c_void_p(pinned[0].data_ptr())) == _lib.OK
    frame(3)
    assert L.rast_framebuffer(r._ctx, ctypes.c_void_p(pinned[0].data_ptr())) == _lib.OK
    assert (pinned[0].numpy().view(np.uint32).reshape(H, W) == want[3]).all()
    r.close()
    assert (want[0] == oracle.render_scene(dict(s, draws=[dict(d, world=worlds[0])]))[0]).all()
