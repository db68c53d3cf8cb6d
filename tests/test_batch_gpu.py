"""Batched rendering (rast_render_batch, CUDA-graph batches, autotuner): every scene of a mixed
batch matches the oracle bit for bit, and is identical to rendering the same scene alone."""
import numpy as np
import pytest

import oracle
from rusterizer_gb300 import scenes
from rusterizer_gb300.batch import BatchRenderer

pytestmark = pytest.mark.gpu


def mixed_scenes():
    rng = np.random.default_rng(17)
    out = [scenes.config0()]
    for k, (w, h, msaa) in enumerate([(256, 256, 1), (200, 150, 4), (320, 180, 1), (97, 61, 4),
                                      (512, 384, 4), (256, 256, 4), (128, 96, 1)]):
        out.append(scenes.soup_scene(int(rng.integers(50, 3000)), w, h, msaa,
                                     np.random.default_rng(100 + k), 64, name=f"b{k}",
                                     fs=[0, 1, 2, 0][k % 4]))
    return out


def test_batch_matches_oracle_and_single_renders():
    sc = mixed_scenes()
    br = BatchRenderer()
    for s in sc:
        br.add_scene(s)
    outs = [np.zeros((s["height"], s["width"]), np.uint32) for s in sc]
    br.render(outs)
    for s, img in zip(sc, outs):
        ref, *_ = oracle.render_scene(s)
        assert (img == ref).all(), s["name"]
    # the same scenes one per launch ("alone") give identical images
    for i, s in enumerate(sc):
        one = np.zeros_like(outs[i])
        br.render([one], indices=[i])
        assert (one == outs[i]).all(), s["name"]
    br.close()


@pytest.mark.parametrize("tile", [8, 16, 32])
def test_batch_fixed_tile_sizes(tile):
    sc = mixed_scenes()[1:5]
    br = BatchRenderer()
    for s in sc:
        br.add_scene(s, tile=tile)
    outs = [np.zeros((s["height"], s["width"]), np.uint32) for s in sc]
    br.render(outs)
    for s, img in zip(sc, outs):
        ref, *_ = oracle.render_scene(s)
        assert (img == ref).all(), s["name"]
    br.close()


def test_graph_batch_replays_identically_and_autotune():
    torch = pytest.importorskip("torch")
    sc = mixed_scenes()
    br = BatchRenderer()
    for s in sc:
        br.add_scene(s)
    dev = [torch.zeros(s["height"] * s["width"], dtype=torch.int32, device="cuda") for s in sc]
    tuned = br.autotune([d.data_ptr() for d in dev])
    assert tuned["msaa1_tile"] in (8, 16, 32) and tuned["msaa4_tile"] in (8, 16, 32)
    g = br.capture([d.data_ptr() for d in dev])
    for rep in range(2):
        for d in dev:
            d.zero_()
        torch.cuda.synchronize()
        BatchRenderer.replay(g)
        for s, d in zip(sc, dev):
            ref, *_ = oracle.render_scene(s)
            img = d.cpu().numpy().view(np.uint32).reshape(s["height"], s["width"])
            assert (img == ref).all(), (rep, s["name"])
    br.close()


def test_graph_batches_with_host_outputs_in_turn():
    """Captured batches writing page-locked host memory (half the scenes) and device memory
    (the other half), two of them launched in turn without waiting so that one's copies overlap
    the other's kernels: after each is waited for, every image equals the oracle's. Pageable
    host outputs are refused (a graph cannot copy into them)."""
    torch = pytest.importorskip("torch")
    import ctypes
    from rusterizer_gb300 import _lib
    sc = mixed_scenes()
    refs = [oracle.render_scene(s)[0] for s in sc]
    br = BatchRenderer()
    for s in sc:
        br.add_scene(s)
    sets = []
    for _ in range(2):
        outs = []
        for i, s in enumerate(sc):
            n = s["height"] * s["width"]
            outs.append(torch.zeros(n, dtype=torch.int32).pin_memory() if i % 2 == 0
                        else torch.zeros(n, dtype=torch.int32, device="cuda"))
        sets.append(outs)
    graphs = [br.capture([o.data_ptr() for o in outs]) for outs in sets]
    for rep in range(3):
        for outs in sets:
            for o in outs:
                o.zero_()
        torch.cuda.synchronize()
        for g in graphs:
            BatchRenderer.replay(g, wait=False)
        for g, outs in zip(graphs, sets):
            torch.cuda.ExternalStream(BatchRenderer.graph_stream(g)).synchronize()
            for s, o, ref in zip(sc, outs, refs):
                img = o.cpu().numpy().view(np.uint32).reshape(s["height"], s["width"])
                assert (img == ref).all(), (rep, s["name"])
    pageable = [np.zeros(s["height"] * s["width"], np.uint32) for s in sc]
    arr = br._array([o.ctypes.data for o in pageable], list(range(len(sc))))
    h = ctypes.c_void_p()
    assert _lib.load().rast_batch_create(br._ctx, arr, len(sc), ctypes.byref(h)) == _lib.INVALID_ARG
    br.close()
