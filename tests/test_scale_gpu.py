"""Parity of the scene-mix paths at their full benchmark scale.

The batched path (rast_batch_create + rast_batch_launch, one CUDA-graph replay) renders the
whole 256-scene batch workload: 100 to 200k triangles per scene, up to 1920x1080, MSAA 1 and
4, one 512x512 texture each, all scenes binned into one grid (frame offsets into the hundreds
of millions of counts) with the autotuned bin sizes. Every scene must equal the same scene
rendered alone through the plain entry point (rast_framebuffer, automatic bin size), and a
dozen of them - the largest of each MSAA, the 1920x1080 ones with the most triangles and some
drawn at random - must equal the oracle. The serving path is checked the same way on a
64-scene pool of the serving workload. The reference renders one scene per Renderer
(src/render.rs:98-114); each scene of a batch must be what that path gives for it alone.
"""
import os

import numpy as np
import pytest

import oracle
from rusterizer_gb300 import _lib, renderer, scenes
from rusterizer_gb300.batch import BatchRenderer
from rusterizer_gb300.server import RenderServer

pytestmark = pytest.mark.gpu


def _alone(scene):
    img, st, r = renderer.render_scene(scene)
    r.close()
    assert st in (_lib.OK, _lib.TEXTURE_OOB), st
    return img


def _oracle_picks(sc, rng, n_random=4, at_least=12):
    """The largest scene of each MSAA, the two 1920x1080 scenes of each MSAA with the most
    triangles, and scenes drawn at random: n_random of them, more if needed to reach at_least."""
    picks = set()
    for m in (1, 4):
        idx = [i for i, s in enumerate(sc) if s["msaa"] == m]
        if not idx:
            continue
        picks.add(max(idx, key=lambda i: scenes.scene_triangles(sc[i])))
        big = [i for i in idx if (sc[i]["width"], sc[i]["height"]) == (1920, 1080)]
        picks.update(sorted(big, key=lambda i: -scenes.scene_triangles(sc[i]))[:2])
    rest = [i for i in range(len(sc)) if i not in picks]
    k = min(max(n_random, at_least - len(picks)), len(rest))
    picks.update(int(i) for i in rng.choice(rest, size=k, replace=False))
    return sorted(picks)


def _check_oracle(sc, imgs, picks):
    cores = os.cpu_count() or 1
    for i in picks:
        ref, *_ = oracle.render_scene(sc[i], nthreads=cores)
        assert (imgs[i] == ref).all(), sc[i]["name"]


def test_full_batch_workload_graph_replay_matches_plain_and_oracle():
    torch = pytest.importorskip("torch")
    sc = scenes.config3()
    assert len(sc) == 256
    br = BatchRenderer()
    for s in sc:
        br.add_scene(s)
    dev = [torch.zeros(s["height"] * s["width"], dtype=torch.int32, device="cuda") for s in sc]
    ptrs = [d.data_ptr() for d in dev]
    tuned = br.autotune(ptrs, cache=False)
    g = br.capture(ptrs)
    for d in dev:
        d.zero_()
    torch.cuda.synchronize()
    BatchRenderer.replay(g)
    imgs = [d.cpu().numpy().view(np.uint32).reshape(s["height"], s["width"]) for s, d in zip(sc, dev)]
    br.close()
    for i, s in enumerate(sc):
        assert (imgs[i] == _alone(s)).all(), (i, s["name"], tuned)
    picks = _oracle_picks(sc, np.random.default_rng(31))
    assert len(picks) >= 12
    _check_oracle(sc, imgs, picks)


def test_serving_pool_matches_plain_and_oracle():
    torch = pytest.importorskip("torch")
    sc = [scenes.batch_scene(s) for s in scenes.config4_specs(seed=4, nscenes=64)]
    br = BatchRenderer()
    for s in sc:
        br.add_scene(s)
    srv = RenderServer(br, streams=2)
    outs, rids = [], []
    rng = np.random.default_rng(12)
    order = list(rng.permutation(len(sc))) + list(rng.integers(0, len(sc), 64))
    for i in order:
        s = sc[i]
        o = torch.zeros(s["height"] * s["width"], dtype=torch.int32, device="cuda")
        outs.append((int(i), o))
        rids.append(srv.submit(int(i), o.data_ptr()))
    for rid in rids:
        st, _ = srv.wait(rid, timeout_ms=120000)
        assert st in (_lib.OK, _lib.TEXTURE_OOB), st
    srv.close()
    br.close()
    alone = {}
    first = {}
    for i, o in outs:
        s = sc[i]
        img = o.cpu().numpy().view(np.uint32).reshape(s["height"], s["width"])
        if i not in alone:
            alone[i] = _alone(s)
            first[i] = img
        assert (img == alone[i]).all(), (i, s["name"])
    picks = _oracle_picks(sc, np.random.default_rng(41), n_random=2, at_least=8)
    _check_oracle(sc, first, picks)
