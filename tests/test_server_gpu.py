"""Render server: requests submitted concurrently are batched on the device, and every result
is identical to the same scene rendered alone (and to the oracle)."""
import numpy as np
import pytest

import oracle
from rusterizer_gb300 import _lib, scenes
from rusterizer_gb300.batch import BatchRenderer
from rusterizer_gb300.server import RenderServer

pytestmark = pytest.mark.gpu


def pool():
    specs = scenes.batch_scene_specs(12, seed=44, min_tris=50, max_tris=4000)
    return [scenes.batch_scene((n, min(w, 512), min(h, 384), m, s)) for n, w, h, m, s in specs]


@pytest.mark.parametrize("mode", ["batched", "plain"])
def test_server_results_same_alone_and_in_the_mix(mode):
    torch = pytest.importorskip("torch")
    sc = pool()
    br = BatchRenderer()
    for s in sc:
        br.add_scene(s)
    alone = []
    for i, s in enumerate(sc):
        img = np.zeros((s["height"], s["width"]), np.uint32)
        br.render([img], indices=[i])
        alone.append(img)
    srv = RenderServer(br, streams=2, one_per_launch=(mode == "plain"))
    outs, rids = [], []
    for rep in range(3):
        for i, s in enumerate(sc):
            o = torch.zeros(s["height"] * s["width"], dtype=torch.int32, device="cuda")
            outs.append((i, o))
            rids.append(srv.submit(i, o.data_ptr()))
    for rid in rids:
        st, lat = srv.wait(rid, timeout_ms=60000)
        assert st in (_lib.OK, _lib.TEXTURE_OOB), st
        assert lat >= 0.0
    for i, o in outs:
        s = sc[i]
        img = o.cpu().numpy().view(np.uint32).reshape(s["height"], s["width"])
        assert (img == alone[i]).all(), (mode, s["name"])
    for i in range(0, len(sc), 4):
        ref, *_ = oracle.render_scene(sc[i])
        assert (alone[i] == ref).all()
    st = srv.stats()
    assert st["completed"] == len(rids)
    if mode == "plain":
        assert st["mean_batch"] == 1.0
    srv.close()
    br.close()


def test_server_admission_budget():
    torch = pytest.importorskip("torch")
    sc = pool()[:4]
    br = BatchRenderer()
    for s in sc:
        br.add_scene(s)
    # a budget below one scene's footprint refuses it outright
    tiny = RenderServer(br, budget_bytes=1024)
    o = torch.zeros(sc[0]["height"] * sc[0]["width"], dtype=torch.int32, device="cuda")
    with pytest.raises(_lib.RastError) as e:
        tiny.submit(0, o.data_ptr())
    assert e.value.status == _lib.ADMISSION_REFUSED
    tiny.close()
    # a budget that fits only a few scenes at a time still completes everything
    one = RenderServer(br, budget_bytes=6 << 20, streams=2)
    outs = [torch.zeros(s["height"] * s["width"], dtype=torch.int32, device="cuda") for s in sc]
    rids = [one.submit(i, outs[i].data_ptr()) for i in range(len(sc))]
    for rid in rids:
        assert one.wait(rid, timeout_ms=60000)[0] in (_lib.OK, _lib.TEXTURE_OOB)
    for i, s in enumerate(sc):
        ref = np.zeros((s["height"], s["width"]), np.uint32)
        br.render([ref], indices=[i])
        assert (outs[i].cpu().numpy().view(np.uint32).reshape(ref.shape) == ref).all()
    one.close()
    br.close()


def test_bounded_waits_and_unknown_requests():
    """A wait that runs out returns RAST_TIMEOUT and leaves the request running (a later wait
    gets its result and releases the record); poll reports NOT_READY meanwhile; an id never
    issued is an invalid argument for poll and wait alike."""
    torch = pytest.importorskip("torch")
    big = scenes.soup_scene(120_000, 1024, 768, 4, np.random.default_rng(5), 256, name="big")
    br = BatchRenderer()
    br.add_scene(big)
    srv = RenderServer(br, streams=1)
    o = torch.zeros(big["height"] * big["width"], dtype=torch.int32, device="cuda")
    rid = srv.submit(0, o.data_ptr())
    st, _ = srv.wait(rid, timeout_ms=0)  # a whole 120k-triangle frame cannot be done already
    assert st == _lib.TIMEOUT
    assert srv.poll(rid)[0] in (_lib.NOT_READY, _lib.OK, _lib.TEXTURE_OOB)
    st, lat = srv.wait(rid, timeout_ms=60000)
    assert st in (_lib.OK, _lib.TEXTURE_OOB) and lat > 0.0
    # the final status has been collected: the record is released
    assert srv.poll(rid)[0] == _lib.INVALID_ARG
    assert srv.info()["tracked"] == 0
    assert srv.poll(rid + 1000)[0] == _lib.INVALID_ARG
    assert srv.wait(rid + 1000, timeout_ms=10)[0] == _lib.INVALID_ARG
    ref = np.zeros((big["height"], big["width"]), np.uint32)
    br.render([ref], indices=[0])
    assert (o.cpu().numpy().view(np.uint32).reshape(ref.shape) == ref).all()
    srv.close()
    br.close()


def test_destroy_drains_requests_never_waited_for():
    """Requests whose submitter never waits (a dropped client) are still rendered and the
    server shuts down cleanly: destroy drains the queue."""
    torch = pytest.importorskip("torch")
    sc = pool()
    br = BatchRenderer()
    for s in sc:
        br.add_scene(s)
    srv = RenderServer(br, streams=2)
    outs = [torch.zeros(s["height"] * s["width"], dtype=torch.int32, device="cuda") for s in sc]
    for i in range(len(sc)):
        srv.submit(i, outs[i].data_ptr())
    srv.close()  # no wait on any request
    torch.cuda.synchronize()
    for i, s in enumerate(sc):
        ref = np.zeros((s["height"], s["width"]), np.uint32)
        br.render([ref], indices=[i])
        assert (outs[i].cpu().numpy().view(np.uint32).reshape(ref.shape) == ref).all(), s["name"]
    br.close()


def test_request_table_stays_bounded():
    """120 000 small requests: collected ones leave the table at once, and of requests nobody
    waits for only the most recent 65 536 finished records are kept, so a server that runs
    indefinitely holds bounded memory; the latency statistics still count every completion."""
    torch = pytest.importorskip("torch")
    tiny = scenes.soup_scene(40, 32, 32, 4, np.random.default_rng(8), 16, name="tiny")
    br = BatchRenderer()
    br.add_scene(tiny)
    ref = np.zeros((32, 32), np.uint32)
    br.render([ref], indices=[0])
    srv = RenderServer(br, streams=2)
    o = torch.zeros(32 * 32, dtype=torch.int32, device="cuda")
    n, peak = 50_000, 0
    for k in range(0, n, 1000):
        rids = [srv.submit(0, o.data_ptr()) for _ in range(1000)]
        for rid in rids:
            assert srv.wait(rid, timeout_ms=60000)[0] in (_lib.OK, _lib.TEXTURE_OOB)
        peak = max(peak, srv.info()["tracked"])
    assert srv.info()["tracked"] == 0 and peak <= 1000
    # 70 000 more that nobody collects
    n2 = 70_000
    for _ in range(n2):
        srv.submit(0, o.data_ptr())
    deadline = 600
    import time
    t0 = time.time()
    while True:
        info = srv.info()
        if info["queued"] == 0 and info["running"] == 0:
            break
        assert time.time() - t0 < deadline
        time.sleep(0.01)
    assert srv.info()["tracked"] == 65536
    assert srv.stats()["completed"] == n + n2
    torch.cuda.synchronize()
    assert (o.cpu().numpy().view(np.uint32).reshape(32, 32) == ref).all()
    srv.close()
    br.close()


def test_invalid_stream_count_is_refused():
    """More than two batches in flight is not offered: the server refuses the configuration
    instead of quietly running one."""
    br = BatchRenderer()
    s = scenes.small_soup(7, ntris=200)
    br.add_scene(s)
    for bad in (3, -1):
        with pytest.raises(_lib.RastError) as e:
            RenderServer(br, streams=bad)
        assert e.value.status == _lib.INVALID_ARG
    RenderServer(br, streams=0).close()  # 0: the default (two)
    br.close()
