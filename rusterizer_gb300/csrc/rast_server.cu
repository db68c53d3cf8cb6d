// rast_server.cu - continuous-batching render server.
//
// Submitters enqueue scenes; one dispatcher thread owns up to two launch slots, each with its
// own engine (scratch buffers, descriptor staging, CUDA stream). Whenever a slot is free, the
// dispatcher takes queued requests in arrival order while they fit the HBM budget, renders
// them as one batch on that slot's stream and enqueues a host callback behind it; the
// callback marks the slot complete and wakes the dispatcher (no polling), so a second batch
// can be launched (on the other slot) while the first still runs and the two overlap on the
// device. A batch that overflowed its bin or clip capacity is re-queued at the front with the
// measured sizes remembered per scene shape.
//
// Memory stays bounded however long the server runs: a request's record is released when a
// wait or poll has returned its final status; finished records nobody collects are kept for
// the most recent kMaxUnclaimed requests only; latency statistics cover the most recent
// kMaxLatencySamples completions.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/rast.h"
#include "rast_internal.h"

using namespace rast;
using Clock = std::chrono::steady_clock;

namespace {

struct Request {
    rast_scene scene;
    Clock::time_point t_submit, t_done;
    uint64_t footprint = 0;
    rast_status status = RAST_NOT_READY;
    bool done = false;
};

constexpr size_t kMaxUnclaimed = size_t(1) << 16;        // finished records kept uncollected
constexpr size_t kMaxLatencySamples = size_t(1) << 20;  // latency window of the statistics

struct Slot {
    Engine E;
    bool busy = false;
    bool complete = false;  // set by the host callback behind the slot's batch
    std::vector<uint64_t> ids;
    std::vector<FrameJob> jobs;
    uint64_t bytes = 0;
    HostBuf<unsigned long long> need;
    void* server = nullptr;
};

using ShapeKey = std::tuple<uint32_t, int, int, int, int>;  // mesh, width, height, msaa, tile

// Device bytes a scene needs while in flight: vertex records, per-triangle rectangles, chunk
// histograms, tile tables, bins (and quadrant lists for 32-pixel bins), clip store and its image.
uint64_t footprint_of(const rast_ctx* c, const rast_scene& s, int ts, uint64_t bins) {
    const MeshRec& m = c->meshes[s.mesh];
    const uint64_t tiles = (uint64_t)((s.width + ts - 1) / ts) * ((s.height + ts - 1) / ts);
    const uint64_t cs = chunk_size_for(m.ntris);
    const uint64_t chunks = (m.ntris + cs - 1) / cs;
    const uint64_t bin_cap = std::max<uint64_t>(bins, 4ull * m.ntris + tiles + 1024ull);
    const uint64_t split = raster_edge(ts) < ts ? 16ull * (bin_cap + tiles) : 0ull;
    return 34ull * m.nverts + 24ull * m.ntris + 4ull * chunks * tiles + 12ull * tiles + 4ull * bin_cap + split +
           4ull * (32ull * m.ntris + 4096ull) + 4ull * (uint64_t)s.width * s.height + 65536ull;
}

}  // namespace

struct rast_server {
    rast_ctx* ctx = nullptr;
    rast_server_config cfg{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread th;
    bool stop = false;
    uint64_t next_id = 1;
    std::deque<uint64_t> queue;
    std::unordered_map<uint64_t, Request> reqs;
    Slot slots[2];
    int nslots = 1;
    uint64_t inflight = 0;
    std::map<ShapeKey, uint64_t> bins_hint;
    std::deque<uint64_t> unclaimed;  // finished requests in completion order (maybe collected)
    // statistics since the last reset: a ring of the most recent latencies
    std::vector<double> lat_ms;
    size_t lat_next = 0;
    uint64_t completed = 0;
    Clock::time_point t_first{}, t_last{};
    uint64_t batches = 0, batch_scenes = 0;

    void record_latency(double ms) {
        if (lat_ms.size() < kMaxLatencySamples) {
            lat_ms.push_back(ms);
        } else {
            lat_ms[lat_next] = ms;
            lat_next = (lat_next + 1) % kMaxLatencySamples;
        }
        ++completed;
    }

    // A request finished: keep its record for the submitter, dropping the oldest uncollected
    // records beyond kMaxUnclaimed (ids already collected are skipped).
    void retire(uint64_t id) {
        unclaimed.push_back(id);
        while (unclaimed.size() > kMaxUnclaimed) {
            reqs.erase(unclaimed.front());
            unclaimed.pop_front();
        }
    }

    // Host callback behind a slot's batch (runs on a CUDA driver thread once the batch and its
    // status copies are complete; it makes no CUDA call).
    static void CUDART_CB on_slot_done(void* p) {
        Slot* sl = static_cast<Slot*>(p);
        rast_server* srv = static_cast<rast_server*>(sl->server);
        {
            std::lock_guard<std::mutex> lk(srv->mu);
            sl->complete = true;
        }
        srv->cv_work.notify_one();
    }

    int tile_of(const rast_scene& s) const {
        int req = s.tile ? s.tile : ctx->tuned_tile[s.msaa == 4 ? 1 : 0];
        const bool mesh_ok = s.mesh < ctx->meshes.size() && ctx->meshes[s.mesh].live;
        return choose_tile(s.width, s.height, s.msaa, req, mesh_ok ? ctx->meshes[s.mesh].ntris : 0u);
    }

    uint64_t hint_of(const rast_scene& s, int ts) const {
        auto it = bins_hint.find(ShapeKey{s.mesh, s.width, s.height, s.msaa, ts});
        return it == bins_hint.end() ? 0 : it->second;
    }

    // Called with the lock held: launch queued requests on a free slot.
    bool launch_one(Slot& sl, std::unique_lock<std::mutex>& lk) {
        if (queue.empty()) return false;
        const uint32_t cap = cfg.one_per_launch ? 1u : (cfg.max_batch ? cfg.max_batch : 0xFFFFFFFFu);
        std::vector<uint64_t> take;
        uint64_t bytes = 0;
        while (!queue.empty() && take.size() < cap) {
            const uint64_t id = queue.front();
            Request& r = reqs[id];
            if (inflight + bytes + r.footprint > cfg.hbm_budget_bytes) break;  // wait for memory
            bytes += r.footprint;
            take.push_back(id);
            queue.pop_front();
        }
        if (take.empty()) return false;
        std::vector<FrameJob> jobs(take.size());
        for (size_t i = 0; i < take.size(); ++i) {
            const rast_scene& s = reqs[take[i]].scene;
            FrameJob& J = jobs[i];
            J.width = s.width;
            J.height = s.height;
            J.msaa = s.msaa;
            J.ts = tile_of(s);
            J.clear_depth = s.clear_depth;
            J.out_dev = s.argb_out;
            DrawJob d;
            d.mesh = &ctx->meshes[s.mesh];
            d.mesh_id = s.mesh;
            d.tex = (s.texture >= 0 && s.texture < (int)ctx->textures.size()) ? &ctx->textures[s.texture] : nullptr;
            d.fs = s.fs_id;
            float pv[16];
            mat4_mul(s.proj, s.view, pv);
            mat4_mul(pv, s.world, d.mvp);
            J.draws.assign(1, d);
            J.ntris_hint = d.mesh->ntris;
            J.bin_hint = hint_of(s, J.ts);
        }
        inflight += bytes;
        sl.busy = true;
        sl.bytes = bytes;
        sl.ids = take;
        lk.unlock();
        sl.jobs = std::move(jobs);
        sl.E.sync_after = false;
        rast_status st = run_frames(sl.E, sl.jobs);
        const size_t nf = sl.jobs.size();
        bool ok = st == RAST_OK && sl.need.reserve(nf);
        if (ok) {
            cudaMemcpyAsync(sl.E.h_state, sl.E.d_state, sizeof(DeviceState), cudaMemcpyDeviceToHost, sl.E.stream);
            cudaMemcpyAsync(sl.need.p, sl.E.frame_need.p, nf * sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, sl.E.stream);
            ok = cudaLaunchHostFunc(sl.E.stream, on_slot_done, &sl) == cudaSuccess;
        }
        lk.lock();
        if (!ok) {
            // fail the batch's requests without waiting on the device
            const Clock::time_point now = Clock::now();
            for (uint64_t id : sl.ids) {
                Request& r = reqs[id];
                r.status = st != RAST_OK ? st : RAST_CUDA_ERROR;
                r.done = true;
                r.t_done = now;
                retire(id);
            }
            inflight -= sl.bytes;
            sl.busy = false;
            cv_done.notify_all();
        }
        return true;
    }

    // Called with the lock held for a slot whose host callback ran: the batch and its status
    // copies are complete (no CUDA call here: the callback of the other slot takes this lock).
    void finish(Slot& sl) {
        sl.complete = false;
        const uint32_t status = sl.E.h_state->status;
        const Clock::time_point now = Clock::now();
        const bool overflow = (status & (ST_BIN_OVERFLOW | ST_CLIP_STORE_OVERFLOW)) != 0;
        // frame k of the launch is job E.h_order[k] (frames are grouped by MSAA and tile size)
        for (size_t k = 0; k < sl.jobs.size() && k < sl.E.h_order.size(); ++k) {
            const FrameJob& J = sl.jobs[sl.E.h_order[k]];
            const rast_scene& s = reqs[sl.ids[sl.E.h_order[k]]].scene;
            uint64_t& h = bins_hint[ShapeKey{s.mesh, s.width, s.height, s.msaa, J.ts}];
            h = std::max<uint64_t>(h, sl.need.p[k] + sl.need.p[k] / 8 + 1024);
        }
        if (status & ST_CLIP_STORE_OVERFLOW)
            sl.E.clip_hint = sl.E.h_state->clip_used + sl.E.h_state->clip_used / 4 + 65536;
        inflight -= sl.bytes;
        sl.busy = false;
        if (overflow) {
            // render again with the measured capacities, ahead of newer requests
            for (auto it = sl.ids.rbegin(); it != sl.ids.rend(); ++it) queue.push_front(*it);
            return;
        }
        rast_status rs = RAST_OK;
        if (status & ST_BAD_INDEX) rs = RAST_INVALID_ARG;
        else if (status & ST_CLIP_OVERFLOW) rs = RAST_CLIP_OVERFLOW;
        else if (status & ST_TEXTURE_OOB) rs = RAST_TEXTURE_OOB;
        for (uint64_t id : sl.ids) {
            Request& r = reqs[id];
            r.status = rs;
            r.done = true;
            r.t_done = now;
            record_latency(std::chrono::duration<double, std::milli>(now - r.t_submit).count());
            if (t_first == Clock::time_point{}) t_first = r.t_submit;
            t_last = now;
            retire(id);
        }
        ++batches;
        batch_scenes += sl.ids.size();
        cv_done.notify_all();
    }

    void run() {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            bool progress = false;
            for (int i = 0; i < nslots; ++i)
                if (slots[i].busy && slots[i].complete) {
                    finish(slots[i]);
                    progress = true;
                }
            for (int i = 0; i < nslots; ++i)
                if (!slots[i].busy && launch_one(slots[i], lk)) progress = true;
            bool any_busy = false;
            for (int i = 0; i < nslots; ++i) any_busy |= slots[i].busy;
            if (stop && queue.empty() && !any_busy) break;
            // woken by a submit, a slot's callback or destroy; the timeout is only a backstop
            if (!progress) cv_work.wait_for(lk, std::chrono::milliseconds(50));
        }
    }
};

extern "C" {

rast_status rast_server_create(rast_ctx* c, const rast_server_config* cfg, rast_server** out) {
    if (!c || !out) return RAST_INVALID_ARG;
    rast_server* s = new (std::nothrow) rast_server();
    if (!s) return RAST_OOM;
    s->ctx = c;
    c->sync_copies();
    if (cfg) s->cfg = *cfg;
    if (s->cfg.streams < 0 || s->cfg.streams > 2) {  // 0 takes the default
        delete s;
        return RAST_INVALID_ARG;
    }
    if (!s->cfg.hbm_budget_bytes) s->cfg.hbm_budget_bytes = 40ull << 30;
    if (!s->cfg.streams) s->cfg.streams = 2;
    s->nslots = (s->cfg.streams == 2 && !s->cfg.one_per_launch) ? 2 : 1;
    for (int i = 0; i < s->nslots; ++i) {
        s->slots[i].server = s;
        // the context's (autotuned) raster settings
        for (int k = 0; k < 2; ++k) {
            s->slots[i].E.heavy_bits[k] = c->E.heavy_bits[k];
            s->slots[i].E.ctas_per_sm[k] = c->E.ctas_per_sm[k];
        }
        if (!s->slots[i].E.init()) {
            delete s;
            return RAST_CUDA_ERROR;
        }
    }
    s->th = std::thread([s] { s->run(); });
    *out = s;
    return RAST_OK;
}

rast_status rast_server_submit(rast_server* s, const rast_scene* sc, uint64_t* id) {
    if (!s || !sc || !id) return RAST_INVALID_ARG;
    const rast_scene& q = *sc;
    if (q.width < 1 || q.height < 1 || q.width > 16384 || q.height > 16384 || (q.msaa != 1 && q.msaa != 4) ||
        q.fs_id < 0 || q.fs_id > 2 || !q.argb_out)
        return RAST_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->stop) return RAST_INVALID_ARG;
    if (q.mesh >= s->ctx->meshes.size() || !s->ctx->meshes[q.mesh].live) return RAST_INVALID_ARG;
    if (q.fs_id == RAST_FS_TEXTURE && (q.texture < 0 || q.texture >= (int)s->ctx->textures.size()))
        return RAST_INVALID_ARG;
    const int ts = s->tile_of(q);
    if (!ts) return RAST_INVALID_ARG;
    Request r;
    r.scene = q;
    r.t_submit = Clock::now();
    r.footprint = footprint_of(s->ctx, q, ts, s->hint_of(q, ts));
    if (r.footprint > s->cfg.hbm_budget_bytes) return RAST_ADMISSION_REFUSED;
    const uint64_t rid = s->next_id++;
    s->reqs.emplace(rid, r);
    s->queue.push_back(rid);
    *id = rid;
    lk.unlock();
    s->cv_work.notify_one();
    return RAST_OK;
}

rast_status rast_server_poll(rast_server* s, uint64_t id, double* latency_ms) {
    if (!s) return RAST_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return RAST_INVALID_ARG;
    if (!it->second.done) return RAST_NOT_READY;
    if (latency_ms)
        *latency_ms = std::chrono::duration<double, std::milli>(it->second.t_done - it->second.t_submit).count();
    const rast_status st = it->second.status;
    s->reqs.erase(it);  // the final status has been collected
    return st;
}

rast_status rast_server_wait(rast_server* s, uint64_t id, int timeout_ms, double* latency_ms) {
    if (!s) return RAST_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto done = [&] {
        auto it = s->reqs.find(id);
        return it == s->reqs.end() || it->second.done;
    };
    if (timeout_ms < 0) {
        s->cv_done.wait(lk, done);
    } else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done)) {
        return RAST_TIMEOUT;
    }
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return RAST_INVALID_ARG;
    if (latency_ms)
        *latency_ms = std::chrono::duration<double, std::milli>(it->second.t_done - it->second.t_submit).count();
    const rast_status st = it->second.status;
    s->reqs.erase(it);  // the final status has been collected
    return st;
}

rast_status rast_server_stats(rast_server* s, double* p50, double* p99, uint64_t* completed,
                              double* rps, double* mean_batch) {
    if (!s) return RAST_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    std::vector<double> v = s->lat_ms;
    std::sort(v.begin(), v.end());
    auto pct = [&](double q) {
        if (v.empty()) return 0.0;
        size_t i = (size_t)(q * (double)(v.size() - 1) + 0.5);
        return v[std::min(i, v.size() - 1)];
    };
    if (p50) *p50 = pct(0.50);
    if (p99) *p99 = pct(0.99);
    if (completed) *completed = s->completed;
    if (rps) {
        const double span = std::chrono::duration<double>(s->t_last - s->t_first).count();
        *rps = span > 0 ? (double)s->completed / span : 0.0;
    }
    if (mean_batch) *mean_batch = s->batches ? (double)s->batch_scenes / (double)s->batches : 0.0;
    return RAST_OK;
}

rast_status rast_server_reset_stats(rast_server* s) {
    if (!s) return RAST_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    s->lat_ms.clear();
    s->lat_next = 0;
    s->completed = 0;
    s->t_first = Clock::time_point{};
    s->t_last = Clock::time_point{};
    s->batches = s->batch_scenes = 0;
    return RAST_OK;
}

rast_status rast_server_info(rast_server* s, uint64_t* queued, uint64_t* running, uint64_t* tracked) {
    if (!s) return RAST_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    uint64_t run = 0;
    for (int i = 0; i < s->nslots; ++i)
        if (s->slots[i].busy) run += s->slots[i].ids.size();
    if (queued) *queued = s->queue.size();
    if (running) *running = run;
    if (tracked) *tracked = s->reqs.size();
    return RAST_OK;
}

rast_status rast_server_destroy(rast_server* s) {
    if (!s) return RAST_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->th.joinable()) s->th.join();
    delete s;
    return RAST_OK;
}

}  // extern "C"
