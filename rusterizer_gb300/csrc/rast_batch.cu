// rast_batch.cu - many independent scenes per launch sequence, CUDA-graph capture of a fixed
// batch, and the autotuner (bin edge, raster kernel split and CTA count, bin capacity).
//
// A batch is a list of frames handed to run_frames at once: the vertex, binning and scan
// kernels run once over every scene, and the persistent raster kernel (one launch per
// (MSAA, tile size) class) takes tiles of all scenes from a single queue, heaviest first, so
// uneven scenes share the GPU instead of each occupying it for a launch of its own. Scenes are
// independent, so each scene's image is bit-identical to rendering it alone. Scenes with host
// outputs resolve into a staging buffer that is copied out at the end (in a captured batch,
// inside the graph, so two batches launched in turn overlap one's copies with the other's
// kernels).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/rast.h"
#include "rast_internal.h"

using namespace rast;

namespace {

bool is_device_ptr(const void* p) {
    cudaPointerAttributes attr;
    const bool dev = cudaPointerGetAttributes(&attr, p) == cudaSuccess &&
                     (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    return dev;
}

// Page-locked (or registered) host memory: the only host memory a captured copy may write.
bool is_pinned_host_ptr(const void* p) {
    cudaPointerAttributes attr;
    const bool pinned = cudaPointerGetAttributes(&attr, p) == cudaSuccess && attr.type == cudaMemoryTypeHost;
    cudaGetLastError();
    return pinned;
}

int scene_tile(const rast_ctx* c, const rast_scene& s) {
    int req = s.tile;
    if (req == 0) req = c->tuned_tile[s.msaa == 4 ? 1 : 0];
    const bool mesh_ok = s.mesh < c->meshes.size() && c->meshes[s.mesh].live;
    return choose_tile(s.width, s.height, s.msaa, req, mesh_ok ? c->meshes[s.mesh].ntris : 0u);
}

// Validates the scenes and turns them into frame jobs. Host outputs (when allowed) are
// redirected to `staging` at the returned offsets.
rast_status build_jobs(rast_ctx* c, const rast_scene* sc, uint32_t n, bool allow_host_out,
                       std::vector<FrameJob>& jobs, std::vector<size_t>* host_off, size_t* staging_px) {
    jobs.clear();
    jobs.resize(n);
    size_t px = 0;
    if (host_off) host_off->assign(n, (size_t)-1);
    for (uint32_t i = 0; i < n; ++i) {
        const rast_scene& s = sc[i];
        if (s.width < 1 || s.height < 1 || s.width > 16384 || s.height > 16384 ||
            (s.msaa != 1 && s.msaa != 4) || s.fs_id < 0 || s.fs_id > 2 || !s.argb_out)
            return RAST_INVALID_ARG;
        if (s.mesh >= c->meshes.size() || !c->meshes[s.mesh].live) return RAST_INVALID_ARG;
        if (s.fs_id == RAST_FS_TEXTURE && (s.texture < 0 || s.texture >= (int)c->textures.size()))
            return RAST_INVALID_ARG;
        const int ts = scene_tile(c, s);
        if (!ts) return RAST_INVALID_ARG;
        FrameJob& J = jobs[i];
        J.width = s.width;
        J.height = s.height;
        J.msaa = s.msaa;
        J.ts = ts;
        J.clear_depth = s.clear_depth;
        if (is_device_ptr(s.argb_out)) {
            J.out_dev = s.argb_out;
        } else {
            if (!allow_host_out) return RAST_INVALID_ARG;
            (*host_off)[i] = px;
            px += (size_t)s.width * (size_t)s.height;
        }
        DrawJob d;
        d.mesh = &c->meshes[s.mesh];
        d.mesh_id = s.mesh;
        d.tex = (s.texture >= 0 && s.texture < (int)c->textures.size()) ? &c->textures[s.texture] : nullptr;
        d.fs = s.fs_id;
        float pv[16];
        mat4_mul(s.proj, s.view, pv);
        mat4_mul(pv, s.world, d.mvp);
        J.draws.assign(1, d);
        J.ntris_hint = d.mesh->ntris;
        if (c->batch_hints.size() == n) J.bin_hint = c->batch_hints[i];
    }
    if (staging_px) *staging_px = px;
    return RAST_OK;
}

rast_status render_jobs(rast_ctx* c, const rast_scene* sc, uint32_t n, std::vector<FrameJob>& jobs,
                        const std::vector<size_t>& host_off, size_t staging_px) {
    if (staging_px && !c->batch_out.reserve(staging_px)) return RAST_OOM;
    for (uint32_t i = 0; i < n; ++i)
        if (host_off[i] != (size_t)-1) jobs[i].out_dev = c->batch_out.p + host_off[i];
    c->E.sync_after = true;
    rast_status st = run_frames(c->E, jobs);
    if (st != RAST_OK && st != RAST_TEXTURE_OOB) return st;
    c->batch_hints.resize(n);
    for (uint32_t i = 0; i < n; ++i)
        c->batch_hints[i] = std::max<uint64_t>(c->batch_hints[i], jobs[i].need + jobs[i].need / 8);
    bool copied = false;
    for (uint32_t i = 0; i < n; ++i) {
        if (host_off[i] == (size_t)-1) continue;
        const size_t bytes = (size_t)sc[i].width * sc[i].height * sizeof(uint32_t);
        if (cudaMemcpyAsync(sc[i].argb_out, c->batch_out.p + host_off[i], bytes, cudaMemcpyDeviceToHost,
                            c->E.stream) != cudaSuccess)
            return RAST_CUDA_ERROR;
        copied = true;
    }
    if (copied && cudaStreamSynchronize(c->E.stream) != cudaSuccess) return RAST_CUDA_ERROR;
    return st;
}

}  // namespace

struct rast_batch {
    rast_ctx* ctx = nullptr;
    Engine E;
    std::vector<FrameJob> jobs;
    DevBuf<uint32_t> stage;          // resolved images of the scenes with host outputs
    std::vector<size_t> host_off;    // per scene: its offset in `stage`, or -1 (device output)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

// The batch's copies of its staged images to the scenes' host outputs, on its stream (one chain
// of copies: 715 MB for the 256-scene mix take about 4.3 ms, under the batch's kernel time).
bool enqueue_host_copies(rast_batch* b, const rast_scene* sc, uint32_t n) {
    for (uint32_t i = 0; i < n; ++i) {
        if (b->host_off[i] == (size_t)-1) continue;
        const size_t bytes = (size_t)sc[i].width * sc[i].height * sizeof(uint32_t);
        if (cudaMemcpyAsync(sc[i].argb_out, b->stage.p + b->host_off[i], bytes, cudaMemcpyDeviceToHost,
                            b->E.stream) != cudaSuccess)
            return false;
    }
    return true;
}

}  // namespace

extern "C" {

rast_status rast_render_batch(rast_ctx* c, const rast_scene* sc, uint32_t n) {
    if (!c || (n && !sc)) return RAST_INVALID_ARG;
    if (n == 0) return RAST_OK;
    c->sync_copies();
    std::vector<FrameJob> jobs;
    std::vector<size_t> host_off;
    size_t staging = 0;
    rast_status st = build_jobs(c, sc, n, true, jobs, &host_off, &staging);
    if (st != RAST_OK) return st;
    return render_jobs(c, sc, n, jobs, host_off, staging);
}

rast_status rast_autotune_batch_ex(rast_ctx* c, const rast_scene* sc, uint32_t n, rast_tuning* out) {
    if (!c || !sc || n == 0) return RAST_INVALID_ARG;
    bool has[2] = {false, false};
    for (uint32_t i = 0; i < n; ++i) has[sc[i].msaa == 4 ? 1 : 0] = true;
    std::vector<rast_scene> trial(sc, sc + n);
    // every trial writes into the staging buffer, not the caller's images
    size_t px = 0;
    for (uint32_t i = 0; i < n; ++i) px += (size_t)sc[i].width * sc[i].height;
    if (!c->batch_out.reserve(px)) return RAST_OOM;
    size_t off = 0;
    for (uint32_t i = 0; i < n; ++i) {
        trial[i].tile = 0;
        trial[i].argb_out = c->batch_out.p + off;
        off += (size_t)sc[i].width * sc[i].height;
    }
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return RAST_CUDA_ERROR;
    Engine& E = c->E;
    const int saved_tile[2] = {c->tuned_tile[0], c->tuned_tile[1]};
    const uint32_t saved_heavy[2] = {E.heavy_bits[0], E.heavy_bits[1]};
    const int saved_ctas[2] = {E.ctas_per_sm[0], E.ctas_per_sm[1]};
    rast_status result = RAST_OK;
    // mean batch time over two timed runs after one sizing run, with the current settings
    auto time_batch = [&](float& ms) {
        ms = 0.0f;
        std::vector<FrameJob> jobs;
        for (int rep = 0; rep < 3 && result == RAST_OK; ++rep) {
            rast_status st = build_jobs(c, trial.data(), n, false, jobs, nullptr, nullptr);
            if (st != RAST_OK) {
                result = st;
                return;
            }
            E.sync_after = true;
            cudaEventRecord(e0, E.stream);
            st = run_frames(E, jobs);
            cudaEventRecord(e1, E.stream);
            cudaEventSynchronize(e1);
            if (st != RAST_OK && st != RAST_TEXTURE_OOB) {
                result = st;
                return;
            }
            c->batch_hints.resize(n);
            for (uint32_t i = 0; i < n; ++i)
                c->batch_hints[i] = std::max<uint64_t>(c->batch_hints[i], jobs[i].need + jobs[i].need / 8);
            float t = 0.0f;
            cudaEventElapsedTime(&t, e0, e1);
            if (rep > 0) ms += t / 2.0f;  // the first run sizes buffers
        }
    };
    // 1. bin edge per MSAA class (8, 16 or 32 pixels), both classes together, under each of the
    // two extreme raster splits (every bin CTA-wide, every bin one warp per tile): the best bin
    // edge depends on the raster kernel
    const int sizes[3] = {8, 16, 32};
    float best_ms = 3.0e38f;
    int best_tile[2] = {0, 0};
    uint32_t best_split = 0;
    auto sweep_tiles = [&](bool keep_split) {
        for (int a = 0; a < (has[0] ? 3 : 1) && result == RAST_OK; ++a)
            for (int b = 0; b < (has[1] ? 3 : 1) && result == RAST_OK; ++b) {
                c->tuned_tile[0] = has[0] ? sizes[a] : 0;
                c->tuned_tile[1] = has[1] ? sizes[b] : 0;
                if (keep_split && c->tuned_tile[0] == best_tile[0] && c->tuned_tile[1] == best_tile[1])
                    continue;  // the current setting was timed already
                float ms = 0.0f;
                time_batch(ms);
                if (result == RAST_OK && ms < best_ms) {
                    best_ms = ms;
                    best_tile[0] = c->tuned_tile[0];
                    best_tile[1] = c->tuned_tile[1];
                    if (!keep_split) best_split = E.heavy_bits[0];
                }
            }
    };
    for (uint32_t split : {0u, 32u}) {
        E.heavy_bits[0] = E.heavy_bits[1] = split;
        E.ctas_per_sm[0] = E.ctas_per_sm[1] = 0;
        sweep_tiles(false);
    }
    E.heavy_bits[0] = E.heavy_bits[1] = best_split;
    c->tuned_tile[0] = best_tile[0];
    c->tuned_tile[1] = best_tile[1];
    // 2. per class, from the best of step 1: the split between the CTA-wide and the
    // warp-per-tile raster kernel, and the persistent raster CTAs per SM
    // every bin CTA-wide; bins of 128+, 512+ or 2048+ entries CTA-wide; every bin one warp each
    const uint32_t heavy_opts[5] = {0u, 7u, 9u, 11u, 32u};
    const int cta_opts[3] = {0, 4, 2};
    for (int cls = 0; cls < 2 && result == RAST_OK; ++cls) {
        if (!has[cls]) continue;
        uint32_t bh = E.heavy_bits[cls];
        int bc = E.ctas_per_sm[cls];
        for (uint32_t h : heavy_opts)
            for (int k : cta_opts) {
                if (result != RAST_OK) break;
                if (h == bh && k == bc) continue;  // the current setting was timed already
                E.heavy_bits[cls] = h;
                E.ctas_per_sm[cls] = k;
                float ms = 0.0f;
                time_batch(ms);
                if (result == RAST_OK && ms < best_ms) {
                    best_ms = ms;
                    bh = h;
                    bc = k;
                }
            }
        E.heavy_bits[cls] = bh;
        E.ctas_per_sm[cls] = bc;
    }
    // the bin edge again, under the chosen splits
    if (result == RAST_OK) {
        sweep_tiles(true);
        c->tuned_tile[0] = best_tile[0];
        c->tuned_tile[1] = best_tile[1];
    }
    // 3. bin capacity: one run with the chosen settings measures each scene's bins; the batch
    // reserves that plus an eighth (batch_hints), instead of the first estimate
    uint64_t cap = 0;
    if (result == RAST_OK) {
        c->batch_hints.assign(n, 0);
        float ms = 0.0f;
        time_batch(ms);
        for (uint32_t i = 0; i < n && result == RAST_OK; ++i) cap += c->batch_hints[i];
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (result != RAST_OK) {
        c->tuned_tile[0] = saved_tile[0];
        c->tuned_tile[1] = saved_tile[1];
        for (int k = 0; k < 2; ++k) {
            E.heavy_bits[k] = saved_heavy[k];
            E.ctas_per_sm[k] = saved_ctas[k];
        }
        return result;
    }
    if (out) {
        for (int k = 0; k < 2; ++k) {
            out->tile[k] = c->tuned_tile[k];
            const uint32_t hb = E.heavy_bits[k];
            out->heavy_entries[k] = hb == 0 ? 0u : hb >= 32 ? 0xFFFFFFFFu : 1u << hb;
            out->raster_ctas_per_sm[k] = E.ctas_per_sm[k];
        }
        out->bin_capacity = cap;
        out->batch_ms = best_ms;
    }
    return RAST_OK;
}

rast_status rast_autotune_batch(rast_ctx* c, const rast_scene* sc, uint32_t n, int best_tiles[2]) {
    rast_tuning t;
    const rast_status st = rast_autotune_batch_ex(c, sc, n, &t);
    if (st == RAST_OK && best_tiles) {
        best_tiles[0] = t.tile[0];
        best_tiles[1] = t.tile[1];
    }
    return st;
}

rast_status rast_batch_create(rast_ctx* c, const rast_scene* sc, uint32_t n, rast_batch** out) {
    if (!c || !sc || n == 0 || !out) return RAST_INVALID_ARG;
    rast_batch* b = new (std::nothrow) rast_batch();
    if (!b) return RAST_OOM;
    b->ctx = c;
    c->sync_copies();
    size_t staging = 0;
    rast_status st = build_jobs(c, sc, n, true, b->jobs, &b->host_off, &staging);
    // host outputs: page-locked only (the graph copies into them); resolved into the batch's
    // own staging buffer
    for (uint32_t i = 0; st == RAST_OK && i < n; ++i)
        if (b->host_off[i] != (size_t)-1 && !is_pinned_host_ptr(sc[i].argb_out)) st = RAST_INVALID_ARG;
    if (st == RAST_OK && staging && !b->stage.reserve(staging)) st = RAST_OOM;
    for (uint32_t i = 0; st == RAST_OK && i < n; ++i)
        if (b->host_off[i] != (size_t)-1) b->jobs[i].out_dev = b->stage.p + b->host_off[i];
    if (st == RAST_OK && !b->E.init()) st = RAST_CUDA_ERROR;
    // the context's (autotuned) raster settings
    for (int k = 0; k < 2; ++k) {
        b->E.heavy_bits[k] = c->E.heavy_bits[k];
        b->E.ctas_per_sm[k] = c->E.ctas_per_sm[k];
    }
    if (st == RAST_OK) {
        // one synchronous run sizes every buffer of this batch's own engine
        b->E.sync_after = true;
        st = run_frames(b->E, b->jobs);
        if (st == RAST_TEXTURE_OOB) st = RAST_OK;
    }
    if (st == RAST_OK) {
        for (FrameJob& J : b->jobs) J.bin_hint = std::max<uint64_t>(J.bin_hint, J.need);
        b->E.sync_after = false;
        if (cudaStreamBeginCapture(b->E.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            st = RAST_CUDA_ERROR;
        } else {
            rast_status rs = run_frames(b->E, b->jobs);
            if (rs == RAST_OK && !enqueue_host_copies(b, sc, n)) rs = RAST_CUDA_ERROR;
            cudaMemcpyAsync(b->E.h_state, b->E.d_state, sizeof(DeviceState), cudaMemcpyDeviceToHost,
                            b->E.stream);
            cudaGraph_t g = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(b->E.stream, &g);
            if (rs != RAST_OK || ce != cudaSuccess || !g) {
                st = rs != RAST_OK ? rs : RAST_CUDA_ERROR;
                if (g) cudaGraphDestroy(g);
            } else {
                b->graph = g;
                if (cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) st = RAST_CUDA_ERROR;
            }
        }
        cudaGetLastError();
    }
    if (st != RAST_OK) {
        rast_batch_destroy(b);
        return st;
    }
    *out = b;
    return RAST_OK;
}

rast_status rast_batch_launch(rast_batch* b, int wait) {
    if (!b || !b->exec) return RAST_INVALID_ARG;
    if (cudaGraphLaunch(b->exec, b->E.stream) != cudaSuccess) return RAST_CUDA_ERROR;
    if (!wait) return RAST_OK;
    if (cudaStreamSynchronize(b->E.stream) != cudaSuccess) return RAST_CUDA_ERROR;
    const uint32_t s = b->E.h_state->status;
    if (s & (ST_BIN_OVERFLOW | ST_CLIP_STORE_OVERFLOW)) return RAST_BIN_OVERFLOW;
    if (s & ST_BAD_INDEX) return RAST_INVALID_ARG;
    if (s & ST_CLIP_OVERFLOW) return RAST_CLIP_OVERFLOW;
    if (s & ST_TEXTURE_OOB) return RAST_TEXTURE_OOB;
    return RAST_OK;
}

void* rast_batch_stream(rast_batch* b) { return b ? (void*)b->E.stream : nullptr; }

rast_status rast_batch_destroy(rast_batch* b) {
    if (!b) return RAST_INVALID_ARG;
    if (b->E.stream) cudaStreamSynchronize(b->E.stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    delete b;
    return RAST_OK;
}

}  // extern "C"
