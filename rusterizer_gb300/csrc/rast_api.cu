// rast_api.cu - host runtime behind the C ABI in include/rast.h.
//
// A context owns: resident meshes and textures, a CUDA stream, the scratch buffers of the
// pipeline (grown on demand and kept across frames), a pinned staging area for the per-frame
// descriptors, and a small device state block (status bits, statistics, allocation counters).
// A frame is one descriptor upload (skipped when the descriptors are unchanged), one state
// reset, seven kernel launches (eight with 32-pixel bins) and one state readback; capacity
// overflows (bins, clip store) are detected on the device and the frame is re-run with the
// measured sizes (at most twice). rast_framebuffer_async skips the readback; into host memory it
// resolves into alternating staging buffers that a side stream copies out.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/rast.h"
#include "rast_internal.h"
#include "rast_kernels.h"

using namespace rast;

namespace rast {

// Mat4 * Mat4 with Vector::dot's order (src/math/matrix.rs:56-79, src/math/vector.rs:17-23).
// Compiled with -ffp-contract=off so each product and sum rounds separately.
void mat4_mul(const float* a, const float* b, float* out) {
    float r[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            float s = 0.0f;
            for (int k = 0; k < 4; ++k) s = s + a[i * 4 + k] * b[k * 4 + j];
            r[i * 4 + j] = s;
        }
    std::memcpy(out, r, sizeof(r));
}

uint32_t heavy_bits_of(uint32_t min_entries) {
    // a power of two: bins with at least 2^bits entries are heavy; all ones: none is
    if (min_entries == 0xFFFFFFFFu) return 32u;
    return min_entries ? 31u - (uint32_t)__builtin_clz(min_entries) : 0u;
}

int choose_tile(int w, int h, int msaa, int req, uint64_t ntris) {
    if (req == 8 || req == 16 || req == 32) {
        long long n = (long long)((w + req - 1) / req) * ((h + req - 1) / req);
        if (n <= kMaxTilesPerFrame) return req;
    }
    (void)msaa;
    const bool big = ntris >= kAutoBigBinTris;
    // the preferred size where one counting pass covers the frame's bins, else the other
    for (int ts : {big ? 32 : 16, big ? 16 : 32}) {
        long long n = (long long)((w + ts - 1) / ts) * ((h + ts - 1) / ts);
        if (n <= kCountBandTiles) return ts;
    }
    // larger frames: the fewest bins (one counting pass per band of them)
    const long long n32 = (long long)((w + 31) / 32) * ((h + 31) / 32);
    return n32 <= kMaxTilesPerFrame ? 32 : 0;
}


rast_status run_frames(Engine& E, std::vector<FrameJob>& jobs) {
    if (jobs.empty()) return RAST_OK;
    cudaStream_t st = E.stream;
    // order frames by raster variant so that each (msaa, tile) group is one launch
    std::vector<size_t> order(jobs.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
        if (jobs[a].msaa != jobs[b].msaa) return jobs[a].msaa < jobs[b].msaa;
        return jobs[a].ts < jobs[b].ts;
    });
    E.h_order = order;

    for (int attempt = 0; attempt < 3; ++attempt) {
        std::vector<FrameDev>& frames = E.h_frames;
        std::vector<DrawDev>& draws = E.h_draws;
        std::vector<ChunkDev>& chunks = E.h_chunks;
        std::vector<uint2>& vblocks = E.h_vblocks;
        frames.clear();
        draws.clear();
        chunks.clear();
        vblocks.clear();
        uint64_t vtot = 0, ttot = 0, count_tot = 0, bin_tot = 0, qbin_tot = 0, clip_est = 0;
        uint32_t tile_tot = 0, group_tot = 0, max_tiles = 1;
        for (size_t oi = 0; oi < order.size(); ++oi) {
            FrameJob& J = jobs[order[oi]];
            FrameDev F{};
            F.width = (uint32_t)J.width;
            F.height = (uint32_t)J.height;
            F.msaa = J.msaa;
            F.ts = J.ts;
            F.tiles_x = (F.width + J.ts - 1) / J.ts;
            F.tiles_y = (F.height + J.ts - 1) / J.ts;
            F.ntiles = F.tiles_x * F.tiles_y;
            F.draw_begin = (uint32_t)draws.size();
            F.draw_count = (uint32_t)J.draws.size();
            F.tile_begin = tile_tot;
            F.group_begin = group_tot;
            F.rect_base = (uint32_t)ttot;
            F.count_base = count_tot;
            F.clear_depth = J.clear_depth;
            F.out = J.out_dev;
            F.dbg_depth = J.dbg_depth;
            F.dbg_color = J.dbg_color;
            uint32_t tb = 0, row = 0;
            for (const DrawJob& DJ : J.draws) {
                DrawDev D{};
                const MeshRec* m = DJ.mesh;
                D.pos = m->pos;
                D.uv = m->uv;
                D.rgba = m->rgba;
                D.idx = m->idx;
                D.tex = DJ.tex ? DJ.tex->data : nullptr;
                D.tex_w = DJ.tex ? (uint32_t)DJ.tex->w : 0u;
                D.tex_h = DJ.tex ? (uint32_t)DJ.tex->h : 0u;
                D.nverts = m->nverts;
                D.ntris = m->ntris;
                D.vbase = (uint32_t)vtot;
                D.tbase = tb;
                D.frame = (uint32_t)frames.size();
                D.fs = DJ.fs;
                std::memcpy(D.mvp, DJ.mvp, sizeof(D.mvp));
                const uint32_t di = (uint32_t)draws.size();
                draws.push_back(D);
                for (uint32_t v = 0; v < m->nverts; v += 256) vblocks.push_back(make_uint2(di, v));
                const uint32_t cs = chunk_size_for(std::max<uint32_t>(J.ntris_hint, m->ntris));
                for (uint32_t t = 0; t < m->ntris; t += cs) {
                    ChunkDev C{};
                    C.draw = di;
                    C.tri_begin = t;
                    C.tri_count = std::min(cs, m->ntris - t);
                    C.row = row++;
                    chunks.push_back(C);
                }
                vtot += m->nverts;
                tb += m->ntris;
            }
            F.ntris = tb;
            if (tb >= kMaxFrameTris) return RAST_INVALID_ARG;  // bin entries hold 27-bit triangle ids
            F.nchunks = row;
            const uint64_t want = std::max<uint64_t>(J.bin_hint, 4ull * tb + F.ntiles + 1024ull);
            F.bin_base = bin_tot;
            F.bin_cap = want;
            bin_tot += want;
            F.qbin_base = qbin_tot;
            if (raster_edge(J.ts) < J.ts) qbin_tot += 4ull * want;
            clip_est += 32ull * tb + 4096ull;
            count_tot += (uint64_t)F.nchunks * F.ntiles;
            ttot += tb;
            tile_tot += F.ntiles;
            group_tot += (F.ntiles + 31) / 32;
            max_tiles = std::max(max_tiles, F.ntiles);
            frames.push_back(F);
        }
        if (vtot >= 0xFFFFFFFFull || ttot >= 0xFFFFFFFFull || bin_tot >= 0xFFFFFFFFull)
            return RAST_INVALID_ARG;
        // scratch
        bool ok = E.vclip.reserve(vtot) && E.vscr.reserve(vtot) && E.vcode.reserve(vtot) &&
                  E.tri_rect.reserve(ttot) && E.tri_aux.reserve(ttot) &&
                  E.counts.reserve(count_tot) && E.tile_start.reserve(tile_tot) &&
                  E.tile_count.reserve(tile_tot) && E.tile_order.reserve(tile_tot) &&
                  E.bins.reserve(bin_tot) && E.qbins.reserve(qbin_tot) && E.clip_list.reserve(3ull * ttot) &&
                  E.qcount.reserve(qbin_tot ? 4ull * tile_tot : 0ull) &&
                  E.clip_store.reserve(std::max<uint64_t>(clip_est, E.clip_hint)) &&
                  E.frame_need.reserve(frames.size());
        if (!ok) return RAST_OOM;
        // descriptors: one pinned staging buffer, one async copy
        const size_t off_frames = 0;
        const size_t off_draws = align_up(off_frames + frames.size() * sizeof(FrameDev), 256);
        const size_t off_chunks = align_up(off_draws + draws.size() * sizeof(DrawDev), 256);
        const size_t off_vblocks = align_up(off_chunks + chunks.size() * sizeof(ChunkDev), 256);
        const size_t total = align_up(off_vblocks + vblocks.size() * sizeof(uint2), 256);
        // the previous upload may still be reading the pinned staging buffer
        if (E.desc_pending) {
            cudaEventSynchronize(E.desc_done);
            E.desc_pending = false;
        }
        if (!E.h_desc.reserve(total) || !E.d_desc.reserve(total)) return RAST_OOM;
        E.h_scratch.resize(total);
        std::memset(E.h_scratch.data(), 0, total);
        std::memcpy(E.h_scratch.data() + off_frames, frames.data(), frames.size() * sizeof(FrameDev));
        std::memcpy(E.h_scratch.data() + off_draws, draws.data(), draws.size() * sizeof(DrawDev));
        std::memcpy(E.h_scratch.data() + off_chunks, chunks.data(), chunks.size() * sizeof(ChunkDev));
        std::memcpy(E.h_scratch.data() + off_vblocks, vblocks.data(), vblocks.size() * sizeof(uint2));
        // identical descriptors (the same scene again) are already on the device
        const bool same = E.desc_valid && E.desc_bytes == total && E.d_desc_ptr == E.d_desc.p &&
                          std::memcmp(E.h_desc.p, E.h_scratch.data(), total) == 0;
        if (!same) {
            std::memcpy(E.h_desc.p, E.h_scratch.data(), total);
            if (cudaMemcpyAsync(E.d_desc.p, E.h_desc.p, total, cudaMemcpyHostToDevice, st) != cudaSuccess)
                return RAST_CUDA_ERROR;
            cudaEventRecord(E.desc_done, st);
            E.desc_pending = true;
            E.desc_valid = true;
            E.desc_bytes = total;
            E.d_desc_ptr = E.d_desc.p;
        }
        if (cudaMemsetAsync(E.d_state, 0, sizeof(DeviceState), st) != cudaSuccess) return RAST_CUDA_ERROR;

        LaunchArgs a{};
        a.stream = st;
        a.frames = reinterpret_cast<const FrameDev*>(E.d_desc.p + off_frames);
        a.nframes = (int)frames.size();
        a.draws = reinterpret_cast<const DrawDev*>(E.d_desc.p + off_draws);
        a.chunks = reinterpret_cast<const ChunkDev*>(E.d_desc.p + off_chunks);
        a.nchunks = (uint32_t)chunks.size();
        a.vblocks = reinterpret_cast<const uint2*>(E.d_desc.p + off_vblocks);
        a.vertex_blocks = (uint32_t)vblocks.size();
        a.scan_groups = group_tot;
        a.max_tiles = max_tiles;
        if (frames.size() == 1) {
            a.scan_order_queue = &E.d_state->queue[0];
            a.scan_heavy_bits = E.heavy_bits[frames[0].msaa == 4 ? 1 : 0];
        }
        Scratch& S = a.scratch;
        S.vclip = E.vclip.p;
        S.vscr = E.vscr.p;
        S.vcode = E.vcode.p;
        S.tri_rect = E.tri_rect.p;
        S.tri_aux = E.tri_aux.p;
        S.counts = E.counts.p;
        S.tile_start = E.tile_start.p;
        S.tile_count = E.tile_count.p;
        S.tile_order = E.tile_order.p;
        S.bins = E.bins.p;
        S.qbins = E.qbins.p;
        S.qcount = E.qcount.p;
        S.clip_store = E.clip_store.p;
        S.clip_cap = E.clip_store.cap;
        S.clip_used = &E.d_state->clip_used;
        S.clip_list = E.clip_list.p;
        S.clip_list_cap = ttot;
        S.clip_n = &E.d_state->clip_n;
        S.status = &E.d_state->status;
        S.stats = E.d_state->stats;
        S.frame_need = E.frame_need.p;
        S.log = E.log_on ? E.log.p : nullptr;
        S.log_n = &E.d_state->log_n;
        S.log_cap = E.log_on ? E.log.cap / 4 : 0;

        cudaError_t err = cudaSuccess;
        if (E.profiling) cudaEventRecord(E.ev[0], st);
        err = launch_vertex(a);
        if (E.profiling) cudaEventRecord(E.ev[1], st);
        if (err == cudaSuccess) err = launch_bin_count(a);
        if (E.profiling) cudaEventRecord(E.ev[2], st);
        if (err == cudaSuccess) err = launch_scans(a);
        if (E.profiling) cudaEventRecord(E.ev[3], st);
        if (err == cudaSuccess) err = launch_bin_scatter(a);
        if (E.profiling) cudaEventRecord(E.ev[4], st);
        // raster: one launch per (msaa, tile) group of consecutive frames; with several groups
        // (batches of mixed MSAA) they alternate between the context stream and its side stream,
        // so one group's tail overlaps the next group's start
        const bool multi = !frames.empty() &&
                           (frames.front().msaa != frames.back().msaa || frames.front().ts != frames.back().ts);
        if (multi && err == cudaSuccess) {
            if (cudaEventRecord(E.fork, st) != cudaSuccess || cudaStreamWaitEvent(E.side, E.fork, 0) != cudaSuccess)
                err = cudaErrorUnknown;
        }
        int group = 0;
        for (size_t i = 0; i < frames.size() && err == cudaSuccess; ++group) {
            if (group >= kMaxRasterGroups) {
                err = cudaErrorInvalidValue;
                break;
            }
            size_t j = i;
            uint32_t blocks = 0;
            while (j < frames.size() && frames[j].msaa == frames[i].msaa && frames[j].ts == frames[i].ts) {
                blocks += frames[j].ntiles;
                ++j;
            }
            a.stream = (multi && (group & 1)) ? E.side : st;
            a.raster_frames = a.frames + i;
            a.raster_nframes = (int)(j - i);
            a.raster_tile_offset = frames[i].tile_begin;
            a.raster_blocks = blocks;
            a.raster_queue = &E.d_state->queue[kQueueSlots * group];
            a.raster_heavy_bits = E.heavy_bits[frames[i].msaa == 4 ? 1 : 0];
            a.raster_ctas_per_sm = E.ctas_per_sm[frames[i].msaa == 4 ? 1 : 0];
            err = launch_raster(a, frames[i].msaa, frames[i].ts);
            i = j;
        }
        a.stream = st;
        if (multi && err == cudaSuccess) {
            if (cudaEventRecord(E.join, E.side) != cudaSuccess || cudaStreamWaitEvent(st, E.join, 0) != cudaSuccess)
                err = cudaErrorUnknown;
        }
        if (E.profiling) cudaEventRecord(E.ev[5], st);
        if (err != cudaSuccess) return RAST_CUDA_ERROR;
        if (E.sync_after) {
            if (cudaMemcpyAsync(E.h_state, E.d_state, sizeof(DeviceState), cudaMemcpyDeviceToHost, st) !=
                cudaSuccess)
                return RAST_CUDA_ERROR;
            if (frames.size() <= E.h_need.size() || E.h_need.reserve(frames.size())) {
                cudaMemcpyAsync(E.h_need.p, E.frame_need.p, frames.size() * sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost, st);
            }
            if (cudaStreamSynchronize(st) != cudaSuccess) return RAST_CUDA_ERROR;
            E.desc_pending = false;  // the stream drained: the staging buffer is free
            const uint32_t status = E.h_state->status;
            bool retry = false;
            if (status & ST_BIN_OVERFLOW) {
                for (size_t k = 0; k < frames.size(); ++k) {
                    FrameJob& J = jobs[order[k]];
                    const uint64_t need = E.h_need.p[k];
                    if (need > frames[k].bin_cap) J.bin_hint = need + need / 4 + 1024;
                }
                retry = true;
            }
            if (status & ST_CLIP_STORE_OVERFLOW) {
                E.clip_hint = E.h_state->clip_used + E.h_state->clip_used / 4 + 65536;
                retry = true;
            }
            if (retry && attempt < 2) continue;
            for (size_t k = 0; k < frames.size(); ++k) jobs[order[k]].need = E.h_need.p[k];
            E.last_status = status;
            std::memcpy(E.last_stats, E.h_state->stats, sizeof(E.last_stats));
            if (status & ST_BIN_OVERFLOW) return RAST_BIN_OVERFLOW;
            if (status & ST_CLIP_STORE_OVERFLOW) return RAST_BIN_OVERFLOW;
            if (status & ST_BAD_INDEX) return RAST_INVALID_ARG;
            if (status & ST_CLIP_OVERFLOW) return RAST_CLIP_OVERFLOW;
            if (status & ST_TEXTURE_OOB) return RAST_TEXTURE_OOB;
        }
        return RAST_OK;
    }
    return RAST_BIN_OVERFLOW;
}

}  // namespace rast

// ============================================================================ C ABI

static void identity16(float* m) {
    for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.0f : 0.0f;
}

extern "C" {

const char* rast_status_string(rast_status s) {
    switch (s) {
        case RAST_OK: return "ok";
        case RAST_INVALID_ARG: return "invalid argument";
        case RAST_OOM: return "device out of memory";
        case RAST_ADMISSION_REFUSED: return "admission refused (HBM budget)";
        case RAST_BIN_OVERFLOW: return "bin capacity overflow";
        case RAST_TIMEOUT: return "timeout";
        case RAST_TEXTURE_OOB: return "texel read past the texture (reference panics)";
        case RAST_CLIP_OVERFLOW: return "clip polygon overflow";
        case RAST_CUDA_ERROR: return "CUDA error";
        case RAST_NOT_READY: return "not ready";
    }
    return "unknown";
}

rast_ctx* rast_create(int width, int height, int msaa, rast_status* status) {
    auto set = [&](rast_status s) {
        if (status) *status = s;
    };
    if (width < 1 || height < 1 || width > 16384 || height > 16384 || (msaa != 1 && msaa != 4)) {
        set(RAST_INVALID_ARG);
        return nullptr;
    }
    rast_ctx* c = new (std::nothrow) rast_ctx();
    if (!c) {
        set(RAST_OOM);
        return nullptr;
    }
    c->width = width;
    c->height = height;
    c->msaa = msaa;
    identity16(c->world);
    identity16(c->view);
    identity16(c->proj);
    if (!c->E.init()) {
        delete c;
        set(RAST_CUDA_ERROR);
        return nullptr;
    }
    set(RAST_OK);
    return c;
}

void rast_destroy(rast_ctx* c) {
    if (!c) return;
    c->sync_copies();
    c->sync_readbacks();
    if (c->copy) cudaStreamDestroy(c->copy);
    if (c->frame_done) cudaEventDestroy(c->frame_done);
    if (c->readback) cudaStreamDestroy(c->readback);
    for (cudaEvent_t e : c->rb_done)
        if (e) cudaEventDestroy(e);
    cudaStreamSynchronize(c->E.stream);
    for (MeshRec& m : c->meshes) m.release();
    for (TexRec& t : c->textures) t.release();
    delete c;
}

rast_status rast_set_clear_depth(rast_ctx* c, float d) {
    if (!c) return RAST_INVALID_ARG;
    c->clear_depth = d;
    return RAST_OK;
}

rast_status rast_set_heavy_tile_entries(rast_ctx* c, uint32_t min_entries) {
    if (!c) return RAST_INVALID_ARG;
    c->E.heavy_bits[0] = c->E.heavy_bits[1] = heavy_bits_of(min_entries);
    return RAST_OK;
}

rast_status rast_set_tile_size(rast_ctx* c, int tile) {
    if (!c || (tile != 0 && tile != 8 && tile != 16 && tile != 32)) return RAST_INVALID_ARG;
    c->tile_req = tile;
    return RAST_OK;
}

rast_status rast_mesh_upload(rast_ctx* c, const float* pos, const float* uv, const float* rgba,
                             uint32_t nverts, const uint32_t* idx, uint32_t ntris, rast_mesh* out) {
    if (!c || !out || (nverts && (!pos || !uv)) || (ntris && !idx)) return RAST_INVALID_ARG;
    for (uint64_t i = 0; i < 3ull * ntris; ++i)
        if (idx[i] >= nverts) return RAST_INVALID_ARG;
    MeshRec m;
    rast_status s = m.upload(pos, uv, rgba, nverts, idx, ntris, c->E.stream);
    if (s != RAST_OK) return s;
    for (size_t i = 0; i < c->meshes.size(); ++i)
        if (!c->meshes[i].live) {
            c->meshes[i] = m;
            *out = (rast_mesh)i;
            return RAST_OK;
        }
    c->meshes.push_back(m);
    *out = (rast_mesh)(c->meshes.size() - 1);
    return RAST_OK;
}

rast_status rast_mesh_free(rast_ctx* c, rast_mesh mesh) {
    if (!c || mesh >= c->meshes.size() || !c->meshes[mesh].live) return RAST_INVALID_ARG;
    c->sync_copies();
    cudaStreamSynchronize(c->E.stream);
    c->meshes[mesh].release();
    return RAST_OK;
}

// Copies new host data over a resident mesh of the same size, on `st`.
static bool copy_mesh(MeshRec& m, const float* pos, const float* uv, const float* rgba, const uint32_t* idx,
                      cudaStream_t st) {
    bool ok = true;
    if (m.nverts) {
        ok &= cudaMemcpyAsync(m.pos, pos, (size_t)m.nverts * 12, cudaMemcpyHostToDevice, st) == cudaSuccess;
        ok &= cudaMemcpyAsync(m.uv, uv, (size_t)m.nverts * 8, cudaMemcpyHostToDevice, st) == cudaSuccess;
        if (rgba)
            ok &= cudaMemcpyAsync(m.rgba, rgba, (size_t)m.nverts * 16, cudaMemcpyHostToDevice, st) == cudaSuccess;
    }
    if (m.ntris) ok &= cudaMemcpyAsync(m.idx, idx, (size_t)m.ntris * 12, cudaMemcpyHostToDevice, st) == cudaSuccess;
    return ok;
}

rast_status rast_mesh_update(rast_ctx* c, rast_mesh mesh, const float* pos, const float* uv,
                             const float* rgba, const uint32_t* idx) {
    if (!c || mesh >= c->meshes.size() || !c->meshes[mesh].live) return RAST_INVALID_ARG;
    MeshRec& m = c->meshes[mesh];
    if ((m.nverts && (!pos || !uv)) || (m.ntris && !idx) || ((rgba != nullptr) != (m.rgba != nullptr)))
        return RAST_INVALID_ARG;
    c->sync_copies();
    cudaStream_t st = c->E.stream;
    bool ok = copy_mesh(m, pos, uv, rgba, idx, st);
    // the caller may reuse its arrays once this returns
    ok &= cudaStreamSynchronize(st) == cudaSuccess;
    return ok ? RAST_OK : RAST_CUDA_ERROR;
}

rast_status rast_mesh_update_async(rast_ctx* c, rast_mesh mesh, const float* pos, const float* uv,
                                   const float* rgba, const uint32_t* idx) {
    if (!c || mesh >= c->meshes.size() || !c->meshes[mesh].live) return RAST_INVALID_ARG;
    MeshRec& m = c->meshes[mesh];
    if ((m.nverts && (!pos || !uv)) || (m.ntris && !idx) || ((rgba != nullptr) != (m.rgba != nullptr)))
        return RAST_INVALID_ARG;
    if (!c->copy && cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking) != cudaSuccess) {
        c->copy = nullptr;
        return RAST_CUDA_ERROR;
    }
    if (!c->frame_done && cudaEventCreateWithFlags(&c->frame_done, cudaEventDisableTiming) != cudaSuccess) {
        c->frame_done = nullptr;
        return RAST_CUDA_ERROR;
    }
    if (!m.ready && cudaEventCreateWithFlags(&m.ready, cudaEventDisableTiming) != cudaSuccess) {
        m.ready = nullptr;
        return RAST_CUDA_ERROR;
    }
    // the frames already enqueued may still read this mesh: the copies start after them
    bool ok = !c->frame_recorded || cudaStreamWaitEvent(c->copy, c->frame_done, 0) == cudaSuccess;
    ok = ok && copy_mesh(m, pos, uv, rgba, idx, c->copy);
    ok = ok && cudaEventRecord(m.ready, c->copy) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        return RAST_CUDA_ERROR;
    }
    m.pending = true;
    return RAST_OK;
}

rast_status rast_texture_upload(rast_ctx* c, int slot, const uint8_t* rgba8, int w, int h) {
    if (!c || !rgba8 || w < 1 || h < 1 || slot != (int)c->textures.size()) return RAST_INVALID_ARG;
    TexRec t;
    rast_status s = t.upload(rgba8, w, h, c->E.stream);
    if (s != RAST_OK) return s;
    c->textures.push_back(t);
    return RAST_OK;
}

rast_status rast_set_uniforms(rast_ctx* c, const float world[16], const float view[16],
                              const float proj[16]) {
    if (!c) return RAST_INVALID_ARG;
    if (world) std::memcpy(c->world, world, sizeof(c->world));
    if (view) std::memcpy(c->view, view, sizeof(c->view));
    if (proj) std::memcpy(c->proj, proj, sizeof(c->proj));
    return RAST_OK;
}

rast_status rast_draw(rast_ctx* c, rast_mesh mesh, int vs_id, int fs_id) {
    if (!c || mesh >= c->meshes.size() || !c->meshes[mesh].live) return RAST_INVALID_ARG;
    if (vs_id != RAST_VS_MVP || fs_id < 0 || fs_id > 2) return RAST_INVALID_ARG;
    if (fs_id == RAST_FS_TEXTURE && c->textures.empty()) return RAST_INVALID_ARG;
    // handles, not pointers: later uploads may reallocate the mesh table before the frame
    DrawJob d;
    d.mesh = nullptr;
    d.mesh_id = mesh;
    d.tex = nullptr;
    d.fs = fs_id;
    float pv[16];
    mat4_mul(c->proj, c->view, pv);
    mat4_mul(pv, c->world, d.mvp);
    c->queue.push_back(d);
    return RAST_OK;
}

static rast_status framebuffer_impl(rast_ctx* c, uint32_t* argb_out, bool sync) {
    if (!c) return RAST_INVALID_ARG;
    uint64_t ntris = 0;
    for (const DrawJob& d : c->queue)
        if (d.mesh_id < c->meshes.size() && c->meshes[d.mesh_id].live) ntris += c->meshes[d.mesh_id].ntris;
    const int ts = choose_tile(c->width, c->height, c->msaa, c->tile_req, ntris);
    if (!ts) return RAST_INVALID_ARG;
    const size_t npx = (size_t)c->width * (size_t)c->height;
    uint32_t* direct = nullptr;  // where the kernels write the image, when not the context's buffer
    if (argb_out) {
        cudaPointerAttributes attr;
        if (cudaPointerGetAttributes(&attr, argb_out) == cudaSuccess) {
            // host memory gets a copy after the frame (a resolve writing page-locked host memory
            // directly over the host link was measured: two host threads' frames slowed from
            // 2079 to 1821 frames/s on the 2M-triangle 4K frame)
            if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) direct = argb_out;
        }
        cudaGetLastError();
    }
    // an asynchronous frame into host memory resolves into a staging buffer of its own and is
    // copied on the readback stream; a synchronous one first lets earlier readbacks land
    const bool host_async = !sync && argb_out && !direct;
    const unsigned slot = c->rb_next;
    if (host_async) {
        if (!c->readback && cudaStreamCreateWithFlags(&c->readback, cudaStreamNonBlocking) != cudaSuccess) {
            c->readback = nullptr;
            return RAST_CUDA_ERROR;
        }
        for (cudaEvent_t* e : {&c->rb_done[0], &c->rb_done[1], &c->frame_done})
            if (!*e && cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) {
                *e = nullptr;
                return RAST_CUDA_ERROR;
            }
        if (!c->rb_stage[slot].reserve(npx)) return RAST_OOM;
        // the staging buffer's previous copy must have read it before this frame resolves
        if (c->rb_pending[slot] && cudaStreamWaitEvent(c->E.stream, c->rb_done[slot], 0) != cudaSuccess)
            return RAST_CUDA_ERROR;
    } else if (sync) {
        c->sync_readbacks();
    }
    if (!direct && !host_async && !c->out.reserve(npx)) return RAST_OOM;
    if (c->capture && (!c->dbg_depth.reserve(npx * c->msaa) || !c->dbg_color.reserve(npx * c->msaa)))
        return RAST_OOM;
    std::vector<FrameJob> jobs(1);
    FrameJob& J = jobs[0];
    J.width = c->width;
    J.height = c->height;
    J.msaa = c->msaa;
    J.ts = ts;
    J.clear_depth = c->clear_depth;
    J.out_dev = direct ? direct : host_async ? c->rb_stage[slot].p : c->out.p;
    J.dbg_depth = c->capture ? c->dbg_depth.p : nullptr;
    J.dbg_color = c->capture ? c->dbg_color.p : nullptr;
    J.draws = c->queue;
    for (DrawJob& d : J.draws) {
        if (d.mesh_id >= c->meshes.size() || !c->meshes[d.mesh_id].live) {
            c->queue.clear();
            return RAST_INVALID_ARG;
        }
        d.mesh = &c->meshes[d.mesh_id];
        d.tex = c->textures.empty() ? nullptr : &c->textures[0];
    }
    J.bin_hint = c->bin_hint;
    uint32_t nt = 0;
    for (const DrawJob& d : J.draws) nt += d.mesh->ntris;
    J.ntris_hint = nt;
    // meshes with an asynchronous update in flight: the frame waits for their copies
    for (DrawJob& d : J.draws) {
        MeshRec& m = c->meshes[d.mesh_id];
        if (!m.pending) continue;
        if (cudaStreamWaitEvent(c->E.stream, m.ready, 0) != cudaSuccess) {
            c->queue.clear();
            return RAST_CUDA_ERROR;
        }
        m.pending = false;
    }
    c->E.sync_after = sync;
    rast_status s = run_frames(c->E, jobs);
    c->queue.clear();
    if (c->frame_done && cudaEventRecord(c->frame_done, c->E.stream) == cudaSuccess) c->frame_recorded = true;
    if (s != RAST_OK && s != RAST_TEXTURE_OOB) return s;
    if (sync && J.need) c->bin_hint = std::max<uint64_t>(c->bin_hint, J.need + J.need / 8);
    if (host_async) {
        // the copy waits for this frame (frame_done was recorded right after it)
        if (!c->frame_recorded || cudaStreamWaitEvent(c->readback, c->frame_done, 0) != cudaSuccess ||
            cudaMemcpyAsync(argb_out, c->rb_stage[slot].p, npx * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                            c->readback) != cudaSuccess ||
            cudaEventRecord(c->rb_done[slot], c->readback) != cudaSuccess)
            return RAST_CUDA_ERROR;
        c->rb_dst[slot] = argb_out;
        c->rb_pending[slot] = true;
        c->rb_next = slot ^ 1u;
    } else if (argb_out && !direct) {
        if (cudaMemcpyAsync(argb_out, c->out.p, npx * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                            c->E.stream) != cudaSuccess)
            return RAST_CUDA_ERROR;
        if (cudaStreamSynchronize(c->E.stream) != cudaSuccess) return RAST_CUDA_ERROR;
    }
    return s;
}

rast_status rast_framebuffer(rast_ctx* c, uint32_t* argb_out) { return framebuffer_impl(c, argb_out, true); }

/* Enqueue-only variant used by throughput loops: no stream synchronisation and no overflow
 * re-run; capacities come from earlier synchronous frames of the same context. */
rast_status rast_framebuffer_async(rast_ctx* c, uint32_t* argb_out) {
    return framebuffer_impl(c, argb_out, false);
}

rast_status rast_wait_output(rast_ctx* c, const uint32_t* argb_out) {
    if (!c) return RAST_INVALID_ARG;
    for (unsigned k = 0; k < 2; ++k) {
        if (!c->rb_pending[k] || (argb_out && c->rb_dst[k] != argb_out)) continue;
        if (cudaEventSynchronize(c->rb_done[k]) != cudaSuccess) return RAST_CUDA_ERROR;
        c->rb_pending[k] = false;
    }
    return RAST_OK;
}

rast_status rast_stats(rast_ctx* c, uint64_t* shaded, uint64_t* fsinv, uint64_t* oob) {
    if (!c) return RAST_INVALID_ARG;
    if (shaded) *shaded = c->E.last_stats[STAT_SHADED];
    if (fsinv) *fsinv = c->E.last_stats[STAT_FSINV];
    if (oob) *oob = c->E.last_stats[STAT_OOB];
    return RAST_OK;
}

void* rast_stream(rast_ctx* c) { return c ? (void*)c->E.stream : nullptr; }

uint64_t rast_kernel_launches(void) { return kernel_launches(); }

rast_status rast_set_profiling(rast_ctx* c, int enable) {
    if (!c) return RAST_INVALID_ARG;
    c->E.profiling = enable != 0;
    return RAST_OK;
}

int rast_stage_times(rast_ctx* c, float* ms, int n) {
    if (!c || !ms || !c->E.profiling) return 0;
    // events of the last enqueued frame; the caller has synchronised the stream
    for (int k = 0; k < 5; ++k)
        if (cudaEventElapsedTime(&c->E.stage_ms[k], c->E.ev[k], c->E.ev[k + 1]) != cudaSuccess) {
            cudaGetLastError();
            return 0;
        }
    int k = std::min(n, 5);
    for (int i = 0; i < k; ++i) ms[i] = c->E.stage_ms[i];
    return k;
}

rast_status rast_debug_capture_samples(rast_ctx* c, int enable) {
    if (!c) return RAST_INVALID_ARG;
    c->capture = enable != 0;
    return RAST_OK;
}

rast_status rast_read_samples(rast_ctx* c, float* depth, uint32_t* color) {
    if (!c || !c->capture || !c->dbg_depth.p) return RAST_INVALID_ARG;
    const size_t n = (size_t)c->width * c->height * c->msaa;
    if (depth && cudaMemcpy(depth, c->dbg_depth.p, n * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
        return RAST_CUDA_ERROR;
    if (color && cudaMemcpy(color, c->dbg_color.p, n * sizeof(uint32_t), cudaMemcpyDeviceToHost) != cudaSuccess)
        return RAST_CUDA_ERROR;
    return RAST_OK;
}

rast_status rast_debug_log_enable(rast_ctx* c, uint64_t capacity) {
    if (!c) return RAST_INVALID_ARG;
    if (capacity == 0) {
        c->E.log_on = false;
        return RAST_OK;
    }
    if (!c->E.log.reserve(capacity * 4)) return RAST_OOM;
    c->E.log_on = true;
    return RAST_OK;
}

rast_status rast_debug_log_read(rast_ctx* c, uint32_t* out, uint64_t capacity, uint64_t* count) {
    if (!c || !c->E.log_on) return RAST_INVALID_ARG;
    const uint64_t n = std::min<uint64_t>(c->E.h_state->log_n, c->E.log.cap / 4);
    if (count) *count = n;
    if (out && capacity) {
        const uint64_t m = std::min(n, capacity);
        if (cudaMemcpy(out, c->E.log.p, m * 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost) != cudaSuccess)
            return RAST_CUDA_ERROR;
    }
    return RAST_OK;
}

rast_status rast_debug_kat(int op, const void* in, size_t in_bytes, void* out, size_t out_bytes) {
    if (!in || !out || in_bytes == 0 || out_bytes == 0) return RAST_INVALID_ARG;
    void *din = nullptr, *dout = nullptr;
    if (cudaMalloc(&din, in_bytes) != cudaSuccess) return RAST_OOM;
    if (cudaMalloc(&dout, out_bytes) != cudaSuccess) {
        cudaFree(din);
        return RAST_OOM;
    }
    rast_status s = RAST_OK;
    if (cudaMemcpy(din, in, in_bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(dout, 0, out_bytes) != cudaSuccess || launch_kat(op, din, dout, 0) != cudaSuccess ||
        cudaMemcpy(out, dout, out_bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
        s = RAST_CUDA_ERROR;
    cudaFree(din);
    cudaFree(dout);
    return s;
}

}  // extern "C"
