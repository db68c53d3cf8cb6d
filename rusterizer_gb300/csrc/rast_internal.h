// rast_internal.h - host-side engine state shared by the plain, batched and serving paths.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/rast.h"
#include "rast_types.h"

namespace rast {

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Device buffer that only grows (one cudaMalloc per growth, never per frame).
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;
    bool reserve(size_t n) {
        if (n <= cap && p) return true;
        size_t c = n > cap + cap / 2 ? n : cap + cap / 2;
        if (c == 0) c = 1;
        T* q = nullptr;
        if (cudaMalloc(&q, c * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (p) cudaFree(p);
        p = q;
        cap = c;
        return true;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    ~DevBuf() { release(); }
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
};

// Pinned host buffer for asynchronous copies.
template <typename T>
struct HostBuf {
    T* p = nullptr;
    size_t cap = 0;
    bool reserve(size_t n) {
        if (n <= cap && p) return true;
        size_t c = n > cap + cap / 2 ? n : cap + cap / 2;
        if (c == 0) c = 1;
        T* q = nullptr;
        if (cudaMallocHost(&q, c * sizeof(T)) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        if (p) cudaFreeHost(p);
        p = q;
        cap = c;
        return true;
    }
    size_t size() const { return cap; }
    ~HostBuf() {
        if (p) cudaFreeHost(p);
    }
    HostBuf() = default;
    HostBuf(const HostBuf&) = delete;
    HostBuf& operator=(const HostBuf&) = delete;
};

// A resident mesh (Mesh{vertices, indices, attributes}, src/mesh.rs:5-12).
struct MeshRec {
    float* pos = nullptr;
    float* uv = nullptr;
    float* rgba = nullptr;
    uint32_t* idx = nullptr;
    uint32_t nverts = 0, ntris = 0;
    bool live = false;
    cudaEvent_t ready = nullptr;  // end of the last rast_mesh_update_async copy
    bool pending = false;         // that copy has not been waited for by a frame yet
    size_t bytes() const {
        return (size_t)nverts * (12 + 8 + (rgba ? 16 : 0)) + (size_t)ntris * 12;
    }
    rast_status upload(const float* hpos, const float* huv, const float* hrgba, uint32_t nv,
                       const uint32_t* hidx, uint32_t nt, cudaStream_t st) {
        nverts = nv;
        ntris = nt;
        auto alloc = [](void** p, size_t b) { return cudaMalloc(p, b ? b : 4) == cudaSuccess; };
        if (!alloc((void**)&pos, (size_t)nv * 12) || !alloc((void**)&uv, (size_t)nv * 8) ||
            (hrgba && !alloc((void**)&rgba, (size_t)nv * 16)) || !alloc((void**)&idx, (size_t)nt * 12)) {
            cudaGetLastError();
            release();
            return RAST_OOM;
        }
        bool ok = true;
        if (nv) {
            ok &= cudaMemcpyAsync(pos, hpos, (size_t)nv * 12, cudaMemcpyHostToDevice, st) == cudaSuccess;
            ok &= cudaMemcpyAsync(uv, huv, (size_t)nv * 8, cudaMemcpyHostToDevice, st) == cudaSuccess;
            if (hrgba)
                ok &= cudaMemcpyAsync(rgba, hrgba, (size_t)nv * 16, cudaMemcpyHostToDevice, st) == cudaSuccess;
        }
        if (nt) ok &= cudaMemcpyAsync(idx, hidx, (size_t)nt * 12, cudaMemcpyHostToDevice, st) == cudaSuccess;
        ok &= cudaStreamSynchronize(st) == cudaSuccess;
        if (!ok) {
            release();
            return RAST_CUDA_ERROR;
        }
        live = true;
        return RAST_OK;
    }
    void release() {
        if (pos) cudaFree(pos);
        if (uv) cudaFree(uv);
        if (rgba) cudaFree(rgba);
        if (idx) cudaFree(idx);
        if (ready) cudaEventDestroy(ready);
        pos = uv = rgba = nullptr;
        idx = nullptr;
        ready = nullptr;
        pending = false;
        live = false;
    }
};

// A resident RGBA8 texture, one u32 per texel (byte 0 = red).
struct TexRec {
    uint32_t* data = nullptr;
    int w = 0, h = 0;
    rast_status upload(const uint8_t* rgba8, int tw, int th, cudaStream_t st) {
        w = tw;
        h = th;
        const size_t b = (size_t)tw * (size_t)th * 4;
        if (cudaMalloc(&data, b) != cudaSuccess) {
            cudaGetLastError();
            data = nullptr;
            return RAST_OOM;
        }
        if (cudaMemcpyAsync(data, rgba8, b, cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            release();
            return RAST_CUDA_ERROR;
        }
        return RAST_OK;
    }
    void release() {
        if (data) cudaFree(data);
        data = nullptr;
    }
};

struct DrawJob {
    const MeshRec* mesh = nullptr;
    uint32_t mesh_id = 0;
    const TexRec* tex = nullptr;
    int fs = 0;
    float mvp[16];
};

struct FrameJob {
    int width = 0, height = 0, msaa = 4, ts = 16;
    float clear_depth = 3.40282347e+38f;
    std::vector<DrawJob> draws;
    uint32_t* out_dev = nullptr;
    float* dbg_depth = nullptr;
    uint32_t* dbg_color = nullptr;
    uint64_t bin_hint = 0;   // bins to reserve (0: default estimate)
    uint32_t ntris_hint = 0;
    uint64_t need = 0;       // bins the frame used (filled after a synchronous run)
};

// Device state block reset at the start of every launch sequence.
struct DeviceState {
    uint32_t status;
    uint32_t pad;
    unsigned long long stats[STAT_COUNT];
    unsigned long long clip_used;
    unsigned long long log_n;
    unsigned int clip_n;     // triangles queued for the warp clipper
    unsigned int pad2;
    unsigned int queue[kQueueSlots * kMaxRasterGroups];  // raster tile queues per (msaa, tile) group
};

struct Engine {
    cudaStream_t stream = nullptr;
    DevBuf<float4> vclip, vscr;
    DevBuf<uint16_t> vcode;
    DevBuf<unsigned long long> tri_rect;
    DevBuf<uint32_t> tri_aux, counts, tile_start, tile_count, tile_order, bins, qbins, qcount, clip_list;
    DevBuf<float> clip_store;
    DevBuf<unsigned long long> frame_need;
    DevBuf<uint32_t> log;
    bool log_on = false;
    DevBuf<unsigned char> d_desc;
    HostBuf<unsigned char> h_desc;
    HostBuf<unsigned long long> h_need;
    DeviceState* d_state = nullptr;
    DeviceState* h_state = nullptr;
    uint64_t clip_hint = 0;
    // raster settings per MSAA class ([0] MSAA 1, [1] MSAA 4): bins of >= 2^heavy_bits entries
    // are rastered CTA-wide, the others one warp per tile; persistent raster CTAs per SM (0: as
    // many as fit)
    uint32_t heavy_bits[2] = {kDefaultHeavyBits, kDefaultHeavyBits};
    int ctas_per_sm[2] = {0, 0};
    bool sync_after = true;
    bool profiling = false;
    cudaEvent_t ev[6] = {};
    float stage_ms[5] = {0, 0, 0, 0, 0};
    uint32_t last_status = 0;
    unsigned long long last_stats[STAT_COUNT] = {0, 0, 0, 0};
    std::vector<FrameDev> h_frames;
    std::vector<DrawDev> h_draws;
    std::vector<ChunkDev> h_chunks;
    std::vector<uint2> h_vblocks;
    std::vector<unsigned char> h_scratch;
    std::vector<size_t> h_order;  // job index of each frame of the last launch (device order)
    cudaEvent_t desc_done = nullptr;  // last descriptor upload finished reading h_desc
    // a second stream for raster launches of different (msaa, tile) groups, which then overlap
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    bool desc_pending = false, desc_valid = false;
    size_t desc_bytes = 0;
    unsigned char* d_desc_ptr = nullptr;

    bool init() {
        if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) return false;
        if (cudaMalloc(&d_state, sizeof(DeviceState)) != cudaSuccess) return false;
        if (cudaMallocHost(&h_state, sizeof(DeviceState)) != cudaSuccess) return false;
        std::memset(h_state, 0, sizeof(DeviceState));
        for (auto& e : ev)
            if (cudaEventCreate(&e) != cudaSuccess) return false;
        if (cudaEventCreateWithFlags(&desc_done, cudaEventDisableTiming) != cudaSuccess) return false;
        if (cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking) != cudaSuccess) return false;
        if (cudaEventCreateWithFlags(&fork, cudaEventDisableTiming) != cudaSuccess) return false;
        if (cudaEventCreateWithFlags(&join, cudaEventDisableTiming) != cudaSuccess) return false;
        return h_need.reserve(64);
    }
    ~Engine() {
        if (stream) cudaStreamSynchronize(stream);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        if (desc_done) cudaEventDestroy(desc_done);
        if (side) cudaStreamSynchronize(side);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (side) cudaStreamDestroy(side);
        if (d_state) cudaFree(d_state);
        if (h_state) cudaFreeHost(h_state);
        if (stream) cudaStreamDestroy(stream);
    }
};

void mat4_mul(const float* a, const float* b, float* out);
// Bin edge for a frame: the requested 8, 16 or 32 when the frame's bin count fits, else
// automatic: 32-pixel bins from kAutoBigBinTris triangles on (the binning work grows with
// chunks x bins, and quadrant rastering keeps 16-pixel raster tiles), 16-pixel bins below.
// 0 when no bin size fits.
constexpr uint64_t kAutoBigBinTris = 8192;
int choose_tile(int w, int h, int msaa, int req, uint64_t ntris);
// rast_set_heavy_tile_entries' threshold as a bit length (32: no bin is heavy)
uint32_t heavy_bits_of(uint32_t min_entries);
rast_status run_frames(Engine& E, std::vector<FrameJob>& jobs);

}  // namespace rast

// The context behind the C ABI: resident meshes and textures, the plain path's draw queue and
// framebuffer, and the tile sizes chosen by the batch autotuner.
struct rast_ctx {
    rast::Engine E;
    int width = 0, height = 0, msaa = 4;
    float clear_depth = 3.40282347e+38f;
    int tile_req = 0;
    std::vector<rast::MeshRec> meshes;
    std::vector<rast::TexRec> textures;
    float world[16], view[16], proj[16];
    std::vector<rast::DrawJob> queue;
    rast::DevBuf<uint32_t> out;
    bool capture = false;
    rast::DevBuf<float> dbg_depth;
    rast::DevBuf<uint32_t> dbg_color;
    uint64_t bin_hint = 0;
    int tuned_tile[2] = {0, 0};             // batch autotuner: MSAA 1, MSAA 4
    std::vector<uint64_t> batch_hints;      // bins needed per scene by the last batch
    rast::DevBuf<uint32_t> batch_out;       // staging for host-pointer batch outputs
    // asynchronous mesh updates: their copies run on `copy` after the frames enqueued before
    // them (`frame_done`, recorded after every frame), and frames wait for the mesh's `ready`
    cudaStream_t copy = nullptr;
    cudaEvent_t frame_done = nullptr;
    bool frame_recorded = false;
    // waits for every asynchronous mesh copy (before synchronous updates, frees and the batch
    // and server paths, which do not track them)
    void sync_copies() {
        if (copy) cudaStreamSynchronize(copy);
        for (rast::MeshRec& m : meshes) m.pending = false;
    }
    // asynchronous frames into host memory: a frame resolves into staging buffer rb_next
    // (alternating), which `readback` copies to the host once the frame is done; a staging
    // buffer is written again only after its previous copy (rb_done). rb_dst/rb_pending name
    // each buffer's last copy for rast_wait_output.
    rast::DevBuf<uint32_t> rb_stage[2];
    cudaStream_t readback = nullptr;
    cudaEvent_t rb_done[2] = {nullptr, nullptr};
    const void* rb_dst[2] = {nullptr, nullptr};
    bool rb_pending[2] = {false, false};
    unsigned rb_next = 0;
    // waits for every asynchronous readback (before synchronous frames, which could otherwise
    // be overtaken by an earlier frame's copy into the same host array)
    void sync_readbacks() {
        if (readback) cudaStreamSynchronize(readback);
        rb_pending[0] = rb_pending[1] = false;
    }
};
