// rast_noalloc.cu - one frame of the raster pipeline without any memory allocation.
//
// Some callers cannot allocate device memory at the moment they want a frame: a plugin or
// engine that owns every byte of device memory through its own pool, code running inside a
// region where cudaMalloc is forbidden or would stall (a real-time loop that must not
// synchronise the device, which cudaMalloc/cudaFree can do), or a process whose allocator
// belongs to another framework. rast_render_noalloc serves them: the caller passes its own
// device buffers for the mesh, the texture and the image, and every intermediate buffer of
// the pipeline (vertex records, tile histograms, bins, clip polygons, descriptors, status)
// lives in one fixed array in device memory that belongs to this library.
//
// That array is kNoAllocScratchBytes (32 MiB) per GPU, reserved on every GPU that loads the
// library until the process exits. Frames that would need more are refused with
// RAST_INVALID_ARG before anything is launched. All calls share the one array: calls whose
// GPU work overlaps (two host threads, or two streams without ordering) race on it and must
// be serialised by the caller.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/rast.h"
#include "rast_internal.h"
#include "rast_kernels.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
constexpr uint32_t kNoAllocMaxVerts = 262144;
constexpr uint32_t kNoAllocMaxTris = 262144;
constexpr uint32_t kMinChunk = 256;  // smallest chunk chunk_size_for returns
constexpr int kMaxDevices = 64;

}  // namespace

// The scratch itself. In host code this name is only a stand-in for the symbol: its device
// address comes from cudaGetSymbolAddress (below), once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

std::mutex g_setup_mu;
unsigned char* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device, looked up on the first call
// made with that device current.
rast_status scratch_for_current_device(unsigned char** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return RAST_CUDA_ERROR;
    }
    if (dev < 0 || dev >= kMaxDevices) return RAST_INVALID_ARG;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return RAST_CUDA_ERROR;
        }
        g_scratch_addr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_addr[dev];
    return RAST_OK;
}

struct Carve {
    size_t off = 0;
    size_t take(size_t bytes) {
        const size_t o = off;
        off = rast::align_up(off + bytes, 256);
        return o;
    }
};

// Offsets of every buffer of one frame inside the scratch array, for the given bin and
// clip-store capacities; `end` is the bytes used.
struct Layout {
    size_t state, frame, draw, chunks, vblocks, vclip, vscr, vcode, rect, aux, counts, tstart, tcount,
        torder, need, bins, qbins, qcount, clip, clist, end;
};

Layout carve_layout(uint32_t nverts, uint32_t ntris, uint32_t nchunks, uint32_t nvb, uint32_t ntiles,
                    bool split, unsigned long long bin_cap, unsigned long long clip_floats) {
    using namespace rast;
    Carve c;
    Layout L;
    L.state = c.take(sizeof(DeviceState));
    L.frame = c.take(sizeof(FrameDev));
    L.draw = c.take(sizeof(DrawDev));
    L.chunks = c.take(sizeof(ChunkDev) * (nchunks ? nchunks : 1));
    L.vblocks = c.take(sizeof(uint2) * (nvb ? nvb : 1));
    L.vclip = c.take(sizeof(float4) * (size_t)nverts);
    L.vscr = c.take(sizeof(float4) * (size_t)nverts);
    L.vcode = c.take(sizeof(uint16_t) * (size_t)nverts);
    L.rect = c.take(sizeof(unsigned long long) * (size_t)ntris);
    L.aux = c.take(sizeof(uint32_t) * (size_t)ntris);
    L.counts = c.take(sizeof(uint32_t) * (size_t)nchunks * ntiles);
    L.tstart = c.take(sizeof(uint32_t) * ntiles);
    L.tcount = c.take(sizeof(uint32_t) * ntiles);
    L.torder = c.take(sizeof(uint32_t) * ntiles);
    L.need = c.take(sizeof(unsigned long long));
    L.bins = c.take(sizeof(uint32_t) * bin_cap);
    // 32-pixel bins are split into quadrant lists for the raster
    L.qbins = c.take(split ? sizeof(uint32_t) * 4ull * bin_cap : 0);
    L.qcount = c.take(split ? sizeof(uint32_t) * 4ull * ntiles : 0);
    L.clip = c.take(sizeof(float) * clip_floats);
    L.clist = c.take(sizeof(uint32_t) * 3ull * (ntris ? ntris : 1));
    L.end = c.off;
    return L;
}

// Host staging of the chunk and vertex-block descriptors: function-level statics instead of
// about 24 KB of stack (callers on small thread stacks), filled and copied under this lock.
// cudaMemcpyAsync from pageable memory returns once the source has been read, so the lock is
// held for the copies' enqueue only.
std::mutex g_desc_mu;
rast::ChunkDev g_chunks[(kNoAllocMaxTris + kMinChunk - 1) / kMinChunk];
uint2 g_vblocks[(kNoAllocMaxVerts + 255) / 256];

}  // namespace

extern "C" rast_status rast_render_noalloc(int width, int height, int msaa, int tile,
                                           float clear_depth, const float* d_pos,
                                           const float* d_uv, const float* d_rgba, uint32_t nverts,
                                           const uint32_t* d_idx, uint32_t ntris,
                                           const float world[16], const float view[16],
                                           const float proj[16], const uint32_t* d_tex,
                                           int tex_w, int tex_h, int fs_id, uint32_t* d_argb,
                                           void* stream) {
    using namespace rast;
    if (width < 1 || height < 1 || width > 16384 || height > 16384 || (msaa != 1 && msaa != 4))
        return RAST_INVALID_ARG;
    if (!d_argb || !world || !view || !proj || fs_id < 0 || fs_id > 2) return RAST_INVALID_ARG;
    if ((nverts && (!d_pos || !d_uv)) || (ntris && !d_idx)) return RAST_INVALID_ARG;
    if (fs_id == RAST_FS_TEXTURE && (!d_tex || tex_w < 1 || tex_h < 1)) return RAST_INVALID_ARG;
    if (nverts > kNoAllocMaxVerts || ntris > kNoAllocMaxTris) return RAST_INVALID_ARG;
    const int ts = choose_tile(width, height, msaa, tile, ntris);
    if (!ts) return RAST_INVALID_ARG;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    const uint32_t cs = chunk_size_for(ntris);
    const uint32_t nchunks = (ntris + cs - 1) / cs;
    const uint32_t nvb = (nverts + 255u) / 256u;
    // chunk_size_for never goes below kMinChunk, so the descriptor arrays always hold them
    if (cs < kMinChunk || nchunks > sizeof(g_chunks) / sizeof(g_chunks[0]) ||
        nvb > sizeof(g_vblocks) / sizeof(g_vblocks[0]))
        return RAST_INVALID_ARG;
    FrameDev F{};
    F.width = (uint32_t)width;
    F.height = (uint32_t)height;
    F.msaa = msaa;
    F.ts = ts;
    F.tiles_x = (F.width + ts - 1) / ts;
    F.tiles_y = (F.height + ts - 1) / ts;
    F.ntiles = F.tiles_x * F.tiles_y;
    F.draw_begin = 0;
    F.draw_count = 1;
    F.ntris = ntris;
    F.nchunks = nchunks;
    F.clear_depth = clear_depth;
    F.out = d_argb;
    DrawDev D{};
    D.pos = d_pos;
    D.uv = d_uv;
    D.rgba = d_rgba;
    D.idx = d_idx;
    D.tex = d_tex;
    D.tex_w = d_tex ? (uint32_t)tex_w : 0u;
    D.tex_h = d_tex ? (uint32_t)tex_h : 0u;
    D.nverts = nverts;
    D.ntris = ntris;
    D.fs = fs_id;
    float pv[16];
    mat4_mul(proj, view, pv);
    mat4_mul(pv, world, D.mvp);
    const bool split = raster_edge(ts) < ts;

    unsigned char* base = nullptr;
    {
        // the first call on a device looks the array's address up (before any launch)
        const rast_status s = scratch_for_current_device(&base);
        if (s != RAST_OK) return s;
    }

    // first guess as rast_framebuffer makes it; a frame whose bins or clipped polygons overflow
    // is run again with the measured sizes while they still fit the array (up to three runs,
    // like rast_framebuffer)
    unsigned long long bin_cap = 4ull * ntris + F.ntiles + 1024ull;
    unsigned long long clip_floats = 32ull * ntris + 4096ull;
    for (int attempt = 0; attempt < 3; ++attempt) {
        const Layout L = carve_layout(nverts, ntris, nchunks, nvb, F.ntiles, split, bin_cap, clip_floats);
        if (L.end > kNoAllocScratchBytes) return RAST_INVALID_ARG;
        F.bin_cap = bin_cap;

        // only the state block must start at zero; every other region is written before it is read
        bool ok = cudaMemsetAsync(base + L.state, 0, sizeof(DeviceState), st) == cudaSuccess;
        ok = ok && cudaMemcpyAsync(base + L.frame, &F, sizeof(F), cudaMemcpyHostToDevice, st) == cudaSuccess;
        ok = ok && cudaMemcpyAsync(base + L.draw, &D, sizeof(D), cudaMemcpyHostToDevice, st) == cudaSuccess;
        {
            std::lock_guard<std::mutex> lock(g_desc_mu);
            for (uint32_t k = 0; k < nchunks; ++k) {
                g_chunks[k].draw = 0;
                g_chunks[k].tri_begin = k * cs;
                g_chunks[k].tri_count = (ntris - k * cs) < cs ? (ntris - k * cs) : cs;
                g_chunks[k].row = k;
            }
            for (uint32_t b = 0; b < nvb; ++b) g_vblocks[b] = make_uint2(0u, b * 256u);
            if (nchunks)
                ok = ok && cudaMemcpyAsync(base + L.chunks, g_chunks, sizeof(ChunkDev) * nchunks,
                                           cudaMemcpyHostToDevice, st) == cudaSuccess;
            if (nvb)
                ok = ok && cudaMemcpyAsync(base + L.vblocks, g_vblocks, sizeof(uint2) * nvb,
                                           cudaMemcpyHostToDevice, st) == cudaSuccess;
        }
        if (!ok) {
            cudaGetLastError();
            return RAST_CUDA_ERROR;
        }

        DeviceState* dstate = reinterpret_cast<DeviceState*>(base + L.state);
        LaunchArgs a{};
        a.stream = st;
        a.frames = reinterpret_cast<const FrameDev*>(base + L.frame);
        a.nframes = 1;
        a.draws = reinterpret_cast<const DrawDev*>(base + L.draw);
        a.chunks = reinterpret_cast<const ChunkDev*>(base + L.chunks);
        a.nchunks = nchunks;
        a.vblocks = reinterpret_cast<const uint2*>(base + L.vblocks);
        a.vertex_blocks = nvb;
        a.scan_groups = (F.ntiles + 31) / 32;
        a.max_tiles = F.ntiles;
        a.raster_frames = a.frames;
        a.raster_nframes = 1;
        a.raster_tile_offset = 0;
        a.raster_blocks = F.ntiles;
        a.raster_queue = dstate->queue;
        a.raster_heavy_bits = kDefaultHeavyBits;
        a.scan_order_queue = dstate->queue;
        a.scan_heavy_bits = kDefaultHeavyBits;
        Scratch& S = a.scratch;
        S.vclip = reinterpret_cast<float4*>(base + L.vclip);
        S.vscr = reinterpret_cast<float4*>(base + L.vscr);
        S.vcode = reinterpret_cast<uint16_t*>(base + L.vcode);
        S.tri_rect = reinterpret_cast<unsigned long long*>(base + L.rect);
        S.tri_aux = reinterpret_cast<uint32_t*>(base + L.aux);
        S.counts = reinterpret_cast<uint32_t*>(base + L.counts);
        S.tile_start = reinterpret_cast<uint32_t*>(base + L.tstart);
        S.tile_count = reinterpret_cast<uint32_t*>(base + L.tcount);
        S.tile_order = reinterpret_cast<uint32_t*>(base + L.torder);
        S.bins = reinterpret_cast<uint32_t*>(base + L.bins);
        S.qbins = split ? reinterpret_cast<uint32_t*>(base + L.qbins) : nullptr;
        S.qcount = split ? reinterpret_cast<uint32_t*>(base + L.qcount) : nullptr;
        S.clip_store = reinterpret_cast<float*>(base + L.clip);
        S.clip_cap = clip_floats;
        S.clip_used = &dstate->clip_used;
        S.clip_list = reinterpret_cast<uint32_t*>(base + L.clist);
        S.clip_list_cap = ntris;
        S.clip_n = &dstate->clip_n;
        S.status = &dstate->status;
        S.stats = dstate->stats;
        S.frame_need = reinterpret_cast<unsigned long long*>(base + L.need);
        S.log = nullptr;
        S.log_n = &dstate->log_n;
        S.log_cap = 0;

        cudaError_t err = launch_vertex(a);
        if (err == cudaSuccess) err = launch_bin_count(a);
        if (err == cudaSuccess) err = launch_scans(a);
        if (err == cudaSuccess) err = launch_bin_scatter(a);
        if (err == cudaSuccess) err = launch_raster(a, msaa, ts);
        if (err != cudaSuccess) {
            cudaGetLastError();
            return RAST_CUDA_ERROR;
        }
        DeviceState h{};
        unsigned long long need = 0;
        if (cudaMemcpyAsync(&h, dstate, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(&need, base + L.need, sizeof(need), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            cudaGetLastError();
            return RAST_CUDA_ERROR;
        }
        if (h.status & (ST_BIN_OVERFLOW | ST_CLIP_STORE_OVERFLOW)) {
            if (attempt == 2) return RAST_BIN_OVERFLOW;
            if ((h.status & ST_BIN_OVERFLOW) && need > bin_cap) bin_cap = need + need / 4 + 1024;
            if (h.status & ST_CLIP_STORE_OVERFLOW) clip_floats = h.clip_used + h.clip_used / 4 + 65536;
            continue;
        }
        if (h.status & ST_BAD_INDEX) return RAST_INVALID_ARG;
        if (h.status & ST_CLIP_OVERFLOW) return RAST_CLIP_OVERFLOW;
        if (h.status & ST_TEXTURE_OOB) return RAST_TEXTURE_OOB;
        return RAST_OK;
    }
    return RAST_BIN_OVERFLOW;
}
