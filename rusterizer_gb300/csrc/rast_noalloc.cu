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

    // descriptors, built on the stack
    const uint32_t cs = chunk_size_for(ntris);
    const uint32_t nchunks = (ntris + cs - 1) / cs;
    const uint32_t nvb = (nverts + 255u) / 256u;
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
    F.bin_cap = 4ull * ntris + F.ntiles + 1024ull;
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

    // scratch layout inside g_noalloc_scratch
    Carve c;
    const size_t o_state = c.take(sizeof(DeviceState));
    const size_t o_frame = c.take(sizeof(FrameDev));
    const size_t o_draw = c.take(sizeof(DrawDev));
    const size_t o_chunks = c.take(sizeof(ChunkDev) * (nchunks ? nchunks : 1));
    const size_t o_vblocks = c.take(sizeof(uint2) * (nvb ? nvb : 1));
    const size_t o_vclip = c.take(sizeof(float4) * (size_t)nverts);
    const size_t o_vscr = c.take(sizeof(float4) * (size_t)nverts);
    const size_t o_vcode = c.take(sizeof(uint16_t) * (size_t)nverts);
    const size_t o_rect = c.take(sizeof(unsigned long long) * (size_t)ntris);
    const size_t o_aux = c.take(sizeof(uint32_t) * (size_t)ntris);
    const size_t o_counts = c.take(sizeof(uint32_t) * (size_t)nchunks * F.ntiles);
    const size_t o_tstart = c.take(sizeof(uint32_t) * F.ntiles);
    const size_t o_tcount = c.take(sizeof(uint32_t) * F.ntiles);
    const size_t o_torder = c.take(sizeof(uint32_t) * F.ntiles);
    const size_t o_need = c.take(sizeof(unsigned long long));
    const size_t o_bins = c.take(sizeof(uint32_t) * F.bin_cap);
    // 32-pixel bins are split into quadrant lists for the raster
    const bool split = raster_edge(ts) < ts;
    const size_t o_qbins = c.take(split ? sizeof(uint32_t) * 4ull * F.bin_cap : 0);
    const size_t o_qcount = c.take(split ? sizeof(uint32_t) * 4ull * F.ntiles : 0);
    const size_t clip_floats = 32ull * ntris + 4096ull;
    const size_t o_clip = c.take(sizeof(float) * clip_floats);
    const size_t o_clist = c.take(sizeof(uint32_t) * 3ull * (ntris ? ntris : 1));
    if (c.off > kNoAllocScratchBytes) return RAST_INVALID_ARG;

    unsigned char* base = nullptr;
    rast_status s = scratch_for_current_device(&base);
    if (s != RAST_OK) return s;

    ChunkDev chunks[(kNoAllocMaxTris + 511) / 512];
    for (uint32_t k = 0; k < nchunks; ++k) {
        chunks[k].draw = 0;
        chunks[k].tri_begin = k * cs;
        chunks[k].tri_count = (ntris - k * cs) < cs ? (ntris - k * cs) : cs;
        chunks[k].row = k;
    }
    uint2 vblocks[(kNoAllocMaxVerts + 255) / 256];
    for (uint32_t b = 0; b < nvb; ++b) vblocks[b] = make_uint2(0u, b * 256u);

    // only the state block must start at zero; every other region is written before it is read
    bool ok = cudaMemsetAsync(base + o_state, 0, sizeof(DeviceState), st) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(base + o_frame, &F, sizeof(F), cudaMemcpyHostToDevice, st) == cudaSuccess;
    ok = ok && cudaMemcpyAsync(base + o_draw, &D, sizeof(D), cudaMemcpyHostToDevice, st) == cudaSuccess;
    if (nchunks)
        ok = ok && cudaMemcpyAsync(base + o_chunks, chunks, sizeof(ChunkDev) * nchunks,
                                   cudaMemcpyHostToDevice, st) == cudaSuccess;
    if (nvb)
        ok = ok && cudaMemcpyAsync(base + o_vblocks, vblocks, sizeof(uint2) * nvb,
                                   cudaMemcpyHostToDevice, st) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        return RAST_CUDA_ERROR;
    }

    DeviceState* dstate = reinterpret_cast<DeviceState*>(base + o_state);
    LaunchArgs a{};
    a.stream = st;
    a.frames = reinterpret_cast<const FrameDev*>(base + o_frame);
    a.nframes = 1;
    a.draws = reinterpret_cast<const DrawDev*>(base + o_draw);
    a.chunks = reinterpret_cast<const ChunkDev*>(base + o_chunks);
    a.nchunks = nchunks;
    a.vblocks = reinterpret_cast<const uint2*>(base + o_vblocks);
    a.vertex_blocks = nvb;
    a.scan_groups = (F.ntiles + 31) / 32;
    a.max_tiles = F.ntiles;
    a.raster_frames = a.frames;
    a.raster_nframes = 1;
    a.raster_tile_offset = 0;
    a.raster_blocks = F.ntiles;
    a.raster_queue = dstate->queue;
    Scratch& S = a.scratch;
    S.vclip = reinterpret_cast<float4*>(base + o_vclip);
    S.vscr = reinterpret_cast<float4*>(base + o_vscr);
    S.vcode = reinterpret_cast<uint16_t*>(base + o_vcode);
    S.tri_rect = reinterpret_cast<unsigned long long*>(base + o_rect);
    S.tri_aux = reinterpret_cast<uint32_t*>(base + o_aux);
    S.counts = reinterpret_cast<uint32_t*>(base + o_counts);
    S.tile_start = reinterpret_cast<uint32_t*>(base + o_tstart);
    S.tile_count = reinterpret_cast<uint32_t*>(base + o_tcount);
    S.tile_order = reinterpret_cast<uint32_t*>(base + o_torder);
    S.bins = reinterpret_cast<uint32_t*>(base + o_bins);
    S.qbins = split ? reinterpret_cast<uint32_t*>(base + o_qbins) : nullptr;
    S.qcount = split ? reinterpret_cast<uint32_t*>(base + o_qcount) : nullptr;
    S.clip_store = reinterpret_cast<float*>(base + o_clip);
    S.clip_cap = clip_floats;
    S.clip_used = &dstate->clip_used;
    S.clip_list = reinterpret_cast<uint32_t*>(base + o_clist);
    S.clip_list_cap = ntris;
    S.clip_n = &dstate->clip_n;
    S.status = &dstate->status;
    S.stats = dstate->stats;
    S.frame_need = reinterpret_cast<unsigned long long*>(base + o_need);
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
    if (cudaMemcpyAsync(&h, dstate, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return RAST_CUDA_ERROR;
    }
    if (h.status & (ST_BIN_OVERFLOW | ST_CLIP_STORE_OVERFLOW)) return RAST_BIN_OVERFLOW;
    if (h.status & ST_BAD_INDEX) return RAST_INVALID_ARG;
    if (h.status & ST_CLIP_OVERFLOW) return RAST_CLIP_OVERFLOW;
    if (h.status & ST_TEXTURE_OOB) return RAST_TEXTURE_OOB;
    return RAST_OK;
}
