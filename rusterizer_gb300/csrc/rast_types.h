// rast_types.h - device-side descriptors and scratch layout of the raster pipeline.
//
// One launch sequence renders a list of frames (scenes); each frame holds an ordered list of
// draws. Plain rendering is one frame; the batched and serving paths pass many.
//
// HBM layout (all scratch owned by the context, grown on demand, never per frame):
//   vclip[v]  float4  clip-space position of vertex v (MVP * (x,y,z,1))
//   vscr[v]   float4  (screen x, screen y, screen z, w) after divide + viewport
//   vcode[v]  u16     clip predicates (rast_device.cuh clip_code)
//   tri_rect[t] u64   pixel box of triangle t (x0,y0,x1,y1 inclusive, 16 bits each),
//                     kRectEmpty when culled
//   tri_aux[t]  u32   offset of the clipped polygon in clip_store, kNone when unclipped
//   clip_list[] u32×3 triangles that straddle a clip plane (draw, triangle, chunk row), clipped
//                     afterwards by one warp each (k_clip)
//   counts[frame][chunk][tile] u32  per-chunk tile histograms, then exclusive prefixes
//   tile_start / tile_count [tile]  each tile's bin range
//   bins[]    u32     per-tile lists in submission order: triangle << 5 | clipped << 4 |
//                     mask of the raster quadrants of the bin that its pixel box touches
//   qbins[]   u32     32-pixel bins only: each bin's entries split into its four 16-pixel
//                     quadrants (stable), quadrant q of bin t at 4 * start(t) + q * count(t)
// Per-sample colour and depth never touch HBM: they live in shared memory of the tile CTA.
#pragma once

#include <cstdint>

namespace rast {

constexpr uint32_t kClearColor = 0xFF191919u;  // src/rasterizer/buffers.rs:5
constexpr float kCullEps = 0.000001f;          // src/rasterizer/clipping.rs:12
constexpr int kMaxPoly = 32;                   // clip polygon capacity (a convex clip needs 9)
constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr unsigned long long kRectEmpty = ~0ull;
// bins of one frame: up to kCountBandTiles are counted in one pass over a chunk's triangles
// (a 32 KB shared histogram); larger frames (any 16384 x 16384 frame fits) take one pass per
// band of kCountBandTiles bins, so the automatic bin size avoids them where it can
constexpr int kCountBandTiles = 16384;
constexpr int kMaxTilesPerFrame = 1 << 22;
// Raster tile queue counters per (msaa, tile) launch group: [0] heavy-tile tickets, [1] empty-bin
// tickets, [2] bins with entries, [3] heavy bins, [4] light-tile tickets
constexpr int kQueueSlots = 8;
constexpr int kMaxRasterGroups = 8;
// Bins with at least 2^kDefaultHeavyBits entries are rastered CTA-wide, the others one warp per
// raster tile (rast_set_heavy_tile_entries)
constexpr uint32_t kDefaultHeavyBits = 0;
// bin entries: triangle << 5 | clipped << 4 | mask of the raster quadrants the box touches
constexpr int kEntShift = 5;
constexpr uint32_t kEntClipped = 1u << 4;
constexpr uint32_t kMaxFrameTris = 1u << (32 - kEntShift);

// Edge of the raster tile that one CTA owns for bins of edge ts: 32-pixel bins are rastered as
// four 16-pixel quadrants (more, smaller units balance the persistent raster kernel better).
#ifdef __CUDACC__
__host__ __device__
#endif
constexpr int raster_edge(int ts) { return ts > 16 ? 16 : ts; }

// Triangles per binning chunk (one CTA of the count and scatter kernels; one row of per-tile
// counts): about 900 chunks for large meshes, a multiple of 256 in [256, 8192].
inline uint32_t chunk_size_for(uint32_t ntris) {
    uint32_t c = (ntris + 899u) / 900u;
    c = (c + 255u) & ~255u;
    return c < 256u ? 256u : (c > 8192u ? 8192u : c);
}

enum StatusBits : uint32_t {
    ST_TEXTURE_OOB = 1u << 0,
    ST_BIN_OVERFLOW = 1u << 1,
    ST_CLIP_OVERFLOW = 1u << 2,
    ST_CLIP_STORE_OVERFLOW = 1u << 3,
    ST_LOG_OVERFLOW = 1u << 4,
    ST_BAD_INDEX = 1u << 5,  // a vertex index >= the mesh's vertex count (triangle skipped)
};

enum StatSlots : int {
    STAT_SHADED = 0,
    STAT_FSINV = 1,
    STAT_OOB = 2,
    STAT_CLIP_NEED = 3,
    STAT_COUNT = 4,
};

struct DrawDev {
    const float* pos;      // nverts * 3
    const float* uv;       // nverts * 2
    const float* rgba;     // nverts * 4 or null
    const uint32_t* idx;   // ntris * 3
    const uint32_t* tex;   // texture 0 (RGBA8 packed in u32), may be null unless fs == 0
    uint32_t tex_w, tex_h;
    uint32_t nverts, ntris;
    uint32_t vbase;        // first vertex record of this draw
    uint32_t tbase;        // first triangle index of this draw within its frame
    uint32_t frame;
    int32_t fs;
    float mvp[16];         // (P * V) * W, row-major
};

struct FrameDev {
    uint32_t width, height;
    int32_t msaa;
    int32_t ts;            // tile edge in pixels
    uint32_t tiles_x, tiles_y, ntiles;
    uint32_t draw_begin, draw_count;
    uint32_t ntris;
    uint32_t nchunks;
    uint32_t tile_begin;   // global index of this frame's first tile
    uint32_t group_begin;  // first 32-tile scan group of this frame
    uint32_t rect_base;    // global index of this frame's first triangle in tri_rect/tri_aux
    unsigned long long count_base;  // offset of counts[frame]
    unsigned long long bin_base;    // offset of this frame's bins
    unsigned long long bin_cap;     // bins reserved for this frame
    unsigned long long qbin_base;   // offset of this frame's quadrant lists (32-pixel bins)
    float clear_depth;
    uint32_t* out;         // width * height ARGB (device)
    float* dbg_depth;      // optional [y][x][s]
    uint32_t* dbg_color;
};

struct ChunkDev {
    uint32_t draw;
    uint32_t tri_begin;    // first triangle within the draw
    uint32_t tri_count;
    uint32_t row;          // chunk index within the frame
};

struct Scratch {
    float4* vclip;
    float4* vscr;
    uint16_t* vcode;
    unsigned long long* tri_rect;
    uint32_t* tri_aux;
    uint32_t* counts;
    uint32_t* tile_start;
    uint32_t* tile_count;
    uint32_t* tile_order;               // raster queue: tiles by decreasing entry count
    uint32_t* bins;
    uint32_t* qbins;                    // per 32-pixel bin: its entries split by raster quadrant
    uint32_t* qcount;                   // [4 * tile + quadrant] entries in each quadrant list
    float* clip_store;
    unsigned long long clip_cap;        // floats
    uint32_t* clip_list;                // triangles needing Sutherland-Hodgman: draw, triangle, chunk row
    unsigned long long clip_list_cap;   // entries
    unsigned int* clip_n;
    unsigned long long* clip_used;      // floats allocated this frame
    uint32_t* status;
    unsigned long long* stats;          // StatSlots
    unsigned long long* frame_need;     // per frame: bin entries needed
    uint32_t* log;
    unsigned long long* log_n;
    unsigned long long log_cap;
};

}  // namespace rast
