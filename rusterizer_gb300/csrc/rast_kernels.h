// rast_kernels.h - launch interface between the host runtime and the kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

#include "rast_types.h"

namespace rast {

struct LaunchArgs {
    cudaStream_t stream;
    const DrawDev* draws;
    const FrameDev* frames;
    int nframes;
    const ChunkDev* chunks;
    uint32_t nchunks;
    const uint2* vblocks;  // (draw, first vertex) per 256-vertex block
    uint32_t vertex_blocks;
    uint32_t scan_groups;  // 32-tile groups over all frames
    uint32_t max_tiles;    // largest per-frame tile count
    // a run of one frame: k_scan_tiles builds the raster tile queue into these counters (with
    // this heavy-tile threshold) and the raster launch skips k_tile_order; null otherwise
    unsigned int* scan_order_queue;
    uint32_t scan_heavy_bits;
    // raster launch over one (msaa, tile) group of consecutive frames
    const FrameDev* raster_frames;
    int raster_nframes;
    uint32_t raster_tile_offset;
    uint32_t raster_blocks;        // tiles in the group
    unsigned int* raster_queue;    // the group's kQueueSlots tile-queue counters (zeroed per frame)
    uint32_t raster_heavy_bits;    // bins of >= 2^bits entries are rastered CTA-wide (32: none)
    int raster_ctas_per_sm;        // persistent raster CTAs per SM (0: as many as fit)
    Scratch scratch;
};

cudaError_t launch_vertex(const LaunchArgs& a);
cudaError_t launch_bin_count(const LaunchArgs& a);
cudaError_t launch_scans(const LaunchArgs& a);
cudaError_t launch_bin_scatter(const LaunchArgs& a);
cudaError_t launch_raster(const LaunchArgs& a, int msaa, int ts);
size_t raster_smem(int msaa, int ts);
unsigned long long kernel_launches();

}  // namespace rast

namespace rast {
cudaError_t launch_kat(int op, const void* in, void* out, cudaStream_t stream);
}
