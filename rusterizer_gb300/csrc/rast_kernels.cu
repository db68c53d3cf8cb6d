// rast_kernels.cu - sm_103a kernels of the raster pipeline.
//
//   k_vertex       per vertex: MVP * v, divide, viewport, clip predicates       (HBM-bound)
//   k_bin_count    per chunk of triangles: classify, tile rectangle, per-chunk tile histogram
//                  in shared memory (band by band for frames of more than 16384 bins)
//   k_clip         one warp per triangle that straddles a clip plane: clip, fan boxes, counts
//   k_scan_cols    per tile: exclusive prefix of the histograms over chunks
//   k_scan_tiles   per frame: exclusive prefix over tiles -> bin ranges, capacity check; for a
//                  one-frame run also the raster tile queue
//   k_bin_scatter  per chunk: order-preserving scatter of triangle ids into tile bins
//   k_tile_order   per raster launch of a batch: the raster tile queue, heaviest first
//   k_bin_split    per 32-pixel bin: its entries split into four 16-pixel quadrant lists
//   k_raster<S,TS> per raster tile, a CTA of 4 warps: replays the tile's triangles in
//                  submission order with all colour/depth samples in shared memory; coverage,
//                  depth test, perspective-correct interpolation, fragment shader, resolve
//   k_raster_warp  the same with one warp per raster tile, for light tiles
//                  (rast_raster_warp.cuh)
//
// No kernel waits on another CTA; every loop is bounded by sizes read from descriptors.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <mutex>

#include "rast_device.cuh"
#include "rast_kernels.h"

namespace rast {

// ===================================================================== helpers

__device__ __forceinline__ unsigned long long pack_rect(uint32_t x0, uint32_t y0, uint32_t x1,
                                                        uint32_t y1) {
    return (unsigned long long)x0 | ((unsigned long long)y0 << 16) |
           ((unsigned long long)x1 << 32) | ((unsigned long long)y1 << 48);
}
__device__ __forceinline__ void unpack_rect(unsigned long long r, uint32_t& x0, uint32_t& y0,
                                            uint32_t& x1, uint32_t& y1) {
    x0 = (uint32_t)(r & 0xFFFFu);
    y0 = (uint32_t)((r >> 16) & 0xFFFFu);
    x1 = (uint32_t)((r >> 32) & 0xFFFFu);
    y1 = (uint32_t)((r >> 48) & 0xFFFFu);
}
// Tile rectangle (inclusive) of a pixel box (inclusive) for tiles of edge ts (a power of two).
__device__ __forceinline__ void tile_rect(unsigned long long r, uint32_t ts, uint32_t& x0, uint32_t& y0,
                                          uint32_t& x1, uint32_t& y1) {
    unpack_rect(r, x0, y0, x1, y1);
    const uint32_t sh = __ffs(ts) - 1;
    x0 >>= sh;
    y0 >>= sh;
    x1 >>= sh;
    y1 >>= sh;
}
__device__ __forceinline__ uint32_t rect_tiles(unsigned long long r, uint32_t ts) {
    if (r == kRectEmpty) return 0;
    uint32_t x0, y0, x1, y1;
    tile_rect(r, ts, x0, y0, x1, y1);
    return (x1 - x0 + 1) * (y1 - y0 + 1);
}
// Bin entry of a triangle for tile (tx, ty): triangle << 5 | clipped << 4 | the raster
// quadrants of the tile that the triangle's pixel box r touches (bit sy * nsx + sx; a single
// bit when nsx == 1).
__device__ __forceinline__ uint32_t bin_entry(uint32_t tri, bool clipped, unsigned long long r, uint32_t tx,
                                              uint32_t ty, uint32_t ts) {
    const uint32_t head = (tri << kEntShift) | (clipped ? kEntClipped : 0u);
    const uint32_t rs = (uint32_t)raster_edge((int)ts);
    if (rs == ts) return head | 1u;
    uint32_t px0, py0, px1, py1;
    unpack_rect(r, px0, py0, px1, py1);
    const uint32_t ox = tx * ts, oy = ty * ts, rsh = __ffs(rs) - 1, nsx = ts >> rsh;
    const uint32_t sx0 = (max(px0, ox) - ox) >> rsh, sx1 = (min(px1, ox + ts - 1) - ox) >> rsh;
    const uint32_t sy0 = (max(py0, oy) - oy) >> rsh, sy1 = (min(py1, oy + ts - 1) - oy) >> rsh;
    const uint32_t xm = (2u << sx1) - (1u << sx0);  // quadrant columns sx0 .. sx1
    uint32_t m = 0;
    for (uint32_t sy = sy0; sy <= sy1; ++sy) m |= xm << (sy * nsx);
    return head | m;
}

// Programmatic dependent launch: wait until the grid launched before this one in the stream has
// completed and its memory is visible (a no-op for a normal launch), then let the next grid's
// CTAs be scheduled once every CTA of this one is running. First statement of every pipeline
// kernel, so that no kernel finishes before its predecessor has.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ uint32_t lanemask_lt() { return (1u << lane_id()) - 1u; }

// Block-wide exclusive scan of one u32 per thread (blockDim.x <= 1024). `tmp` holds 33 words.
template <bool kTrailingBarrier = true>
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* tmp, uint32_t& total) {
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) tmp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < nw ? tmp[lane] : 0u;
        uint32_t s = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, o);
            if (lane >= (uint32_t)o) s += y;
        }
        tmp[lane] = s - w;
        if (lane == 31) tmp[32] = s;
    }
    __syncthreads();
    uint32_t r = tmp[warp] + x - v;
    total = tmp[32];
    // without it, the caller must pass a barrier before tmp is written again
    if (kTrailingBarrier) __syncthreads();
    return r;
}

// ===================================================================== vertex stage

__global__ void __launch_bounds__(256) k_vertex(const DrawDev* __restrict__ draws,
                                                const FrameDev* __restrict__ frames,
                                                const uint2* __restrict__ vblocks, Scratch s) {
    pdl_enter();
    __shared__ float m[16];
    const uint2 vb = vblocks[blockIdx.x];
    const DrawDev* d = &draws[vb.x];
    if (threadIdx.x < 16) m[threadIdx.x] = d->mvp[threadIdx.x];
    __syncthreads();
    const uint32_t v = vb.y + threadIdx.x;
    if (v >= d->nverts) return;
    const FrameDev* f = &frames[d->frame];
    const float x = __ldg(d->pos + 3ull * v), y = __ldg(d->pos + 3ull * v + 1),
                z = __ldg(d->pos + 3ull * v + 2);
    // vertex shader P*V*W*v (upstream src/main.rs:147-152) with MVP folded on the host in the
    // same dot order; Mat4 * Vec4 is src/math/vector.rs:219-240
    float4 c = make_float4(dot4(m + 0, x, y, z, 1.0f), dot4(m + 4, x, y, z, 1.0f),
                           dot4(m + 8, x, y, z, 1.0f), dot4(m + 12, x, y, z, 1.0f));
    const uint32_t o = d->vbase + v;
    s.vclip[o] = c;
    s.vscr[o] = to_screen(c, (float)f->width, (float)f->height);
    s.vcode[o] = (uint16_t)clip_code(c);
}

// ===================================================================== triangle classify

// try_clip + divide + viewport + bounding box for one triangle (src/rasterizer/mod.rs:425-441).
// Returns its pixel box (kRectEmpty when nothing can be covered) and, for a clipped
// triangle, the offset of its polygon in the clip store.
__device__ void classify_triangle(const DrawDev& d, const FrameDev& f, uint32_t di, uint32_t tri, uint32_t row,
                                  const Scratch& s, unsigned long long& rect, uint32_t& aux) {
    rect = kRectEmpty;
    aux = kNone;
    const uint32_t i0 = __ldg(d.idx + 3ull * tri), i1 = __ldg(d.idx + 3ull * tri + 1),
                   i2 = __ldg(d.idx + 3ull * tri + 2);
    // primitive_assembly indexes the vertex list (src/render.rs:75-96) and panics past its end;
    // here the triangle is skipped and the frame reports an invalid argument
    if (i0 >= d.nverts || i1 >= d.nverts || i2 >= d.nverts) {
        atomicOr(s.status, ST_BAD_INDEX);
        return;
    }
    const uint32_t v[3] = {d.vbase + i0, d.vbase + i1, d.vbase + i2};
    const float4 c0 = s.vclip[v[0]], c1 = s.vclip[v[1]], c2 = s.vclip[v[2]];
    const int cls = clip_classify(tri2x_area(c0.x, c0.y, c1.x, c1.y, c2.x, c2.y), s.vcode[v[0]],
                                  s.vcode[v[1]], s.vcode[v[2]]);
    if (cls == 0) return;
    uint32_t bx0 = 0xFFFFFFFFu, bx1 = 0, by0 = 0xFFFFFFFFu, by1 = 0;
    if (cls == 1) {
        const float4 sv[3] = {s.vscr[v[0]], s.vscr[v[1]], s.vscr[v[2]]};
        pixel_bbox(sv, f.width, f.height, bx0, bx1, by0, by1);
        if (bx0 >= bx1 || by0 >= by1) return;
    } else {
        // straddles a clip plane: queued for k_clip, which clips it with one warp and adds its
        // tiles to this chunk's counts
        const uint32_t slot = atomicAdd(s.clip_n, 1u);
        if (slot < s.clip_list_cap) {
            uint32_t* L = s.clip_list + 3ull * slot;
            L[0] = di;
            L[1] = tri;
            L[2] = row;
        } else {
            atomicOr(s.status, ST_CLIP_STORE_OVERFLOW);
        }
        return;
    }
    rect = pack_rect(bx0, by0, bx1 - 1, by1 - 1);
}

// Sutherland-Hodgman against the six clip planes in CLIP_PLANES order
// (src/rasterizer/clipping.rs:113-177) with the polygon spread over a warp: lane i holds
// vertex i. Per plane every lane looks at its edge (previous vertex -> its vertex) and emits
// nothing, the intersection, its vertex, or both, in the reference's order; an exclusive scan
// of the emit counts places them. A plane every vertex is inside leaves the polygon as it is.
// Returns the new vertex count, or -1 past 32 vertices. Called by a whole warp.
__device__ __forceinline__ int warp_clip(ClipVert& v, int cn) {
    const uint32_t lane = lane_id();
    for (int plane = 0; plane < 6; ++plane) {
        const bool live = lane < (uint32_t)cn;
        const float dc = live ? distance_measure(plane, v.p) : 0.0f;
        const bool cin = dc >= 0.0f;
        if (__all_sync(0xFFFFFFFFu, !live || cin)) continue;
        const uint32_t prev = live ? (lane + (uint32_t)cn - 1u) % (uint32_t)cn : lane;
        ClipVert pv;
#pragma unroll
        for (int k = 0; k < 4; ++k) pv.p[k] = __shfl_sync(0xFFFFFFFFu, v.p[k], prev);
#pragma unroll
        for (int k = 0; k < 6; ++k) pv.a[k] = __shfl_sync(0xFFFFFFFFu, v.a[k], prev);
        const float dp = __shfl_sync(0xFFFFFFFFu, dc, prev);
        const bool pin = dp >= 0.0f;
        uint32_t emit = 0;
        if (live) emit = (pin && cin) ? 1u : (pin && !cin) ? 1u : (!pin && cin) ? 2u : 0u;
        ClipVert first = v;  // both inside: the vertex itself
        if (live && pin != cin) clip_intersect(pv, dp, v, dc, first);
        uint32_t incl = emit;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
        if (total > (uint32_t)kMaxPoly) return -1;
        // new vertex `lane`: emitted by the lane whose inclusive count first exceeds it
        uint32_t src = 0;
#pragma unroll
        for (int st = 16; st > 0; st >>= 1) {
            const uint32_t c = __shfl_sync(0xFFFFFFFFu, incl, src + st - 1);
            if (c <= lane) src += st;
        }
        src = min(src, 31u);
        const uint32_t second = lane - (__shfl_sync(0xFFFFFFFFu, incl, src) - __shfl_sync(0xFFFFFFFFu, emit, src));
        ClipVert nv;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float a = __shfl_sync(0xFFFFFFFFu, first.p[k], src), b = __shfl_sync(0xFFFFFFFFu, v.p[k], src);
            nv.p[k] = second ? b : a;
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const float a = __shfl_sync(0xFFFFFFFFu, first.a[k], src), b = __shfl_sync(0xFFFFFFFFu, v.a[k], src);
            nv.a[k] = second ? b : a;
        }
        v = nv;
        cn = (int)total;
        if (cn == 0) break;
    }
    return cn;
}

// Clips the queued straddling triangles, one warp per triangle: the polygon goes to the clip
// store in screen space (to_screen per vertex, as the reference divides and maps the fan's
// triangles, src/rasterizer/mod.rs:425-441), the union of the fan's pixel boxes
// (clipping.rs:185-190) becomes the triangle's box, and its tiles are added to its chunk's
// counts. Grid-stride over the queue.
__global__ void __launch_bounds__(256) k_clip(const DrawDev* __restrict__ draws,
                                              const FrameDev* __restrict__ frames, Scratch s) {
    pdl_enter();
    const uint32_t lane = lane_id();
    const uint32_t nq = min(*(volatile unsigned int*)s.clip_n, (unsigned int)s.clip_list_cap);
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < nq; e += nwarps) {
        const uint32_t di = s.clip_list[3ull * e], tri = s.clip_list[3ull * e + 1], row = s.clip_list[3ull * e + 2];
        const DrawDev& d = draws[di];
        const FrameDev& f = frames[d.frame];
        ClipVert v;
        if (lane < 3) {
            const uint32_t vi = __ldg(d.idx + 3ull * tri + lane);
            const float4 c = s.vclip[d.vbase + vi];
            v.p[0] = c.x;
            v.p[1] = c.y;
            v.p[2] = c.z;
            v.p[3] = c.w;
#pragma unroll
            for (int q = 0; q < 4; ++q) v.a[q] = d.rgba ? __ldg(d.rgba + 4ull * vi + q) : 0.0f;
            v.a[4] = __ldg(d.uv + 2ull * vi);
            v.a[5] = __ldg(d.uv + 2ull * vi + 1);
        } else {
#pragma unroll
            for (int k = 0; k < 4; ++k) v.p[k] = 0.0f;
#pragma unroll
            for (int k = 0; k < 6; ++k) v.a[k] = 0.0f;
        }
        const int n = warp_clip(v, 3);
        if (n < 0) {
            if (lane == 0) atomicOr(s.status, ST_CLIP_OVERFLOW);
            continue;
        }
        if (n < 3) continue;
        const unsigned long long need = 1ull + 10ull * (unsigned long long)n;
        unsigned long long off = 0;
        if (lane == 0) off = atomicAdd(s.clip_used, need);
        off = __shfl_sync(0xFFFFFFFFu, off, 0);
        if (off + need > s.clip_cap) {
            if (lane == 0) atomicOr(s.status, ST_CLIP_STORE_OVERFLOW);
            continue;
        }
        float* st = s.clip_store + off;
        const float4 sc = to_screen(make_float4(v.p[0], v.p[1], v.p[2], v.p[3]), (float)f.width, (float)f.height);
        if (lane == 0) st[0] = __int_as_float(n);
        if (lane < (uint32_t)n) {
            float* o = st + 1 + 10 * lane;
            o[0] = sc.x;
            o[1] = sc.y;
            o[2] = sc.z;
            o[3] = sc.w;
#pragma unroll
            for (int q = 0; q < 6; ++q) o[4 + q] = v.a[q];
        }
        // fan triangle `lane`: vertices 0, lane + 1, lane + 2
        float4 tv[3];
        tv[0] = make_float4(__shfl_sync(0xFFFFFFFFu, sc.x, 0), __shfl_sync(0xFFFFFFFFu, sc.y, 0),
                            __shfl_sync(0xFFFFFFFFu, sc.z, 0), __shfl_sync(0xFFFFFFFFu, sc.w, 0));
        const uint32_t l1 = min(lane + 1, 31u), l2 = min(lane + 2, 31u);
        tv[1] = make_float4(__shfl_sync(0xFFFFFFFFu, sc.x, l1), __shfl_sync(0xFFFFFFFFu, sc.y, l1),
                            __shfl_sync(0xFFFFFFFFu, sc.z, l1), __shfl_sync(0xFFFFFFFFu, sc.w, l1));
        tv[2] = make_float4(__shfl_sync(0xFFFFFFFFu, sc.x, l2), __shfl_sync(0xFFFFFFFFu, sc.y, l2),
                            __shfl_sync(0xFFFFFFFFu, sc.z, l2), __shfl_sync(0xFFFFFFFFu, sc.w, l2));
        uint32_t a0 = 0xFFFFFFFFu, a1 = 0, b0 = 0xFFFFFFFFu, b1 = 0;
        if (lane + 2 < (uint32_t)n) {
            uint32_t x0, x1, y0, y1;
            pixel_bbox(tv, f.width, f.height, x0, x1, y0, y1);
            if (x0 < x1 && y0 < y1) {
                a0 = x0;
                a1 = x1;
                b0 = y0;
                b1 = y1;
            }
        }
        a0 = __reduce_min_sync(0xFFFFFFFFu, a0);
        a1 = __reduce_max_sync(0xFFFFFFFFu, a1);
        b0 = __reduce_min_sync(0xFFFFFFFFu, b0);
        b1 = __reduce_max_sync(0xFFFFFFFFu, b1);
        if (a0 >= a1 || b0 >= b1) continue;
        const unsigned long long rect = pack_rect(a0, b0, a1 - 1, b1 - 1);
        const uint32_t g = f.rect_base + d.tbase + tri;
        if (lane == 0) {
            s.tri_rect[g] = rect;
            s.tri_aux[g] = (uint32_t)off;
        }
        uint32_t x0, y0, x1, y1;
        tile_rect(rect, (uint32_t)f.ts, x0, y0, x1, y1);
        const uint32_t w = x1 - x0 + 1, nt = (y1 - y0 + 1) * w;
        uint32_t* crow = s.counts + f.count_base + (unsigned long long)row * f.ntiles;
        for (uint32_t k = lane; k < nt; k += 32) atomicAdd(&crow[(y0 + k / w) * f.tiles_x + x0 + k % w], 1u);
    }
}

// ===================================================================== binning: count

__global__ void __launch_bounds__(256, 8) k_bin_count(const ChunkDev* __restrict__ chunks,
                                                   const DrawDev* __restrict__ draws,
                                                   const FrameDev* __restrict__ frames,
                                                   Scratch s) {
    pdl_enter();
    // per-bin counts of the chunk, two 16-bit counters per word (bin t in half t & 1 of word
    // t / 2): a chunk holds at most 8192 triangles, so no counter carries into its neighbour,
    // and the histogram of kCountBandTiles = 16384 bins takes 32 KB (8 CTAs per SM for the
    // largest frames). Frames with more bins are counted band by band: the first pass
    // classifies the triangles and stores their boxes, later passes read the boxes back and
    // count the bins of their band (rows of the box outside the band are skipped).
    extern __shared__ uint32_t hist[];
    const ChunkDev ch = chunks[blockIdx.x];
    const DrawDev& d = draws[ch.draw];
    const FrameDev& f = frames[d.frame];
    const uint32_t nt = f.ntiles, tx = f.tiles_x;
    uint32_t* row = s.counts + f.count_base + (unsigned long long)ch.row * nt;
    for (uint32_t b0 = 0; b0 < nt; b0 += (uint32_t)kCountBandTiles) {
        const uint32_t b1 = min(nt, b0 + (uint32_t)kCountBandTiles);
        for (uint32_t t = threadIdx.x; t < (b1 - b0 + 1) / 2; t += blockDim.x) hist[t] = 0;
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < ch.tri_count; i += blockDim.x) {
            const uint32_t tri = ch.tri_begin + i;
            const uint32_t g = f.rect_base + d.tbase + tri;
            unsigned long long rect;
            if (b0 == 0) {
                uint32_t aux;
                classify_triangle(d, f, ch.draw, tri, ch.row, s, rect, aux);
                s.tri_rect[g] = rect;
                s.tri_aux[g] = aux;
            } else {
                rect = s.tri_rect[g];  // stored by this thread in the first pass
            }
            if (rect != kRectEmpty) {
                uint32_t x0, y0, x1, y1;
                tile_rect(rect, (uint32_t)f.ts, x0, y0, x1, y1);
                if (nt <= (uint32_t)kCountBandTiles) {  // one band: every bin of the box counts
                    for (uint32_t y = y0; y <= y1; ++y)
                        for (uint32_t x = x0; x <= x1; ++x) {
                            const uint32_t t = y * tx + x;
                            atomicAdd(&hist[t >> 1], (t & 1u) ? 0x10000u : 1u);
                        }
                } else {
                    // rows of the box whose bins can fall in [b0, b1)
                    const uint32_t ya = max(y0, b0 / tx), yb = min(y1, (b1 - 1) / tx);
                    for (uint32_t y = ya; y <= yb; ++y)
                        for (uint32_t x = x0; x <= x1; ++x) {
                            const uint32_t t = y * tx + x;
                            if (t >= b0 && t < b1) atomicAdd(&hist[(t - b0) >> 1], ((t - b0) & 1u) ? 0x10000u : 1u);
                        }
                }
            }
        }
        __syncthreads();
        for (uint32_t t = b0 + threadIdx.x; t < b1; t += blockDim.x)
            row[t] = (hist[(t - b0) >> 1] >> (((t - b0) & 1u) * 16u)) & 0xFFFFu;
        if (b1 < nt) __syncthreads();  // the histogram is cleared again for the next band
    }
}

// ===================================================================== binning: scans

// One block per 32-tile group of a frame; 32 segments of chunks per tile.
__global__ void __launch_bounds__(1024) k_scan_cols(const FrameDev* __restrict__ frames,
                                                    int nframes, Scratch s) {
    pdl_enter();
    __shared__ uint32_t part[32][33];
    __shared__ int s_frame;
    if (threadIdx.x == 0) {
        int lo = 0, hi = nframes;
        while (hi - lo > 1) {
            int mid = (lo + hi) >> 1;
            if (frames[mid].group_begin <= blockIdx.x) lo = mid; else hi = mid;
        }
        s_frame = lo;
    }
    __syncthreads();
    const FrameDev& f = frames[s_frame];
    const uint32_t tl = threadIdx.x & 31u, seg = threadIdx.x >> 5;
    const uint32_t t = (blockIdx.x - f.group_begin) * 32u + tl;
    const uint32_t R = f.nchunks, nt = f.ntiles;
    const uint32_t r0 = (uint32_t)((unsigned long long)R * seg / 32u);
    const uint32_t r1 = (uint32_t)((unsigned long long)R * (seg + 1) / 32u);
    uint32_t* base = s.counts + f.count_base;
    uint32_t sum = 0;
    if (t < nt)
        for (uint32_t r = r0; r < r1; ++r) sum += base[(unsigned long long)r * nt + t];
    part[seg][tl] = sum;
    __syncthreads();
    if (seg == 0) {
        uint32_t run = 0;
        for (int k = 0; k < 32; ++k) {
            uint32_t c = part[k][tl];
            part[k][tl] = run;
            run += c;
        }
        if (t < nt) s.tile_count[f.tile_begin + t] = run;
    }
    __syncthreads();
    if (t < nt) {
        uint32_t run = part[seg][tl];
        for (uint32_t r = r0; r < r1; ++r) {
            uint32_t* p = &base[(unsigned long long)r * nt + t];
            const uint32_t c = *p;
            // the scatter reads a chunk's offset only for bins the chunk has entries in: empty
            // cells keep their 0 (most of the matrix for dense meshes) and are not written
            if (c) *p = run;
            run += c;
        }
    }
}

__device__ void tile_order_block(uint32_t tile0, uint32_t n, const uint32_t* __restrict__ tile_count,
                                 uint32_t* __restrict__ order, unsigned int* __restrict__ queue, bool overflow,
                                 uint32_t heavy_bits, uint32_t* cnt, uint32_t* off);

// One block (1024 threads) per frame: tile_start = exclusive prefix of tile_count, capacity
// check. For a run of one frame (order_queue set) the block also builds the raster tile queue
// (tile_order_block), which saves the separate k_tile_order launch.
__global__ void __launch_bounds__(1024) k_scan_tiles(const FrameDev* __restrict__ frames,
                                                     Scratch s, uint32_t* __restrict__ order,
                                                     unsigned int* __restrict__ order_queue,
                                                     uint32_t heavy_bits) {
    pdl_enter();
    __shared__ uint32_t tmp[33];
    __shared__ uint32_t cnt[33], off[33];
    const FrameDev& f = frames[blockIdx.x];
    const uint32_t nt = f.ntiles;
    const uint32_t per = (nt + blockDim.x - 1) / blockDim.x;
    const uint32_t a = threadIdx.x * per, b = min(nt, a + per);
    uint32_t loc = 0;
    for (uint32_t t = a; t < b; ++t) loc += s.tile_count[f.tile_begin + t];
    uint32_t total;
    uint32_t run = block_excl_scan(loc, tmp, total);
    for (uint32_t t = a; t < b; ++t) {
        uint32_t c = s.tile_count[f.tile_begin + t];
        s.tile_start[f.tile_begin + t] = run;
        run += c;
    }
    if (threadIdx.x == 0) {
        s.frame_need[blockIdx.x] = total;
        if ((unsigned long long)total > f.bin_cap) atomicOr(s.status, ST_BIN_OVERFLOW);
    }
    if (order_queue) {
        __syncthreads();  // every tile_count read above is done before the queue is built
        tile_order_block(f.tile_begin, nt, s.tile_count, order, order_queue,
                         (unsigned long long)total > f.bin_cap, heavy_bits, cnt, off);
    }
}

// ===================================================================== binning: scatter

constexpr int kScatterThreads = 256;
constexpr int kScatterWarps = kScatterThreads / 32;
constexpr int kScatterTriPerThread = 2;
constexpr int kScatterWindow = kScatterThreads * kScatterTriPerThread;  // triangles per batch
constexpr int kPairsPerBatch = 512;  // (triangle, tile) pairs ranked per batch
constexpr uint32_t kBigTri = 32;     // triangles over more tiles are binned alone, tile-parallel
constexpr int kHashSlots = 1024;     // open-addressing table over tile ids, load <= 0.5
constexpr uint32_t kHashEmpty = 0xFFFFFFFFu;
constexpr unsigned long long kRectClippedBit = 1ull << 63;  // pixel boxes stay below 2^15

__device__ __forceinline__ uint32_t hash_slot(uint32_t t) {
    return (t * 2654435761u) >> (32 - 10);
}

// Bins the (triangle, tile) pairs of a chunk in submission order. Per batch of up to
// kScatterWindow triangles (two consecutive ones per thread, so each warp holds a contiguous
// run) and kPairsPerBatch pairs, every warp walks its pairs 32 at a time: lanes with the same
// tile (match_any) take consecutive ranks from the warp's counter for that tile (wcnt, found
// through a small hash of the batch's tiles). A pair's position is then the tile's running
// offset + the counts of the earlier warps + its rank in its warp. A triangle over more than
// kBigTri tiles ends a batch and is binned alone, tile-parallel.
__global__ void __launch_bounds__(kScatterThreads) k_bin_scatter(
    const ChunkDev* __restrict__ chunks, const DrawDev* __restrict__ draws,
    const FrameDev* __restrict__ frames, Scratch s) {
    pdl_enter();
    __shared__ uint32_t hkey[kHashSlots];
    __shared__ uint16_t wcnt[kHashSlots][kScatterWarps];
    __shared__ uint16_t slot_list[kPairsPerBatch];
    __shared__ uint32_t pxy[kPairsPerBatch];  // tile x | tile y << 16
    __shared__ uint16_t pslot[kPairsPerBatch], prank[kPairsPerBatch];
    __shared__ uint16_t ptri[kPairsPerBatch];
    __shared__ unsigned long long trect[kScatterWindow];  // pixel box, bit 63: clipped
    __shared__ uint32_t sbase[kHashSlots];  // per slot: the tile's position before the batch
    __shared__ uint32_t nslots, take_s, npairs_s;
    __shared__ uint32_t tmp[33];
    if (*(volatile uint32_t*)s.status & ST_BIN_OVERFLOW) return;
    const ChunkDev ch = chunks[blockIdx.x];
    const DrawDev& d = draws[ch.draw];
    const FrameDev& f = frames[d.frame];
    const uint32_t nt = f.ntiles, tx = f.tiles_x, ts = (uint32_t)f.ts;
    // the chunk's row of scanned counts: its offset within each tile's list, advanced in place
    // as the chunk's entries are placed (the row is the chunk's own and dead after this
    // kernel); the chunk's next position in tile t is tile_start[t] + crow[t]
    uint32_t* crow = s.counts + f.count_base + (unsigned long long)ch.row * nt;
    const uint32_t* tstart = s.tile_start + f.tile_begin;
    for (uint32_t h = threadIdx.x; h < (uint32_t)kHashSlots; h += blockDim.x) {
        hkey[h] = kHashEmpty;
#pragma unroll
        for (int w = 0; w < kScatterWarps; ++w) wcnt[h][w] = 0;
    }
    if (threadIdx.x == 0) nslots = 0;
    __syncthreads();
    uint32_t* bins = s.bins + f.bin_base;
    const unsigned long long cap = f.bin_cap;
    const uint32_t gbase = f.rect_base + d.tbase + ch.tri_begin;
    const uint32_t fbase = d.tbase + ch.tri_begin;  // frame triangle index of the chunk's first
    const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
    uint32_t base = 0;
    while (base < ch.tri_count) {
        // ---- this thread's two triangles: pixel boxes, clipped flags, tile counts
        unsigned long long r[kScatterTriPerThread];
        uint32_t n[kScatterTriPerThread];
        uint32_t mine = 0;
#pragma unroll
        for (int j = 0; j < kScatterTriPerThread; ++j) {
            const uint32_t v = threadIdx.x * kScatterTriPerThread + j;
            const uint32_t i = base + v;
            const bool live = i < ch.tri_count;
            r[j] = live ? s.tri_rect[gbase + i] : kRectEmpty;
            const bool clipped = live && r[j] != kRectEmpty && s.tri_aux[gbase + i] != kNone;
            n[j] = rect_tiles(r[j], ts);
            trect[v] = clipped ? (r[j] | kRectClippedBit) : r[j];
            mine += n[j];
        }
        if (threadIdx.x == 0) take_s = kScatterWindow;
        uint32_t total;
        const uint32_t excl = block_excl_scan(mine, tmp, total);  // its barriers order take_s
        // the batch: a prefix of the window within the pair budget
        {
            uint32_t run = excl;
#pragma unroll
            for (int j = 0; j < kScatterTriPerThread; ++j) {
                const uint32_t v = threadIdx.x * kScatterTriPerThread + j;
                run += n[j];
                if (run > (uint32_t)kPairsPerBatch || n[j] > kBigTri) {
                    atomicMin(&take_s, v);
                    break;
                }
            }
        }
        __syncthreads();
        uint32_t take = take_s;
        if (take == 0) {
            // a single triangle over more than kBigTri tiles: its tiles are distinct, each
            // takes the next position
            const bool c0 = (trect[0] & kRectClippedBit) != 0;
            const unsigned long long r0 = trect[0] & ~kRectClippedBit;
            uint32_t x0, y0, x1, y1;
            tile_rect(r0, ts, x0, y0, x1, y1);
            const uint32_t w = x1 - x0 + 1, n0 = rect_tiles(r0, ts);
            for (uint32_t k = threadIdx.x; k < n0; k += blockDim.x) {
                const uint32_t ttx = x0 + k % w, tty = y0 + k / w;
                const uint32_t t = tty * tx + ttx;
                const uint32_t pos = tstart[t] + crow[t];
                if (pos < cap) bins[pos] = bin_entry(fbase + base, c0, r0, ttx, tty, ts);
                crow[t] += 1;
            }
            __syncthreads();
            base += 1;
            continue;
        }
        take = min(take, ch.tri_count - base);
        // ---- per warp, its pairs in order, 32 at a time: rank within the warp per tile
        uint32_t pc = 0;  // this thread's pairs in the batch
#pragma unroll
        for (int j = 0; j < kScatterTriPerThread; ++j)
            if (threadIdx.x * kScatterTriPerThread + j < take) pc += n[j];
        uint32_t winc = pc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, winc, o);
            if (lane >= (uint32_t)o) winc += y;
        }
        const uint32_t wtotal = __shfl_sync(0xFFFFFFFFu, winc, 31);
        const uint32_t wbase = __shfl_sync(0xFFFFFFFFu, excl, 0);  // block index of the warp's first pair
        for (uint32_t rb = 0; rb < wtotal; rb += 32) {
            const uint32_t pi = rb + lane;
            uint32_t sl = 0;
#pragma unroll
            for (int st = 16; st > 0; st >>= 1) {
                const uint32_t v = __shfl_sync(0xFFFFFFFFu, winc, sl + st - 1);
                if (v <= pi) sl += st;
            }
            const uint32_t src = min(sl, 31u);
            const uint32_t o = pi - __shfl_sync(0xFFFFFFFFu, winc - pc, src);
            const uint32_t n0 = __shfl_sync(0xFFFFFFFFu, n[0], src);
            uint32_t key = 0xFFFFFFFFu - lane, v = 0, xy = 0;
            if (pi < wtotal) {
                const uint32_t j = o < n0 ? 0u : 1u, k = o < n0 ? o : o - n0;
                v = (warp * 32 + src) * kScatterTriPerThread + j;
                uint32_t x0, y0, x1, y1;
                tile_rect(trect[v] & ~kRectClippedBit, ts, x0, y0, x1, y1);
                const uint32_t w = x1 - x0 + 1;
                const uint32_t ky = k < w ? 0u : k / w;
                const uint32_t ttx = x0 + (k - ky * w), tty = y0 + ky;
                key = tty * tx + ttx;
                xy = ttx | (tty << 16);
            }
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
            const uint32_t leader = __ffs(peers) - 1;
            uint32_t slot = 0, old = 0;
            if (pi < wtotal && lane == leader) {
                uint32_t h = hash_slot(key);
                while (true) {
                    const uint32_t prev = atomicCAS(&hkey[h], kHashEmpty, key);
                    if (prev == kHashEmpty) {
                        slot_list[atomicAdd(&nslots, 1u)] = (uint16_t)h;
                        break;
                    }
                    if (prev == key) break;
                    h = (h + 1) & (kHashSlots - 1);
                }
                slot = h;
                old = wcnt[h][warp];
                wcnt[h][warp] = (uint16_t)(old + __popc(peers));
            }
            slot = __shfl_sync(0xFFFFFFFFu, slot, leader);
            old = __shfl_sync(0xFFFFFFFFu, old, leader);
            if (pi < wtotal) {
                const uint32_t bp = wbase + pi;
                pxy[bp] = xy;
                pslot[bp] = (uint16_t)slot;
                prank[bp] = (uint16_t)(old + __popc(peers & lanemask_lt()));
                ptri[bp] = (uint16_t)v;
            }
        }
        {
            const uint32_t t_last = take - 1;  // its thread holds the end of the batch's pairs
            if (threadIdx.x == t_last / kScatterTriPerThread) {
                uint32_t e = excl;
#pragma unroll
                for (int j = 0; j < kScatterTriPerThread; ++j)
                    if (threadIdx.x * kScatterTriPerThread + j < take) e += n[j];
                npairs_s = e;
            }
        }
        __syncthreads();
        // ---- per tile of the batch: its position before the batch, the warps' counts turned
        // into exclusive prefixes, and the chunk's offset advanced past the batch
        const uint32_t ns = nslots, npairs = npairs_s;
        for (uint32_t j = threadIdx.x; j < ns; j += blockDim.x) {
            const uint32_t h = slot_list[j], t = hkey[h];
            const uint32_t c = crow[t];
            const uint32_t b = tstart[t] + c;
            uint32_t tot = 0;
#pragma unroll
            for (int w2 = 0; w2 < kScatterWarps; ++w2) {
                const uint32_t c = wcnt[h][w2];
                wcnt[h][w2] = (uint16_t)tot;
                tot += c;
            }
            sbase[h] = b;
            crow[t] = c + tot;
        }
        __syncthreads();
        // ---- positions: the tile's position + earlier warps' counts + rank in the warp
        for (uint32_t bp = threadIdx.x; bp < npairs; bp += blockDim.x) {
            const uint32_t xy = pxy[bp], slot = pslot[bp], v = ptri[bp];
            const uint32_t pw = v / (32 * kScatterTriPerThread);
            const uint32_t pos = sbase[slot] + wcnt[slot][pw] + prank[bp];
            const unsigned long long rv = trect[v];
            const bool clipped = (rv & kRectClippedBit) != 0;
            if (pos < cap)
                bins[pos] = bin_entry(fbase + base + v, clipped, rv & ~kRectClippedBit, xy & 0xFFFFu, xy >> 16, ts);
        }
        __syncthreads();
        for (uint32_t j = threadIdx.x; j < ns; j += blockDim.x) {
            const uint32_t h = slot_list[j];
#pragma unroll
            for (int w2 = 0; w2 < kScatterWarps; ++w2) wcnt[h][w2] = 0;
            hkey[h] = kHashEmpty;
        }
        if (threadIdx.x == 0) nslots = 0;
        __syncthreads();
        base += take;
    }
}

// ===================================================================== raster

constexpr int kRasterThreads = 128;
constexpr int kRasterWarps = kRasterThreads / 32;
constexpr int kRasterCtasPerSm = 7;  // occupancy the launch bounds aim at (shared memory allows 7)
constexpr int kEmptyRun = 8;  // bins without entries taken per queue update
constexpr uint32_t kTrimMin = 4;  // shortest box line that line_span trims

// A raster CTA owns one TS x TS tile: a whole bin (bin edge == TS) or one quadrant of a bin
// twice as wide. Bin entries carry, in their low 4 bits, the quadrants the triangle's pixel box
// touches, so a quadrant CTA skips the other entries without loading them.
template <int S, int TS>
struct RasterCfg {
    static constexpr int NPIX = TS * TS;
    static constexpr int IC = kRasterThreads;  // items (triangles after clipping) per batch
    static constexpr int QC = 64;              // per-warp fragment ring
    static_assert(TS <= 16 && IC <= 256, "ring entries hold item and pixel in one byte each");
    static constexpr int LINES = (TS + kRasterWarps - 1) / kRasterWarps;  // lines of a tile per warp
    static_assert(LINES <= 4, "an item meets a warp on at most four lines of a tile");
};

template <int S, int TS>
struct RasterSmem {
    using C = RasterCfg<S, TS>;
    float zb[C::NPIX * S];     // sample-major: sample k of pixel p at k * NPIX + p
    uint32_t cb[C::NPIX * S];
    // items of the current batch (struct of arrays)
    float ipx[3][C::IC], ipy[3][C::IC], iz[3][C::IC], iw[3][C::IC], iinv[C::IC];
    float iuv[6][C::IC];  // texture coordinates (u, v) of the three corners
    uint32_t irect[C::IC];  // tile-local pixel box: x0 | y0 << 8 | x1 << 16 | y1 << 24
    uint32_t itri[C::IC];
    uint32_t imeta[C::IC];  // draw << 8 | sub-triangle
    uint32_t member[kRasterWarps][C::IC / 32];  // bit: item overlaps the warp's rows/columns
    uint16_t wlist[kRasterWarps][C::IC];         // the warp's items, in submission order
    // per-warp rings of covered fragments, in submission order
    float qz[kRasterWarps][S][C::QC];
    uint8_t qitem[kRasterWarps][C::QC];
    uint8_t qpix[kRasterWarps][C::QC];
    uint8_t qcov[kRasterWarps][C::QC];
    // per-warp rings of depth-passed fragments waiting for the fragment shader, in order
    float sz0[kRasterWarps][C::QC];
    uint8_t sitem[kRasterWarps][C::QC];
    uint8_t spix[kRasterWarps][C::QC];
    uint8_t sdm[kRasterWarps][C::QC];
    float inv255[256];
    int rowd[TS + 1], cold[TS + 1];  // candidate work of the batch, difference arrays
    uint32_t tmp[40];
    uint32_t misc[8];  // [0] tile ticket, [1] items staged, [2..4] statistics
    uint32_t zmaxw[kRasterWarps];  // per warp: largest stored depth of its share of the tile

};

template <int S, int TS>
size_t raster_smem_bytes() { return sizeof(RasterSmem<S, TS>); }

__device__ __forceinline__ uint32_t find_draw(const DrawDev* __restrict__ draws,
                                              const FrameDev& f, uint32_t g) {
    uint32_t lo = f.draw_begin, hi = f.draw_begin + f.draw_count;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (draws[mid].tbase <= g) lo = mid; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ uint32_t frame_of_tile(const FrameDev* __restrict__ frames, int nframes,
                                                  uint32_t gt) {
    int lo = 0, hi = nframes;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (frames[mid].tile_begin <= gt) lo = mid; else hi = mid;
    }
    return (uint32_t)lo;
}

// Inward edge normal k of an item (RasterizerTriangle::new, src/rasterizer/mod.rs:199-204),
// recomputed from the stored points with the same two subtractions.
template <typename SM>
__device__ __forceinline__ void item_normal(const SM& sm, uint32_t it, int k, float& nx,
                                            float& ny) {
    const int n = k == 2 ? 0 : k + 1;
    const float vx = sm.ipx[n][it] - sm.ipx[k][it];
    const float vy = sm.ipy[n][it] - sm.ipy[k][it];
    nx = -vy;
    ny = vx;
}

// Room added to edge k's value at a pixel centre so that it bounds the computed edge value at
// every sample of the pixel: s_k + m_k, derived at line_span.
template <int S>
__device__ __forceinline__ float edge_room(float nx, float ny, float Px, float Py) {
    const float sk = S == 1 ? 0.0f : 0.125f * fmaxf(fabsf(nx - 3.0f * ny), fabsf(3.0f * nx + ny));
    return sk + 1e-6f * (fabsf(nx) * (fabsf(Px) + 16400.0f) + fabsf(ny) * (fabsf(Py) + 16400.0f)) + 1e-37f;
}

// The pixels of one line of an item's box that can hold a covered sample: line lc (a tile-local
// row in mode 0, a column in mode 1), candidates [a0, a1) along it, trimmed in place. A pixel is
// dropped only where some edge k is negative at every sample with room to spare: with E_k the
// edge function in exact arithmetic over the stored f32 normal and point, the computed
// edge_eval value differs from E_k by at most 3 * 2^-24 * (|nx| |x - Px| + |ny| |y - Py|)
// (two subtractions, two products and one sum, each correctly rounded; the leading 0 + is
// exact). E_k is linear, so over the pixel's samples it is at most E_k(centre) + s_k, s_k the
// largest of nx ox + ny oy over the sample offsets (ox, oy) from the centre: for the 4-sample
// pattern (1/8, -3/8), (3/8, 1/8) and their negatives, s_k = max(|nx - 3 ny|, |3 nx + ny|) / 8;
// 0 for the single centre sample. So E_k(centre) + s_k + m_k < 0, m_k = 1e-6 (|nx| (|Px| +
// 16400) + |ny| (|Py| + 16400)) + 1e-37, makes every sample's computed value negative, and the
// edge test fails whatever the tie rule (screen coordinates stay below 16400; m_k also covers
// the f32 rounding of s_k and of the line offset below). Along the line the bound is linear in
// the pixel index, so the pixels that keep it are an interval [ceil(t), ...) or (..., t]; t is
// computed in f32 to within 0.03 pixel whenever it falls near the tile (|pal - gk / nal| below
// 2^16; farther out only its sign matters), and the interval is widened by 1/8 pixel.
// Non-finite points are not trimmed.
template <int S, int TS>
__device__ __forceinline__ void line_span_pts(const float px[3], const float py[3], uint32_t mode, uint32_t lc,
                                              uint32_t X0, uint32_t Y0, uint32_t& a0, uint32_t& a1) {
    bool finite = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) finite = finite && isfinite(px[k]) && isfinite(py[k]);
    if (!finite) return;
    // line centre across, and the pixel-centre origin along the line (global coordinates)
    const float cacross = (float)((mode == 0 ? Y0 : X0) + lc) + 0.5f;
    const float oalong = (float)(mode == 0 ? X0 : Y0) + 0.5f;
    int lo = (int)a0, hi = (int)a1;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int n = k == 2 ? 0 : k + 1;
        const float nx = -(py[n] - py[k]), ny = px[n] - px[k];
        const float R = edge_room<S>(nx, ny, px[k], py[k]);
        const float nal = mode == 0 ? nx : ny, nac = mode == 0 ? ny : nx;
        const float pal = mode == 0 ? px[k] : py[k], pac = mode == 0 ? py[k] : px[k];
        const float gk = nac * (cacross - pac) + R;  // E_k + R = nal * (c_along - pal) + gk
        if (fabsf(nal) <= 1e-20f) {
            // (almost) constant along the line
            if (gk + fabsf(nal) * (fabsf(pal) + 16400.0f) < 0.0f) hi = lo;
            continue;
        }
        // E_k + R >= 0  <=>  nal * (oalong + x - pal) >= -gk
        const float t = pal - __fdividef(gk, nal) - oalong;  // 2-ulp division is enough
        if (!isfinite(t)) continue;
        const float tc = fminf(fmaxf(t, -8.0f), (float)TS + 8.0f);
        if (nal > 0.0f) lo = max(lo, (int)ceilf(tc - 0.125f));
        else hi = min(hi, (int)floorf(tc + 0.125f) + 1);
    }
    if (hi < lo) hi = lo;
    a0 = (uint32_t)lo;
    a1 = (uint32_t)hi;
}

// line_span of item `it` of a shared-memory item batch.
template <int S, int TS, typename SM>
__device__ __forceinline__ void line_span(const SM& sm, uint32_t it, uint32_t mode, uint32_t lc,
                                          uint32_t X0, uint32_t Y0, uint32_t& a0, uint32_t& a1) {
    const float px[3] = {sm.ipx[0][it], sm.ipx[1][it], sm.ipx[2][it]};
    const float py[3] = {sm.ipy[0][it], sm.ipy[1][it], sm.ipy[2][it]};
    line_span_pts<S, TS>(px, py, mode, lc, X0, Y0, a0, a1);
}

// Order-preserving map of floats to unsigned integers (NaN above +inf) and back.
__device__ __forceinline__ uint32_t float_to_ordered(float x) {
    const uint32_t b = __float_as_uint(x);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ordered_to_float(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// True when no sample of the triangle with screen depths z0..z2 can pass the strict depth
// test against a tile whose stored depths are all <= ztile. A sample depth is (b0 z0 + b1 z1)
// + b2 z2 with clamped b0, b1 in [0, 1] and b2 = clamp((1 - b0) - b1): a convex combination,
// or with b2 = 0 a combination with b0 + b1 >= 1, so for depths >= 0 it is at least
// min(z0, z1, z2) up to the rounding of the products and sums (well below 2^-20 relative).
// Never true with a negative or NaN corner depth or a NaN ztile.
__device__ __forceinline__ bool depth_cull(float z0, float z1, float z2, float ztile) {
    const float zmin = fminf(fminf(z0, z1), z2);
    const bool ok = z0 >= 0.0f && z1 >= 0.0f && z2 >= 0.0f;  // false for NaN
    return ok && zmin * (1.0f - 0x1p-20f) >= ztile;
}

// Stages the items of one bin entry (one triangle, or the fan of its clipped polygon) at
// positions first.. of the batch: screen points, depths, w, attributes, 1 / 2x area and the
// tile-local pixel box, and adds the box to the batch's row and column work.
template <int S, int TS>
__device__ __forceinline__ void stage_entry(RasterSmem<S, TS>& sm, const FrameDev& f,
                                            const DrawDev* __restrict__ draws, const Scratch& s,
                                            uint32_t g, uint32_t aux, uint32_t nitems, uint32_t first,
                                            uint32_t X0, uint32_t Y0, float ztile) {
    const uint32_t di = find_draw(draws, f, g);
    const DrawDev& d = draws[di];
    const int fs = d.fs;
    for (uint32_t k = 0; k < nitems; ++k) {
        const uint32_t it = first + k;
        float4 sv[3];
        float uv[3][2] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
        if (aux == kNone) {
            const uint32_t tri = g - d.tbase;
            const uint32_t ii[3] = {__ldg(d.idx + 3ull * tri), __ldg(d.idx + 3ull * tri + 1),
                                    __ldg(d.idx + 3ull * tri + 2)};
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                sv[q] = s.vscr[d.vbase + ii[q]];
                if (fs == 0) {
                    uv[q][0] = __ldg(d.uv + 2ull * ii[q]);
                    uv[q][1] = __ldg(d.uv + 2ull * ii[q] + 1);
                }
            }
        } else {
            const float* st = s.clip_store + aux + 1;
            const uint32_t vi[3] = {0u, k + 1, k + 2};
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const float* o = st + 10 * vi[q];
                sv[q] = make_float4(o[0], o[1], o[2], o[3]);
                uv[q][0] = o[8];
                uv[q][1] = o[9];
            }
        }
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            sm.ipx[q][it] = sv[q].x;
            sm.ipy[q][it] = sv[q].y;
            sm.iz[q][it] = sv[q].z;
            sm.iw[q][it] = sv[q].w;
            sm.iuv[2 * q][it] = uv[q][0];
            sm.iuv[2 * q + 1][it] = uv[q][1];
        }
        // 1 / triangle_2x_area (RasterizerTriangle::new, src/rasterizer/mod.rs:206)
        sm.iinv[it] = 1.0f / tri2x_area(sv[0].x, sv[0].y, sv[1].x, sv[1].y, sv[2].x, sv[2].y);
        uint32_t bx0, bx1, by0, by1;
        pixel_bbox(sv, f.width, f.height, bx0, bx1, by0, by1);
        const uint32_t cx0 = max(bx0, X0), cx1 = min(bx1, X0 + TS);
        const uint32_t cy0 = max(by0, Y0), cy1 = min(by1, Y0 + TS);
        // hidden: no sample depth can get below the largest depth stored in the tile
        // (depth_cull), so the strict depth test (mod.rs:363-378) fails everywhere
        const bool nonempty = bx0 < bx1 && by0 < by1 && cx0 < cx1 && cy0 < cy1 &&
                              !depth_cull(sv[0].z, sv[1].z, sv[2].z, ztile);
        uint32_t r = 0;
        if (nonempty) {
            const uint32_t lx0 = cx0 - X0, ly0 = cy0 - Y0, lx1 = cx1 - X0, ly1 = cy1 - Y0;
            r = lx0 | (ly0 << 8) | (lx1 << 16) | (ly1 << 24);
            const int cw = (int)(lx1 - lx0), chh = (int)(ly1 - ly0);
            atomicAdd(&sm.rowd[ly0], cw);
            atomicAdd(&sm.rowd[ly1], -cw);
            atomicAdd(&sm.cold[lx0], chh);
            atomicAdd(&sm.cold[lx1], -chh);
        }
        sm.irect[it] = r;
        sm.itri[it] = g;
        sm.imeta[it] = (di << 8) | k;
    }
}

// Chooses how the tile's pixels are divided among the warps for one batch: interleaved rows
// (row r to warp r % kRasterWarps; suits scattered triangles) or interleaved columns (suits
// runs of small triangles along a screen row, which crowd into a few rows), whichever gives
// the lighter heaviest warp by candidate-pixel work. Either way each warp owns its pixels for
// the batch, which keeps every pixel's fragments in one warp and in submission order, and an
// item meets each warp on at most TS / kRasterWarps lines. Returns 0 for rows, 1 for columns.
// Called by one warp.
template <int TS>
__device__ __forceinline__ uint32_t split_work(const int* rowd, const int* cold) {
    const uint32_t lane = lane_id();
    // per-line work from the difference arrays (lane = line)
    int rw = lane < (uint32_t)TS ? rowd[lane] : 0, cw = lane < (uint32_t)TS ? cold[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xFFFFFFFFu, rw, o), z = __shfl_up_sync(0xFFFFFFFFu, cw, o);
        if (lane >= (uint32_t)o) {
            rw += y;
            cw += z;
        }
    }
    uint32_t wr = lane < (uint32_t)TS ? (uint32_t)rw : 0u;
    uint32_t wc = lane < (uint32_t)TS ? (uint32_t)cw : 0u;
    // each warp's load: the sum of its lines (lane % kRasterWarps), then the heaviest warp
#pragma unroll
    for (int o = kRasterWarps; o < 32; o <<= 1) {
        wr += __shfl_down_sync(0xFFFFFFFFu, wr, o);
        wc += __shfl_down_sync(0xFFFFFFFFu, wc, o);
    }
#pragma unroll
    for (int o = kRasterWarps / 2; o > 0; o >>= 1) {
        wr = max(wr, __shfl_xor_sync(0xFFFFFFFFu, wr, o));
        wc = max(wc, __shfl_xor_sync(0xFFFFFFFFu, wc, o));
    }
    return wc < wr ? 1u : 0u;  // lane 0's values cover lanes 0 .. kRasterWarps - 1
}

// Appends one fragment record to the debug log (rast_debug_log_enable); kept out of line.
__device__ __noinline__ void log_fragment(const Scratch& s, uint32_t tri, uint32_t sub, uint32_t yx,
                                          uint32_t masks) {
    const unsigned long long slot = atomicAdd(s.log_n, 1ull);
    if (slot < s.log_cap) {
        uint32_t* L = s.log + 4ull * slot;
        L[0] = tri;
        L[1] = sub;
        L[2] = yx;
        L[3] = masks;
    } else {
        atomicOr(s.status, ST_LOG_OVERFLOW);
    }
}

// FS::Color's input for an item: the vertex colours of its three corners (Color vertex
// attribute, src/graphics_primitives.rs:9-13), from the mesh or from the clipped polygon.
__device__ __noinline__ void item_colours(const DrawDev& d, const FrameDev& f, const Scratch& s, uint32_t g,
                                          uint32_t k, float col[3][4]) {
    const uint32_t aux = s.tri_aux[f.rect_base + g];
    if (aux == kNone) {
        const uint32_t tri = g - d.tbase;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const uint32_t vi = __ldg(d.idx + 3ull * tri + q);
#pragma unroll
            for (int c = 0; c < 4; ++c) col[q][c] = d.rgba ? __ldg(d.rgba + 4ull * vi + c) : 0.0f;
        }
    } else {
        const float* st = s.clip_store + aux + 1;
        const uint32_t vi[3] = {0u, k + 1, k + 2};
#pragma unroll
        for (int q = 0; q < 3; ++q)
#pragma unroll
            for (int c = 0; c < 4; ++c) col[q][c] = st[10 * vi[q] + 4 + c];
    }
}

// Depth test of up to 32 queued fragments of one warp (lane = one fragment, queue order =
// submission order). Fragments of the same pixel run in rounds of increasing rank, so the
// depth test (depth_coverage, src/rasterizer/mod.rs:363-378) happens in submission order.
// Fragments with samples that passed go, in the same order, to the warp's shade ring.
template <int S, int TS>
__device__ __forceinline__ void warp_depth(RasterSmem<S, TS>& sm, uint32_t w, uint32_t head, uint32_t n,
                                           uint32_t& stail, const Scratch& s, uint32_t X0, uint32_t Y0,
                                           uint32_t& shaded, uint32_t& fsinv) {
    using C = RasterCfg<S, TS>;
    const uint32_t lane = lane_id();
    const bool valid = lane < n;
    const uint32_t q = (head + lane) & (C::QC - 1);
    uint32_t it = 0, pix = 0, cov = 0;
    float z[S];
#pragma unroll
    for (int k = 0; k < S; ++k) z[k] = 0.0f;
    if (valid) {
        it = sm.qitem[w][q];
        pix = sm.qpix[w][q];
        cov = sm.qcov[w][q];
#pragma unroll
        for (int k = 0; k < S; ++k) z[k] = sm.qz[w][k][q];
    }
    const uint32_t key = valid ? pix : 0x10000u + lane;
    const uint32_t grp = __match_any_sync(0xFFFFFFFFu, key);
    const uint32_t rank = __popc(grp & lanemask_lt());
    const uint32_t maxr = __reduce_max_sync(0xFFFFFFFFu, rank);
    uint32_t dm = 0;
    for (uint32_t r = 0; r <= maxr; ++r) {
        // this round's lanes: no two share a pixel; the test and the store are predicated
        const bool act = valid && rank == r;
#pragma unroll
        for (int k = 0; k < S; ++k) {
            const float old = sm.zb[k * C::NPIX + pix];
            const bool pass = act & (((cov >> k) & 1u) != 0) & (z[k] < old);
            if (pass) sm.zb[k * C::NPIX + pix] = z[k];
            dm |= (uint32_t)pass << k;
        }
        if (s.log && act)
            log_fragment(s, sm.itri[it], sm.imeta[it] & 0xFFu, ((Y0 + pix / TS) << 16) | (X0 + pix % TS),
                         (dm << 8) | cov);
        __syncwarp();
    }
    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, dm != 0);
    if (dm) {
        const uint32_t sq = (stail + __popc(bal & lanemask_lt())) & (C::QC - 1);
        sm.sitem[w][sq] = (uint8_t)it;
        sm.spix[w][sq] = (uint8_t)pix;
        sm.sdm[w][sq] = (uint8_t)dm;
        sm.sz0[w][sq] = z[0];
        shaded += __popc(dm);
        fsinv += 1;
    }
    stail += __popc(bal);
    __syncwarp();
}

// Fragment shader and colour write of up to 32 fragments of the warp's shade ring (kept out of
// line: the coverage loop that calls it stays small enough for the instruction cache):
// Fragment::interpolate (src/rasterizer/mod.rs:69-100) at the point its depth-passed mask
// selects, the draw's shader by id, then write_pixel (mod.rs:380-397) to the passed samples,
// same-pixel fragments in rounds of increasing rank (submission order).
template <int S, int TS>
__device__ __noinline__ void warp_shade(RasterSmem<S, TS>& sm, uint32_t w, uint32_t head, uint32_t n,
                                           const DrawDev* __restrict__ draws, const FrameDev& f,
                                           const Scratch& s, uint32_t X0, uint32_t Y0, uint32_t& oobc) {
    using C = RasterCfg<S, TS>;
    const uint32_t lane = lane_id();
    const bool valid = lane < n;
    const uint32_t q = (head + lane) & (C::QC - 1);
    uint32_t argb = 0, pix = 0, dm = 0;
    if (valid) {
        const uint32_t it = sm.sitem[w][q];
        pix = sm.spix[w][q];
        dm = sm.sdm[w][q];
        const uint32_t x = X0 + pix % TS, y = Y0 + pix / TS;
        float xs, ys;
        interp_point<S>(x, y, dm, xs, ys);
        float e[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            float nx, ny;
            item_normal(sm, it, k, nx, ny);
            e[k] = edge_eval(nx, ny, sm.ipx[k][it], sm.ipy[k][it], xs, ys);
        }
        float u, v, ww;
        persp_bary(e[0], e[1], e[2], sm.iw[0][it], sm.iw[1][it], sm.iw[2][it], u, v, ww);
        const DrawDev& d = draws[sm.imeta[it] >> 8];
        float col[4];
        if (d.fs == 0) {
            // FS::Texture (upstream src/main.rs:214-216)
            const float tu = sm.iuv[0][it] * u + sm.iuv[2][it] * v + sm.iuv[4][it] * ww;
            const float tv = sm.iuv[1][it] * u + sm.iuv[3][it] * v + sm.iuv[5][it] * ww;
            bool oob = false;
            tex_sample(d.tex, d.tex_w, d.tex_h, tu, tv, sm.inv255, col, oob);
            if (oob) ++oobc;
        } else if (d.fs == 1) {
            // FS::Color (upstream src/main.rs:217)
            float vc[3][4];
            item_colours(d, f, s, sm.itri[it], sm.imeta[it] & 0xFFu, vc);
#pragma unroll
            for (int c = 0; c < 4; ++c) col[c] = vc[0][c] * u + vc[1][c] * v + vc[2][c] * ww;
        } else {
            // FS::Debug (upstream src/main.rs:218-220): grayscale(frag_coords.depths[0])
            const float z0 = sm.sz0[w][q];
            col[0] = z0;
            col[1] = z0;
            col[2] = z0;
            col[3] = 1.0f;
        }
        argb = to_argb(col[0], col[1], col[2], col[3]);
    }
    const uint32_t key = valid ? pix : 0x10000u + lane;
    const uint32_t grp = __match_any_sync(0xFFFFFFFFu, key);
    const uint32_t rank = __popc(grp & lanemask_lt());
    const uint32_t maxr = __reduce_max_sync(0xFFFFFFFFu, rank);
    for (uint32_t r = 0; r <= maxr; ++r) {
        const bool act = valid && rank == r;
#pragma unroll
        for (int k = 0; k < S; ++k)
            if (act & (((dm >> k) & 1u) != 0)) sm.cb[k * C::NPIX + pix] = argb;
        __syncwarp();
    }
}

// Writes the clear colour (and, when captured, clear samples) over one tile of a frame.
__device__ __forceinline__ void clear_tile_warp(const FrameDev& f, uint32_t x0, uint32_t y0,
                                                uint32_t edge, int S) {
    const uint32_t lane = lane_id();
    if (!f.dbg_depth && (f.width & 3u) == 0 && x0 + edge <= f.width &&
        (reinterpret_cast<uintptr_t>(f.out) & 15u) == 0) {
        // whole rows of 16-byte stores: the image starts on a 16-byte boundary (checked; batch
        // outputs can start anywhere), width % 4 == 0 and x0 is a multiple of the bin edge, so
        // every row segment does too
        const uint32_t q = edge / 4, sh = __ffs(q) - 1;  // uint4 per row (2, 4 or 8), its log2
        const uint4 c = make_uint4(kClearColor, kClearColor, kClearColor, kClearColor);
        for (uint32_t i = lane; i < edge * q; i += 32) {
            const uint32_t y = y0 + (i >> sh);
            if (y >= f.height) break;
            uint4* row = reinterpret_cast<uint4*>(f.out + (unsigned long long)y * f.width + x0);
            row[i & (q - 1)] = c;
        }
        return;
    }
    for (uint32_t i = lane; i < edge * edge; i += 32) {
        const uint32_t x = x0 + i % edge, y = y0 + i / edge;
        if (x >= f.width || y >= f.height) continue;
        const unsigned long long o = (unsigned long long)y * f.width + x;
        f.out[o] = kClearColor;
        if (f.dbg_depth) {
            for (int q = 0; q < S; ++q) {
                f.dbg_depth[o * S + q] = f.clear_depth;
                f.dbg_color[o * S + q] = kClearColor;
            }
        }
    }
}

// Persistent raster kernel for the heavy tiles. Units are (bin, quadrant) pairs of the first
// queue[3] bins of the raster queue (the bins with the most entries; the others go one warp per
// tile to k_raster_warp), taken heaviest bin first from queue[0]; per unit the CTA replays the
// bin in submission order in batches of up to IC items: stage the items (A), split the tile's rows or columns over the warps by work
// (B), then each warp walks the candidate pixels of its items inside its range — coverage
// (EdgeFunctions::eval, mod.rs:134-146) and sample depths (RasterizerTriangle::fragment,
// mod.rs:225-253) — and depth-tests, shades and writes the covered fragments in order (C).
// Bins without entries are then cleared by single warps from queue[1].
template <int S, int TS>
__global__ void __launch_bounds__(kRasterThreads, kRasterCtasPerSm) k_raster(const FrameDev* __restrict__ frames,
                                                           int nframes,
                                                           const uint32_t* __restrict__ order,
                                                           uint32_t ntotal, uint32_t nsx,
                                                           unsigned int* __restrict__ queue,
                                                           const DrawDev* __restrict__ draws,
                                                           Scratch s) {
    pdl_enter();
    using C = RasterCfg<S, TS>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    RasterSmem<S, TS>& sm = *reinterpret_cast<RasterSmem<S, TS>*>(smem_raw);
    const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
    for (uint32_t b = threadIdx.x; b < 256u; b += blockDim.x) sm.inv255[b] = (float)b / 255.0f;
    uint32_t shaded = 0, fsinv = 0, oobc = 0;
    const uint32_t nbusy = *(volatile unsigned int*)&queue[2];  // written by k_tile_order
    const uint32_t nheavy = *(volatile unsigned int*)&queue[3];  // the first nheavy bins of the queue
    const uint32_t nsub = nsx * nsx;

    // unit tickets (heaviest first); the next one is taken when the current unit starts its
    // resolve, so the queue update is in flight during the resolve
    if (threadIdx.x == 0) sm.misc[0] = atomicAdd(&queue[0], 1u);
    for (;;) {
    __syncthreads();
    // misc[0] is written again only after this unit's resolve, many barriers later
    const uint32_t qi = sm.misc[0];
    if (qi >= nheavy * nsub) break;
    const uint32_t gt = order[qi / nsub], sub = qi % nsub;
    const FrameDev& f = frames[frame_of_tile(frames, nframes, gt)];
    const uint32_t lt = gt - f.tile_begin;
    const uint32_t X0 = (lt % f.tiles_x) * (uint32_t)f.ts + (sub % nsx) * TS;
    const uint32_t Y0 = (lt / f.tiles_x) * (uint32_t)f.ts + (sub / nsx) * TS;
    const uint32_t W = f.width, H = f.height;
    for (uint32_t i = threadIdx.x; i < (uint32_t)(C::NPIX * S); i += blockDim.x) {
        sm.zb[i] = f.clear_depth;
        sm.cb[i] = kClearColor;
    }
    // the bin's entries, or for a quadrant of a 32-pixel bin its own split list
    uint32_t nent;
    const uint32_t* bins;
    if (nsub > 1) {
        nent = s.qcount[4ull * gt + sub];
        bins = s.qbins + f.qbin_base + 4ull * s.tile_start[gt] + (unsigned long long)sub * s.tile_count[gt];
    } else {
        nent = s.tile_count[gt];
        bins = s.bins + f.bin_base + s.tile_start[gt];
    }
    const uint32_t mybit = 1u << sub;

    uint32_t pos = 0;  // next entry of the bin
    while (pos < nent) {
        // ---- A. fill a batch with the items of the next entries that touch this tile
        if (threadIdx.x <= (uint32_t)TS) {
            sm.rowd[threadIdx.x] = 0;
            sm.cold[threadIdx.x] = 0;
        }
        // largest depth stored in the tile before this batch, for depth_cull: the clear depth
        // for the unit's first batch; else reduced here and combined after the scan's barriers.
        // NaN (no culling) while the fragment log records depth-failed fragments too.
        float zt = s.log ? __int_as_float(0x7FC00000) : f.clear_depth;
        bool zt_ready = s.log || pos == 0;
        if (!zt_ready) {
            uint32_t zm = 0;
            for (uint32_t i = threadIdx.x; i < (uint32_t)(C::NPIX * S); i += blockDim.x)
                zm = max(zm, float_to_ordered(sm.zb[i]));
            zm = __reduce_max_sync(0xFFFFFFFFu, zm);
            if (lane == 0) sm.zmaxw[warp] = zm;
        }
        uint32_t nit = 0;
        while (pos < nent) {
            const uint32_t e = pos + threadIdx.x;
            uint32_t g = 0, aux = kNone, nitems = 0;
            if (e < nent) {
                const uint32_t ent = bins[e];
                if (ent & mybit) {
                    g = ent >> kEntShift;
                    nitems = 1;
                    if (ent & kEntClipped) {
                        aux = s.tri_aux[f.rect_base + g];
                        nitems = (uint32_t)__float_as_int(s.clip_store[aux]) - 2u;
                    }
                }
            }
            if (threadIdx.x == 0) sm.misc[1] = nit;
            uint32_t itot;
            // the __syncthreads_count below orders the reads of tmp before its next use
            const uint32_t iex = block_excl_scan<false>(nitems, sm.tmp, itot);
            // entries fit while the running item count stays within the batch (a prefix)
            const bool part = (e < nent) && (nit + iex + nitems <= (uint32_t)C::IC);
            const uint32_t take = __syncthreads_count(part);
            if (part && threadIdx.x == take - 1) sm.misc[1] = nit + iex + nitems;
            if (part && nitems) {
                if (!zt_ready) {
                    uint32_t zm = sm.zmaxw[0];
#pragma unroll
                    for (int w = 1; w < kRasterWarps; ++w) zm = max(zm, sm.zmaxw[w]);
                    zt = ordered_to_float(zm);
                    zt_ready = true;
                }
                stage_entry<S, TS>(sm, f, draws, s, g, aux, nitems, nit + iex, X0, Y0, zt);
            }
            __syncthreads();
            nit = sm.misc[1];
            const uint32_t window = min(nent - pos, (uint32_t)kRasterThreads);
            pos += take;
            if (take < window) break;  // the batch is full
        }
        // ---- B. divide the tile's pixels among the warps (every warp computes the same
        // choice from the batch's work histograms: no barrier to wait for one warp's);
        // which warps each item reaches
        const uint32_t mode = __shfl_sync(0xFFFFFFFFu, split_work<TS>(sm.rowd, sm.cold), 0);
        {
            const uint32_t t = threadIdx.x;
            uint32_t wm = 0;
            if (t < nit) {
                const uint32_t r = sm.irect[t];
                // the warps of lines a0 .. a1 - 1 (rows, or columns in column mode)
                const uint32_t a0 = mode ? (r & 0xFFu) : ((r >> 8) & 0xFFu);
                const uint32_t a1 = mode ? ((r >> 16) & 0xFFu) : (r >> 24);
                if (a1 > a0) {
                    const uint32_t nl = a1 - a0;
                    wm = nl >= (uint32_t)kRasterWarps ? (1u << kRasterWarps) - 1u
                                                      : (((1u << nl) - 1u) << (a0 % kRasterWarps));
                    wm = (wm | (wm >> kRasterWarps)) & ((1u << kRasterWarps) - 1u);
                }
            }
#pragma unroll
            for (int w = 0; w < kRasterWarps; ++w) {
                const uint32_t bal = __ballot_sync(0xFFFFFFFFu, (wm >> w) & 1u);
                if (lane == 0) sm.member[w][warp] = bal;
            }
        }
        __syncthreads();
        // ---- C. per warp, in submission order: the candidate pixels of its items on its
        // lines (each line trimmed to the pixels that can hold a covered sample, line_span);
        // coverage (EdgeFunctions::eval, mod.rs:134-146) and
        // sample depths (RasterizerTriangle::fragment, mod.rs:225-253) of each; then ordered
        // depth test and shading of the covered fragments
        uint32_t nmine = 0;
#pragma unroll
        for (int src = 0; src < C::IC / 32; ++src) {
            const uint32_t bits = sm.member[warp][src];
            if ((bits >> lane) & 1u) sm.wlist[warp][nmine + __popc(bits & lanemask_lt())] = (uint16_t)(src * 32 + lane);
            nmine += __popc(bits);
        }
        __syncwarp();
        uint32_t head = 0, tail = 0, shead = 0, stail = 0;
        for (uint32_t gb = 0; gb < nmine; gb += 32) {
            const bool act = gb + lane < nmine;
            const uint32_t it_l = act ? sm.wlist[warp][gb + lane] : 0u;
            // candidates of the lane's item: its lines owned by this warp (rows, or columns in
            // column mode: first, first + kRasterWarps, ... up to C::LINES of them), each
            // trimmed by line_span; geo = first line | start 1 << 5 | length 1 << 10 |
            // start 2 << 15 | length 2 << 20 | start 3 << 25, geo2 = length 3 | start 4 << 5
            // (the fourth length is what remains of the count)
            uint32_t c = 0, geo = 0, geo2 = 0;
            if (act) {
                const uint32_t r = sm.irect[it_l];
                const uint32_t lx0 = r & 0xFFu, ly0 = (r >> 8) & 0xFFu, lx1 = (r >> 16) & 0xFFu, ly1 = r >> 24;
                const uint32_t l0 = mode ? lx0 : ly0, l1 = mode ? lx1 : ly1;  // lines
                const uint32_t b0 = mode ? ly0 : lx0, b1 = mode ? ly1 : lx1;  // along each line
                const uint32_t first = l0 + ((warp + kRasterWarps - (l0 % kRasterWarps)) % kRasterWarps);
                const uint32_t nlines = first < l1 ? (l1 - first + kRasterWarps - 1) / kRasterWarps : 0u;
                uint32_t sa[4] = {b0, b0, b0, b0}, ea[4] = {b1, b1, b1, b1};
                // lines shorter than kTrimMin pixels are cheaper to test whole than to trim
                const uint32_t ntrim = b1 - b0 >= kTrimMin ? nlines : 0u;
#pragma unroll 1
                for (uint32_t ln = 0; ln < ntrim; ++ln) {
                    uint32_t a0 = b0, a1 = b1;
                    line_span<S, TS>(sm, it_l, mode, first + ln * kRasterWarps, X0, Y0, a0, a1);
                    // selects, not an indexed store (the arrays stay in registers)
#pragma unroll
                    for (uint32_t q = 0; q < (uint32_t)C::LINES; ++q) {
                        sa[q] = ln == q ? a0 : sa[q];
                        ea[q] = ln == q ? a1 : ea[q];
                    }
                }
                uint32_t w[4];
#pragma unroll
                for (uint32_t q = 0; q < 4; ++q) w[q] = nlines > q ? ea[q] - sa[q] : 0u;
                c = w[0] + w[1] + w[2] + w[3];
                geo = first | (sa[0] << 5) | (w[0] << 10) | (sa[1] << 15) | (w[1] << 20) | (sa[2] << 25);
                geo2 = w[2] | (sa[3] << 5);
            }
            uint32_t incl = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
                if (lane >= (uint32_t)o) incl += y;
            }
            const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
            for (uint32_t pb = 0; pb < total; pb += 32) {
                const uint32_t p = pb + lane;
                // source lane: number of lanes whose inclusive count is <= p
                uint32_t j = 0;
#pragma unroll
                for (int st = 16; st > 0; st >>= 1) {
                    const uint32_t v = __shfl_sync(0xFFFFFFFFu, incl, j + st - 1);
                    if (v <= p) j += st;
                }
                const uint32_t sj = min(j, 31u);
                const uint32_t it = __shfl_sync(0xFFFFFFFFu, it_l, sj);
                const uint32_t exc = __shfl_sync(0xFFFFFFFFu, incl - c, sj);
                const uint32_t gg = __shfl_sync(0xFFFFFFFFu, geo, sj);
                const uint32_t gg2 = C::LINES > 2 ? __shfl_sync(0xFFFFFFFFu, geo2, sj) : 0u;
                uint32_t cov = 0, pix = 0;
                float z[S];
#pragma unroll
                for (int k = 0; k < S; ++k) z[k] = 0.0f;
                if (p < total) {
                    const uint32_t rr = p - exc;
                    // which of the item's lines: cumulative lengths c1 <= c2 <= c3
                    const uint32_t c1 = (gg >> 10) & 31u, c2 = c1 + ((gg >> 20) & 31u), c3 = c2 + (gg2 & 31u);
                    uint32_t k = (uint32_t)(rr >= c1);
                    uint32_t start = k ? (gg >> 15) & 31u : (gg >> 5) & 31u, base = k ? c1 : 0u;
                    if (C::LINES > 2) {
                        start = rr >= c2 ? (rr >= c3 ? (gg2 >> 5) & 31u : gg >> 25) : start;
                        base = rr >= c2 ? (rr >= c3 ? c3 : c2) : base;
                        k += (uint32_t)(rr >= c2) + (uint32_t)(rr >= c3);
                    }
                    const uint32_t along = start + (rr - base);
                    const uint32_t line = (gg & 31u) + k * (uint32_t)kRasterWarps;
                    const uint32_t lx = mode ? line : along, ly = mode ? along : line;
                    pix = ly * TS + lx;
                    const float fx = (float)(X0 + lx), fy = (float)(Y0 + ly);
                    float n0x, n0y, n1x, n1y, n2x, n2y;
                    item_normal(sm, it, 0, n0x, n0y);
                    item_normal(sm, it, 1, n1x, n1y);
                    item_normal(sm, it, 2, n2x, n2y);
                    const float p0x = sm.ipx[0][it], p0y = sm.ipy[0][it];
                    const float p1x = sm.ipx[1][it], p1y = sm.ipy[1][it];
                    const float p2x = sm.ipx[2][it], p2y = sm.ipy[2][it];
                    // tie rule per edge (EdgeFunctions::inside, mod.rs:148-170), once per pixel
                    const bool t0 = edge_tie(n0x, n0y), t1 = edge_tie(n1x, n1y), t2 = edge_tie(n2x, n2y);
                    const float inv = sm.iinv[it];
                    const float z0 = sm.iz[0][it], z1 = sm.iz[1][it], z2 = sm.iz[2][it];
#pragma unroll
                    for (int k = 0; k < S; ++k) {
                        const float xs = fx + sample_dx<S>(k), ys = fy + sample_dy<S>(k);
                        const float e0 = edge_eval_test(n0x, n0y, p0x, p0y, xs, ys);
                        const float e1 = edge_eval_test(n1x, n1y, p1x, p1y, xs, ys);
                        const float e2 = edge_eval_test(n2x, n2y, p2x, p2y, xs, ys);
                        // branch-free: every sample's depth is computed, the covered ones kept
                        const bool in = edge_pass_t(e0, t0) & edge_pass_t(e1, t1) & edge_pass_t(e2, t2);
                        const float zk = interp_depth_fast(e1, e2, inv, z0, z1, z2);
                        cov |= (uint32_t)in << k;
                        z[k] = in ? zk : 0.0f;
                    }
                }
                const uint32_t bal = __ballot_sync(0xFFFFFFFFu, cov != 0);
                if (cov) {
                    const uint32_t q = (tail + __popc(bal & lanemask_lt())) & (C::QC - 1);
                    sm.qitem[warp][q] = (uint8_t)it;
                    sm.qpix[warp][q] = (uint8_t)pix;
                    sm.qcov[warp][q] = (uint8_t)cov;
#pragma unroll
                    for (int k = 0; k < S; ++k) sm.qz[warp][k][q] = z[k];
                }
                tail += __popc(bal);
                __syncwarp();
                if (tail - head >= 32) {
                    warp_depth<S, TS>(sm, warp, head, 32, stail, s, X0, Y0, shaded, fsinv);
                    head += 32;
                    if (stail - shead >= 32) {
                        warp_shade<S, TS>(sm, warp, shead, 32, draws, f, s, X0, Y0, oobc);
                        shead += 32;
                    }
                }
            }
        }
        if (tail != head) warp_depth<S, TS>(sm, warp, head, tail - head, stail, s, X0, Y0, shaded, fsinv);
        while (stail != shead) {
            const uint32_t nsh = min(stail - shead, 32u);
            warp_shade<S, TS>(sm, warp, shead, nsh, draws, f, s, X0, Y0, oobc);
            shead += nsh;
        }
        __syncthreads();
    }

    // ---- resolve (resolve_and_clear + box_filter_color, mod.rs:478-518, buffers.rs:111-125)
    __syncthreads();
    uint32_t next_ticket = 0;
    if (threadIdx.x == 0) next_ticket = atomicAdd(&queue[0], 1u);
    for (uint32_t p = threadIdx.x; p < (uint32_t)C::NPIX; p += blockDim.x) {
        const uint32_t x = X0 + p % TS, y = Y0 + p / TS;
        if (x >= W || y >= H) continue;
        const unsigned long long o = (unsigned long long)y * W + x;
        uint32_t smp[S];
#pragma unroll
        for (int q = 0; q < S; ++q) smp[q] = sm.cb[q * C::NPIX + p];
        f.out[o] = box_filter<S>(smp);
        if (f.dbg_depth) {
#pragma unroll
            for (int q = 0; q < S; ++q) {
                f.dbg_depth[o * S + q] = sm.zb[q * C::NPIX + p];
                f.dbg_color[o * S + q] = sm.cb[q * C::NPIX + p];
            }
        }
    }
    if (threadIdx.x == 0) sm.misc[0] = next_ticket;
    }  // units with entries

    // ---- bins without entries: warps take runs of kEmptyRun bins (one counter update per run,
    // not per bin) and write the clear colour
    for (;;) {
        uint32_t q0 = 0;
        if (lane == 0) q0 = atomicAdd(&queue[1], (unsigned)kEmptyRun);
        q0 = __shfl_sync(0xFFFFFFFFu, q0, 0) + nbusy;
        if (q0 >= ntotal) break;
        const uint32_t q1 = min(q0 + (uint32_t)kEmptyRun, ntotal);
        for (uint32_t qi = q0; qi < q1; ++qi) {
            const uint32_t gt = order[qi];
            const FrameDev& f = frames[frame_of_tile(frames, nframes, gt)];
            const uint32_t lt = gt - f.tile_begin;
            const uint32_t edge = (uint32_t)f.ts;
            clear_tile_warp(f, (lt % f.tiles_x) * edge, (lt / f.tiles_x) * edge, edge, S);
        }
    }
    // per-block statistics
    __syncthreads();
    if (threadIdx.x == 0) {
        sm.misc[2] = 0;
        sm.misc[3] = 0;
        sm.misc[4] = 0;
    }
    __syncthreads();
    if (shaded) atomicAdd(&sm.misc[2], shaded);
    if (fsinv) atomicAdd(&sm.misc[3], fsinv);
    if (oobc) atomicAdd(&sm.misc[4], oobc);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (sm.misc[2]) atomicAdd(&s.stats[STAT_SHADED], (unsigned long long)sm.misc[2]);
        if (sm.misc[3]) atomicAdd(&s.stats[STAT_FSINV], (unsigned long long)sm.misc[3]);
        if (sm.misc[4]) {
            atomicAdd(&s.stats[STAT_OOB], (unsigned long long)sm.misc[4]);
            atomicOr(s.status, ST_TEXTURE_OOB);
        }
    }
}

#include "rast_raster_warp.cuh"

// Splits each 32-pixel bin with entries into its four quadrant lists, keeping submission
// order within each (an entry goes to every quadrant its mask names). Persistent CTAs walk the
// bins with entries in the raster queue's order (k_tile_order runs first); the quadrant raster
// CTAs then read only their own entries. Windows of 4 consecutive entries per thread; the
// per-quadrant counts travel as 16-bit fields (two quadrants per word) through one block scan.
__global__ void __launch_bounds__(256) k_bin_split(const FrameDev* __restrict__ frames, int nframes,
                                                   const uint32_t* __restrict__ order,
                                                   const unsigned int* __restrict__ queue, Scratch s) {
    pdl_enter();
    constexpr int kPer = 4;
    __shared__ uint32_t tmp[2][33];
    __shared__ uint32_t base[4];
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const uint32_t nbusy = *(volatile const unsigned int*)&queue[2];
    for (uint32_t qi = blockIdx.x; qi < nbusy; qi += gridDim.x) {
        const uint32_t gt = order[qi];
        const uint32_t n = s.tile_count[gt];
        const FrameDev& f = frames[frame_of_tile(frames, nframes, gt)];
        const unsigned long long start = s.tile_start[gt];
        const uint32_t* src = s.bins + f.bin_base + start;
        uint32_t* dst = s.qbins + f.qbin_base + 4ull * start;
        if (threadIdx.x < 4) base[threadIdx.x] = 0;
        for (uint32_t e0 = 0; e0 < n; e0 += blockDim.x * kPer) {
            uint32_t ent[kPer];
            uint32_t c01 = 0, c23 = 0;  // this thread's count per quadrant, 16 bits each
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                const uint32_t e = e0 + threadIdx.x * kPer + j;
                ent[j] = e < n ? src[e] : 0u;
                c01 += (ent[j] & 1u) + (((ent[j] >> 1) & 1u) << 16);
                c23 += ((ent[j] >> 2) & 1u) + (((ent[j] >> 3) & 1u) << 16);
            }
            // block-wide exclusive scan of both words at once
            uint32_t x01 = c01, x23 = c23;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y01 = __shfl_up_sync(0xFFFFFFFFu, x01, o), y23 = __shfl_up_sync(0xFFFFFFFFu, x23, o);
                if (lane >= (uint32_t)o) {
                    x01 += y01;
                    x23 += y23;
                }
            }
            if (lane == 31) {
                tmp[0][warp] = x01;
                tmp[1][warp] = x23;
            }
            __syncthreads();
            if (warp == 0) {
                const uint32_t w01 = lane < nw ? tmp[0][lane] : 0u, w23 = lane < nw ? tmp[1][lane] : 0u;
                uint32_t s01 = w01, s23 = w23;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t y01 = __shfl_up_sync(0xFFFFFFFFu, s01, o), y23 = __shfl_up_sync(0xFFFFFFFFu, s23, o);
                    if (lane >= (uint32_t)o) {
                        s01 += y01;
                        s23 += y23;
                    }
                }
                tmp[0][lane] = s01 - w01;
                tmp[1][lane] = s23 - w23;
                if (lane == 31) {
                    tmp[0][32] = s01;
                    tmp[1][32] = s23;
                }
            }
            __syncthreads();
            const uint32_t p01 = tmp[0][warp] + x01 - c01, p23 = tmp[1][warp] + x23 - c23;
            uint32_t o[4] = {base[0] + (p01 & 0xFFFFu), base[1] + (p01 >> 16), base[2] + (p23 & 0xFFFFu),
                             base[3] + (p23 >> 16)};
#pragma unroll
            for (int j = 0; j < kPer; ++j)
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if ((ent[j] >> q) & 1u) dst[(unsigned long long)q * n + o[q]++] = ent[j];
            __syncthreads();
            if (threadIdx.x < 4) {
                const uint32_t t = tmp[threadIdx.x >> 1][32];
                base[threadIdx.x] += (threadIdx.x & 1u) ? (t >> 16) : (t & 0xFFFFu);
            }
            __syncthreads();
        }
        if (threadIdx.x < 4) s.qcount[4ull * gt + threadIdx.x] = base[threadIdx.x];
        __syncthreads();
    }
}

// Tile queue of one raster launch (block-wide, 1024 threads): tiles with entries first, in
// decreasing order of entry count (bucketed by bit length), then tiles without entries;
// queue[2] = tiles with entries, queue[3] = the leading tiles with at least 2^heavy_bits entries
// (rastered CTA-wide by k_raster; the rest one warp per tile by k_raster_warp). After a bin
// overflow every tile counts as empty (each is cleared and the host re-runs the frame).
__device__ void tile_order_block(uint32_t tile0, uint32_t n, const uint32_t* __restrict__ tile_count,
                                 uint32_t* __restrict__ order, unsigned int* __restrict__ queue, bool overflow,
                                 uint32_t heavy_bits, uint32_t* cnt, uint32_t* off) {
    if (threadIdx.x < 33) cnt[threadIdx.x] = 0;
    __syncthreads();
    // lanes with the same bucket add once per warp (thousands of tiles share a few buckets)
    for (uint32_t i0 = 0; i0 < n; i0 += blockDim.x) {
        const uint32_t i = i0 + threadIdx.x;
        const uint32_t b = i < n ? 32 - __clz(overflow ? 0u : tile_count[tile0 + i]) : 33u;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, b);
        if (b < 33u && lane_id() == (uint32_t)(__ffs(peers) - 1)) atomicAdd(&cnt[b], (uint32_t)__popc(peers));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0, heavy = 0;
        for (int b = 32; b >= 0; --b) {
            off[b] = run;
            run += cnt[b];
            // bins of at least 2^heavy_bits entries (bit length above heavy_bits), never empty ones
            if (b > (int)heavy_bits && b > 0) heavy += cnt[b];
        }
        queue[2] = n - cnt[0];
        queue[3] = heavy;
    }
    __syncthreads();
    for (uint32_t i0 = 0; i0 < n; i0 += blockDim.x) {
        const uint32_t i = i0 + threadIdx.x;
        const uint32_t b = i < n ? 32 - __clz(overflow ? 0u : tile_count[tile0 + i]) : 33u;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, b);
        const uint32_t leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (b < 33u && lane_id() == leader) base = atomicAdd(&off[b], (uint32_t)__popc(peers));
        base = __shfl_sync(0xFFFFFFFFu, base, leader);
        if (b < 33u) order[tile0 + base + __popc(peers & lanemask_lt())] = tile0 + i;
    }
}

// The tile queue of one raster launch over a group of frames (tile_order_block). One block.
__global__ void __launch_bounds__(1024) k_tile_order(uint32_t tile0, uint32_t n,
                                                     const uint32_t* __restrict__ tile_count,
                                                     uint32_t* __restrict__ order,
                                                     unsigned int* __restrict__ queue,
                                                     const uint32_t* __restrict__ status,
                                                     uint32_t heavy_bits) {
    pdl_enter();
    __shared__ uint32_t cnt[33], off[33];
    const bool overflow = (*(volatile const uint32_t*)status & ST_BIN_OVERFLOW) != 0;
    tile_order_block(tile0, n, tile_count, order, queue, overflow, heavy_bits, cnt, off);
}

// ===================================================================== launchers

// Launch with programmatic stream serialization (see pdl_enter): the kernel may be scheduled
// while its predecessor in the stream is still running and waits for it on entry.
// Pipeline kernels launched by this process (counted at enqueue, or at capture for graphs).
static std::atomic<unsigned long long> g_launches{0};
unsigned long long kernel_launches() { return g_launches.load(std::memory_order_relaxed); }

template <typename... KArgs, typename... Args>
static cudaError_t launch_pdl(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem,
                              cudaStream_t stream, Args... args) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Per-device launch set-up (multiprocessor count, raised shared-memory limits, persistent grid
// sizes), looked up once per device: a process may render on several GPUs, and
// cudaFuncSetAttribute applies to the current device only. Host threads may launch at once.
constexpr int kMaxDevices = 64;

static int current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return -1;
    }
    return dev;
}

// Multiprocessor count of the current device.
static int sm_count() {
    static std::atomic<int> sms[kMaxDevices];
    const int dev = current_device();
    if (dev < 0) return 1;
    int n = sms[dev].load(std::memory_order_relaxed);
    if (!n) {
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
        sms[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

// Persistent grid of a kernel on the current device: resident CTAs per SM x SMs, with its
// dynamic shared-memory limit raised to `bytes` (done once per device and kernel; every host
// thread computes the same).
template <typename K>
static cudaError_t persistent_grid(K kernel, int threads, size_t bytes, std::atomic<int>* cache, int& grid) {
    const int dev = current_device();
    if (dev < 0) return cudaErrorInvalidDevice;
    grid = cache[dev].load(std::memory_order_acquire);
    if (grid) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    int per = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, bytes);
    if (e != cudaSuccess) return e;
    grid = (per > 0 ? per : 1) * sm_count();
    cache[dev].store(grid, std::memory_order_release);
    return cudaSuccess;
}

template <int S, int TS>
static cudaError_t launch_raster_t(const LaunchArgs& a, uint32_t nsx) {
    const size_t bytes = sizeof(RasterSmem<S, TS>);
    const size_t wbytes = sizeof(WarpRasterSmem<S, TS>);
    static std::atomic<int> cta_cap[kMaxDevices], warp_cap[kMaxDevices];
    int grid_cap = 0, wgrid_cap = 0;
    cudaError_t e = persistent_grid(k_raster<S, TS>, kRasterThreads, bytes, cta_cap, grid_cap);
    if (e != cudaSuccess) return e;
    e = persistent_grid(k_raster_warp<S, TS>, 32 * kWarpUnitWarps, wbytes, warp_cap, wgrid_cap);
    if (e != cudaSuccess) return e;
    if (a.raster_ctas_per_sm > 0) {
        const int cap = a.raster_ctas_per_sm * sm_count();
        grid_cap = grid_cap < cap ? grid_cap : cap;
        wgrid_cap = wgrid_cap < cap ? wgrid_cap : cap;
    }
    if (a.raster_blocks == 0) return cudaSuccess;
    if (!a.scan_order_queue) {  // else k_scan_tiles built the queue
        e = launch_pdl(k_tile_order, 1, 1024, 0, a.stream, a.raster_tile_offset, a.raster_blocks,
                       a.scratch.tile_count, a.scratch.tile_order, a.raster_queue, a.scratch.status,
                       a.raster_heavy_bits);
        if (e != cudaSuccess) return e;
    }
    if (nsx > 1) {
        const unsigned sgrid = a.raster_blocks < (uint32_t)grid_cap ? a.raster_blocks : (unsigned)grid_cap;
        e = launch_pdl(k_bin_split, sgrid, 256, 0, a.stream, a.raster_frames, a.raster_nframes,
                       (const uint32_t*)(a.scratch.tile_order + a.raster_tile_offset),
                       (const unsigned int*)a.raster_queue, a.scratch);
        if (e != cudaSuccess) return e;
    }
    const unsigned long long units = (unsigned long long)a.raster_blocks * nsx * nsx;
    // heavy tiles CTA-wide (none when every bin is below the threshold: the launch then only
    // helps with the bins without entries), then the light tiles one warp each
    if (a.raster_heavy_bits < 32) {
        const unsigned grid = units < (unsigned long long)grid_cap ? (unsigned)units : (unsigned)grid_cap;
        e = launch_pdl(k_raster<S, TS>, grid, kRasterThreads, bytes, a.stream, a.raster_frames, a.raster_nframes,
                       (const uint32_t*)(a.scratch.tile_order + a.raster_tile_offset), a.raster_blocks, nsx,
                       a.raster_queue, a.draws, a.scratch);
        if (e != cudaSuccess) return e;
    }
    if (a.raster_heavy_bits == 0) return cudaSuccess;  // every bin with entries is heavy
    const unsigned long long wunits = (units + kWarpUnitWarps - 1) / kWarpUnitWarps;
    const unsigned wgrid = wunits < (unsigned long long)wgrid_cap ? (unsigned)wunits : (unsigned)wgrid_cap;
    return launch_pdl(k_raster_warp<S, TS>, wgrid, 32 * kWarpUnitWarps, wbytes, a.stream, a.raster_frames,
                      a.raster_nframes, (const uint32_t*)(a.scratch.tile_order + a.raster_tile_offset),
                      a.raster_blocks, nsx, a.raster_queue, a.draws, a.scratch);
}

cudaError_t launch_vertex(const LaunchArgs& a) {
    if (a.vertex_blocks == 0) return cudaSuccess;
    return launch_pdl(k_vertex, a.vertex_blocks, 256, 0, a.stream, a.draws, a.frames, a.vblocks, a.scratch);
}

cudaError_t launch_bin_count(const LaunchArgs& a) {
    if (a.nchunks == 0) return cudaSuccess;
    // the kernel's dynamic shared-memory limit (per device) only ever grows, under a lock: a
    // smaller value set by another host thread must not undercut a concurrent larger launch
    static std::mutex mu;
    static int configured[kMaxDevices] = {};
    const uint32_t band = a.max_tiles < (uint32_t)kCountBandTiles ? a.max_tiles : (uint32_t)kCountBandTiles;
    const int bytes = (int)(((band + 1) / 2) * sizeof(uint32_t));
    const int dev = current_device();
    if (dev < 0) return cudaErrorInvalidDevice;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (bytes > configured[dev]) {
            cudaError_t e = cudaFuncSetAttribute(k_bin_count, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
            if (e != cudaSuccess) return e;
            configured[dev] = bytes;
        }
    }
    cudaError_t e = launch_pdl(k_bin_count, a.nchunks, 256, (size_t)bytes, a.stream, a.chunks, a.draws, a.frames,
                               a.scratch);
    if (e != cudaSuccess) return e;
    // the straddling triangles the count queued: a grid-stride pass, one warp per triangle
    const int sms = sm_count();
    // up to four resident CTAs per SM (57 registers a thread), 32 warps per chunk: a frame of
    // a few chunks spreads its straddlers over every SM, a tiny frame launches a few CTAs
    const uint32_t grid = a.nchunks < (uint32_t)sms ? 4u * a.nchunks : (uint32_t)(4 * sms);
    return launch_pdl(k_clip, grid, 256, 0, a.stream, a.draws, a.frames, a.scratch);
}

cudaError_t launch_scans(const LaunchArgs& a) {
    if (a.scan_groups) {
        cudaError_t e = launch_pdl(k_scan_cols, a.scan_groups, 1024, 0, a.stream, a.frames, a.nframes, a.scratch);
        if (e != cudaSuccess) return e;
    }
    if (a.nframes)
        return launch_pdl(k_scan_tiles, (unsigned)a.nframes, 1024, 0, a.stream, a.frames, a.scratch,
                          a.scratch.tile_order, a.scan_order_queue, a.scan_heavy_bits);
    return cudaSuccess;
}

cudaError_t launch_bin_scatter(const LaunchArgs& a) {
    if (a.nchunks == 0) return cudaSuccess;
    return launch_pdl(k_bin_scatter, a.nchunks, kScatterThreads, 0, a.stream, a.chunks, a.draws, a.frames,
                      a.scratch);
}

cudaError_t launch_raster(const LaunchArgs& a, int msaa, int ts) {
    // bins of edge ts are rastered as tiles of edge raster_edge(ts) (quadrants of 32-pixel bins)
    if (ts != 8 && ts != 16 && ts != 32) return cudaErrorInvalidValue;
    const int rs = raster_edge(ts);
    const uint32_t nsx = (uint32_t)(ts / rs);
    if (msaa == 4) return rs == 8 ? launch_raster_t<4, 8>(a, nsx) : launch_raster_t<4, 16>(a, nsx);
    if (msaa == 1) return rs == 8 ? launch_raster_t<1, 8>(a, nsx) : launch_raster_t<1, 16>(a, nsx);
    return cudaErrorInvalidValue;
}

size_t raster_smem(int msaa, int ts) {
    if (ts != 8 && ts != 16 && ts != 32) return 0;
    const int rs = raster_edge(ts);
    if (msaa == 4) return rs == 8 ? raster_smem_bytes<4, 8>() : raster_smem_bytes<4, 16>();
    if (msaa == 1) return rs == 8 ? raster_smem_bytes<1, 8>() : raster_smem_bytes<1, 16>();
    return 0;
}

}  // namespace rast

// ===================================================================== known-answer kernel

namespace rast {

// Evaluates one pipeline device function on caller-supplied inputs (single thread). Layouts
// per op are documented beside rast_debug_kat in rast_api.cu.
__global__ void k_kat(int op, const unsigned char* __restrict__ in, unsigned char* __restrict__ out) {
    const float* fi = reinterpret_cast<const float*>(in);
    float* fo = reinterpret_cast<float*>(out);
    uint32_t* uo = reinterpret_cast<uint32_t*>(out);
    const int32_t* ii = reinterpret_cast<const int32_t*>(in);
    if (op != 5 && threadIdx.x != 0) return;
    switch (op) {
        case 0: {  // perspective divide of 3 clip vertices
            for (int v = 0; v < 3; ++v) {
                float4 n = persp_divide(make_float4(fi[4 * v], fi[4 * v + 1], fi[4 * v + 2], fi[4 * v + 3]));
                fo[4 * v] = n.x; fo[4 * v + 1] = n.y; fo[4 * v + 2] = n.z; fo[4 * v + 3] = n.w;
            }
            break;
        }
        case 1: {  // viewport + setup: in {i32 w, i32 h, f32 ndc[12]}
            const float* ndc = fi + 2;
            float4 sv[3];
            for (int v = 0; v < 3; ++v)
                sv[v] = viewport(make_float4(ndc[4 * v], ndc[4 * v + 1], ndc[4 * v + 2], ndc[4 * v + 3]),
                                 (float)ii[0], (float)ii[1]);
            TriSetup t;
            tri_setup(t, sv);
            for (int v = 0; v < 3; ++v) {
                fo[2 * v] = t.px[v]; fo[2 * v + 1] = t.py[v];
                fo[6 + v] = t.z[v]; fo[9 + v] = t.w[v];
                fo[13 + 2 * v] = t.nx[v]; fo[14 + 2 * v] = t.ny[v];
            }
            fo[12] = t.inv_area;
            break;
        }
        case 2:    // fragment at pixel: in {f32 screen[9], i32 x, i32 y}; out {u32 mask, f32 d[4]}
        case 4: {  // interpolate: in {screen[9], i32 x, i32 y, w[3], attrs[18]}; out attr[6]
            float4 sv[3];
            for (int v = 0; v < 3; ++v) sv[v] = make_float4(fi[3 * v], fi[3 * v + 1], fi[3 * v + 2], 1.0f);
            const uint32_t x = (uint32_t)ii[9], y = (uint32_t)ii[10];
            if (op == 4)
                for (int v = 0; v < 3; ++v) sv[v].w = fi[11 + v];
            TriSetup t;
            tri_setup(t, sv);
            // the raster kernel's coverage and sample-depth arithmetic
            uint32_t cov = 0;
            float d[4] = {0, 0, 0, 0};
            for (int q = 0; q < 4; ++q) {
                const float xs = (float)x + sample_dx<4>(q), ys = (float)y + sample_dy<4>(q);
                float e[3];
                for (int k = 0; k < 3; ++k) e[k] = edge_eval_test(t.nx[k], t.ny[k], t.px[k], t.py[k], xs, ys);
                bool in3 = true;
                for (int k = 0; k < 3; ++k) in3 = in3 && edge_pass_t(e[k], edge_tie(t.nx[k], t.ny[k]));
                if (in3) {
                    cov |= 1u << q;
                    d[q] = interp_depth_fast(e[1], e[2], t.inv_area, t.z[0], t.z[1], t.z[2]);
                }
            }
            if (op == 2) {
                uo[0] = cov;
                for (int q = 0; q < 4; ++q) fo[1 + q] = d[q];
            } else {
                const float* at = fi + 14;
                float xs, ys;
                interp_point<4>(x, y, cov, xs, ys);
                float e[3];
                for (int k = 0; k < 3; ++k) e[k] = edge_eval(t.nx[k], t.ny[k], t.px[k], t.py[k], xs, ys);
                float u, v, w;
                persp_bary(e[0], e[1], e[2], t.w[0], t.w[1], t.w[2], u, v, w);
                for (int c = 0; c < 6; ++c) fo[c] = at[c] * u + at[6 + c] * v + at[12 + c] * w;
            }
            break;
        }
        case 3: {  // eval_single: in {screen[9], f32 x, f32 y}; out {e[3], u32 inside}
            float4 sv[3];
            for (int v = 0; v < 3; ++v) sv[v] = make_float4(fi[3 * v], fi[3 * v + 1], fi[3 * v + 2], 1.0f);
            TriSetup t;
            tri_setup(t, sv);
            bool in3 = true;
            for (int k = 0; k < 3; ++k) {
                fo[k] = edge_eval(t.nx[k], t.ny[k], t.px[k], t.py[k], fi[9], fi[10]);
                in3 = in3 && edge_pass_t(fo[k], edge_tie(t.nx[k], t.ny[k]));
            }
            uo[3] = in3;
            break;
        }
        case 5: {  // try_clip: in {verts[12], attrs[18]}; out {i32 result, i32 ntris, verts[ntris*12]}
            // the product path's warp clipper (k_clip): the whole warp runs this op
            const uint32_t lane = lane_id();
            ClipVert v;
            for (int k = 0; k < 4; ++k) v.p[k] = lane < 3 ? fi[4 * lane + k] : 0.0f;
            for (int k = 0; k < 6; ++k) v.a[k] = lane < 3 ? fi[12 + 6 * lane + k] : 0.0f;
            uint32_t codes[3];
            for (int q = 0; q < 3; ++q)
                codes[q] = clip_code(make_float4(fi[4 * q], fi[4 * q + 1], fi[4 * q + 2], fi[4 * q + 3]));
            int cls = clip_classify(tri2x_area(fi[0], fi[1], fi[4], fi[5], fi[8], fi[9]), codes[0], codes[1], codes[2]);
            int32_t* io = reinterpret_cast<int32_t*>(out);
            const int n = cls == 2 ? warp_clip(v, 3) : 0;
            // gather the polygon's positions to lane 0's view through shared memory
            __shared__ float poly[kMaxPoly][4];
            if (cls == 2 && n > 0 && lane < (uint32_t)n)
                for (int k = 0; k < 4; ++k) poly[lane][k] = v.p[k];
            __syncwarp();
            if (lane != 0) break;
            io[1] = 0;
            if (cls == 2) {
                if (n < 3) {
                    cls = 0;
                } else {
                    io[1] = n - 2;
                    for (int t = 0; t + 2 < n; ++t) {
                        const int vi[3] = {0, t + 1, t + 2};
                        for (int q = 0; q < 3; ++q)
                            for (int k = 0; k < 4; ++k) fo[2 + (3 * t + q) * 4 + k] = poly[vi[q]][k];
                    }
                }
            }
            io[0] = cls;
            break;
        }
        case 6: {  // bbox (unclamped viewport 65535): in points[6]; out u64[4]
            float4 sv[3];
            for (int v = 0; v < 3; ++v) sv[v] = make_float4(fi[2 * v], fi[2 * v + 1], 0.0f, 1.0f);
            uint32_t x0, x1, y0, y1;
            pixel_bbox(sv, 0xFFFFu, 0xFFFFu, x0, x1, y0, y1);
            unsigned long long* lo = reinterpret_cast<unsigned long long*>(out);
            lo[0] = x0; lo[1] = x1; lo[2] = y0; lo[3] = y1;
            break;
        }
        case 7: {  // box filter: in u32[4]; out u32
            uo[0] = box_filter<4>(reinterpret_cast<const uint32_t*>(in));
            break;
        }
        case 8: {  // to_argb: in rgba f32[4]; out u32
            uo[0] = to_argb(fi[0], fi[1], fi[2], fi[3]);
            break;
        }
        case 9: {  // texture sample: in {i32 w, i32 h, f32 u, f32 v, u32 texels[w*h]}; out {f32[4], u32 oob}
            float inv255[256];
            for (int b = 0; b < 256; ++b) inv255[b] = (float)b / 255.0f;
            bool oob = false;
            tex_sample(reinterpret_cast<const uint32_t*>(in) + 4, (uint32_t)ii[0], (uint32_t)ii[1], fi[2], fi[3],
                       inv255, fo, oob);
            uo[4] = oob;
            break;
        }
        case 10: {  // Mat4 * Vec4: in {m[16], v[4]}; out f32[4]
            for (int r = 0; r < 4; ++r) fo[r] = dot4(fi + 4 * r, fi[16], fi[17], fi[18], fi[19]);
            break;
        }
        default:
            break;
    }
}

cudaError_t launch_kat(int op, const void* in, void* out, cudaStream_t stream) {
    // one warp: op 5 (the warp clipper) uses every lane, the others run on lane 0
    k_kat<<<1, 32, 0, stream>>>(op, static_cast<const unsigned char*>(in), static_cast<unsigned char*>(out));
    return cudaGetLastError();
}

}  // namespace rast
