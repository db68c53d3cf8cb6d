// rast_raster_warp.cuh - warp-per-tile raster for light tiles (included by rast_kernels.cu).
//
// A raster tile with few bin entries leaves the warps of the CTA-wide kernel (k_raster) running
// partial warps between block barriers. Here one warp owns a whole tile: it stages the tile's
// items 32 at a time, one per lane and held in that lane's registers (other lanes read them
// with shuffles, which keeps shared memory for the samples and rings: 5 CTAs of 4 warps per
// SM with four samples per pixel, 6 with one), walks their candidate pixels 32 at a time, depth-tests the covered fragments in
// submission order and shades the passed ones, with full warps and no block barrier. The
// arithmetic is the same device functions as k_raster (coverage, sample depths, tie rule,
// interpolation, shaders, resolve), so results are bit-identical; only the work split differs.
//
// The persistent kernel takes light tiles (bins past the first `nheavy` of the raster queue,
// which k_tile_order or, for a one-frame run, k_scan_tiles sorts heaviest first) from their own
// counter, then helps clear the bins without entries. k_raster takes the heavy tiles.

constexpr int kWarpUnitWarps = 4;  // warps (independent tiles) per CTA of k_raster_warp
// CTAs per SM the launch bounds aim at: with 4 samples the shared sample tiles allow 5; with
// one sample 6 (79 registers, no spills; 7 spills and ran 2% slower on the scene mix, 5 3% slower)
constexpr int kWarpUnitCtas = 5;
constexpr int kWarpUnitCtas1 = 6;

template <int S, int TS>
struct alignas(16) WarpUnitSmem {
    static constexpr int NPIX = TS * TS;
    static constexpr int IB = 32;  // items per batch (one per lane)
    static constexpr int QC = 64;  // ring entries
    float zb[NPIX * S];            // sample-major: sample k of pixel p at k * NPIX + p
    uint32_t cb[NPIX * S];
    uint8_t rpre[IB][TS];          // rows trimmed by line_span: candidates before each box row
                                   // (at most 15 rows of 16 before the last: fits a byte)
    uint8_t rsta[IB][TS];          // rows trimmed by line_span: first column of each box row
    float qz[S][QC];               // ring of covered fragments, in submission order
    uint8_t qitem[QC], qpix[QC], qcov[QC];
    float sz0[QC];                 // ring of depth-passed fragments waiting for the shader
    uint8_t sitem[QC], spix[QC], sdm[QC];
};

template <int S, int TS>
struct WarpRasterSmem {
    float inv255[256];
    WarpUnitSmem<S, TS> u[kWarpUnitWarps];
};

template <int S, int TS>
size_t warp_raster_smem_bytes() { return sizeof(WarpRasterSmem<S, TS>); }

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    const uint32_t lane = lane_id();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, v, o);
        if (lane >= (uint32_t)o) v += y;
    }
    return v;
}

// One item of a warp batch (a triangle, or one fan triangle of a clipped polygon), held by the
// lane of its slot: screen points, depths, w, texture coordinates, 1 / 2x area, tile-local box
// (x0 | y0 << 8 | x1 << 16 | y1 << 24, 0: nothing to do), frame triangle and draw << 8 | sub.
struct WItem {
    float px[3], py[3], z[3], w[3], inv;
    float uv[6];
    uint32_t rect, tri, meta;
};

// Stages item k of a bin entry (triangle g, clipped polygon at aux or kNone) into `it`, as
// stage_entry does for k_raster.
template <int TS>
__device__ __forceinline__ void wstage_item(WItem& it, const FrameDev& f, const DrawDev* __restrict__ draws,
                                            const Scratch& s, uint32_t g, uint32_t aux, uint32_t k, uint32_t X0,
                                            uint32_t Y0, float ztile) {
    const uint32_t di = find_draw(draws, f, g);
    const DrawDev& d = draws[di];
    float4 sv[3];
    float uv[3][2] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
    if (aux == kNone) {
        const uint32_t tri = g - d.tbase;
        const uint32_t ii[3] = {__ldg(d.idx + 3ull * tri), __ldg(d.idx + 3ull * tri + 1),
                                __ldg(d.idx + 3ull * tri + 2)};
        const bool tex = d.fs == 0;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            sv[q] = s.vscr[d.vbase + ii[q]];
            if (tex) {
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
        it.px[q] = sv[q].x;
        it.py[q] = sv[q].y;
        it.z[q] = sv[q].z;
        it.w[q] = sv[q].w;
        it.uv[2 * q] = uv[q][0];
        it.uv[2 * q + 1] = uv[q][1];
    }
    // 1 / triangle_2x_area (RasterizerTriangle::new, src/rasterizer/mod.rs:206)
    it.inv = 1.0f / tri2x_area(sv[0].x, sv[0].y, sv[1].x, sv[1].y, sv[2].x, sv[2].y);
    uint32_t bx0, bx1, by0, by1;
    pixel_bbox(sv, f.width, f.height, bx0, bx1, by0, by1);
    const uint32_t cx0 = max(bx0, X0), cx1 = min(bx1, X0 + TS);
    const uint32_t cy0 = max(by0, Y0), cy1 = min(by1, Y0 + TS);
    // hidden items (depth_cull) cover nothing that could pass the strict depth test
    const bool nonempty = bx0 < bx1 && by0 < by1 && cx0 < cx1 && cy0 < cy1 &&
                          !depth_cull(sv[0].z, sv[1].z, sv[2].z, ztile);
    it.rect = nonempty ? ((cx0 - X0) | ((cy0 - Y0) << 8) | ((cx1 - X0) << 16) | ((cy1 - Y0) << 24)) : 0u;
    it.tri = g;
    it.meta = (di << 8) | k;
}

__device__ __forceinline__ float shfl_f(float v, uint32_t src) { return __shfl_sync(0xFFFFFFFFu, v, src); }
__device__ __forceinline__ uint32_t shfl_u(uint32_t v, uint32_t src) { return __shfl_sync(0xFFFFFFFFu, v, src); }

// Depth test of up to 32 queued fragments (lane = fragment, ring order = submission order):
// fragments of one pixel in rounds of increasing rank, as warp_depth does for k_raster.
template <int S, int TS>
__device__ __forceinline__ void wdepth(WarpUnitSmem<S, TS>& sm, const WItem& my, uint32_t head, uint32_t n,
                                       uint32_t& stail, const Scratch& s, uint32_t X0, uint32_t Y0,
                                       uint32_t& shaded, uint32_t& fsinv) {
    using U = WarpUnitSmem<S, TS>;
    const uint32_t lane = lane_id();
    const bool valid = lane < n;
    const uint32_t q = (head + lane) & (U::QC - 1);
    uint32_t it = 0, pix = 0, cov = 0;
    float z[S];
#pragma unroll
    for (int k = 0; k < S; ++k) z[k] = 0.0f;
    if (valid) {
        it = sm.qitem[q];
        pix = sm.qpix[q];
        cov = sm.qcov[q];
#pragma unroll
        for (int k = 0; k < S; ++k) z[k] = sm.qz[k][q];
    }
    // the fragment log (debug) names the fragment's triangle: read from the item's lane
    uint32_t ltri = 0, lmeta = 0;
    if (s.log) {
        ltri = shfl_u(my.tri, it);
        lmeta = shfl_u(my.meta, it);
    }
    const uint32_t key = valid ? pix : 0x10000u + lane;
    const uint32_t grp = __match_any_sync(0xFFFFFFFFu, key);
    const uint32_t rank = __popc(grp & lanemask_lt());
    const uint32_t maxr = __reduce_max_sync(0xFFFFFFFFu, rank);
    uint32_t dm = 0;
    for (uint32_t r = 0; r <= maxr; ++r) {
        const bool act = valid && rank == r;
#pragma unroll
        for (int k = 0; k < S; ++k) {
            const float old = sm.zb[k * U::NPIX + pix];
            const bool pass = act & (((cov >> k) & 1u) != 0) & (z[k] < old);
            if (pass) sm.zb[k * U::NPIX + pix] = z[k];
            dm |= (uint32_t)pass << k;
        }
        if (s.log && act)
            log_fragment(s, ltri, lmeta & 0xFFu, ((Y0 + pix / TS) << 16) | (X0 + pix % TS), (dm << 8) | cov);
        __syncwarp();
    }
    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, dm != 0);
    if (dm) {
        const uint32_t sq = (stail + __popc(bal & lanemask_lt())) & (U::QC - 1);
        sm.sitem[sq] = (uint8_t)it;
        sm.spix[sq] = (uint8_t)pix;
        sm.sdm[sq] = (uint8_t)dm;
        sm.sz0[sq] = z[0];
        shaded += __popc(dm);
        fsinv += 1;
    }
    stail += __popc(bal);
    __syncwarp();
}

// Fragment shader and colour write of up to 32 fragments of the shade ring, as warp_shade does
// for k_raster; each lane reads its fragment's item from the item's lane.
template <int S, int TS>
__device__ __forceinline__ void wshade(WarpUnitSmem<S, TS>& sm, const WItem& my, const float* inv255,
                                      uint32_t head, uint32_t n, const DrawDev* __restrict__ draws,
                                      const FrameDev& f, const Scratch& s, uint32_t X0, uint32_t Y0,
                                      uint32_t& oobc) {
    using U = WarpUnitSmem<S, TS>;
    const uint32_t lane = lane_id();
    const bool valid = lane < n;
    const uint32_t q = (head + lane) & (U::QC - 1);
    const uint32_t it = valid ? sm.sitem[q] : 0u;
    float px[3], py[3], w[3], tuv[6];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        px[k] = shfl_f(my.px[k], it);
        py[k] = shfl_f(my.py[k], it);
        w[k] = shfl_f(my.w[k], it);
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) tuv[k] = shfl_f(my.uv[k], it);
    const uint32_t meta = shfl_u(my.meta, it), tri = shfl_u(my.tri, it);
    uint32_t argb = 0, pix = 0, dm = 0;
    if (valid) {
        pix = sm.spix[q];
        dm = sm.sdm[q];
        const uint32_t x = X0 + pix % TS, y = Y0 + pix / TS;
        float xs, ys;
        interp_point<S>(x, y, dm, xs, ys);
        float e[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            // inward normal of edge k (RasterizerTriangle::new, src/rasterizer/mod.rs:199-204)
            const int nk = k == 2 ? 0 : k + 1;
            const float nx = -(py[nk] - py[k]), ny = px[nk] - px[k];
            e[k] = edge_eval(nx, ny, px[k], py[k], xs, ys);
        }
        float u, v, ww;
        persp_bary(e[0], e[1], e[2], w[0], w[1], w[2], u, v, ww);
        const DrawDev& d = draws[meta >> 8];
        float col[4];
        if (d.fs == 0) {
            // FS::Texture (upstream src/main.rs:214-216)
            const float tu = tuv[0] * u + tuv[2] * v + tuv[4] * ww;
            const float tv = tuv[1] * u + tuv[3] * v + tuv[5] * ww;
            bool oob = false;
            tex_sample(d.tex, d.tex_w, d.tex_h, tu, tv, inv255, col, oob);
            if (oob) ++oobc;
        } else if (d.fs == 1) {
            // FS::Color (upstream src/main.rs:217)
            float vc[3][4];
            item_colours(d, f, s, tri, meta & 0xFFu, vc);
#pragma unroll
            for (int c = 0; c < 4; ++c) col[c] = vc[0][c] * u + vc[1][c] * v + vc[2][c] * ww;
        } else {
            // FS::Debug (upstream src/main.rs:218-220): grayscale(frag_coords.depths[0])
            const float z0 = sm.sz0[q];
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
            if (act & (((dm >> k) & 1u) != 0)) sm.cb[k * U::NPIX + pix] = argb;
        __syncwarp();
    }
}

// Resolve (resolve_and_clear + box_filter_color, mod.rs:478-518, buffers.rs:111-125) of the
// warp's tile: four consecutive pixels of a row per lane with 16-byte stores where the image
// row allows them, one pixel per lane otherwise (image edges, unaligned outputs, sample capture).
template <int S, int TS>
__device__ __forceinline__ void wresolve(const WarpUnitSmem<S, TS>& sm, const FrameDev& f, uint32_t X0, uint32_t Y0) {
    using U = WarpUnitSmem<S, TS>;
    const uint32_t lane = lane_id();
    const uint32_t W = f.width, H = f.height;
    const bool vec = !f.dbg_depth && (W & 3u) == 0 && X0 + TS <= W &&
                     (reinterpret_cast<uintptr_t>(f.out) & 15u) == 0;
    if (vec) {
        for (uint32_t p = 4 * lane; p < (uint32_t)U::NPIX; p += 128) {
            const uint32_t y = Y0 + p / TS;
            if (y >= H) break;  // rows go down with p
            uint4 c[S];
#pragma unroll
            for (int k = 0; k < S; ++k) c[k] = *reinterpret_cast<const uint4*>(&sm.cb[k * U::NPIX + p]);
            uint32_t px[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                uint32_t smp[S];
#pragma unroll
                for (int k = 0; k < S; ++k) smp[k] = j == 0 ? c[k].x : j == 1 ? c[k].y : j == 2 ? c[k].z : c[k].w;
                px[j] = box_filter<S>(smp);
            }
            *reinterpret_cast<uint4*>(f.out + (unsigned long long)y * W + X0 + p % TS) =
                make_uint4(px[0], px[1], px[2], px[3]);
        }
        return;
    }
    for (uint32_t p = lane; p < (uint32_t)U::NPIX; p += 32) {
        const uint32_t x = X0 + p % TS, y = Y0 + p / TS;
        if (x >= W || y >= H) continue;
        const unsigned long long o = (unsigned long long)y * W + x;
        uint32_t smp[S];
#pragma unroll
        for (int k = 0; k < S; ++k) smp[k] = sm.cb[k * U::NPIX + p];
        f.out[o] = box_filter<S>(smp);
        if (f.dbg_depth) {
#pragma unroll
            for (int k = 0; k < S; ++k) {
                f.dbg_depth[o * S + k] = sm.zb[k * U::NPIX + p];
                f.dbg_color[o * S + k] = sm.cb[k * U::NPIX + p];
            }
        }
    }
}

// One light tile by one warp: the bin's entries in submission order, 32 items at a time.
// (A) the items of the next entries, one per lane (a lane finds its entry and fan triangle
// from the entries' running item counts); (B) per item (lane) its candidate pixels: the whole
// tile-local box, or for boxes of kTrimMin+ columns each row trimmed by line_span; (C) the
// candidates 32 at a time - coverage (EdgeFunctions::eval, mod.rs:134-146) and sample depths
// (RasterizerTriangle::fragment, mod.rs:225-253) - into the fragment ring, ordered depth test
// into the shade ring, shading; both rings are drained before the next batch replaces the items
// they refer to. Then the resolve.
template <int S, int TS>
__device__ __forceinline__ void warp_unit(WarpUnitSmem<S, TS>& sm, const float* inv255, const FrameDev& f,
                                          const DrawDev* __restrict__ draws, const Scratch& s,
                                          const uint32_t* __restrict__ bins, uint32_t nent, uint32_t mybit,
                                          uint32_t X0, uint32_t Y0, uint32_t& shaded, uint32_t& fsinv,
                                          uint32_t& oobc) {
    using U = WarpUnitSmem<S, TS>;
    const uint32_t lane = lane_id();
    {
        const float4 zc = make_float4(f.clear_depth, f.clear_depth, f.clear_depth, f.clear_depth);
        const uint4 cc = make_uint4(kClearColor, kClearColor, kClearColor, kClearColor);
        float4* z4 = reinterpret_cast<float4*>(sm.zb);
        uint4* c4 = reinterpret_cast<uint4*>(sm.cb);
        for (uint32_t i = lane; i < (uint32_t)(U::NPIX * S / 4); i += 32) {
            z4[i] = zc;
            c4[i] = cc;
        }
    }
    __syncwarp();
    WItem my;  // the item of this lane's slot in the current batch
    uint32_t pos = 0, batch = 0;
    // depth_cull bound: the clear depth at first; NaN (no culling) while the fragment log
    // records depth-failed fragments too
    float zt = s.log ? __int_as_float(0x7FC00000) : f.clear_depth;
    while (pos < nent) {
        // the largest stored depth, refreshed before batches 1, 2, 4, 8, ...
        if (!s.log && batch > 0 && (batch & (batch - 1)) == 0) {
            uint32_t zm = 0;
            for (uint32_t i = lane; i < (uint32_t)(U::NPIX * S); i += 32) zm = max(zm, float_to_ordered(sm.zb[i]));
            zt = ordered_to_float(__reduce_max_sync(0xFFFFFFFFu, zm));
        }
        ++batch;
        // ---- A. items of the next entries that touch this tile, while they fit the batch
        uint32_t nit = 0;
        my.rect = 0;
        while (pos < nent) {
            const uint32_t e = pos + lane;
            uint32_t g = 0, aux = kNone, nitems = 0;
            if (e < nent) {
                const uint32_t ent = bins[e];
                if (ent & mybit) {
                    g = ent >> kEntShift;
                    nitems = 1;
                    if (ent & kEntClipped) {
                        aux = s.tri_aux[f.rect_base + g];
                        // a fan of at most kMaxPoly - 2 <= IB triangles (k_clip stores 3..kMaxPoly
                        // vertices); the bound keeps every entry within one batch
                        nitems = min((uint32_t)__float_as_int(s.clip_store[aux]) - 2u, (uint32_t)U::IB);
                    }
                }
            }
            const uint32_t incl = warp_incl_scan(nitems);
            // running item counts only grow along the lanes, so the entries that fit are a prefix
            const bool fits = e < nent && nit + incl <= (uint32_t)U::IB;
            const uint32_t take = __popc(__ballot_sync(0xFFFFFFFFu, fits));
            const uint32_t win = take ? __shfl_sync(0xFFFFFFFFu, incl, take - 1) : 0u;  // items taken
            // slot lane gets item q = lane - nit of this window: entry src, fan triangle k
            const uint32_t qi = lane - nit;  // wraps for lanes below nit (not staged)
            uint32_t src = 0;
#pragma unroll
            for (int st = 16; st > 0; st >>= 1) {
                const uint32_t v = __shfl_sync(0xFFFFFFFFu, incl, src + st - 1);
                if (v <= qi) src += st;
            }
            src = min(src, 31u);
            const uint32_t sg = __shfl_sync(0xFFFFFFFFu, g, src), saux = __shfl_sync(0xFFFFFFFFu, aux, src);
            const uint32_t sk = qi - (__shfl_sync(0xFFFFFFFFu, incl, src) - __shfl_sync(0xFFFFFFFFu, nitems, src));
            if (lane >= nit && lane < nit + win) wstage_item<TS>(my, f, draws, s, sg, saux, sk, X0, Y0, zt);
            nit += win;
            pos += take;
            if (take < 32) break;  // the batch is full, or the entries ran out
        }
        // ---- B. candidates of each item (lane = item): the whole box, or for boxes of kTrimMin+
        // columns each row trimmed by line_span
        uint32_t c = 0, geo = 0, nrows = 0;  // geo: x0 | y0 << 5 | w << 10 | h << 16 | trimmed << 21
        if (lane < nit) {
            const uint32_t r = my.rect;
            const uint32_t x0 = r & 0xFFu, y0 = (r >> 8) & 0xFFu, x1 = (r >> 16) & 0xFFu, y1 = r >> 24;
            const uint32_t w = x1 - x0, h = y1 - y0;
            const bool trim = w >= kTrimMin && h > 0;
            nrows = trim ? h : 0u;
            c = w * h;
            geo = x0 | (y0 << 5) | (w << 10) | (h << 16) | ((uint32_t)trim << 21);
        }
        // the rows to trim, spread over the lanes 32 at a time (a warp would otherwise run as many
        // rounds as its tallest item has rows): task t is row t - (rows of earlier items) of the
        // item whose running row count first exceeds t, read from that item's lane; the span's
        // start goes to rsta, its length to rpre until the prefix pass below
        const uint32_t rincl = warp_incl_scan(nrows);
        const uint32_t rtot = __shfl_sync(0xFFFFFFFFu, rincl, 31);
        for (uint32_t tb = 0; tb < rtot; tb += 32) {
            const uint32_t t = tb + lane;
            uint32_t j = 0;
#pragma unroll
            for (int st = 16; st > 0; st >>= 1) {
                const uint32_t v = __shfl_sync(0xFFFFFFFFu, rincl, j + st - 1);
                if (v <= t) j += st;
            }
            j = min(j, 31u);
            const float px[3] = {shfl_f(my.px[0], j), shfl_f(my.px[1], j), shfl_f(my.px[2], j)};
            const float py[3] = {shfl_f(my.py[0], j), shfl_f(my.py[1], j), shfl_f(my.py[2], j)};
            const uint32_t gj = __shfl_sync(0xFFFFFFFFu, geo, j);
            const uint32_t row = t - __shfl_sync(0xFFFFFFFFu, rincl - nrows, j);
            if (t < rtot) {
                const uint32_t x0 = gj & 31u, y0 = (gj >> 5) & 31u;
                uint32_t a0 = x0, a1 = x0 + ((gj >> 10) & 31u);
                line_span_pts<S, TS>(px, py, 0u, y0 + row, X0, Y0, a0, a1);
                sm.rsta[j][row] = (uint8_t)a0;
                sm.rpre[j][row] = (uint8_t)(a1 - a0);
            }
        }
        __syncwarp();
        if (nrows) {
            uint32_t run = 0;  // candidates before each row
            for (uint32_t row = 0; row < nrows; ++row) {
                const uint32_t len = sm.rpre[lane][row];
                sm.rpre[lane][row] = (uint8_t)run;
                run += len;
            }
            c = run;
        }
        const uint32_t incl = warp_incl_scan(c);
        const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
        __syncwarp();
        // ---- C. the candidates, 32 at a time, in submission order
        uint32_t head = 0, tail = 0, shead = 0, stail = 0;
        for (uint32_t pb = 0; pb < total; pb += 32) {
            const uint32_t p = pb + lane;
            uint32_t j = 0;  // source item: number of items whose inclusive count is <= p
#pragma unroll
            for (int st = 16; st > 0; st >>= 1) {
                const uint32_t v = __shfl_sync(0xFFFFFFFFu, incl, j + st - 1);
                if (v <= p) j += st;
            }
            const uint32_t it = min(j, 31u);
            const uint32_t exc = __shfl_sync(0xFFFFFFFFu, incl - c, it);
            const uint32_t gg = __shfl_sync(0xFFFFFFFFu, geo, it);
            // the item's points, depths and 1 / 2x area from its lane
            const float p0x = shfl_f(my.px[0], it), p0y = shfl_f(my.py[0], it);
            const float p1x = shfl_f(my.px[1], it), p1y = shfl_f(my.py[1], it);
            const float p2x = shfl_f(my.px[2], it), p2y = shfl_f(my.py[2], it);
            const float z0 = shfl_f(my.z[0], it), z1 = shfl_f(my.z[1], it), z2 = shfl_f(my.z[2], it);
            const float inv = shfl_f(my.inv, it);
            uint32_t cov = 0, pix = 0;
            float z[S];
#pragma unroll
            for (int k = 0; k < S; ++k) z[k] = 0.0f;
            if (p < total) {
                const uint32_t rr = p - exc;
                const uint32_t x0 = gg & 31u, y0 = (gg >> 5) & 31u, w = (gg >> 10) & 31u, h = (gg >> 16) & 31u;
                uint32_t row, col;
                if (gg & (1u << 21)) {
                    // last box row whose prefix is <= rr (rows trimmed to nothing are skipped)
                    row = 0;
#pragma unroll
                    for (int st = TS / 2; st > 0; st >>= 1)
                        if (row + st < h && sm.rpre[it][row + st] <= rr) row += st;
                    col = sm.rsta[it][row] + (rr - sm.rpre[it][row]);
                } else {
                    // w < kTrimMin = 4: rr / w with a multiply (exact for rr < 128)
                    row = w == 1 ? rr : w == 2 ? (rr >> 1) : ((rr * 43u) >> 7);
                    col = x0 + (rr - row * w);
                }
                const uint32_t ly = y0 + row;
                pix = ly * TS + col;
                const float fx = (float)(X0 + col), fy = (float)(Y0 + ly);
                // inward normals (RasterizerTriangle::new, src/rasterizer/mod.rs:199-204)
                const float n0x = -(p1y - p0y), n0y = p1x - p0x;
                const float n1x = -(p2y - p1y), n1y = p2x - p1x;
                const float n2x = -(p0y - p2y), n2y = p0x - p2x;
                // tie rule per edge (EdgeFunctions::inside, mod.rs:148-170)
                const bool t0 = edge_tie(n0x, n0y), t1 = edge_tie(n1x, n1y), t2 = edge_tie(n2x, n2y);
#pragma unroll
                for (int k = 0; k < S; ++k) {
                    const float xs = fx + sample_dx<S>(k), ys = fy + sample_dy<S>(k);
                    const float e0 = edge_eval_test(n0x, n0y, p0x, p0y, xs, ys);
                    const float e1 = edge_eval_test(n1x, n1y, p1x, p1y, xs, ys);
                    const float e2 = edge_eval_test(n2x, n2y, p2x, p2y, xs, ys);
                    const bool in = edge_pass_t(e0, t0) & edge_pass_t(e1, t1) & edge_pass_t(e2, t2);
                    const float zk = interp_depth_fast(e1, e2, inv, z0, z1, z2);
                    cov |= (uint32_t)in << k;
                    z[k] = in ? zk : 0.0f;
                }
            }
            const uint32_t bal = __ballot_sync(0xFFFFFFFFu, cov != 0);
            if (cov) {
                const uint32_t q = (tail + __popc(bal & lanemask_lt())) & (U::QC - 1);
                sm.qitem[q] = (uint8_t)it;
                sm.qpix[q] = (uint8_t)pix;
                sm.qcov[q] = (uint8_t)cov;
#pragma unroll
                for (int k = 0; k < S; ++k) sm.qz[k][q] = z[k];
            }
            tail += __popc(bal);
            __syncwarp();
            if (tail - head >= 32) {
                wdepth<S, TS>(sm, my, head, 32, stail, s, X0, Y0, shaded, fsinv);
                head += 32;
                if (stail - shead >= 32) {
                    wshade<S, TS>(sm, my, inv255, shead, 32, draws, f, s, X0, Y0, oobc);
                    shead += 32;
                }
            }
        }
        if (tail != head) wdepth<S, TS>(sm, my, head, tail - head, stail, s, X0, Y0, shaded, fsinv);
        while (stail != shead) {
            const uint32_t nsh = min(stail - shead, 32u);
            wshade<S, TS>(sm, my, inv255, shead, nsh, draws, f, s, X0, Y0, oobc);
            shead += nsh;
        }
        __syncwarp();
    }
    __syncwarp();
    wresolve<S, TS>(sm, f, X0, Y0);
    __syncwarp();
}

// Persistent warp-per-tile raster kernel over the light tiles of one raster launch: the bins
// order[nheavy .. nbusy) (queue[3] = nheavy, queue[2] = nbusy, both written by k_tile_order),
// times nsx * nsx quadrants, taken one tile per warp from queue[4]; then bins without entries
// from queue[1], like k_raster.
template <int S, int TS>
__global__ void __launch_bounds__(32 * kWarpUnitWarps, S == 1 ? kWarpUnitCtas1 : kWarpUnitCtas) k_raster_warp(const FrameDev* __restrict__ frames,
                                                                     int nframes,
                                                                     const uint32_t* __restrict__ order,
                                                                     uint32_t ntotal, uint32_t nsx,
                                                                     unsigned int* __restrict__ queue,
                                                                     const DrawDev* __restrict__ draws,
                                                                     Scratch s) {
    pdl_enter();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    WarpRasterSmem<S, TS>& sh = *reinterpret_cast<WarpRasterSmem<S, TS>*>(smem_raw);
    for (uint32_t i = threadIdx.x; i < 256u; i += blockDim.x) sh.inv255[i] = (float)i / 255.0f;
    __syncthreads();
    const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
    WarpUnitSmem<S, TS>& sm = sh.u[warp];
    const uint32_t nbusy = *(volatile unsigned int*)&queue[2];
    const uint32_t nheavy = *(volatile unsigned int*)&queue[3];
    const uint32_t nsub = nsx * nsx;
    const uint32_t nlight = (nbusy - nheavy) * nsub;
    uint32_t shaded = 0, fsinv = 0, oobc = 0;
    for (;;) {
        uint32_t qi = 0;
        if (lane == 0) qi = atomicAdd(&queue[4], 1u);
        qi = __shfl_sync(0xFFFFFFFFu, qi, 0);
        if (qi >= nlight) break;
        const uint32_t gt = order[nheavy + qi / nsub], sub = qi % nsub;
        const FrameDev& f = frames[frame_of_tile(frames, nframes, gt)];
        const uint32_t lt = gt - f.tile_begin;
        const uint32_t X0 = (lt % f.tiles_x) * (uint32_t)f.ts + (sub % nsx) * TS;
        const uint32_t Y0 = (lt / f.tiles_x) * (uint32_t)f.ts + (sub / nsx) * TS;
        uint32_t nent;
        const uint32_t* bins;
        if (nsub > 1) {
            nent = s.qcount[4ull * gt + sub];
            bins = s.qbins + f.qbin_base + 4ull * s.tile_start[gt] + (unsigned long long)sub * s.tile_count[gt];
        } else {
            nent = s.tile_count[gt];
            bins = s.bins + f.bin_base + s.tile_start[gt];
        }
        warp_unit<S, TS>(sm, sh.inv255, f, draws, s, bins, nent, 1u << sub, X0, Y0, shaded, fsinv, oobc);
    }
    // bins without entries: runs of kEmptyRun bins per counter update, the clear colour
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
    shaded = __reduce_add_sync(0xFFFFFFFFu, shaded);
    fsinv = __reduce_add_sync(0xFFFFFFFFu, fsinv);
    oobc = __reduce_add_sync(0xFFFFFFFFu, oobc);
    if (lane == 0) {
        if (shaded) atomicAdd(&s.stats[STAT_SHADED], (unsigned long long)shaded);
        if (fsinv) atomicAdd(&s.stats[STAT_FSINV], (unsigned long long)fsinv);
        if (oobc) {
            atomicAdd(&s.stats[STAT_OOB], (unsigned long long)oobc);
            atomicOr(s.status, ST_TEXTURE_OOB);
        }
    }
}
