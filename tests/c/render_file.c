/* C caller of include/rast.h, for the ABI test: reads one scene from a binary file, renders it
 * through rast_create / rast_texture_upload / rast_mesh_upload / rast_set_uniforms / rast_draw /
 * rast_framebuffer (the reference demo's call order), and writes the ARGB frame.
 *
 * Input (little-endian): int32 width, height, msaa, nverts, ntris, tex_w, tex_h, fs_id;
 * f32 clear_depth; f32 world[16], view[16], proj[16]; f32 pos[nverts*3], uv[nverts*2];
 * u32 idx[ntris*3]; u8 tex[tex_w*tex_h*4]. Output: u32 argb[width*height], then u32 status.
 */
#include <stdio.h>
#include <stdlib.h>

#include "rast.h"

static void* read_n(FILE* f, size_t bytes) {
    void* p = malloc(bytes ? bytes : 1);
    if (!p || fread(p, 1, bytes, f) != bytes) {
        fprintf(stderr, "short read\n");
        exit(2);
    }
    return p;
}

int main(int argc, char** argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: %s scene.bin out.bin\n", argv[0]);
        return 2;
    }
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    int* hdr = (int*)read_n(f, 8 * sizeof(int));
    const int W = hdr[0], H = hdr[1], msaa = hdr[2], tw = hdr[5], th = hdr[6], fs = hdr[7];
    const uint32_t nv = (uint32_t)hdr[3], nt = (uint32_t)hdr[4];
    float* cd = (float*)read_n(f, sizeof(float));
    float* mats = (float*)read_n(f, 48 * sizeof(float));
    float* pos = (float*)read_n(f, (size_t)nv * 3 * sizeof(float));
    float* uv = (float*)read_n(f, (size_t)nv * 2 * sizeof(float));
    uint32_t* idx = (uint32_t*)read_n(f, (size_t)nt * 3 * sizeof(uint32_t));
    uint8_t* tex = (uint8_t*)read_n(f, (size_t)tw * th * 4);
    fclose(f);

    rast_status st = RAST_OK;
    rast_ctx* ctx = rast_create(W, H, msaa, &st);
    if (!ctx) {
        fprintf(stderr, "rast_create: %s\n", rast_status_string(st));
        return 1;
    }
    rast_mesh mesh = 0;
    if ((st = rast_set_clear_depth(ctx, *cd)) != RAST_OK ||
        (st = rast_texture_upload(ctx, 0, tex, tw, th)) != RAST_OK ||
        (st = rast_mesh_upload(ctx, pos, uv, NULL, nv, idx, nt, &mesh)) != RAST_OK ||
        (st = rast_set_uniforms(ctx, mats, mats + 16, mats + 32)) != RAST_OK ||
        (st = rast_draw(ctx, mesh, RAST_VS_MVP, fs)) != RAST_OK) {
        fprintf(stderr, "setup: %s\n", rast_status_string(st));
        rast_destroy(ctx);
        return 1;
    }
    uint32_t* out = (uint32_t*)malloc((size_t)W * H * sizeof(uint32_t));
    st = rast_framebuffer(ctx, out);
    FILE* o = fopen(argv[2], "wb");
    if (!o) return 2;
    fwrite(out, sizeof(uint32_t), (size_t)W * H, o);
    uint32_t s32 = (uint32_t)st;
    fwrite(&s32, sizeof(s32), 1, o);
    fclose(o);
    rast_destroy(ctx);
    free(out);
    free(hdr);
    free(cd);
    free(mats);
    free(pos);
    free(uv);
    free(idx);
    free(tex);
    return st == RAST_OK || st == RAST_TEXTURE_OOB ? 0 : 1;
}
