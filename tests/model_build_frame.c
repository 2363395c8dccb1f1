/*
 * Builds the three models of oracle/build_scene.h from raw-mesh files (tests/raw_models.py's
 * format) with this library's sft_model_build (meshlets and proxies on the host, BLAS on the GPU)
 * and renders the scene's frames through the sft_* API, writing each frame's colour: the calls
 * oracle/build_harness.c makes on the reference.  Built and run by tests/test_gpu_model_build.py
 * against libsofren2_gb300.so.
 *
 * usage: model_build_frame <out.bin> <samples> <ground.bin> <shapes.bin> <humanoid.bin>
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#define SFT_FUNC
#include "sofren2.h"
#include "../oracle/build_scene.h"

static const unsigned char* rd(const unsigned char** p, size_t n) { const unsigned char* r = *p; *p += n; return r; }
static u32 rd32(const unsigned char** p) { u32 v; memcpy(&v, rd(p, 4), 4); return v; }

static sft_model* build(const char* path, sft_mat_handle mat, sft_arena* arena) {
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END); const long n = ftell(f); fseek(f, 0, SEEK_SET);
    unsigned char* blob = (unsigned char*)malloc((size_t)n + 16);
    if (fread(blob, 1, (size_t)n, f) != (size_t)n) { fclose(f); return NULL; }
    fclose(f);
    const unsigned char* p = blob;
    if (memcmp(rd(&p, 4), "SFTR", 4) || rd32(&p) != 1) return NULL;
    const u32 seed = rd32(&p);
    const i32 budget = (i32)rd32(&p);
    const u32 nb = rd32(&p);
    sft_raw_bone* bones = (sft_raw_bone*)calloc(nb + 1, sizeof(sft_raw_bone));
    for (u32 b = 0; b < nb; b++) { bones[b].parent_ind = (i32)rd32(&p); memcpy(&bones[b].bind_pos, rd(&p, 12), 12); }
    const u32 nm = rd32(&p);
    sft_raw_mesh* ms = (sft_raw_mesh*)calloc(nm + 1, sizeof(sft_raw_mesh));
    for (u32 k = 0; k < nm; k++) {
        sft_raw_mesh* r = &ms[k];
        r->vertex_count = rd32(&p); r->triangle_count = rd32(&p);
        const u32 skinned = rd32(&p), nv = r->vertex_count;
        r->pos = (const f32*)rd(&p, (size_t)nv * 12);
        r->nrm = (const f32*)rd(&p, (size_t)nv * 12);
        r->uv = (const f32*)rd(&p, (size_t)nv * 8);
        if (skinned) { r->joints = (const u16*)rd(&p, (size_t)nv * 8); r->weights = rd(&p, (size_t)nv * 4); }
        r->indices = (const i32*)rd(&p, (size_t)r->triangle_count * 12);
        r->material = mat;
    }
    srand(seed);
    sft_model* m = sft_model_build(ms, nm, bones, nb, budget, arena);
    free(ms); free(bones);   /* the model keeps no pointer into the caller's arrays */
    free(blob);
    return m;
}

int main(int argc, char** argv) {
    if (argc < 6) { fprintf(stderr, "usage: %s out.bin samples ground.bin shapes.bin humanoid.bin\n", argv[0]); return 2; }
    const int w = BUILD_SCENE_W, h = BUILD_SCENE_H;
    sft_init(w, h, 0);
    sft_set_msaa_samples(atoi(argv[2]));
    static sft_arena arena;
    sft_arena_init(&arena, 1ull << 26);
    const sft_mat_handle mat = build_scene_material();
    sft_model* ms[3];
    for (int k = 0; k < 3; k++) if (!(ms[k] = build(argv[3 + k], mat, &arena))) return 3;
    u32* color = (u32*)calloc((size_t)w * h, 4);
    FILE* out = fopen(argv[1], "wb");
    if (!out) return 5;
    for (int f = 0; f < BUILD_SCENE_FRAMES; f++) {
        build_scene_frame(f, ms[0], ms[1], ms[2], color, w, h);
        fwrite(color, 4, (size_t)w * h, out);
    }
    fclose(out);
    sft_release();
    return 0;
}
