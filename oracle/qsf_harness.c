/*
 * Test infrastructure: loads a QSF2 file with the unmodified reference's sft_model_load_qsf and
 * renders one of two scenes over it, writing each frame's colour buffer (u32 ARGB, width *
 * height) to <out>:
 *   atrium   oracle/qsf_scene.h (a generated file: two instances, moving camera)
 *   map      oracle/map_scene.h (the viewer's frame loop over a map), followed by its ray
 *            queries written to <out>.rays (8 words per ray)
 * MSAA is compile-time in the reference (SFT_USE_AA / SFT_AA_SAMPLES).
 *
 * usage: qsf_harness <atrium|map> <model.qsf> <out.bin> [width=640] [height=360]
 */
#define _GNU_SOURCE
#define SFT_IMPL
#define SFT_NO_DEBUG
#include "sofren2.c"
#include "qsf_scene.h"
#include "map_scene.h"

int main(int argc, char** argv) {
    if (argc < 4) { fprintf(stderr, "usage: %s atrium|map model.qsf out.bin [width] [height]\n", argv[0]); return 2; }
    const int map = strcmp(argv[1], "map") == 0;
    const int w = argc > 4 ? atoi(argv[4]) : 640, h = argc > 5 ? atoi(argv[5]) : 360;
    sft_init(w, h, 1);
    static sft_arena arena;
    sft_arena_init(&arena, 1ull << 30);
    if (!(map ? map_scene_setup(argv[2], &arena) : qsf_scene_setup(argv[2], &arena))) return 4;
    u32* color = (u32*)calloc((size_t)w * h, 4);
    FILE* out = fopen(argv[3], "wb");
    if (!out) return 3;
    const int frames = map ? MAP_SCENE_FRAMES : QSF_SCENE_FRAMES;
    for (int f = 0; f < frames; f++) {
        if (map) map_scene_frame(f, color, w, h);
        else qsf_scene_frame(f, color, w, h);
        fwrite(color, 4, (size_t)w * h, out);
    }
    fclose(out);
    if (map) {
        static u32 hits[MAP_RAYS * 8];
        map_scene_rays(hits);
        char rp[4096];
        snprintf(rp, sizeof(rp), "%s.rays", argv[3]);
        FILE* rf = fopen(rp, "wb");
        if (!rf) return 3;
        fwrite(hits, 4, (size_t)MAP_RAYS * 8, rf);
        fclose(rf);
    }
    return 0;
}
