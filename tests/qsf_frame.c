/*
 * Loads a QSF2 file with this library's sft_model_load_qsf and renders one of the scenes of
 * oracle/qsf_harness.c over it through the sft_* API (the same calls the harness makes on the
 * reference), writing each frame's colour to <out>, and for the map scene its ray queries to
 * <out>.rays.  Also checks the loader's soft failures: a missing file and a file with the wrong
 * magic give NULL.  Built and run by tests/test_gpu_qsf.py against libsofren2_gb300.so.
 *
 * usage: qsf_frame <atrium|map> <model.qsf> <out.bin> <samples> [width=640] [height=360]
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#define SFT_FUNC
#include "sofren2.h"
#include "../oracle/qsf_scene.h"
#include "../oracle/map_scene.h"

int main(int argc, char** argv) {
    if (argc < 5) { fprintf(stderr, "usage: %s atrium|map model.qsf out.bin samples [width] [height]\n", argv[0]); return 2; }
    const int map = strcmp(argv[1], "map") == 0;
    const int S = atoi(argv[4]);
    const int w = argc > 5 ? atoi(argv[5]) : 640, h = argc > 6 ? atoi(argv[6]) : 360;
    sft_init(w, h, 0);
    sft_set_msaa_samples(S);
    static sft_arena arena;
    sft_arena_init(&arena, 1ull << 26);
    if (sft_model_load_qsf("/nonexistent/model.qsf", &arena)) return 5;
    if (sft_model_load_qsf(argv[0], &arena)) return 6;   /* an ELF file: wrong magic */
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
    sft_release();
    return 0;
}
