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
    {   /* the same file cut short, at several points: NULL, no crash */
        FILE* f = fopen(argv[2], "rb");
        if (!f) return 7;
        fseek(f, 0, SEEK_END);
        const long size = ftell(f);
        fseek(f, 0, SEEK_SET);
        unsigned char* buf = (unsigned char*)malloc((size_t)size);
        if (fread(buf, 1, (size_t)size, f) != (size_t)size) return 7;
        fclose(f);
        char cut[4096];
        snprintf(cut, sizeof(cut), "%s.cut", argv[3]);
        /* cut points inside the model data; near the end only when no game-data section (which
         * the loader does not read) follows the model */
        unsigned long long game_off = 0;
        memcpy(&game_off, buf + 8, 8);
        const long points[6] = { 10, 40, size / 3, size / 2, size - 300, size - 1 };
        const int n_points = game_off ? 4 : 6;
        for (int k = 0; k < n_points; k++) {
            FILE* o = fopen(cut, "wb");
            if (!o) return 7;
            fwrite(buf, 1, (size_t)points[k], o);
            fclose(o);
            if (sft_model_load_qsf(cut, &arena)) return 8;
        }
        remove(cut);
        free(buf);
    }
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
