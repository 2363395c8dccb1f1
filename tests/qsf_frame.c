/*
 * Loads a QSF2 file with this library's sft_model_load_qsf and renders the QSF scene
 * (oracle/qsf_scene.h) through the sft_* API, the same calls oracle/qsf_harness.c makes on the
 * reference, writing each frame's colour.  Also checks the loader's soft failures: a missing
 * file and a file with the wrong magic give NULL.  Built and run by tests/test_gpu_qsf.py
 * against libsofren2_gb300.so.
 *
 * usage: qsf_frame <model.qsf> <out.bin> <samples> [width=640] [height=360]
 */
#include <stdio.h>
#include <stdlib.h>
#define SFT_FUNC
#include "sofren2.h"
#include "../oracle/qsf_scene.h"

int main(int argc, char** argv) {
    if (argc < 4) { fprintf(stderr, "usage: %s model.qsf out.bin samples [width] [height]\n", argv[0]); return 2; }
    const int S = atoi(argv[3]);
    const int w = argc > 4 ? atoi(argv[4]) : 640, h = argc > 5 ? atoi(argv[5]) : 360;
    sft_init(w, h, 0);
    sft_set_msaa_samples(S);
    static sft_arena arena;
    sft_arena_init(&arena, 1ull << 26);
    if (sft_model_load_qsf("/nonexistent/model.qsf", &arena)) return 5;
    if (sft_model_load_qsf(argv[0], &arena)) return 6;   /* an ELF file: wrong magic */
    if (!qsf_scene_setup(argv[1], &arena)) return 4;
    u32* color = (u32*)calloc((size_t)w * h, 4);
    FILE* out = fopen(argv[2], "wb");
    if (!out) return 3;
    for (int f = 0; f < QSF_SCENE_FRAMES; f++) {
        qsf_scene_frame(f, color, w, h);
        fwrite(color, 4, (size_t)w * h, out);
    }
    fclose(out);
    sft_release();
    return 0;
}
