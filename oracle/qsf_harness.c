/*
 * Test infrastructure: loads a QSF2 file with the unmodified reference's sft_model_load_qsf,
 * renders the QSF scene (oracle/qsf_scene.h) and writes each frame's colour buffer (u32 ARGB,
 * width * height).  MSAA is compile-time in the reference (SFT_USE_AA / SFT_AA_SAMPLES).
 *
 * usage: qsf_harness <model.qsf> <out.bin> [width=640] [height=360]
 */
#define _GNU_SOURCE
#define SFT_IMPL
#define SFT_NO_DEBUG
#include "sofren2.c"
#include "qsf_scene.h"

int main(int argc, char** argv) {
    if (argc < 3) { fprintf(stderr, "usage: %s model.qsf out.bin [width] [height]\n", argv[0]); return 2; }
    const int w = argc > 3 ? atoi(argv[3]) : 640, h = argc > 4 ? atoi(argv[4]) : 360;
    sft_init(w, h, 1);
    static sft_arena arena;
    sft_arena_init(&arena, 1ull << 30);
    if (!qsf_scene_setup(argv[1], &arena)) return 4;
    u32* color = (u32*)calloc((size_t)w * h, 4);
    FILE* out = fopen(argv[2], "wb");
    if (!out) return 3;
    for (int f = 0; f < QSF_SCENE_FRAMES; f++) {
        qsf_scene_frame(f, color, w, h);
        fwrite(color, 4, (size_t)w * h, out);
    }
    fclose(out);
    return 0;
}
