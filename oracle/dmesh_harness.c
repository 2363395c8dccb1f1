/*
 * Test infrastructure: renders the dynamic-mesh scene (oracle/dmesh_scene.h) with the
 * unmodified reference and writes each frame's colour buffer (u32 ARGB, width * height).
 * MSAA is compile-time in the reference (SFT_USE_AA / SFT_AA_SAMPLES).
 *
 * usage: dmesh_harness <out.bin> [width=640] [height=360]
 */
#define _GNU_SOURCE
#define SFT_IMPL
#define SFT_NO_DEBUG
#include "sofren2.c"
#include "dmesh_scene.h"

int main(int argc, char** argv) {
    if (argc < 2) { fprintf(stderr, "usage: %s out.bin [width] [height]\n", argv[0]); return 2; }
    const int w = argc > 2 ? atoi(argv[2]) : 640, h = argc > 3 ? atoi(argv[3]) : 360;
    sft_init(w, h, 1);
    dmesh_scene_setup();
    u32* color = (u32*)calloc((size_t)w * h, 4);
    FILE* out = fopen(argv[1], "wb");
    if (!out) return 3;
    for (int f = 0; f < DMESH_SCENE_FRAMES; f++) {
        dmesh_scene_frame(f, color, w, h);
        fwrite(color, 4, (size_t)w * h, out);
    }
    fclose(out);
    return 0;
}
