/*
 * Renders the dynamic-mesh scene (oracle/dmesh_scene.h) through this library's sft_* API, the
 * same calls oracle/dmesh_harness.c makes on the reference, and writes each frame's colour.
 * Built and run by tests/test_gpu_dmesh.py against libsofren2_gb300.so.
 *
 * usage: dmesh_frame <out.bin> <samples> [width=640] [height=360]
 */
#include <stdio.h>
#include <stdlib.h>
#define SFT_FUNC
#include "sofren2.h"
#include "../oracle/dmesh_scene.h"

int main(int argc, char** argv) {
    if (argc < 3) { fprintf(stderr, "usage: %s out.bin samples [width] [height]\n", argv[0]); return 2; }
    const int S = atoi(argv[2]);
    const int w = argc > 3 ? atoi(argv[3]) : 640, h = argc > 4 ? atoi(argv[4]) : 360;
    sft_init(w, h, 0);
    sft_set_msaa_samples(S);
    dmesh_scene_setup();
    u32* color = (u32*)calloc((size_t)w * h, 4);
    FILE* out = fopen(argv[1], "wb");
    if (!out) return 3;
    for (int f = 0; f < DMESH_SCENE_FRAMES; f++) {
        dmesh_scene_frame(f, color, w, h);
        fwrite(color, 4, (size_t)w * h, out);
    }
    fclose(out);
    sft_release();
    return 0;
}
