/*
 * The SoA math helpers of include/sofren2.h (sofren2.c:780-792) on groups of eight lanes read
 * from a file; writes every result in the layout of oracle/soa_harness.c, which runs the
 * reference's own helpers on the same file.
 *
 * usage: soa_math <in.bin> <out.bin>
 */
#define SFT_FUNC
#include "sofren2.h"

#define IN_F (3 * 8 + 3 * 8 + 8 + 16)
#define OUT_V (3 + 3 + 3 + 1 + 3 + 1 + 1 + 3 + 3 + 3 + 3 + 16)

static vf32 ld(const f32* p) { vf32 v; memcpy(&v, p, 32); return v; }
static void put(f32** o, vf32 v) { memcpy(*o, &v, 32); *o += 8; }
static void put3(f32** o, sftvvec v) { put(o, v.x); put(o, v.y); put(o, v.z); }

int main(int argc, char** argv) {
    if (argc < 3) { fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]); return 2; }
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 3;
    fseek(f, 0, SEEK_END); const long n = ftell(f); fseek(f, 0, SEEK_SET);
    const long groups = n / (long)(IN_F * 4);
    f32* in = (f32*)malloc((size_t)n + 4);
    if (fread(in, 1, (size_t)n, f) != (size_t)n) return 3;
    fclose(f);
    f32* out = (f32*)malloc((size_t)groups * OUT_V * 8 * 4 + 4);
    f32* o = out;
    for (long g = 0; g < groups; g++) {
        const f32* p = in + g * IN_F;
        sftvvec a = { ld(p), ld(p + 8), ld(p + 16) };
        sftvvec b = { ld(p + 24), ld(p + 32), ld(p + 40) };
        const vf32 s = ld(p + 48);
        sftmat m; memcpy(&m, p + 56, 64);
        const sftvmat vm = sft_vm_broadcast(m);
        put3(&o, sft_vv_add(a, b));
        put3(&o, sft_vv_sub(a, b));
        put3(&o, sft_vv_scale(a, s));
        put(&o, sft_vv_dot(a, b));
        put3(&o, sft_vv_cross(a, b));
        put(&o, sft_vv_length2(a));
        put(&o, sft_vv_length(a));
        put3(&o, sft_vv_norm(a));
        put3(&o, sft_vv_norm_fast(a));
        put3(&o, sft_vv_transform(a, vm));
        put3(&o, sft_vv_transform_dir(a, vm));
        for (int i = 0; i < 4; i++) for (int j = 0; j < 4; j++) put(&o, vm.m[i][j]);
    }
    f = fopen(argv[2], "wb");
    if (!f) return 4;
    fwrite(out, 4, (size_t)(o - out), f);
    fclose(f);
    free(in); free(out);
    return 0;
}
