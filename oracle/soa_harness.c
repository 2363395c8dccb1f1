/*
 * Test infrastructure: runs the unmodified reference's SoA math helpers (sofren2.c:1921-2060,
 * declared at 780-792) in its AVX2 build on groups of eight lanes read from a file, and writes
 * every result.  Built by oracle/Makefile from the reference sources where they lie; its
 * counterpart on the product side is tests/soa_math.c, which reads the same input file and
 * writes the same layout through include/sofren2.h.
 *
 * input, per group (f32): a.x a.y a.z (8 each), b.x b.y b.z (8 each), s (8), m (16, row-major)
 * output, per group (f32, 8 lanes per vector component): add(3) sub(3) scale(3) dot(1) cross(3)
 * length2(1) length(1) norm(3) norm_fast(3) transform(3) transform_dir(3) broadcast(16)
 *
 * usage: soa_harness <in.bin> <out.bin>
 */
#define _GNU_SOURCE
#define SFT_IMPL
#define SFT_NO_DEBUG
#include "sofren2.c"

#define IN_F (3 * 8 + 3 * 8 + 8 + 16)
#define OUT_V (3 + 3 + 3 + 1 + 3 + 1 + 1 + 3 + 3 + 3 + 3 + 16)

static void put(f32** o, vf32 v) { sft_vf_storeu(*o, v); *o += 8; }
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
        sftvvec a = { sft_vf_loadu(p), sft_vf_loadu(p + 8), sft_vf_loadu(p + 16) };
        sftvvec b = { sft_vf_loadu(p + 24), sft_vf_loadu(p + 32), sft_vf_loadu(p + 40) };
        const vf32 s = sft_vf_loadu(p + 48);
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
    return 0;
}
