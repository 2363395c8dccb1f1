/*
 * The load-time builders of include/sofren2.h (sft_mesh_build_meshlets,
 * sft_model_fit_shadow_proxies) on the raw meshes of an input file in oracle/build_harness.c's
 * format, writing the same output layout (meshlets per mesh, then the proxies), so the two can be
 * compared byte for byte.  The proxies need the model's BLAS: node images from a file (a BLAS built
 * from these meshlets), or none (then no proxies are written).  Compiled with tests/sftg_fake.c:
 * nothing here touches a GPU.
 *
 * usage: model_build <in.bin> <out.bin> [<blas.bin> <root>]
 */
#define SFT_IMPL
#define SFT_NO_DEBUG
#include "sofren2.h"

static const unsigned char* rd(const unsigned char** p, size_t n) { const unsigned char* r = *p; *p += n; return r; }
static u32 rd32(const unsigned char** p) { u32 v; memcpy(&v, rd(p, 4), 4); return v; }
static unsigned char* slurp(const char* path, size_t* n) {
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END); *n = (size_t)ftell(f); fseek(f, 0, SEEK_SET);
    unsigned char* b = (unsigned char*)malloc(*n + 16);
    if (fread(b, 1, *n, f) != *n) { fclose(f); free(b); return NULL; }
    fclose(f);
    return b;
}

int main(int argc, char** argv) {
    if (argc < 3) { fprintf(stderr, "usage: %s in.bin out.bin [blas.bin root]\n", argv[0]); return 2; }
    size_t n_in = 0;
    unsigned char* blob = slurp(argv[1], &n_in);
    if (!blob) return 3;
    const unsigned char* p = blob;
    if (memcmp(rd(&p, 4), "SFTR", 4) || rd32(&p) != 1) return 4;
    const u32 seed = rd32(&p);
    const i32 budget = (i32)rd32(&p);
    const u32 nb = rd32(&p);
    sft_raw_bone* bones = (sft_raw_bone*)calloc(nb + 1, sizeof(sft_raw_bone));
    for (u32 b = 0; b < nb; b++) { bones[b].parent_ind = (i32)rd32(&p); memcpy(&bones[b].bind_pos, rd(&p, 12), 12); }
    const u32 nm = rd32(&p);
    sft_mesh_data* md = (sft_mesh_data*)calloc(nm + 1, sizeof(sft_mesh_data));
    FILE* o = fopen(argv[2], "wb");
    if (!o) return 5;
    srand(seed);
    for (u32 mi = 0; mi < nm; mi++) {
        sft_raw_mesh r;
        memset(&r, 0, sizeof(r));
        r.vertex_count = rd32(&p); r.triangle_count = rd32(&p);
        const u32 skinned = rd32(&p), nv = r.vertex_count, nt = r.triangle_count;
        r.pos = (const f32*)rd(&p, (size_t)nv * 12);
        r.nrm = (const f32*)rd(&p, (size_t)nv * 12);
        r.uv = (const f32*)rd(&p, (size_t)nv * 8);
        if (skinned) { r.joints = (const u16*)rd(&p, (size_t)nv * 8); r.weights = rd(&p, (size_t)nv * 4); }
        r.indices = (const i32*)rd(&p, (size_t)nt * 12);
        r.material = SFT_INVALID_HANDLE;
        const u32 cap = nt ? nt : 1;
        f32* attr = (f32*)calloc((size_t)cap * 640, 4);
        u8* inds = (u8*)calloc((size_t)cap * 512, 1);
        f32* cull = (f32*)calloc((size_t)cap * 8, 4);
        u16* jn = skinned ? (u16*)calloc((size_t)cap * 256, 2) : NULL;
        u8* wt = skinned ? (u8*)calloc((size_t)cap * 256, 1) : NULL;
        i32* cb = skinned ? (i32*)calloc(cap, 4) : NULL;
        const u32 n = sft_mesh_build_meshlets(&r, nb, cap, attr, inds, cull, jn, wt, cb);
        fwrite(&n, 4, 1, o);
        fwrite(attr, 4, (size_t)n * 640, o);
        fwrite(inds, 1, (size_t)n * 512, o);
        fwrite(cull, 4, (size_t)n * 8, o);
        if (skinned) { fwrite(jn, 2, (size_t)n * 256, o); fwrite(wt, 1, (size_t)n * 256, o); fwrite(cb, 4, n, o); }
        md[mi].meshlet_count = n; md[mi].attr = attr; md[mi].inds = inds; md[mi].cull = cull;
        md[mi].joints = jn; md[mi].weights = wt; md[mi].culling_bones = cb;
    }
    u32 np = 0;
    sft_shadow_proxy* px = NULL;
    if (argc >= 5) {
        size_t nbytes = 0;
        unsigned char* blas = slurp(argv[3], &nbytes);
        const u32 root = (u32)strtoul(argv[4], NULL, 10);
        if (!blas) return 6;
        np = sft_model_fit_shadow_proxies(md, nm, blas, (u32)(nbytes / 256), root, bones, nb, budget, NULL, 0);
        px = (sft_shadow_proxy*)calloc(np + 1, sizeof(sft_shadow_proxy));
        sft_model_fit_shadow_proxies(md, nm, blas, (u32)(nbytes / 256), root, bones, nb, budget, px, np);
        free(blas);
    }
    fwrite(&np, 4, 1, o);
    for (u32 i = 0; i < np; i++) {
        const f32 v[7] = { px[i].posa.x, px[i].posa.y, px[i].posa.z, px[i].posb.x, px[i].posb.y, px[i].posb.z, px[i].radius };
        fwrite(v, 4, 7, o); fwrite(&px[i].bone_ind, 4, 1, o);
    }
    fclose(o);
    return 0;
}
