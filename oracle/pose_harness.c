/*
 * Test infrastructure: runs the unmodified reference's sft_pose_update (sofren2.c:8952-9108)
 * on a pose blob (format in sft_oracle.c, sfto_pose_eval) and writes, per request, the posed
 * bone matrices then the global matrices (f32, bones x 16 each).  Built by oracle/Makefile
 * from the reference sources where they lie.
 *
 * usage: pose_harness <pose.bin> <out.bin>
 */
#define _GNU_SOURCE
#define SFT_IMPL
#define SFT_NO_DEBUG
#include "sofren2.c"

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
    if (argc < 3) { fprintf(stderr, "usage: %s pose.bin out.bin\n", argv[0]); return 2; }
    size_t n = 0;
    unsigned char* blob = slurp(argv[1], &n);
    if (!blob || n < 8 || memcmp(blob, "SFTP", 4)) return 3;
    const unsigned char* p = blob + 4;
    u32 nb; memcpy(&nb, p, 4); p += 4;
    struct sft_model m; memset(&m, 0, sizeof(m));
    m.skeleton.bone_count = (i32)nb;
    m.skeleton.bones = (struct sft_bone*)calloc(nb, sizeof(struct sft_bone));
    for (u32 b = 0; b < nb; b++) {
        struct sft_bone* B = &m.skeleton.bones[b];
        memcpy(&B->inverse_bind_matrix, p, 64); memcpy(&B->local_bind_matrix, p + 64, 64);
        memcpy(&B->parent_ind, p + 128, 4);
        memcpy(&B->base_t, p + 132, 12); memcpy(&B->base_r, p + 144, 16); memcpy(&B->base_s, p + 160, 12);
        p += 172;
    }
    u32 na; memcpy(&na, p, 4); p += 4;
    m.anim_count = (i32)na;
    m.animations = (struct sft_animation*)calloc(na + 1, sizeof(struct sft_animation));
    for (u32 a = 0; a < na; a++) {
        struct sft_animation* A = &m.animations[a];
        u32 ns, nc;
        memcpy(&A->duration, p, 4); memcpy(&ns, p + 4, 4); memcpy(&nc, p + 8, 4); p += 12;
        A->sampler_count = (i32)ns; A->channel_count = (i32)nc;
        A->samplers = (struct sft_anim_sampler*)calloc(ns + 1, sizeof(struct sft_anim_sampler));
        A->channels = (struct sft_anim_channel*)calloc(nc + 1, sizeof(struct sft_anim_channel));
        for (u32 k = 0; k < ns; k++) {
            u32 cnt, step; memcpy(&cnt, p, 4); memcpy(&step, p + 4, 4); p += 8;
            A->samplers[k].count = (i32)cnt; A->samplers[k].is_step = (u8)step;
            A->samplers[k].inputs = (f32*)malloc(cnt * 4); memcpy(A->samplers[k].inputs, p, cnt * 4); p += cnt * 4;
            A->samplers[k].outputs = (f32*)malloc(cnt * 16); memcpy(A->samplers[k].outputs, p, cnt * 16); p += cnt * 16;
        }
        for (u32 k = 0; k < nc; k++) {
            i32 v[3]; memcpy(v, p, 12); p += 12;
            A->channels[k].sampler_ind = v[0]; A->channels[k].node_ind = v[1]; A->channels[k].path = (enum sft_anim_path)v[2];
        }
    }
    u32 nr; memcpy(&nr, p, 4); p += 4;
    sft_pose pose; memset(&pose, 0, sizeof(pose));
    pose.model = &m;
    pose.global_matrices = (sftmat*)calloc(nb, sizeof(sftmat));
    pose.posed_bone_matrices = (sftmat*)calloc(nb, sizeof(sftmat));
    FILE* out = fopen(argv[2], "wb");
    if (!out) return 4;
    for (u32 r = 0; r < nr; r++) {
        i32 ai; f32 t; memcpy(&ai, p + 8 * r, 4); memcpy(&t, p + 8 * r + 4, 4);
        memset(pose.global_matrices, 0, nb * sizeof(sftmat));
        memset(pose.posed_bone_matrices, 0, nb * sizeof(sftmat));
        sft_pose_update(&pose, ai, t);
        fwrite(pose.posed_bone_matrices, sizeof(sftmat), nb, out);
        fwrite(pose.global_matrices, sizeof(sftmat), nb, out);
    }
    fclose(out);
    return 0;
}
