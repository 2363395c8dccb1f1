/* A fake of the GPU ABI (include/sftg.h) for testing the host runtime of include/sofren2.h on the
 * CPU.  Uploads are counted; a model's BLAS query answers with a one-slot root node holding the
 * union of the boxes of its live triangles (which is what the runtime reads from the root: the
 * model's bounds); a rendered frame's TLAS (built by the host runtime) is kept for inspection.
 * Nothing is drawn. */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "sftg.h"

struct sftg_ctx { int32_t n_tex, n_models, n_skel; };
typedef struct { float mn[3], mx[3]; int live; } fk_box;

static struct sftg_ctx fake;
static fk_box boxes[4096];
static unsigned char* tlas;
static uint32_t tlas_n, tlas_root, frames_seen;

int sftg_create(int device, sftg_ctx** out) { (void)device; memset(&fake, 0, sizeof(fake)); *out = &fake; return 0; }
void sftg_destroy(sftg_ctx* ctx) { (void)ctx; }
const char* sftg_last_error(const sftg_ctx* ctx) { (void)ctx; return "fake GPU layer"; }

int sftg_texture_upload(sftg_ctx* ctx, const uint32_t* texels, uint64_t n_texels, const sftg_texture_desc* desc, int32_t* out_index) {
    (void)texels; (void)n_texels; (void)desc;
    *out_index = ctx->n_tex++;
    return 0;
}
int sftg_material_set(sftg_ctx* ctx, int32_t index, int32_t texture, uint32_t base_color, float shininess) {
    (void)ctx; (void)index; (void)texture; (void)base_color; (void)shininess;
    return 0;
}

static int upload(sftg_ctx* ctx, const sftg_model_desc* d, int32_t* out) {
    const int32_t id = ctx->n_models++;
    fk_box b = { { 1e30f, 1e30f, 1e30f }, { -1e30f, -1e30f, -1e30f }, 0 };
    for (uint32_t k = 0; k < d->mesh_count; k++)
        for (uint32_t j = 0; j < d->meshes[k].meshlet_count; j++) {
            const uint8_t* in = d->meshes[k].inds + (size_t)j * 512;
            const float* at = d->meshes[k].attr + (size_t)j * 640;
            for (uint32_t t = 0; t < 128; t++) {
                const uint32_t bt = t >> 3, l = t & 7;
                const uint32_t i0 = in[bt * 32 + l], i1 = in[bt * 32 + 8 + l], i2 = in[bt * 32 + 16 + l];
                if (i0 == i1 && i1 == i2) continue;
                for (int a = 0; a < 3; a++) {
                    const float p0 = at[a * 64 + i0], p1 = at[a * 64 + i1], p2 = at[a * 64 + i2];
                    const float m12 = p1 < p2 ? p1 : p2, x12 = p1 > p2 ? p1 : p2;
                    const float mn = p0 < m12 ? p0 : m12, mx = p0 > x12 ? p0 : x12;
                    if (mn < b.mn[a]) b.mn[a] = mn;
                    if (mx > b.mx[a]) b.mx[a] = mx;
                }
                b.live = 1;
            }
        }
    if (id >= 0 && id < 4096) boxes[id] = b;
    *out = id;
    return 0;
}
int sftg_model_upload(sftg_ctx* ctx, const sftg_model_desc* desc, int32_t* out_model) { return upload(ctx, desc, out_model); }
int sftg_model_upload_transient(sftg_ctx* ctx, const sftg_model_desc* desc, int32_t* out_model) { return upload(ctx, desc, out_model); }
void sftg_transient_reset(sftg_ctx* ctx) { (void)ctx; }

int sftg_model_blas(sftg_ctx* ctx, int32_t model, uint32_t first, uint32_t count, void* dst, uint32_t* out_count, uint32_t* out_root) {
    (void)ctx; (void)first;
    const int live = model >= 0 && model < 4096 && boxes[model].live;
    if (out_count) *out_count = live ? 1u : 0u;
    if (out_root) *out_root = 0;
    if (dst && count && live) {   /* sft_bvh_node: mn[3][8], mx[3][8], child[8], count, leaf */
        unsigned char node[256];
        float f[48];
        uint32_t child[8];
        memset(node, 0, sizeof(node));
        for (int i = 0; i < 48; i++) f[i] = i < 24 ? 1e30f : -1e30f;
        for (int a = 0; a < 3; a++) { f[a * 8] = boxes[model].mn[a]; f[24 + a * 8] = boxes[model].mx[a]; }
        for (int i = 0; i < 8; i++) child[i] = 0xFFFFFFFFu;
        memcpy(node, f, 192); memcpy(node + 192, child, 32);
        node[224] = 1;
        memcpy(dst, node, 256);
    }
    return 0;
}

static int capture(const sftg_frame_desc* f) {
    free(tlas); tlas = NULL; tlas_n = 0;
    if (f->tlas_nodes && f->tlas_count) {
        tlas = (unsigned char*)malloc((size_t)f->tlas_count * 256);
        memcpy(tlas, f->tlas_nodes, (size_t)f->tlas_count * 256);
        tlas_n = f->tlas_count;
    }
    tlas_root = f->tlas_root;
    frames_seen++;
    return 0;
}
int sftg_frame_render(sftg_ctx* ctx, const sftg_frame_desc* frame, uint32_t* color, int32_t pitch_bytes, sftg_debug_out* dbg) {
    (void)ctx; (void)color; (void)pitch_bytes; (void)dbg;
    return capture(frame);
}
int sftg_frames_render(sftg_ctx* ctx, const sftg_frame_desc* frames, uint32_t n_views, uint32_t* const* colors, const int32_t* pitch_bytes,
                       const uint32_t** out_device_colors) {
    (void)ctx; (void)colors; (void)pitch_bytes; (void)out_device_colors;
    return n_views ? capture(&frames[0]) : 0;
}
int sftg_frames_submit(sftg_ctx* ctx, uint32_t lane, const sftg_frame_desc* frames, uint32_t n_views, uint32_t* const* colors,
                       const int32_t* pitch_bytes) {
    (void)ctx; (void)lane; (void)colors; (void)pitch_bytes;
    return n_views ? capture(&frames[0]) : 0;
}
int sftg_lane_done(sftg_ctx* ctx, uint32_t lane) { (void)ctx; (void)lane; return 1; }
int sftg_lane_wait(sftg_ctx* ctx, uint32_t lane) { (void)ctx; (void)lane; return 0; }
int sftg_autotune(sftg_ctx* ctx, const sftg_frame_desc* frames, uint32_t n_views, int32_t reps, sftg_tuning* out) {
    (void)ctx; (void)frames; (void)n_views; (void)reps; (void)out;
    return 0;
}
int sftg_skeleton_upload(sftg_ctx* ctx, const sftg_bone_desc* bones, uint32_t bone_count, const sftg_animation_desc* anims,
                         uint32_t anim_count, int32_t* out_skeleton) {
    (void)bones; (void)bone_count; (void)anims; (void)anim_count;
    *out_skeleton = ctx->n_skel++;
    return 0;
}
int sftg_pose_eval(sftg_ctx* ctx, const sftg_pose_request* requests, uint32_t n, float* posed, float* global) {
    (void)ctx; (void)requests; (void)n; (void)posed; (void)global;
    return 0;
}
int sftg_raycast(sftg_ctx* ctx, const sftg_ray* rays, uint32_t n, sftg_ray_hit* hits) {
    (void)ctx; (void)rays;
    memset(hits, 0, (size_t)n * sizeof(sftg_ray_hit));
    return 0;
}
int sftg_last_timings(const sftg_ctx* ctx, float* out5) { (void)ctx; memset(out5, 0, 20); return 0; }
int sftg_last_launch_count(const sftg_ctx* ctx) { (void)ctx; return 0; }
void* sftg_stream(const sftg_ctx* ctx) { (void)ctx; return NULL; }

/* the TLAS of the last frame rendered: node count (images copied to out when it holds them) */
uint32_t fk_tlas(unsigned char* out, uint32_t cap_nodes, uint32_t* root, uint32_t* frames) {
    if (out && cap_nodes >= tlas_n && tlas) memcpy(out, tlas, (size_t)tlas_n * 256);
    if (root) *root = tlas_root;
    if (frames) *frames = frames_seen;
    return tlas_n;
}
