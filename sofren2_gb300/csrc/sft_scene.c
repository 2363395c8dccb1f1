/*
 * Scene player: loads an SFTS scene blob (layout in sofren2_gb300/scenes.py) and renders its
 * frames through the public sft_* API only, the way an application's frame loop does
 * (lights, sft_set_color_buffer, sft_frame_begin, sft_set_camera, sft_draw_instance,
 * sft_present, sft_frame_end).  Used by the Python runtime, the tests and bench.py.
 */
#define SFT_FUNC __attribute__((visibility("default")))
#include "../../include/sofren2.h"

#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define SFTX_EXPORT __attribute__((visibility("default")))

typedef struct { const uint8_t* p; const uint8_t* e; int bad; } sftx_cur;
static const void* sftx_take(sftx_cur* c, size_t n) {
    if (c->bad || (size_t)(c->e - c->p) < n) { c->bad = 1; return NULL; }
    const void* r = c->p; c->p += n; return r;
}
static uint32_t sftx_u32(sftx_cur* c) { const void* q = sftx_take(c, 4); uint32_t v = 0; if (q) memcpy(&v, q, 4); return v; }
static float sftx_f32(sftx_cur* c) { const void* q = sftx_take(c, 4); float v = 0; if (q) memcpy(&v, q, 4); return v; }

typedef struct {
    uint32_t width, height;
    const float* cam; const float* view; const float* proj; const float* ambient;
    float lm_brightness; uint32_t clear, clear_color, shadows;
    uint32_t n_dir; const float* dir;       /* 7 floats each */
    uint32_t n_point; const float* point;   /* 8 floats each */
    uint32_t n_inst; uint32_t* inst_model; const float** inst_T; uint32_t* inst_nb; const float** inst_bones;
} sftx_frame;

typedef struct {
    uint8_t* data;
    uint32_t n_tex, n_mat, n_model, n_frame;
    sft_tex_handle* tex; sft_mat_handle* mat; sft_model** model;
    sftx_frame* frames;
    sftmat* bone_scratch; uint32_t bone_cap;
} sftx_scene;

SFTX_EXPORT void sftx_scene_free(void* p);

SFTX_EXPORT void* sftx_scene_load(const uint8_t* blob, uint64_t size) {
    sftx_scene* s = (sftx_scene*)calloc(1, sizeof(sftx_scene));
    s->data = (uint8_t*)malloc(size + 16);
    memcpy(s->data, blob, size);
    sftx_cur c = { s->data, s->data + size, 0 };
    if (sftx_u32(&c) != 0x53544653u || sftx_u32(&c) != 1u) { sftx_scene_free(s); return NULL; }
    s->n_tex = sftx_u32(&c);
    s->tex = (sft_tex_handle*)calloc(s->n_tex + 1, sizeof(sft_tex_handle));
    for (uint32_t i = 0; i < s->n_tex && !c.bad; i++) {
        const uint32_t w = sftx_u32(&c), h = sftx_u32(&c);
        const uint32_t* px = (const uint32_t*)sftx_take(&c, (size_t)w * h * 4);
        if (!px) break;
        uint32_t* tmp = (uint32_t*)malloc((size_t)w * h * 4);
        memcpy(tmp, px, (size_t)w * h * 4);
        s->tex[i] = sft_texture_create((i32)w, (i32)h, tmp);
        free(tmp);
    }
    s->n_mat = sftx_u32(&c);
    s->mat = (sft_mat_handle*)calloc(s->n_mat + 1, sizeof(sft_mat_handle));
    for (uint32_t i = 0; i < s->n_mat && !c.bad; i++) {
        const int32_t t = (int32_t)sftx_u32(&c); const uint32_t base = sftx_u32(&c); const float shin = sftx_f32(&c);
        s->mat[i] = sft_material_create(t >= 0 ? s->tex[t] : SFT_INVALID_HANDLE, base, shin);
    }
    s->n_model = sftx_u32(&c);
    s->model = (sft_model**)calloc(s->n_model + 1, sizeof(sft_model*));
    for (uint32_t i = 0; i < s->n_model && !c.bad; i++) {
        const uint32_t n_meshes = sftx_u32(&c), bone_count = sftx_u32(&c), n_lm = sftx_u32(&c);
        const int32_t* lms = (const int32_t*)sftx_take(&c, 4u * n_lm);
        sft_tex_handle* lmh = (sft_tex_handle*)calloc(n_lm + 1, sizeof(sft_tex_handle));
        for (uint32_t k = 0; k < n_lm && lms; k++) { int32_t q; memcpy(&q, lms + k, 4); lmh[k] = q >= 0 ? s->tex[q] : SFT_INVALID_HANDLE; }
        const uint32_t n_prox = sftx_u32(&c);
        sft_shadow_proxy* px = (sft_shadow_proxy*)calloc(n_prox + 1, sizeof(sft_shadow_proxy));
        for (uint32_t p = 0; p < n_prox && !c.bad; p++) {
            float v[7];
            for (int k = 0; k < 7; k++) v[k] = sftx_f32(&c);
            px[p].posa.x = v[0]; px[p].posa.y = v[1]; px[p].posa.z = v[2];
            px[p].posb.x = v[3]; px[p].posb.y = v[4]; px[p].posb.z = v[5];
            px[p].radius = v[6]; px[p].bone_ind = sftx_u32(&c);
        }
        sft_mesh_data* md = (sft_mesh_data*)calloc(n_meshes + 1, sizeof(sft_mesh_data));
        void** owned = (void**)calloc(8 * (n_meshes + 1), sizeof(void*));
        for (uint32_t k = 0; k < n_meshes && !c.bad; k++) {
            const uint32_t n = sftx_u32(&c); const int32_t mat = (int32_t)sftx_u32(&c);
            const uint32_t page = sftx_u32(&c), skin = sftx_u32(&c);
            float* attr = (float*)malloc((size_t)n * 2560 + 16); uint8_t* inds = (uint8_t*)malloc((size_t)n * 512 + 16);
            float* cull = (float*)malloc((size_t)n * 32 + 16); int32_t* bones = (int32_t*)malloc((size_t)n * 4 + 16);
            uint16_t* js = skin ? (uint16_t*)malloc((size_t)n * 512 + 16) : NULL; uint8_t* ws = skin ? (uint8_t*)malloc((size_t)n * 256 + 16) : NULL;
            for (uint32_t j = 0; j < n && !c.bad; j++) {
                const void* a = sftx_take(&c, 2560); if (a) memcpy(attr + (size_t)j * 640, a, 2560);
                if (skin) {
                    const void* jj = sftx_take(&c, 512); if (jj) memcpy(js + (size_t)j * 256, jj, 512);
                    const void* ww = sftx_take(&c, 256); if (ww) memcpy(ws + (size_t)j * 256, ww, 256);
                }
                const void* ii = sftx_take(&c, 512); if (ii) memcpy(inds + (size_t)j * 512, ii, 512);
                const void* cc = sftx_take(&c, 32); if (cc) memcpy(cull + (size_t)j * 8, cc, 32);
                bones[j] = (int32_t)sftx_u32(&c);
            }
            md[k].meshlet_count = n; md[k].attr = attr; md[k].inds = inds; md[k].cull = cull;
            md[k].joints = js; md[k].weights = ws; md[k].culling_bones = skin ? bones : NULL;
            md[k].material = mat >= 0 ? s->mat[mat] : SFT_INVALID_HANDLE;
            md[k].lightmap_page = page;
            owned[8 * k + 0] = attr; owned[8 * k + 1] = inds; owned[8 * k + 2] = cull; owned[8 * k + 3] = bones;
            owned[8 * k + 4] = js; owned[8 * k + 5] = ws;
        }
        if (!c.bad) s->model[i] = sft_model_create(md, n_meshes, px, n_prox, bone_count, lmh, n_lm, NULL);
        for (uint32_t k = 0; k < 8 * (n_meshes + 1); k++) free(owned[k]);
        free(owned); free(md); free(px); free(lmh);
    }
    s->n_frame = sftx_u32(&c);
    s->frames = (sftx_frame*)calloc(s->n_frame + 1, sizeof(sftx_frame));
    for (uint32_t i = 0; i < s->n_frame && !c.bad; i++) {
        sftx_frame* f = &s->frames[i];
        f->width = sftx_u32(&c); f->height = sftx_u32(&c);
        f->cam = (const float*)sftx_take(&c, 12); f->view = (const float*)sftx_take(&c, 64); f->proj = (const float*)sftx_take(&c, 64);
        f->ambient = (const float*)sftx_take(&c, 12); f->lm_brightness = sftx_f32(&c);
        f->clear = sftx_u32(&c); f->clear_color = sftx_u32(&c); f->shadows = sftx_u32(&c);
        f->n_dir = sftx_u32(&c); f->dir = (const float*)sftx_take(&c, 28u * f->n_dir);
        f->n_point = sftx_u32(&c); f->point = (const float*)sftx_take(&c, 32u * f->n_point);
        f->n_inst = sftx_u32(&c);
        f->inst_model = (uint32_t*)calloc(f->n_inst + 1, 4); f->inst_T = (const float**)calloc(f->n_inst + 1, sizeof(float*));
        f->inst_nb = (uint32_t*)calloc(f->n_inst + 1, 4); f->inst_bones = (const float**)calloc(f->n_inst + 1, sizeof(float*));
        for (uint32_t k = 0; k < f->n_inst && !c.bad; k++) {
            f->inst_model[k] = sftx_u32(&c); f->inst_T[k] = (const float*)sftx_take(&c, 64);
            f->inst_nb[k] = sftx_u32(&c);
            f->inst_bones[k] = f->inst_nb[k] ? (const float*)sftx_take(&c, 64u * f->inst_nb[k]) : NULL;
        }
    }
    if (c.bad) { sftx_scene_free(s); return NULL; }
    return s;
}

SFTX_EXPORT uint32_t sftx_scene_frame_count(const void* p) { return p ? ((const sftx_scene*)p)->n_frame : 0; }
SFTX_EXPORT uint32_t sftx_scene_frame_size(const void* p, uint32_t frame, uint32_t* w, uint32_t* h) {
    const sftx_scene* s = (const sftx_scene*)p;
    if (!s || frame >= s->n_frame) return 0;
    *w = s->frames[frame].width; *h = s->frames[frame].height;
    return 1;
}

static float sftx_ld(const float* p, int i) { float v; memcpy(&v, p + i, 4); return v; }

SFTX_EXPORT int sftx_scene_render(void* p, uint32_t frame, uint32_t* color, int32_t pitch_bytes);

/* Issues one frame's API calls and sft_present into `color` (pitch in bytes), drawing at most
 * max_point_lights of the frame's point lights (the first ones). */
SFTX_EXPORT int sftx_scene_render_ex(void* p, uint32_t frame, uint32_t* color, int32_t pitch_bytes, uint32_t max_point_lights) {
    sftx_scene* s = (sftx_scene*)p;
    if (!s || frame >= s->n_frame) return -1;
    const sftx_frame* f = &s->frames[frame];
    const uint32_t n_point = f->n_point < max_point_lights ? f->n_point : max_point_lights;
    sft_resize((i32)f->width, (i32)f->height);
    sft_set_ambient_light(sftx_ld(f->ambient, 0), sftx_ld(f->ambient, 1), sftx_ld(f->ambient, 2));
    for (uint32_t l = 0; l < f->n_dir; l++) {
        const float* d = f->dir + 7 * l;
        sft_draw_directional_light(SFT_V(sftx_ld(d, 0), sftx_ld(d, 1), sftx_ld(d, 2)), sftx_ld(d, 3), sftx_ld(d, 4), sftx_ld(d, 5), sftx_ld(d, 6));
    }
    for (uint32_t l = 0; l < n_point; l++) {
        const float* q = f->point + 8 * l;
        sft_draw_point_light(SFT_V(sftx_ld(q, 0), sftx_ld(q, 1), sftx_ld(q, 2)), sftx_ld(q, 3), sftx_ld(q, 4), sftx_ld(q, 5), sftx_ld(q, 6), sftx_ld(q, 7), l);
    }
    sft_set_shadows_enabled((u8)f->shadows);
    sft_set_lightmap_brightness(f->lm_brightness);
    sft_set_clear((u8)f->clear);
    sft_set_clear_color(f->clear_color);
    sft_set_color_buffer(color, pitch_bytes);
    sft_frame_begin();
    sftmat view, proj;
    memcpy(&view, f->view, 64); memcpy(&proj, f->proj, 64);
    sft_set_camera(SFT_V(sftx_ld(f->cam, 0), sftx_ld(f->cam, 1), sftx_ld(f->cam, 2)), view, proj);
    uint32_t nb = 0;
    for (uint32_t k = 0; k < f->n_inst; k++) nb += f->inst_nb[k];
    if (nb > s->bone_cap) { s->bone_cap = nb; s->bone_scratch = (sftmat*)realloc(s->bone_scratch, (size_t)nb * sizeof(sftmat)); }
    uint32_t bo = 0;
    for (uint32_t k = 0; k < f->n_inst; k++) {
        sft_instance inst;
        memset(&inst, 0, sizeof(inst));
        inst.model = s->model[f->inst_model[k]];
        memcpy(&inst.transform, f->inst_T[k], 64);
        if (f->inst_nb[k]) {
            memcpy(s->bone_scratch + bo, f->inst_bones[k], 64u * f->inst_nb[k]);
            inst.posed_bone_matrices = s->bone_scratch + bo;
            bo += f->inst_nb[k];
        }
        sft_draw_instance(&inst);
    }
    sft_present();
    sft_frame_end();
    return 0;
}

/* Renders n (scene, frame, samples) views in one batched submission; colors (optional) holds a
 * host buffer per view (entries may be null: that view's colour stays on the device). */
SFTX_EXPORT int sftx_scene_render_batch(void* const* scenes, const uint32_t* frames, const int32_t* samples, uint32_t n,
                                        uint32_t* const* colors, const int32_t* pitch_bytes) {
    sft_batch_begin();
    for (uint32_t i = 0; i < n; i++) {
        sft_set_msaa_samples(samples[i]);
        if (sftx_scene_render(scenes[i], frames[i], colors ? colors[i] : NULL, pitch_bytes ? pitch_bytes[i] : 0)) {
            sft_batch_submit();
            return -1;
        }
    }
    return sft_batch_submit();
}

/* Renders n views as `lanes` batches queued on submission lanes 1..lanes without waiting in
 * between, so that they overlap on the GPU, then waits for all of them.  Views go to the batch
 * with the least work so far (pixels x samples), heaviest first. */
SFTX_EXPORT int sftx_scene_render_lanes(void* const* scenes, const uint32_t* frames, const int32_t* samples, uint32_t n,
                                        uint32_t* const* colors, const int32_t* pitch_bytes, uint32_t lanes) {
    if (lanes < 1 || lanes > SFTG_MAX_LANES - 1) return -1;
    uint32_t* order = (uint32_t*)malloc((size_t)(n ? n : 1) * 4);
    uint32_t* group = (uint32_t*)malloc((size_t)(n ? n : 1) * 4);
    double* cost = (double*)malloc((size_t)(n ? n : 1) * sizeof(double));
    double load[SFTG_MAX_LANES] = { 0 };
    for (uint32_t i = 0; i < n; i++) {
        uint32_t w = 0, h = 0;
        sftx_scene_frame_size(scenes[i], frames[i], &w, &h);
        cost[i] = (double)w * h * samples[i];
        order[i] = i;
    }
    for (uint32_t i = 1; i < n; i++)   /* heaviest first (insertion sort; n is small) */
        for (uint32_t j = i; j > 0 && cost[order[j]] > cost[order[j - 1]]; j--) { const uint32_t t = order[j]; order[j] = order[j - 1]; order[j - 1] = t; }
    for (uint32_t k = 0; k < n; k++) {
        uint32_t g = 0;
        for (uint32_t q = 1; q < lanes; q++) if (load[q] < load[g]) g = q;
        group[order[k]] = g;
        load[g] += cost[order[k]];
    }
    int rc = 0;
    for (uint32_t g = 0; g < lanes; g++) {
        sft_batch_begin();
        for (uint32_t i = 0; i < n; i++) {
            if (group[i] != g) continue;
            sft_set_msaa_samples(samples[i]);
            if (sftx_scene_render(scenes[i], frames[i], colors ? colors[i] : NULL, pitch_bytes ? pitch_bytes[i] : 0)) rc = -1;
        }
        if (sft_batch_submit_async(g + 1)) rc = -1;
    }
    for (uint32_t g = 0; g < lanes; g++) if (sft_batch_wait(g + 1)) rc = -1;
    free(order); free(group); free(cost);
    return rc;
}

/* Tunes the scheduling knobs on n (scene, frame, samples) views rendered as one batch. */
SFTX_EXPORT int sftx_scene_autotune_batch(void* const* scenes, const uint32_t* frames, const int32_t* samples, uint32_t n,
                                          int32_t reps) {
    sft_batch_begin();
    for (uint32_t i = 0; i < n; i++) {
        sft_set_msaa_samples(samples[i]);
        if (sftx_scene_render(scenes[i], frames[i], NULL, 0)) {
            sft_batch_submit();
            return -1;
        }
    }
    return sft_batch_autotune(reps);
}

SFTX_EXPORT int sftx_scene_render(void* p, uint32_t frame, uint32_t* color, int32_t pitch_bytes) {
    return sftx_scene_render_ex(p, frame, color, pitch_bytes, 0xFFFFFFFFu);
}

/* the i-th model of a loaded scene (for direct sft_* calls on it), or NULL */
SFTX_EXPORT void* sftx_scene_model(void* p, uint32_t i) {
    sftx_scene* s = (sftx_scene*)p;
    return (s && i < s->n_model) ? (void*)s->model[i] : NULL;
}

SFTX_EXPORT void sftx_scene_free(void* p) {
    sftx_scene* s = (sftx_scene*)p;
    if (!s) return;
    for (uint32_t i = 0; i < s->n_frame; i++) {
        free(s->frames[i].inst_model); free((void*)s->frames[i].inst_T); free(s->frames[i].inst_nb); free((void*)s->frames[i].inst_bones);
    }
    free(s->frames); free(s->tex); free(s->mat); free(s->model); free(s->bone_scratch); free(s->data); free(s);
}
