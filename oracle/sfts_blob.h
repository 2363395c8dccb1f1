/*
 * Test infrastructure (oracle side): a minimal reader for SFTS scene blobs, shared by the
 * CPU oracle and the reference harness.  The blob layout is documented in
 * sofren2_gb300/scenes.py.  Nothing in the shipped library includes this file.
 */
#ifndef SFTS_BLOB_H
#define SFTS_BLOB_H

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct { uint32_t w, h; const uint32_t* argb; } sfts_texture;
typedef struct { int32_t tex; uint32_t base_color; float shininess; } sfts_material;
typedef struct { float posa[3], posb[3], radius; uint32_t bone; } sfts_proxy;

typedef struct {
    const float* attr;      /* [10][64] x y z nx ny nz u v lu lv */
    const uint16_t* joints; /* [4][64] or NULL */
    const uint8_t* weights; /* [4][64] or NULL */
    const uint8_t* inds;    /* [512] */
    const float* cull;      /* center[3], radius, axis[3], cutoff */
    int32_t culling_bone;
} sfts_meshlet;

typedef struct {
    uint32_t meshlet_count;
    int32_t material;
    uint32_t lightmap_page;
    uint32_t has_skin;
    sfts_meshlet* meshlets;
} sfts_mesh;

typedef struct {
    uint32_t n_meshes, bone_count, n_lightmaps, n_proxies;
    const int32_t* lightmaps;
    sfts_proxy* proxies;
    sfts_mesh* meshes;
} sfts_model;

typedef struct { float dir[3], r, g, b, intensity; } sfts_dir_light;
typedef struct { float pos[3], r, g, b, intensity, radius; } sfts_point_light;
typedef struct { uint32_t model; const float* transform; uint32_t n_bones; const float* bones; } sfts_instance;

typedef struct {
    uint32_t width, height;
    const float* cam_pos; const float* view; const float* proj;
    const float* ambient; float lightmap_brightness;
    uint32_t clear, clear_color, shadows;
    uint32_t n_dir; const sfts_dir_light* dir;
    uint32_t n_point; const sfts_point_light* point;
    uint32_t n_inst; sfts_instance* inst;
} sfts_frame;

typedef struct {
    uint8_t* data; size_t size;
    uint32_t n_textures, n_materials, n_models, n_frames;
    sfts_texture* textures;
    sfts_material* materials;
    sfts_model* models;
    sfts_frame* frames;
} sfts_scene;

typedef struct { const uint8_t* p; const uint8_t* end; int bad; } sfts_cursor;

static const void* sfts__take(sfts_cursor* c, size_t n) {
    if (c->bad || (size_t)(c->end - c->p) < n) { c->bad = 1; return NULL; }
    const void* r = c->p; c->p += n; return r;
}
static uint32_t sfts__u32(sfts_cursor* c) {
    const void* q = sfts__take(c, 4); uint32_t v = 0; if (q) memcpy(&v, q, 4); return v;
}
static float sfts__f32(sfts_cursor* c) {
    const void* q = sfts__take(c, 4); float v = 0; if (q) memcpy(&v, q, 4); return v;
}

/* Parses a blob already in memory (the scene keeps pointers into `data`). Returns 0 on success. */
static int sfts_parse(sfts_scene* s, uint8_t* data, size_t size) {
    memset(s, 0, sizeof(*s));
    s->data = data; s->size = size;
    sfts_cursor c = { data, data + size, 0 };
    if (sfts__u32(&c) != 0x53544653u || sfts__u32(&c) != 1u) return -1;
    s->n_textures = sfts__u32(&c);
    s->textures = (sfts_texture*)calloc(s->n_textures + 1, sizeof(sfts_texture));
    for (uint32_t i = 0; i < s->n_textures && !c.bad; i++) {
        s->textures[i].w = sfts__u32(&c); s->textures[i].h = sfts__u32(&c);
        s->textures[i].argb = (const uint32_t*)sfts__take(&c, (size_t)s->textures[i].w * s->textures[i].h * 4);
    }
    s->n_materials = sfts__u32(&c);
    s->materials = (sfts_material*)calloc(s->n_materials + 1, sizeof(sfts_material));
    for (uint32_t i = 0; i < s->n_materials && !c.bad; i++) {
        s->materials[i].tex = (int32_t)sfts__u32(&c);
        s->materials[i].base_color = sfts__u32(&c);
        s->materials[i].shininess = sfts__f32(&c);
    }
    s->n_models = sfts__u32(&c);
    s->models = (sfts_model*)calloc(s->n_models + 1, sizeof(sfts_model));
    for (uint32_t i = 0; i < s->n_models && !c.bad; i++) {
        sfts_model* m = &s->models[i];
        m->n_meshes = sfts__u32(&c); m->bone_count = sfts__u32(&c); m->n_lightmaps = sfts__u32(&c);
        m->lightmaps = (const int32_t*)sfts__take(&c, 4u * m->n_lightmaps);
        m->n_proxies = sfts__u32(&c);
        m->proxies = (sfts_proxy*)calloc(m->n_proxies + 1, sizeof(sfts_proxy));
        for (uint32_t p = 0; p < m->n_proxies && !c.bad; p++) {
            const void* q = sfts__take(&c, 28);
            if (q) memcpy(&m->proxies[p], q, 28);
            m->proxies[p].bone = sfts__u32(&c);
        }
        m->meshes = (sfts_mesh*)calloc(m->n_meshes + 1, sizeof(sfts_mesh));
        for (uint32_t k = 0; k < m->n_meshes && !c.bad; k++) {
            sfts_mesh* ms = &m->meshes[k];
            ms->meshlet_count = sfts__u32(&c); ms->material = (int32_t)sfts__u32(&c);
            ms->lightmap_page = sfts__u32(&c); ms->has_skin = sfts__u32(&c);
            ms->meshlets = (sfts_meshlet*)calloc(ms->meshlet_count + 1, sizeof(sfts_meshlet));
            for (uint32_t j = 0; j < ms->meshlet_count && !c.bad; j++) {
                sfts_meshlet* ml = &ms->meshlets[j];
                ml->attr = (const float*)sfts__take(&c, 10 * 64 * 4);
                if (ms->has_skin) {
                    ml->joints = (const uint16_t*)sfts__take(&c, 4 * 64 * 2);
                    ml->weights = (const uint8_t*)sfts__take(&c, 4 * 64);
                }
                ml->inds = (const uint8_t*)sfts__take(&c, 512);
                ml->cull = (const float*)sfts__take(&c, 8 * 4);
                ml->culling_bone = (int32_t)sfts__u32(&c);
            }
        }
    }
    s->n_frames = sfts__u32(&c);
    s->frames = (sfts_frame*)calloc(s->n_frames + 1, sizeof(sfts_frame));
    for (uint32_t i = 0; i < s->n_frames && !c.bad; i++) {
        sfts_frame* f = &s->frames[i];
        f->width = sfts__u32(&c); f->height = sfts__u32(&c);
        f->cam_pos = (const float*)sfts__take(&c, 12);
        f->view = (const float*)sfts__take(&c, 64);
        f->proj = (const float*)sfts__take(&c, 64);
        f->ambient = (const float*)sfts__take(&c, 12);
        f->lightmap_brightness = sfts__f32(&c);
        f->clear = sfts__u32(&c); f->clear_color = sfts__u32(&c); f->shadows = sfts__u32(&c);
        f->n_dir = sfts__u32(&c); f->dir = (const sfts_dir_light*)sfts__take(&c, 28u * f->n_dir);
        f->n_point = sfts__u32(&c); f->point = (const sfts_point_light*)sfts__take(&c, 32u * f->n_point);
        f->n_inst = sfts__u32(&c);
        f->inst = (sfts_instance*)calloc(f->n_inst + 1, sizeof(sfts_instance));
        for (uint32_t k = 0; k < f->n_inst && !c.bad; k++) {
            f->inst[k].model = sfts__u32(&c);
            f->inst[k].transform = (const float*)sfts__take(&c, 64);
            f->inst[k].n_bones = sfts__u32(&c);
            f->inst[k].bones = f->inst[k].n_bones ? (const float*)sfts__take(&c, 64u * f->inst[k].n_bones) : NULL;
        }
    }
    return c.bad ? -2 : 0;
}

static int sfts_load_file(sfts_scene* s, const char* path) {
    FILE* f = fopen(path, "rb");
    if (!f) return -10;
    fseek(f, 0, SEEK_END); long n = ftell(f); fseek(f, 0, SEEK_SET);
    uint8_t* d = (uint8_t*)malloc((size_t)n + 16);
    if (!d || fread(d, 1, (size_t)n, f) != (size_t)n) { fclose(f); free(d); return -11; }
    fclose(f);
    return sfts_parse(s, d, (size_t)n);
}

/* ---- dump writer: a flat list of named sections, read by tests/oracle_io.py ---- */
typedef struct { FILE* f; } sfts_dump;

static void sfts_dump_section(sfts_dump* d, const char* name, const char* dtype, const void* data, uint64_t bytes) {
    char nm[32] = {0}, dt[8] = {0};
    strncpy(nm, name, 31); strncpy(dt, dtype, 7);
    fwrite("SEC1", 1, 4, d->f); fwrite(nm, 1, 32, d->f); fwrite(dt, 1, 8, d->f);
    fwrite(&bytes, 8, 1, d->f);
    if (bytes) fwrite(data, 1, (size_t)bytes, d->f);
}

#endif
