/*
 * Data layouts shared by the host runtime and the CUDA kernels of the sofren2 render path.
 *
 * Resident (uploaded once per asset), all in device memory:
 *   texel heap        u32 ARGB texels; every texture keeps its full mip chain, each level
 *                     padded to 4x4 and stored 4x4 block-linear (row-major texels inside a
 *                     block, row-major blocks), as sft_texture_create lays it out
 *                     (sofren2.c:9181-9310)
 *   sftg_tex          per texture: size, levels, pot flag, per-level texel offset / blocks_w / shift
 *   sftg_mat          per material: texture index (-1 none), base colour, shininess
 *   meshlet pool      per meshlet g: attr[g] = f32[10][64] (x y z nx ny nz u v lu lv),
 *                     inds[g] = u8[512] (16 batches x [v0 x8, v1 x8, v2 x8, pad x8]),
 *                     cull[g] = f32[8] (sphere centre, radius, cone axis, cone cutoff),
 *                     info[g] (culling bone, skin slot, mesh material, lightmap texture);
 *                     skinned meshlets also own skin[slot] = u16 j[4][64] + u8 w[4][64]
 *   BLAS node pool    sft_bvh_node images (256 B: SoA child AABBs, child ids, count, leaf flag)
 *   sftg_model        per model: meshlet range in the pool, BLAS range, bone count
 *
 * Per frame (one upload of a few KB, then a bump arena for scratch):
 *   sftg_frame        camera, frustum, display, lighting constants and array pointers
 *   sftg_inst         per instance: model, transform, screen-space cache offset, bones offset
 *   ss cache          SFTG_SS_FLOATS f32 per drawn meshlet: the values of the reference's
 *                     sft_ss_meshlet (sofren2.c:1464-1477: sx sy inv_w wx wy wz wnx wny wnz per
 *                     vertex) and the vertex's texture and lightmap coordinates, held vertex-
 *                     major so that the resolve reads a vertex with three 16-byte loads and one
 *                     word: float4[64] (sx, sy, inv_w, wx) at SFTG_SS_A, float4[64] (wy, wz,
 *                     wnx, wny) at SFTG_SS_B, float4[64] (wnz, u, v, lu) at SFTG_SS_C, f32[64] lv
 *                     at SFTG_SS_D; debug captures return the reference's [9][64] rows
 *   batch records     per (drawn meshlet, batch): u64 payload + tile rect + clip count
 *   tile lists        u64 payloads per tile, in the reference's single-worker order
 *   colour            u32 ARGB8888, pitch = width
 */
#ifndef SFTG_TYPES_H
#define SFTG_TYPES_H

#include <stdint.h>

#define SFTG_TILE 64
#define SFTG_TILE_PX 4096
#define SFTG_MAX_TILE_LIGHTS 16
#define SFTG_MAX_LIGHT_PROXIES 16
#define SFTG_MAX_INSTANCES 64
#define SFTG_INVALID 0xFFFFFFFFu
#define SFTG_SS_A 0                /* ss cache record: float offsets of its parts */
#define SFTG_SS_B 256
#define SFTG_SS_C 512
#define SFTG_SS_D 768
#define SFTG_SS_FLOATS 832         /* floats per record (3328 B) */

typedef struct sftg_tex {
    int32_t w, h, levels, is_pot;
    uint32_t offs[14];     /* texel offset of each level from the heap base */
    int32_t bw[14];        /* 4x4 blocks per row */
    int32_t shift[14];     /* log2(bw) when pot */
} sftg_tex;

typedef struct sftg_mat {
    int32_t tex;           /* texture index or -1 */
    uint32_t base_color;
    float shininess;
    uint32_t pad;
} sftg_mat;

typedef struct sftg_meshlet_info {
    int32_t culling_bone;  /* -1 when static */
    int32_t skin_slot;     /* -1 when static */
    int32_t material;      /* material index or -1 (reference default: white, shininess 4) */
    int32_t lightmap_tex;  /* texture index or -1 */
} sftg_meshlet_info;

typedef struct sftg_model {
    uint32_t meshlet_base, total_meshlets;
    uint32_t blas_base, blas_root, blas_count;
    uint32_t bone_count;
    uint32_t mesh_count, pad;
} sftg_model;

typedef struct sftg_bvh_node {  /* sft_bvh_node, sofren2.c:967-983 */
    float mn[3][8];
    float mx[3][8];
    uint32_t child[8];
    uint8_t count, leaf, pad[30];
} sftg_bvh_node;

typedef struct sftg_inst {
    float T[16];           /* row-major 4x4, row vectors (translation in row 3) */
    uint32_t model;
    uint32_t ss_offset;    /* first screen-space cache slot of this instance */
    int32_t bones;         /* offset into the frame's bone matrices, -1 when none */
    uint32_t meshlet_base; /* copy of the model's pool base */
} sftg_inst;

typedef struct sftg_job {   /* up to 8 consecutive meshlets of one mesh, sft_geom_job (sofren2.c:1264) */
    uint32_t inst;
    uint32_t first;        /* model-relative meshlet index */
    uint16_t count;        /* 1..8 */
    uint16_t skinned;      /* mesh has skin and the instance has bones */
    uint32_t view;         /* view of the batch this job belongs to */
    uint32_t group_first;  /* first meshlet of the reference's 8-meshlet group: its culling bone is
                              the whole group's (sofren2.c:4939-4960), also when a job covers part of it */
} sftg_job;

typedef struct sftg_point_light {
    float pos[3];
    float color[3];        /* rgb * intensity */
    float radius;
    float inv_radius_sqr;  /* 1 / (radius * radius) */
} sftg_point_light;

typedef struct sftg_dir_light {
    float dir[3];          /* normalised */
    float color[3];
} sftg_dir_light;

typedef struct sftg_proxy {    /* world-space capsule, sft_world_shadow_proxy (sofren2.c:1429) */
    float posa[3], posb[3], radius;
    uint32_t pad;
} sftg_proxy;

typedef struct sftg_frame {
    /* display */
    int32_t width, height, samples, pitch;
    float hw, hh, vpx, vpy;
    int32_t cols, rows, tiles, debug_mode;
    uint32_t clear, clear_color, shadows, pad0;
    /* camera */
    float cam[3], pad1;
    float vp[16];
    float fn[6][3], fan[6][3], fd[6];
    float pad2[2];
    /* lighting */
    float ambient[3], lightmap_brightness;
    uint32_t n_point, n_dir, n_proxies, n_inst;
    uint32_t total_ss, n_jobs, tlas_root, tlas_count;
    uint32_t clip_cap, tile_cap;                 /* capacities of the clip pool and tile payload buffer */
    int32_t debug_tex;                           /* checkerboard texture of the debug view */
    uint32_t stile_cap;                          /* capacity of the super-tile meshlet lists */
    /* where this view's rows start in the batch-wide arrays (all 0 for a single frame) */
    uint32_t view, ss_base;        /* screen-space cache slot; batch records start at ss_base * 16 */
    uint32_t tile_base, prox_base; /* global tile index; global proxy index (light_vis rows) */
    uint32_t packet_base, n_packets;
    uint32_t stile_base, scols;    /* global index of the first super-tile (4 x 4 tiles); super-tile columns */
    uint64_t vis_base;             /* float2 offset of this view's visibility buffer */
    uint32_t* color_dev;           /* this view's colour buffer, width * height */
    /* per-frame arrays */
    const sftg_inst* inst;
    const float* bones;            /* 16 floats per matrix */
    const sftg_job* jobs;
    const sftg_point_light* point;
    const sftg_dir_light* dir;
    const sftg_proxy* proxies;
    const sftg_bvh_node* tlas;
    /* resident tables */
    const sftg_model* models;
    const sftg_tex* texs;
    const uint32_t* texels;
    const sftg_mat* mats;
    const float* ml_attr;          /* [g][10][64] */
    const uint8_t* ml_inds;        /* [g][512] */
    const float* ml_cull;          /* [g][8] */
    const sftg_meshlet_info* ml_info;
    const uint16_t* skin_j;        /* [slot][4][64] */
    const uint8_t* skin_w;         /* [slot][4][64] */
    const sftg_bvh_node* blas;     /* pool */
    const uint32_t* lightmaps_of_model; /* unused: lightmap textures are resolved per meshlet */
} sftg_frame;

#endif
