/* Device-side records exchanged between the render-path kernels, and the kernel entry points. */
#pragma once
#include <stdint.h>
#include "sftg_types.h"
#include "../../include/sftg.h"

/* one 8-triangle batch of a drawn meshlet after setup (sofren2.c:4775-4884) */
struct __align__(16) sftg_batch_rec {
    uint64_t payload;      /* inst | meshlet << 24 | batch << 48 | lane mask << 56; 0 = nothing binned */
    int16_t x0, x1, y0, y1;/* tile rectangle (inclusive, unclamped) */
};

/* sft_clipped_triangle (sofren2.c:1271-1280), same field order */
struct sftg_clip_tri {
    float sx[3], sy[3], iw[3], u[3], v[3], lu[3], lv[3], px[3], py[3], pz[3], nx[3], ny[3], nz[3];
    uint32_t inst, m;
};

/* Arguments of the tile kernels.  Tiles are numbered batch-wide: tile_view maps a tile to its
 * view's frame block, whose tile_base, ss_base, prox_base and vis_base locate the view's rows in
 * the shared arrays. */
/* A tile's lights and proxy selection, computed once per tile by k_tile_lights for all of the
 * tile's resolve CTAs: the first SFTG_MAX_TILE_LIGHTS point lights in index order that reach the
 * tile's depth range and rectangle (sofren2.c:5855-5934), and per light the first
 * SFTG_MAX_LIGHT_PROXIES proxies in index order that see the light and can reach it (5936-5990). */
struct sftg_tile_lights {
    uint32_t proxy[SFTG_MAX_TILE_LIGHTS][SFTG_MAX_LIGHT_PROXIES];
    uint16_t light[SFTG_MAX_TILE_LIGHTS];
    uint8_t npc[SFTG_MAX_TILE_LIGHTS];
    uint32_t nlights;
    uint32_t pad[3];
};

struct sftg_tile_args {
    const sftg_frame* frames;
    const uint16_t* tile_view;
    const float* ss;
    const sftg_clip_tri* clips;
    const uint32_t* clip_base;     /* exclusive scan of clip counts: a view's first slot is clip_base[ss_base * 16] */
    const uint32_t* tile_order;    /* launch order of the tiles (heaviest first within each sample count) */
    uint8_t* tile_nlights;         /* per tile: light list length, for the debug overlays (k_tile_lights or the resolve) */
    sftg_tile_lights* tile_lights; /* per tile, written by k_tile_lights, read by every resolve CTA of the tile
                                      where the range's resolve is launched with records */
    const uint32_t* tile_start;
    const uint32_t* tile_count;
    const uint64_t* tile_pay;
    const uint8_t* light_vis;      /* [proxy][64] */
    float2* vis;                   /* (depth, vis id) per sample */
    float2* zrange;                /* per tile and raster band (sftg_raster_bands() entries per tile) */
    float* vis_depth;              /* debug capture of a single view, or null */
    uint32_t* vis_id;
    float* shadow_out;
};

__global__ void k_geometry(const sftg_frame* frames, const sftg_job* jobs, uint32_t n_jobs, float* ss, sftg_batch_rec* recs,
                           uint32_t* clip_cnt, int4* mrect);
__global__ void k_clip(const sftg_frame* frames, uint32_t n_views, const float* ss, const uint32_t* clip_cnt,
                       const uint32_t* clip_base, sftg_clip_tri* clips, int4* clip_rect, int4* mrect, uint32_t n_records);
#define SFTG_STILE 4   /* tiles per side of a super-tile (coarse binning) */
__global__ void k_coarse(const sftg_frame* frames, const uint16_t* stile_view, const int4* mrect, uint32_t* stile_count,
                         const uint32_t* stile_start, uint32_t* stile_list);
__global__ void k_bin(const sftg_frame* frames, const uint16_t* tile_view, const sftg_batch_rec* recs, const uint32_t* clip_cnt,
                      const uint32_t* clip_base, const int4* clip_rect, const int4* mrect, const uint32_t* stile_count,
                      const uint32_t* stile_start, const uint32_t* stile_list, uint32_t* tile_count,
                      const uint32_t* tile_start, uint64_t* tile_pay);
__global__ void k_scan_reduce(const uint32_t* in, uint32_t n, uint32_t* sums);
__global__ void k_scan_top(uint32_t* sums, uint32_t nb, uint32_t* total_out);
__global__ void k_scan_down(const uint32_t* in, uint32_t n, const uint32_t* sums, uint32_t* out);
#define SFTG_SCAN_SMALL (1024u * 32u)   /* inputs up to this size are scanned by one CTA */
__global__ void k_scan_small(const uint32_t* in, uint32_t n, uint32_t* out, uint32_t* total_out);
size_t sftg_packet_bytes();
/* BLAS sub-walk items per (packet, instance) pair: the pair buffer holds max_pairs pairs, then
 * max_pairs * items_per_pair items; the counter word after n_pairs counts the items.  A walk
 * whose items do not fit keeps the rest of its subtree on its own stack. */
#define SFTG_OCC_ITEMS_PER_PAIR 64
#define SFTG_OCC_ITEMS_PER_PAIR_NOALLOC 64
/* packet_view maps a batch-wide shadow packet to its view, prox_view a batch-wide proxy */
void sftg_launch_occlusion(const sftg_frame* frames, const uint16_t* packet_view, uint32_t n_packets, const uint16_t* prox_view,
                           uint32_t n_proxies, uint32_t max_inst, void* packets, uint2* pairs, uint32_t* n_pairs,
                           uint32_t max_pairs, uint32_t items_per_pair, uint8_t* light_vis, uint32_t* status, int ray_prune,
                           cudaStream_t st);
cudaError_t sftg_tile_configure(int max_dynamic_smem);
int sftg_raster_bands(void);   /* raster CTAs (row bands) per 64x64 tile */
/* order[] = the batch's tiles, heaviest first inside each sample-count range; scratch holds 192 words */
int sftg_launch_tile_order(const sftg_frame* frames, const uint16_t* tile_view, const uint32_t* tile_count, uint32_t n_tiles,
                            uint32_t* scratch, uint32_t* order, cudaStream_t st);
/* slab_rows: rows of one raster work item (4..64); split: resolve CTAs per tile (1, 2, 4, 8 or 16) */
void sftg_launch_raster(int S, uint32_t tile0, uint32_t tiles, int slab_rows, int bands, uint32_t* queue, cudaStream_t st,
                        const sftg_tile_args& A);
void sftg_launch_tile_lights(uint32_t tile0, uint32_t tiles, cudaStream_t st, const sftg_tile_args& A);
/* queue: null for one CTA per (tile, part) item, else a zeroed counter for one persistent launch
 * whose CTAs take the items in launch order (k_resolve_queue); likewise for the raster */
void sftg_launch_resolve(int S, uint32_t tile0, uint32_t tiles, int split, bool records, uint32_t* queue, cudaStream_t st,
                         const sftg_tile_args& A);
/* tile overlays of the debug views 2-4 (sft__debug_draw_tile_overlay), after every resolve */
void sftg_launch_debug_overlay(uint32_t tiles, cudaStream_t st, const sftg_tile_args& A);

/* skeletons and animations on the device (sftg_skeleton_upload) */
struct sftg_bone_dev {
    float inverse_bind[16], local_bind[16];
    int32_t parent;
    float base_t[3], base_r[4], base_s[3];
};
struct sftg_skel_dev { uint32_t bone_base, bone_count, anim_base, anim_count, order_base, level_base, level_count, pad; };
struct sftg_anim_dev { uint32_t sampler_base, channel_base; int32_t sampler_count, channel_count; float duration; uint32_t pad[3]; };
struct sftg_sampler_dev { uint32_t input_base, output_base; int32_t count, is_step; };
struct sftg_pose_tables {
    uint32_t n_skels;              /* requests naming another skeleton leave their matrices untouched */
    const sftg_skel_dev* skels;
    const sftg_bone_dev* bones;
    const sftg_anim_dev* anims;
    const sftg_sampler_dev* samplers;
    const sftg_channel_desc* channels;
    const float* keys;
    const uint16_t* order;         /* per skeleton: bones parents-first */
    const uint16_t* levels;        /* per skeleton: level_count + 1 starts into order */
};
void sftg_launch_raycast(const sftg_ray* rays, uint32_t n, const sftg_model* models, uint32_t n_models, const sftg_bvh_node* blas,
                         const float* ml_attr, const uint8_t* ml_inds, sftg_ray_hit* hits, cudaStream_t st);
/* BLAS construction on the device (sftg_blas.cu): begin counts the model's triangles and lays
 * out the tree's shape (node count known on return), finish builds the node images into dst
 * (status 1: a device work list overflowed), end releases the job. */
struct sftg_blas_job;
cudaError_t sftg_blas_begin(sftg_blas_job** out, const float* attr, const uint8_t* inds, uint32_t nm, cudaStream_t st,
                            uint32_t* n_items, uint32_t* n_nodes);
cudaError_t sftg_blas_finish(sftg_blas_job* job, sftg_bvh_node* dst, uint32_t* status);
uint32_t sftg_blas_launches(const sftg_blas_job* job);
void sftg_blas_end(sftg_blas_job* job);
void sftg_launch_pose(const sftg_pose_tables& T, const sftg_pose_request* reqs, const uint32_t* out_off, uint32_t n, float* posed,
                      float* global, cudaStream_t st);

#define SFTG_SCAN_ELEMS_PER_BLOCK 4096
