/*
 * sftg — the C ABI between sofren2's host runtime (include/sofren2.h, SFT_IMPL) and the
 * GB300 kernels.  Plain pointers and sizes only.  Every call returns 0 on success or a
 * negative SFTG_E* code; sftg_last_error() gives the text.  One context drives one GPU.
 *
 * Each entry point replaces a piece of the reference's CPU frame machinery (sofren2.c):
 *   sftg_create / sftg_destroy      thread pool, barriers and arenas of sft_init / sft_release
 *                                   (sofren2.c:7974-8137); here a stream plus device arenas
 *   sftg_texture_upload             the texture heap of sft_texture_create (sofren2.c:9181-9310):
 *                                   the caller passes the block-linear mip chain it built
 *   sftg_material_set               the static material pool (sofren2.c:9393-9424)
 *   sftg_model_upload               the meshlet / BLAS data a loaded sft_model carries
 *                                   (sft_model, sofren2.c:1057-1123)
 *   sftg_frame_render               sft_present (sofren2.c:8139-8289): proxy occlusion, geometry
 *                                   and binning jobs, tile raster and resolve, written to the
 *                                   caller's colour buffer (sft_set_color_buffer, 8405-8408)
 */
#ifndef SFTG_H
#define SFTG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SFTG_OK 0
#define SFTG_E_CUDA (-1)          /* a CUDA call failed (text in sftg_last_error) */
#define SFTG_E_ARG (-2)           /* invalid argument */
#define SFTG_E_NOMEM (-3)         /* device allocation failed */
#define SFTG_E_LIMIT (-4)         /* a reference limit was exceeded (e.g. > 64 instances) */
#define SFTG_E_DEVICE_STATUS (-5) /* a kernel reported a bounded-walk overflow */

typedef struct sftg_ctx sftg_ctx;

/* texture description: level offsets are relative to the first texel passed */
typedef struct sftg_texture_desc {
    int32_t width, height, levels, is_pot;
    uint32_t level_offset[14];
    int32_t blocks_w[14];
    int32_t stride_shift[14];
} sftg_texture_desc;

/* one mesh of a model: meshlet_count meshlets, each with
 *   attr     f32[10][64]  x y z nx ny nz u v lu lv
 *   inds     u8[512]      16 batches x [v0 x8, v1 x8, v2 x8, pad x8]
 *   cull     f32[8]       sphere centre xyz, radius, cone axis xyz, cone cutoff
 *   joints   u16[4][64], weights u8[4][64], culling_bone i32   (skinned meshes only, else NULL) */
typedef struct sftg_mesh_desc {
    uint32_t meshlet_count;
    const float* attr;
    const uint8_t* inds;
    const float* cull;
    const uint16_t* joints;
    const uint8_t* weights;
    const int32_t* culling_bones;
    int32_t material;          /* material index, -1 = none */
    int32_t lightmap_texture;  /* texture index, -1 = no lightmap */
} sftg_mesh_desc;

typedef struct sftg_model_desc {
    uint32_t mesh_count;
    const sftg_mesh_desc* meshes;
    uint32_t bone_count;
    const void* blas_nodes;    /* sft_bvh_node images, 256 B each */
    uint32_t blas_count, blas_root;
    uint32_t build_blas;       /* 1 with no blas_nodes: build the BLAS on the device at upload,
                                  sft__blas_build_model (sofren2.c:3526-3617) */
} sftg_model_desc;

typedef struct sftg_instance_desc {
    int32_t model;
    float transform[16];
    const float* bones;        /* posed matrices (16 floats each) or NULL */
    uint32_t bone_count;
} sftg_instance_desc;

typedef struct sftg_frame_desc {
    int32_t width, height, samples;          /* samples: 1, 2 or 4 */
    float cam_pos[3];
    float view_proj[16];
    float frustum_n[6][3], frustum_d[6];     /* normalised planes (sft_set_camera) */
    float ambient[3], lightmap_brightness;
    uint32_t clear, clear_color, shadows, debug_mode;   /* debug_mode: enum sft_debug_mode (sofren2.c:59-67) */
    uint32_t n_point;
    const float* point_lights;               /* per light: pos[3], color[3] (rgb * intensity), radius, 1/radius^2 */
    uint32_t n_dir;
    const float* dir_lights;                 /* per light: dir[3] (normalised), color[3] */
    uint32_t n_instances;
    const sftg_instance_desc* instances;
    uint32_t n_proxies;
    const float* proxies;                    /* per world proxy: posa[3], posb[3], radius, pad */
    const void* tlas_nodes;                  /* sft_bvh_node images built on the host */
    uint32_t tlas_count, tlas_root;
    int32_t debug_texture;                   /* texture of SFT_DEBUG_CHECKERBOARD (the base material's albedo) */
} sftg_frame_desc;

/* optional per-frame outputs for parity checks (any pointer may be NULL; host memory) */
typedef struct sftg_debug_out {
    float* vis_depth;          /* tiles * samples * 4096 */
    uint32_t* vis_id;          /* tiles * samples * 4096 */
    uint32_t* tile_counts;     /* tiles */
    uint64_t* tile_payloads;   /* capacity tile_payload_cap */
    uint64_t tile_payload_cap;
    uint64_t* tile_payload_total;
    float* ss_cache;           /* total screen-space meshlets * 576 */
    uint8_t* light_vis;        /* proxies * 64 */
    void* clip_tris;           /* clip_cap * 164 bytes */
    uint64_t clip_cap;
    uint64_t* clip_total;
    float* shadow;             /* width * height * 16, 1x only */
    uint32_t* status;          /* kernel status bits */
} sftg_debug_out;

int sftg_create(int device, sftg_ctx** out);
void sftg_destroy(sftg_ctx* ctx);
const char* sftg_last_error(const sftg_ctx* ctx);

int sftg_texture_upload(sftg_ctx* ctx, const uint32_t* texels, uint64_t n_texels, const sftg_texture_desc* desc, int32_t* out_index);
int sftg_texture_update_desc(sftg_ctx* ctx, int32_t index, const sftg_texture_desc* desc_or_null);
int sftg_material_set(sftg_ctx* ctx, int32_t index, int32_t texture, uint32_t base_color, float shininess);
int sftg_model_upload(sftg_ctx* ctx, const sftg_model_desc* desc, int32_t* out_model);
/* A resident model's BLAS: node count and root index, and `count` node images from `first`
 * copied into `dst` (256 B each) when dst is not NULL.  Replaces reading sft_model.blas_nodes
 * (sofren2.c:1107-1108) for a BLAS that was built on the device. */
int sftg_model_blas(sftg_ctx* ctx, int32_t model, uint32_t first, uint32_t count, void* dst, uint32_t* out_count, uint32_t* out_root);
/* A model for one frame only: the geometry of the reference's dynamic meshes (sft_dmesh_*,
 * sofren2.c:8720-8951), which lives in its per-frame scratch arena.  sftg_transient_reset drops
 * every transient model uploaded since the last reset (after the frames that draw them);
 * transient models uploaded before a resident one stay until the context is destroyed. */
int sftg_model_upload_transient(sftg_ctx* ctx, const sftg_model_desc* desc, int32_t* out_model);
void sftg_transient_reset(sftg_ctx* ctx);

/* Renders one frame into `color` (host memory, pitch in bytes; width*4 when 0).  When the frame
 * does not clear, the current content of `color` is read first (the reference keeps it). */
int sftg_frame_render(sftg_ctx* ctx, const sftg_frame_desc* frame, uint32_t* color, int32_t pitch_bytes, sftg_debug_out* dbg);

/* Same as sftg_frame_render but leaves the result in device memory: *out_device_color points at
 * width*height u32 owned by the context (valid until the next frame). No host copies of pixels. */
int sftg_frame_render_device(sftg_ctx* ctx, const sftg_frame_desc* frame, const uint32_t** out_device_color);

/* Renders n_views independent frames (each with its own camera, size, sample count, instances,
 * lights and proxies; all drawing from the context's resident models) in one submission: every
 * pipeline stage is one launch over all views' work, so small views fill the GPU together.
 * Each view's result is identical to rendering it alone with sftg_frame_render.
 * colors (optional) holds one host pointer per view (entries may be null), pitch_bytes
 * (optional) one pitch per view (0 = width*4); out_device_colors (optional) receives one device
 * pointer per view, valid until the next render call.  No counterpart in the reference, which
 * renders one view per sft_present. */
int sftg_frames_render(sftg_ctx* ctx, const sftg_frame_desc* frames, uint32_t n_views, uint32_t* const* colors,
                       const int32_t* pitch_bytes, const uint32_t** out_device_colors);

/* Light visibility of a frame's shadow proxies (the occlusion pass of sft_present,
 * sofren2.c:8163-8280) computed without allocating anything: no cudaMalloc / cudaFree, no
 * growth of the context's arena or pinned staging, no host heap.  For callers that must not
 * allocate while they run (a serving loop whose device-memory budget is already committed,
 * per-frame code on a latency deadline).  Scratch is a static device array of
 * SFTG_NOALLOC_SCRATCH_BYTES; a frame needing more (many proxies x lights x instances) is
 * rejected with SFTG_E_LIMIT before any device work.  light_vis (host, n_proxies * 64 bytes)
 * receives 3 - rays blocked per (proxy, light), 0 in columns past the light count: the rows
 * sftg_frame_render computes for the same frame.  The models must be on the device already
 * (a render since the last model upload).  sftg_create looks up the scratch's device address
 * once per device, so the 4 MiB are committed on the device when its first context is created,
 * not during a call.  The scratch is shared by all contexts on a
 * device, so overlapping calls race: serialise them.  No counterpart in the reference, whose
 * CPU frame always has its arenas. */
#define SFTG_NOALLOC_SCRATCH_BYTES (4u << 20)
int sftg_light_vis_noalloc(sftg_ctx* ctx, const sftg_frame_desc* frame, uint8_t* light_vis);

/* Scheduling knobs.  None but occl_ray_prune changes a result: they set how the same work is cut
 * into CTAs and warps.  No counterpart in the reference (its SIMD width and tile size are fixed;
 * the 64x64 tile stays fixed here too, because the per-tile payload lists are part of the
 * render path's observable output). */
typedef struct sftg_tuning {
    int32_t resolve_split[3];     /* resolve CTAs per 64x64 tile at 1x, 2x, 4x: 1, 2, 4, 8 or 16 (default 16, 8, 16) */
    int32_t raster_slab_rows[3];  /* tile rows per raster work item at 1x, 2x, 4x: 4..64 (default 8, 8, 4) */
    int32_t geom_job_width;       /* meshlets per geometry warp: 1..8 (default 1; the reference's job is 8) */
    int32_t occl_ray_prune;       /* 1: also cull BLAS children no unblocked shadow ray reaches (faster; can differ
                                     from the reference only where a ray grazes a triangle's plane); default 0.
                                     The only knob that is not result-neutral: sftg_autotune leaves it as set */
    int32_t raster_bands[3];      /* raster CTAs per 64x64 tile at 1x, 2x, 4x, each a band of its rows: 0 = by the
                                     tile's payload count (default: 1, 2 above 48 payloads, 4 above 128; at 4x 2),
                                     1, 2 or 4 = every tile (at 4x at least 2) */
    int32_t tile_lights[3];       /* where a tile's light list and proxy selection are made at 1x, 2x, 4x: 1 = by each of
                                     its resolve CTAs, 2 = once per tile by a launch before the resolve (its CTAs read
                                     the result), 0 = 2 where the range has 16 CTAs per tile and at least 256 tiles,
                                     else 1 (default) */
    int32_t tile_queue;           /* bit 0 raster, bit 1 resolve: set, the phase is one persistent launch of as many CTAs
                                     as are resident at once, which take its (tile, band) / (tile, part) items, heaviest
                                     tiles first, from a device counter; clear (default 0), one CTA per item */
} sftg_tuning;
int sftg_get_tuning(const sftg_ctx* ctx, sftg_tuning* out);
int sftg_set_tuning(sftg_ctx* ctx, const sftg_tuning* tuning);
/* Times the given views with each candidate setting (median of reps renders per candidate,
 * coordinate search: job width, then per sample count slab rows, raster bands, and resolve split
 * with where the tile light lists are made, jointly, then the persistent tile queue), keeps the
 * fastest in the context and copies it to *out (optional). */
int sftg_autotune(sftg_ctx* ctx, const sftg_frame_desc* frames, uint32_t n_views, int32_t reps, sftg_tuning* out);

/* Skeletal animation on the GPU (sft_pose_update, sofren2.c:8952-9108).  A skeleton (bones in
 * sft_bone's layout, sofren2.c:1000-1009) with its animations (samplers / channels,
 * sofren2.c:1023-1049) is uploaded once; sftg_pose_eval then evaluates any number of
 * (skeleton, animation, time) requests in one launch, one warp per request.  Results are the
 * reference's posed bone matrices (inverse bind x global) and, optionally, the globals; they
 * equal the reference's up to the rounding of the device's acosf / sinf / cosf against the host
 * libm's inside the quaternion slerp (a few ulp). */
typedef struct sftg_bone_desc {
    float inverse_bind[16], local_bind[16];   /* row-major sftmat */
    int32_t parent;                           /* -1 for a root; any order */
    float base_t[3], base_r[4], base_s[3];    /* rest pose TRS (quaternion x y z w) */
} sftg_bone_desc;
typedef struct sftg_sampler_desc {
    const float* inputs;                      /* count keyframe times, ascending */
    const float* outputs;                     /* count * 4 floats (xyz or xyzw per key) */
    int32_t count, is_step;
} sftg_sampler_desc;
typedef struct sftg_channel_desc { int32_t sampler, node, path; } sftg_channel_desc;   /* path: 0 T, 1 R, 2 S */
typedef struct sftg_animation_desc {
    const sftg_sampler_desc* samplers;
    const sftg_channel_desc* channels;
    int32_t sampler_count, channel_count;
    float duration;
} sftg_animation_desc;
typedef struct sftg_pose_request { int32_t skeleton, animation; float time; } sftg_pose_request;
#define SFTG_MAX_BONES 128
int sftg_skeleton_upload(sftg_ctx* ctx, const sftg_bone_desc* bones, uint32_t bone_count, const sftg_animation_desc* anims,
                         uint32_t anim_count, int32_t* out_skeleton);
/* posed (and global, optional) receive for request k, at float offset 16 * (sum of the bone counts
 * of requests 0..k-1), its bones' matrices; host memory.  A request whose animation index is out
 * of range leaves its matrices untouched, as sft_pose_update returns early. */
int sftg_pose_eval(sftg_ctx* ctx, const sftg_pose_request* requests, uint32_t n, float* posed, float* global);
/* The same on device arrays, asynchronous on the context's stream (sftg_stream): request k
 * writes its bone_count matrices at d_posed + 16 * d_off[k] (and d_global, when not NULL); the
 * caller sizes the outputs for its offsets.  Requests naming no uploaded skeleton, or an
 * animation out of range, leave their matrices untouched. */
int sftg_pose_eval_device(sftg_ctx* ctx, const sftg_pose_request* d_requests, const uint32_t* d_off, uint32_t n, float* d_posed,
                          float* d_global);

/* Ray queries against resident models (sft_raycast_instance, sofren2.c:3733-3837), any number in
 * one launch, one thread per ray.  A ray names a model and its instance transform; results equal
 * the reference's bit for bit, including its treatment of the transform: the ray enters model
 * space through the transposed rotation rows alone (sft_m_mul_vec adds no translation) and the
 * hit position leaves it the same way.  Skinned models are queried in their bind pose, as in the
 * reference.  A ray whose model is not resident, or has no BLAS, gives hit 0 and distance
 * max_dist; hit 2 marks a walk whose stack overflowed (a BLAS deeper than 18 levels). */
typedef struct sftg_ray {
    float transform[16];       /* the instance's transform, row-major sftmat */
    float origin[3], dir[3];   /* world space; dir need not be normalised */
    float max_dist;
    int32_t model;             /* resident model (sftg_model_upload) */
} sftg_ray;
typedef struct sftg_ray_hit {  /* sft_ray_hit (sofren2.c:895-900) */
    uint32_t hit;
    float distance, pos[3], normal[3];
} sftg_ray_hit;
/* host arrays; returns when hits is filled (SFTG_E_DEVICE_STATUS if a walk overflowed) */
int sftg_raycast(sftg_ctx* ctx, const sftg_ray* rays, uint32_t n, sftg_ray_hit* hits);
/* device arrays, queued on the context's stream (sftg_stream); returns without waiting */
int sftg_raycast_device(sftg_ctx* ctx, const sftg_ray* d_rays, uint32_t n, sftg_ray_hit* d_hits);

/* Overlapping batches.  A context has SFTG_MAX_LANES submission lanes, each with its own streams,
 * frame arena and colour pool; lane 0 serves the synchronous calls above.  sftg_frames_submit
 * queues a batch (as sftg_frames_render would render it) on lane 1..SFTG_MAX_LANES-1 and returns
 * without waiting, so that batches submitted on different lanes run on the GPU at the same time;
 * the frame descriptions, everything they point at and the colour buffers must stay valid until
 * sftg_lane_wait returns.  sftg_lane_done is 1 once the lane's batch has finished (or the lane is
 * idle) and 0 while it runs; sftg_lane_wait waits for it, re-renders it when a capacity had to
 * grow, and returns its status.  A batch with a view that keeps the caller's pixels (clear off)
 * completes inside sftg_frames_submit.  Each view's pixels are those it would get alone. */
#define SFTG_MAX_LANES 8
int sftg_frames_submit(sftg_ctx* ctx, uint32_t lane, const sftg_frame_desc* frames, uint32_t n_views, uint32_t* const* colors,
                       const int32_t* pitch_bytes);
int sftg_lane_done(sftg_ctx* ctx, uint32_t lane);
int sftg_lane_wait(sftg_ctx* ctx, uint32_t lane);
/* Kernels launched by every batch finished so far, on all lanes (a running total). */
uint64_t sftg_launch_total(const sftg_ctx* ctx);
/* The last BLAS built on the device at model upload (no counterpart in the reference, whose build
 * is host code): wall time in ms, the span of the build on the upload stream between two CUDA
 * events in ms, its triangle count and the kernels it launched. */
int sftg_last_blas_build(const sftg_ctx* ctx, double* wall_ms, double* stream_ms, uint32_t* items, uint32_t* launches);

/* Device time in ms of the last frame, split as [occlusion, geometry+clip, binning, raster, resolve]. */
int sftg_last_timings(const sftg_ctx* ctx, float* out5);
/* Number of kernels launched by the last frame. */
int sftg_last_launch_count(const sftg_ctx* ctx);
/* The cudaStream_t the context renders on (for callers that time or order work around frames). */
void* sftg_stream(const sftg_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif
