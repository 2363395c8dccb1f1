/*
 * sofren2 for GB300 — drop-in replacement for the reference's single-header C API.
 *
 * Same names, signatures and frame contract as the reference's public API
 * (sofren2.c:744-863): lights, sft_set_color_buffer, sft_frame_begin, sft_set_camera,
 * sft_draw_instance ..., sft_present, sft_frame_end.  As with the reference, exactly one
 * translation unit defines SFT_IMPL before including this header; that TU gets the host
 * runtime below, which keeps the frame state in C and renders through the sftg C ABI
 * (include/sftg.h, libsofren2_gb300.so) on the GPU.  There is no CPU rendering path:
 * sft_init fails loudly when no CUDA device or library is available.
 *
 * Compile-time options kept from the reference: SFT_USE_AA / SFT_AA_SAMPLES (1, 2, 4),
 * SFT_FUNC, SFT_NO_DEBUG.  Additions (not in the reference) are marked "extension".
 */
#ifndef SOFREN2_GB300_H
#define SOFREN2_GB300_H

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "sftg.h"
#include "x86_approx_tables.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef int8_t i8; typedef uint8_t u8; typedef int16_t i16; typedef uint16_t u16;
typedef int32_t i32; typedef uint32_t u32; typedef int64_t i64; typedef uint64_t u64;
typedef float f32; typedef double f64;

enum sft_debug_mode {
    SFT_DEBUG_NONE, SFT_DEBUG_WIREFRAME, SFT_DEBUG_TILES, SFT_DEBUG_DEPTH,
    SFT_DEBUG_LIGHT_COUNT, SFT_DEBUG_CHECKERBOARD, SFT_DEBUG_COUNT
};
enum sft_dmesh_type { SFT_DMESH_QUADS, SFT_DMESH_TRIANGLES };

typedef u32 sft_tex_handle;
typedef u32 sft_mat_handle;
#define SFT_INVALID_HANDLE 0xFFFFFFFF
#define SFT_HANDLE_INDEX_MASK 0x0000FFFF
#define SFT_HANDLE_GEN_SHIFT 16
#define SFT_HANDLE_INDEX(h) ((h) & SFT_HANDLE_INDEX_MASK)
#define SFT_MAT_TRANSIENT_BIT 0x80000000
#define SFT_MAT_GEN_SHIFT 16
#define SFT_MAT_GEN_MASK 0x7FFF0000
#define SFT_MAT_INDEX_MASK 0x0000FFFF
#define SFT_MAT_IS_TRANSIENT(h) (0 != ((h) & SFT_MAT_TRANSIENT_BIT))
#define SFT_MAT_INDEX(h) ((h) & SFT_MAT_INDEX_MASK)

#define SFT_PI (3.14159265358979323846)
#define SFT_EPSILON (1e-6f)
#define SFT_V(a, b, c) (sftvec){ .x = (a), .y = (b), .z = (c) }
#define SFT_MAX_INSTANCES_PER_FRAME 64
#define SFT_VERTS_PER_MESHLET 64

#ifdef SFT_USE_AA
    #ifndef SFT_AA_SAMPLES
        #define SFT_AA_SAMPLES 4
    #endif
#else
    #ifndef SFT_AA_SAMPLES
        #define SFT_AA_SAMPLES 1
    #endif
#endif

#ifndef SFT_FUNC
    #define SFT_FUNC static
#endif

typedef struct sftvec { f32 x, y, z; } sftvec;
typedef struct sftquat { f32 x, y, z, w; } sftquat;
typedef union sftmat { sftquat rows[4]; f32 m[4][4]; } sftmat;

typedef struct sft_arena { u8* base; u64 max_size; u64 committed_size; u64 offset; volatile i32 commit_lock; } sft_arena;

typedef struct sft_model sft_model;      /* host mirror of a device-resident model */
typedef struct sft_dmesh sft_dmesh;
/* a batch of quads reserved in a dynamic mesh's current meshlet: the caller writes 4 vertices
 * per quad at vert_offset .. (sofren2.c:1167-1173) */
typedef struct sft_dmesh_qb {
    f32 *x, *y, *z;
    f32 *nx, *ny, *nz;
    f32 *u, *v;
    u32 vert_offset;
    u32 allocated_count;
} sft_dmesh_qb;

typedef struct sft_pose {
    const sft_model* model;
    sftmat* global_matrices;
    sftmat* posed_bone_matrices;
} sft_pose;

typedef struct sft_instance {
    const sft_model* model;
    sftmat transform;
    u32 ss_meshlet_offset;
    sftmat* posed_bone_matrices;
} sft_instance;

/* sofren2.c:895-900 */
typedef struct sft_ray_hit { u8 hit; f32 distance; sftvec pos; sftvec normal; } sft_ray_hit;

/* capsule shadow proxy in model (or bone) space, sofren2.c:985-989 */
typedef struct sft_shadow_proxy { sftvec posa, posb; f32 radius; u32 bone_ind; } sft_shadow_proxy;

/* extension: meshlet arrays of one mesh in the reference's layout (sofren2.c:914-953, 1071-1092) */
typedef struct sft_mesh_data {
    u32 meshlet_count;
    const f32* attr;            /* [meshlet][10][64]: x y z nx ny nz u v lu lv */
    const u8* inds;             /* [meshlet][512] */
    const f32* cull;            /* [meshlet][8]: sphere centre, radius, cone axis, cone cutoff */
    const u16* joints;          /* [meshlet][4][64] or NULL */
    const u8* weights;          /* [meshlet][4][64] or NULL */
    const i32* culling_bones;   /* [meshlet] or NULL */
    sft_mat_handle material;
    u32 lightmap_page;          /* index into the model's lightmaps, 0xFFFFFFFF = none */
} sft_mesh_data;

/* math (sofren2.c:745-792) */
SFT_FUNC sftvec sft_v_add(sftvec a, sftvec b);
SFT_FUNC sftvec sft_v_sub(sftvec a, sftvec b);
SFT_FUNC sftvec sft_v_mul(sftvec a, f32 b);
SFT_FUNC sftvec sft_v_div(sftvec a, f32 b);
SFT_FUNC f32 sft_v_dot(sftvec a, sftvec b);
SFT_FUNC sftvec sft_v_cross(sftvec a, sftvec b);
SFT_FUNC f32 sft_v_length(sftvec v);
SFT_FUNC f32 sft_v_length2(sftvec v);
SFT_FUNC sftvec sft_v_norm(sftvec v);
SFT_FUNC sftvec sft_v_normf(f32 x, f32 y, f32 z);
SFT_FUNC sftvec sft_v_lerp(sftvec a, sftvec b, f32 t);
SFT_FUNC sftmat sft_m_identity(void);
SFT_FUNC sftmat sft_m_rot_x(f32 a);
SFT_FUNC sftmat sft_m_rot_y(f32 a);
SFT_FUNC sftmat sft_m_rot_z(f32 a);
SFT_FUNC sftmat sft_m_translate(f32 x, f32 y, f32 z);
SFT_FUNC sftmat sft_m_scale(f32 x, f32 y, f32 z);
SFT_FUNC sftmat sft_m_proj(f32 fov_deg, f32 aspect, f32 near_z, f32 far_z);
SFT_FUNC sftmat sft_m_mul(sftmat a, sftmat b);
SFT_FUNC sftmat sft_m_qinv(sftmat m);
SFT_FUNC sftmat sft_m_view_look_at(sftvec pos, sftvec target, sftvec up);
SFT_FUNC sftmat sft_m_model_look_at(sftvec pos, sftvec target, sftvec up);
SFT_FUNC sftmat sft_m_ortho(f32 left, f32 right, f32 bottom, f32 top, f32 near_z, f32 far_z);
SFT_FUNC sftvec sft_m_mul_vec(sftmat m, sftvec v);
SFT_FUNC sftvec sft_m_mul_quat(sftmat m, sftquat v);
SFT_FUNC void sft_m_decompose(sftmat m, sftvec* pos, sftvec* rot, sftvec* scale);
SFT_FUNC sftquat sft_q_invert(sftquat q);
SFT_FUNC sftvec sft_v_face_normal(sftvec a, sftvec b, sftvec c);
SFT_FUNC sftvec sft_v_perpendicular(sftvec v);
SFT_FUNC sftvec sft_v_rotate_by_quat(sftvec v, sftquat q);
SFT_FUNC sftmat sft_m_from_quat(sftquat q);
SFT_FUNC sftquat sft_q_mul(sftquat a, sftquat b);
SFT_FUNC sftquat sft_q_slerp(sftquat a, sftquat b, f32 t);
SFT_FUNC sftquat sft_q_norm(sftquat q);

/* SoA math (sofren2.c:780-792, 1921-2060): eight lanes, the width of the reference's AVX2 build,
 * whose results these reproduce bit for bit on any host (x86-64 or aarch64): IEEE add, sub, mul,
 * div and sqrt per lane, a fused multiply-add exactly where the reference calls fmadd / fnmadd,
 * _mm256_max_ps's operand order, and RSQRTPS through the instruction's measured table
 * (x86_approx_tables.h).  Compile the calling TU with -ffp-contract=off, as the reference must be.
 * vf32 is a GCC/Clang vector of 8 floats (the same vector shape as __m256), so lanes can be
 * read and written as v[i] or with ordinary operators.  Like the reference's SFT_INLINE helpers,
 * these are static inline in every TU that includes this header, not library exports. */
#ifndef SFT_INLINE
    #define SFT_INLINE static inline
#endif
/* the helpers are static inline, so the calling convention of 32-byte vectors never crosses a TU */
#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Wpsabi"
typedef float vf32 __attribute__((vector_size(32)));
typedef struct sftvvec { vf32 x, y, z; } sftvvec;
typedef struct sftvquat { vf32 x, y, z, w; } sftvquat;
typedef union sftvmat { sftvquat rows[4]; vf32 m[4][4]; } sftvmat;

SFT_INLINE sftvvec sft_vv_add(sftvvec a, sftvvec b);
SFT_INLINE sftvvec sft_vv_sub(sftvvec a, sftvvec b);
SFT_INLINE sftvvec sft_vv_scale(sftvvec a, vf32 b);
SFT_INLINE vf32 sft_vv_dot(sftvvec a, sftvvec b);
SFT_INLINE sftvvec sft_vv_cross(sftvvec a, sftvvec b);
SFT_INLINE vf32 sft_vv_length2(sftvvec v);
SFT_INLINE vf32 sft_vv_length(sftvvec v);
SFT_INLINE sftvvec sft_vv_norm(sftvvec v);
SFT_INLINE sftvvec sft_vv_norm_fast(sftvvec v);
SFT_INLINE sftvvec sft_vv_transform(sftvvec v, sftvmat vm);
SFT_INLINE sftvvec sft_vv_transform_dir(sftvvec v, sftvmat vm);
SFT_INLINE sftvmat sft_vm_broadcast(sftmat m);

/* lane-wise fused multiply-add (_mm256_fmadd_ps) and -(a*b)+c (_mm256_fnmadd_ps) */
SFT_INLINE vf32 sft__vfma(vf32 a, vf32 b, vf32 c) { vf32 r; for (int i = 0; i < 8; i++) r[i] = fmaf(a[i], b[i], c[i]); return r; }
SFT_INLINE vf32 sft__vfnma(vf32 a, vf32 b, vf32 c) { vf32 r; for (int i = 0; i < 8; i++) r[i] = fmaf(-a[i], b[i], c[i]); return r; }
SFT_INLINE vf32 sft__vset1(f32 s) { vf32 r = { s, s, s, s, s, s, s, s }; return r; }
/* NaN lanes as x86 leaves them: from NaN-free inputs every NaN is born of an invalid operation
 * (0 * inf, inf - inf, inf / inf), whose SSE/AVX result is the default NaN 0xFFC00000, and later
 * arithmetic passes it on unchanged; aarch64 would give 0x7FC00000.  (NaN inputs also come out as
 * 0xFFC00000, where x86 would keep their payload.) */
SFT_INLINE vf32 sft__xnan(vf32 v) {
    const u32 dnan = 0xFFC00000u;
    for (int i = 0; i < 8; i++) if (v[i] != v[i]) memcpy((char*)&v + 4 * i, &dnan, 4);
    return v;
}
SFT_INLINE sftvvec sft__xnan3(sftvvec v) { v.x = sft__xnan(v.x); v.y = sft__xnan(v.y); v.z = sft__xnan(v.z); return v; }

SFT_INLINE sftvvec sft_vv_add(sftvvec a, sftvvec b) { sftvvec r = { a.x + b.x, a.y + b.y, a.z + b.z }; return sft__xnan3(r); }
SFT_INLINE sftvvec sft_vv_sub(sftvvec a, sftvvec b) { sftvvec r = { a.x - b.x, a.y - b.y, a.z - b.z }; return sft__xnan3(r); }
SFT_INLINE sftvvec sft_vv_scale(sftvvec a, vf32 b) { sftvvec r = { a.x * b, a.y * b, a.z * b }; return sft__xnan3(r); }
/* x*x' + (y*y' + z*z'), three products rounded separately */
SFT_INLINE vf32 sft_vv_dot(sftvvec a, sftvvec b) { const vf32 x = a.x * b.x, y = a.y * b.y, z = a.z * b.z; return sft__xnan(x + (y + z)); }
SFT_INLINE sftvvec sft_vv_cross(sftvvec a, sftvvec b) {
    sftvvec r = { a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x };
    return sft__xnan3(r);
}
SFT_INLINE vf32 sft_vv_length2(sftvvec v) { return sft_vv_dot(v, v); }
SFT_INLINE vf32 sft_vv_length(sftvvec v) {
    const vf32 d = sft_vv_dot(v, v);
    vf32 r; for (int i = 0; i < 8; i++) r[i] = sqrtf(d[i]);
    return sft__xnan(r);
}
/* v / max(|v|, SFT_EPSILON); max keeps _mm256_max_ps's rule (the second operand unless a > b) */
SFT_INLINE sftvvec sft_vv_norm(sftvvec v) {
    vf32 len = sft_vv_length(v);
    for (int i = 0; i < 8; i++) len[i] = len[i] > SFT_EPSILON ? len[i] : SFT_EPSILON;
    sftvvec r = { v.x / len, v.y / len, v.z / len };
    return sft__xnan3(r);
}
/* RSQRTPS of one lane: the measured 11-bit estimate of x86 (zero and denormals give +-inf,
 * negatives the default NaN, +inf gives 0, NaN stays NaN, quieted) */
SFT_INLINE f32 sft__x86_rsqrt(f32 xf) {
    static const u32 tab[2048] = SFT_X86_RSQRT_TABLE_INIT;
    u32 x, s, e, m, out;
    memcpy(&x, &xf, 4);
    s = x & 0x80000000u; e = (x >> 23) & 0xFF; m = x & 0x7FFFFF;
    if (e == 0xFF) out = m ? (x | 0x00400000u) : (s ? 0xFFC00000u : 0u);
    else if (e == 0) out = s | 0x7F800000u;
    else if (s) out = 0xFFC00000u;
    else {
        const u32 t = tab[(e & 1) * 1024 + (m >> 13)];
        out = ((u32)(((380 - (i32)e) >> 1) + (i32)(t >> 23) - 1) << 23) | (t & 0x7FFFFF);
    }
    memcpy(&xf, &out, 4);
    return xf;
}
/* one Newton step on the estimate: (0.5 * a) * fnmadd(|v|^2, a*a, 3); a zero vector gives
 * 0 * inf there, so NaN lanes */
SFT_INLINE sftvvec sft_vv_norm_fast(sftvvec v) {
    const vf32 sq = sft_vv_dot(v, v);
    vf32 a; for (int i = 0; i < 8; i++) a[i] = sft__x86_rsqrt(sq[i]);
    const vf32 refined = (sft__vset1(0.5f) * a) * sft__vfnma(sq, a * a, sft__vset1(3.f));
    sftvvec r = { v.x * refined, v.y * refined, v.z * refined };
    return sft__xnan3(r);
}
/* row-vector transform, each component accumulated z, then y, then x, fused */
SFT_INLINE sftvvec sft_vv_transform(sftvvec v, sftvmat vm) {
    sftvvec r;
    r.x = sft__vfma(v.x, vm.m[0][0], sft__vfma(v.y, vm.m[1][0], sft__vfma(v.z, vm.m[2][0], vm.m[3][0])));
    r.y = sft__vfma(v.x, vm.m[0][1], sft__vfma(v.y, vm.m[1][1], sft__vfma(v.z, vm.m[2][1], vm.m[3][1])));
    r.z = sft__vfma(v.x, vm.m[0][2], sft__vfma(v.y, vm.m[1][2], sft__vfma(v.z, vm.m[2][2], vm.m[3][2])));
    return sft__xnan3(r);
}
SFT_INLINE sftvvec sft_vv_transform_dir(sftvvec v, sftvmat vm) {
    sftvvec r;
    r.x = sft__vfma(v.x, vm.m[0][0], sft__vfma(v.y, vm.m[1][0], v.z * vm.m[2][0]));
    r.y = sft__vfma(v.x, vm.m[0][1], sft__vfma(v.y, vm.m[1][1], v.z * vm.m[2][1]));
    r.z = sft__vfma(v.x, vm.m[0][2], sft__vfma(v.y, vm.m[1][2], v.z * vm.m[2][2]));
    return sft__xnan3(r);
}
SFT_INLINE sftvmat sft_vm_broadcast(sftmat m) {
    sftvmat vm;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) vm.m[i][j] = sft__vset1(m.m[i][j]);
    return vm;
}
#pragma GCC diagnostic pop

/* core (sofren2.c:795-800) */
SFT_FUNC void sft_init(i32 width, i32 height, i32 requested_threads);
SFT_FUNC void sft_release(void);
SFT_FUNC void sft_present(void);
SFT_FUNC void sft_frame_begin(void);
SFT_FUNC void sft_frame_end(void);
SFT_FUNC void sft_resize(i32 width, i32 height);

/* misc (803-808) */
SFT_FUNC void sft_set_camera(sftvec cam_pos, sftmat view, sftmat proj);
SFT_FUNC void sft_set_debug_mode(enum sft_debug_mode mode);
SFT_FUNC const char* sft_get_debug_name(enum sft_debug_mode mode);
SFT_FUNC void sft_set_clear(u8 enabled);
SFT_FUNC void sft_set_clear_color(u32 color);
SFT_FUNC void sft_set_color_buffer(u32* buf, i32 pitch_in_bytes);

/* drawing (811-824) */
SFT_FUNC void sft_draw_instance(const sft_instance* instance);
SFT_FUNC void sft_draw_cube(sft_dmesh* dm);
SFT_FUNC void sft_draw_cube_inv(sft_dmesh* dm);
SFT_FUNC void sft_draw_sphere(sft_dmesh* dm, i32 rings, i32 slices);
SFT_FUNC void sft_draw_capsule(sft_dmesh* dm, sftvec start_pos, sftvec end_pos, f32 radius, i32 slices, i32 rings);
SFT_FUNC void sft_draw_cylinder(sft_dmesh* dm, sftvec start_pos, sftvec end_pos, f32 start_radius, f32 end_radius, i32 sides);
SFT_FUNC sft_dmesh* sft_dmesh_begin(enum sft_dmesh_type type, sft_mat_handle material, u32 max_prims);
SFT_FUNC void sft_dmesh_push_quad(sft_dmesh* dm, sftvec p0, sftvec p1, sftvec p2, sftvec p3, f32 u0, f32 v0, f32 u1, f32 v1, sftvec normal);
SFT_FUNC void sft_dmesh_push_quad_4n(sft_dmesh* dm, sftvec p0, sftvec p1, sftvec p2, sftvec p3, f32 u0, f32 v0, f32 u1, f32 v1,
                                     sftvec n0, sftvec n1, sftvec n2, sftvec n3);
SFT_FUNC void sft_dmesh_push_tri(sft_dmesh* dm, sftvec p0, sftvec p1, sftvec p2, f32 u0, f32 v0, f32 u1, f32 v1, f32 u2, f32 v2, sftvec normal);
SFT_FUNC u8 sft_dmesh_alloc_quads(sft_dmesh* dm, u32 count, sft_dmesh_qb* out_batch);
SFT_FUNC void sft_dmesh_end(sft_dmesh* dm, const sftmat* opt_transform);
SFT_FUNC sft_pose* sft_pose_create(const sft_model* model, sft_arena* arena);
SFT_FUNC void sft_pose_update(sft_pose* pose, i32 anim_id, f32 time);
/* ray queries (sofren2.c:3733): answered on the GPU; the batch form is one launch for n rays,
 * ray k against insts[k] */
SFT_FUNC sft_ray_hit sft_raycast_instance(const sft_instance* inst, sftvec origin, sftvec dir, f32 max_dist);
SFT_FUNC void sft_raycast_batch(const sft_instance* const* insts, const sftvec* origins, const sftvec* dirs, const f32* max_dists,
                                u32 n, sft_ray_hit* out);

/* lights (827-832) */
SFT_FUNC void sft_set_ambient_light(f32 r, f32 g, f32 b);
SFT_FUNC void sft_draw_directional_light(sftvec dir, f32 r, f32 g, f32 b, f32 intensity);
SFT_FUNC void sft_draw_point_light(sftvec pos, f32 r, f32 g, f32 b, f32 intensity, f32 radius, u32 light_id);
SFT_FUNC void sft_set_shadows_enabled(u8 enabled);
SFT_FUNC void sft_set_lightmap_brightness(f32 b);

/* textures (839-844) */
SFT_FUNC sft_tex_handle sft_texture_create(i32 width, i32 height, const u32* pixels);
SFT_FUNC sft_tex_handle sft_texture_create_solid(u32 color);
SFT_FUNC i32 sft_texture_get_width(sft_tex_handle tex);
SFT_FUNC i32 sft_texture_get_height(sft_tex_handle tex);
SFT_FUNC u32* sft_texture_get_linear_pixels(sft_tex_handle tex);
SFT_FUNC void sft_texture_release(sft_tex_handle tex);

/* materials (847-849) */
SFT_FUNC sft_mat_handle sft_material_create(sft_tex_handle tex, u32 base_color, f32 shininess);
SFT_FUNC sft_mat_handle sft_material_clone(sft_mat_handle base_mat);
SFT_FUNC void sft_material_release(sft_mat_handle mat);

/* arenas (852-855) */
SFT_FUNC void sft_arena_init(sft_arena* arena, u64 reserve_size);
SFT_FUNC void* sft_arena_alloc(sft_arena* arena, u64 size);
SFT_FUNC void sft_arena_commit_if_needed(sft_arena* arena, u64 required_bytes);
SFT_FUNC void sft_arena_frame_begin(sft_arena* arena);

/* extension: build a model from meshlet data (the reference's loaders produce the same
 * arrays, sofren2.c:6918-7045); uploads everything to the GPU and builds the BLAS there like
 * sft__blas_build_model (3526-3617).  lightmaps are texture handles indexed by lightmap_page. */
SFT_FUNC sft_model* sft_model_create(const sft_mesh_data* meshes, u32 mesh_count, const sft_shadow_proxy* proxies,
                                     u32 proxy_count, u32 bone_count, const sft_tex_handle* lightmaps, u32 lightmap_count,
                                     sft_arena* arena);
SFT_FUNC u32 sft_model_get_meshlet_count(const sft_model* model);
/* extension: load-time builders of the reference's GLB loader (sofren2.c:7426-7700), for callers
 * that hold raw triangles instead of a .glb file.  One raw mesh is what the loader gathers per
 * material before it builds meshlets: vertex streams and a triangle list. */
typedef struct sft_raw_mesh {
    u32 vertex_count, triangle_count;
    const f32* pos;        /* [vertex][3] */
    const f32* nrm;        /* [vertex][3] */
    const f32* uv;         /* [vertex][2] */
    const u16* joints;     /* [vertex][4] skeleton joint indices, or NULL for a static mesh */
    const u8* weights;     /* [vertex][4], 255 = 1 (with joints) */
    const i32* indices;    /* [triangle][3] vertex indices, in the winding the renderer draws */
    sft_mat_handle material;
} sft_raw_mesh;
/* extension: a skeleton joint as the shadow-proxy fitter sees it: parent (-1 for a root) and the
 * joint's bind position (sft_bone.parent_ind / bind_pos, sofren2.c:1000-1010) */
typedef struct sft_raw_bone { i32 parent_ind; sftvec bind_pos; } sft_raw_bone;
/* extension: the meshlets of one raw mesh as the reference's loader builds them (sofren2.c:
 * 7467-7660): greedy growth over triangle adjacency (vertex reuse first, normal cone second, at
 * most 64 vertices and 128 triangles), the 8-lane index swizzle, Welzl bounding spheres
 * (2255-2289), normal cones, and for a skinned mesh the per-meshlet culling joint (6918-7045).
 * Arrays in sft_mesh_data's layout; up to `cap` meshlets are written and the meshlet count is
 * returned (call again with larger arrays when it exceeds cap).  joints, weights and
 * culling_bones may be NULL for a static mesh.  Like the reference, Welzl draws from the C
 * library's rand(): seed it (srand) for repeatable results. */
SFT_FUNC u32 sft_mesh_build_meshlets(const sft_raw_mesh* mesh, u32 bone_count, u32 cap, f32* attr, u8* inds, f32* cull,
                                     u16* joints, u8* weights, i32* culling_bones);
/* extension: the shadow proxies the reference fits at load (sofren2.c:3064-3524): with a
 * skeleton, one capsule per joint cluster (triangles voted to their heaviest joint, clusters
 * merged by area into their parents down to `budget`, capsules anchored at the joints); without
 * one, capsules fitted to the vertices under the BLAS nodes that splitting the largest volumes
 * gives.  blas_nodes: the model's sft_bvh_node images (256 B each).  Writes up to cap proxies and
 * returns their count (0 for budget <= 0 or no BLAS). */
SFT_FUNC u32 sft_model_fit_shadow_proxies(const sft_mesh_data* meshes, u32 mesh_count, const void* blas_nodes, u32 blas_count,
                                          u32 blas_root, const sft_raw_bone* bones, u32 bone_count, i32 budget,
                                          sft_shadow_proxy* out, u32 cap);
/* extension: a model from raw meshes, as sft_model_load_glb makes one from a file: meshlets built
 * on the host (sft_mesh_build_meshlets), the BLAS on the GPU, then the shadow proxies fitted
 * (sft_model_fit_shadow_proxies).  bones may be NULL (bone_count 0) for a static model. */
SFT_FUNC sft_model* sft_model_build(const sft_raw_mesh* meshes, u32 mesh_count, const sft_raw_bone* bones, u32 bone_count,
                                    i32 shadow_proxy_budget, sft_arena* arena);
/* model loading (sofren2.c:859-862): QSF2 files; GLB needs cgltf and is not provided */
SFT_FUNC sft_model* sft_model_load_qsf(const char* path, sft_arena* arena);
/* extension: the model's skeleton and animation tracks, what the reference's GLB loader fills
 * (sft_bone / sft_animation, sofren2.c:1000-1049); uploaded for sft_pose_update, which then
 * evaluates poses on the GPU.  bone_count must be the model's.  Returns 0 or an sftg error. */
SFT_FUNC i32 sft_model_set_skeleton(sft_model* model, const sftg_bone_desc* bones, u32 bone_count,
                                    const sftg_animation_desc* anims, u32 anim_count);
/* extension: MSAA samples (1, 2, 4) of the shared library build; SFT_AA_SAMPLES sets it in SFT_IMPL builds */
SFT_FUNC void sft_set_msaa_samples(i32 samples);
/* extension: last error text of the GPU runtime ("" when none) */
SFT_FUNC const char* sft_get_last_error(void);
/* extension: capture parity buffers for the next sft_present (struct sftg_debug_out from sftg.h, or NULL) */
SFT_FUNC void sft_set_debug_capture(void* sftg_debug_out_or_null);
/* extension: BLAS of a model as sft_bvh_node images (256 B each) */
SFT_FUNC const void* sft_model_get_blas(const sft_model* model, u32* out_count, u32* out_root);
/* extension: device time of the last present, ms: [occlusion, geometry, binning, raster, resolve] */
SFT_FUNC void sft_get_frame_timings(f32* out5);
/* extension: kernels launched by the last present, and the CUDA stream the runtime renders on */
SFT_FUNC i32 sft_get_launch_count(void);
SFT_FUNC void* sft_get_cuda_stream(void);
/* extension: batched submission.  Between sft_batch_begin and sft_batch_submit, sft_present
 * records the frame (camera, size, instances, poses, lights, proxies, colour buffer) instead of
 * rendering it; sft_batch_submit renders every recorded frame in one GPU submission
 * (sftg_frames_render) and writes each into the colour buffer that was set for it, leaving the
 * colour in device memory for frames recorded without one.  Each frame's pixels are those
 * sft_present would have produced alone.  Returns 0 or a negative sftg error code. */
SFT_FUNC void sft_batch_begin(void);
SFT_FUNC i32 sft_batch_submit(void);
/* extension: the i-th frame recorded since sft_batch_begin (a struct sftg_frame_desc, valid until
 * sft_batch_submit), and the sftg context the runtime renders with, for direct sftg_* calls */
SFT_FUNC const void* sft_batch_peek(u32 i);
/* extension: instead of rendering the recorded frames, tune the scheduling knobs on them
 * (sftg_autotune, reps renders per candidate) and drop them; ends the batch */
SFT_FUNC i32 sft_batch_autotune(i32 reps);
SFT_FUNC void* sft_get_gpu_context(void);
/* extension: overlapping batches.  sft_batch_submit_async ends the batch like sft_batch_submit
 * but queues it on submission lane `lane` (1 to SFTG_MAX_LANES - 1) and returns at once (a
 * batch still on that lane is waited for first); the colour buffers must stay untouched until
 * sft_batch_wait(lane) returns, which waits for the batch and gives its status.  sft_batch_done(lane) is 1 once the lane's batch has finished
 * (or the lane is idle), 0 while it runs.  Batches on different lanes overlap on the GPU. */
SFT_FUNC i32 sft_batch_submit_async(u32 lane);
SFT_FUNC i32 sft_batch_done(u32 lane);
SFT_FUNC i32 sft_batch_wait(u32 lane);

#ifdef __cplusplus
}
#endif

/*================================================================ implementation */
#ifdef SFT_IMPL

#include "sftg.h"
#include <sys/mman.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifdef SFT_NO_DEBUG
    #define SFT__LOG(...)
#else
    #define SFT__LOG(...) do { fprintf(stdout, "[sofren2-gb300]: "); fprintf(stdout, __VA_ARGS__); } while (0)
#endif
#define SFT__FATAL(...) do { fprintf(stderr, "fatal sofren2-gb300 error in %s: ", __func__); fprintf(stderr, __VA_ARGS__); exit(1); } while (0)

/* sft_bvh_node image (sofren2.c:967-983) */
typedef struct sft__node {
    f32 mn[3][8]; f32 mx[3][8];
    u32 child[8]; u8 count; u8 leaf; u8 pad[30];
} sft__node;

typedef struct sft__item { u32 id; f32 mn[3], mx[3], c[3]; } sft__item;

struct sft_model {
    i32 device_id;
    i32 skeleton_id;              /* sftg skeleton with the model's animations, -1 when none */
    u32 mesh_count, total_meshlets, bone_count;
    u32* mesh_first;              /* per mesh: first model meshlet */
    u32* mesh_meshlets;
    sft_shadow_proxy* proxies; u32 proxy_count;
    sft__node* blas; u32 blas_count, blas_root;
    f32 root_min[3], root_max[3]; /* from the BLAS root children, for the TLAS */
};

typedef struct sft__tex {
    u32 generation; i32 next_free; i32 device_index;
    i32 w, h, levels; u8 is_pot;
    u32* level0;                  /* linear copy of level 0 for sft_texture_get_linear_pixels */
    u8 live;
} sft__tex;

static struct sft__state {
    sftg_ctx* gpu;
    i32 width, height, samples;
    u32* color; i32 pitch;
    u8 clear; u32 clear_color; u8 shadows; enum sft_debug_mode debug_mode;
    sftvec cam; sftmat view, proj, view_proj;
    f32 fn[6][3], fd[6];
    sftvec ambient; f32 lightmap_brightness;
    f32* point; u32 n_point, cap_point;        /* 8 floats per light */
    f32* dir; u32 n_dir, cap_dir;              /* 6 floats per light */
    sftg_instance_desc inst[SFT_MAX_INSTANCES_PER_FRAME]; i32 n_inst_claimed; u32 n_inst;
    const sft_model* inst_model[SFT_MAX_INSTANCES_PER_FRAME];
    f32* bones; u32 n_bones, cap_bones;        /* copies of posed matrices for this frame */
    u32 inst_bone_off[SFT_MAX_INSTANCES_PER_FRAME];
    f32* proxies; u32 n_prox, cap_prox;        /* 8 floats per world proxy */
    u32 total_ss;
    sft__tex* tex; i32 tex_cap, tex_free;
    u32* mat_gen; i32* mat_next; i32 mat_cap, mat_free;
    i32 n_transient;
    sft_mat_handle base_mat;
    sft_tex_handle checker_tex;    /* the base material's albedo, for SFT_DEBUG_CHECKERBOARD */
    sftg_debug_out* debug;
    char err[512];
    /* dynamic meshes of the current frame: index templates, open meshes, transient models */
    u8 dmesh_quad_inds[512], dmesh_tri_inds[512];
    struct sft_dmesh* dmesh_list;
    struct sft__transient* transient_list;
    /* batched submission: frames recorded by sft_present between sft_batch_begin / _submit */
    u8 batching; u32 n_batch, cap_batch;
    sftg_frame_desc* batch_fd; u32** batch_color; i32* batch_pitch; void** batch_mem;
    /* batches handed to submission lanes, kept until sft_batch_wait */
    struct { sftg_frame_desc* fd; u32** color; i32* pitch; void** mem; u32 n; } lane[SFTG_MAX_LANES];
} *sft__s;

/* ---------------------------------------------------------------- math (sofren2.c:1503-1918) */
SFT_FUNC sftvec sft_v_add(sftvec a, sftvec b) { sftvec r = { a.x + b.x, a.y + b.y, a.z + b.z }; return r; }
SFT_FUNC sftvec sft_v_sub(sftvec a, sftvec b) { sftvec r = { a.x - b.x, a.y - b.y, a.z - b.z }; return r; }
SFT_FUNC sftvec sft_v_mul(sftvec a, f32 b) { sftvec r = { a.x * b, a.y * b, a.z * b }; return r; }
SFT_FUNC sftvec sft_v_div(sftvec a, f32 b) { const f32 ib = 1.f / b; sftvec r = { a.x * ib, a.y * ib, a.z * ib }; return r; }
SFT_FUNC f32 sft_v_dot(sftvec a, sftvec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
SFT_FUNC sftvec sft_v_cross(sftvec a, sftvec b) { sftvec r = { a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x }; return r; }
SFT_FUNC f32 sft_v_length(sftvec v) { return sqrtf(sft_v_dot(v, v)); }
SFT_FUNC f32 sft_v_length2(sftvec v) { return sft_v_dot(v, v); }
SFT_FUNC sftvec sft_v_norm(sftvec v) { const f32 l = sft_v_length(v); if (l > SFT_EPSILON) return sft_v_mul(v, 1.f / l); sftvec z = { 0, 0, 0 }; return z; }
SFT_FUNC sftvec sft_v_normf(f32 x, f32 y, f32 z) { sftvec v = { x, y, z }; return sft_v_norm(v); }
SFT_FUNC sftvec sft_v_lerp(sftvec a, sftvec b, f32 t) { return sft_v_add(a, sft_v_mul(sft_v_sub(b, a), t)); }
SFT_FUNC sftmat sft_m_identity(void) { sftmat r; memset(&r, 0, sizeof(r)); r.m[0][0] = r.m[1][1] = r.m[2][2] = r.m[3][3] = 1.f; return r; }
SFT_FUNC sftmat sft_m_rot_x(f32 a) { sftmat r = sft_m_identity(); const f32 c = cosf(a), s = sinf(a); r.m[1][1] = c; r.m[1][2] = s; r.m[2][1] = -s; r.m[2][2] = c; return r; }
SFT_FUNC sftmat sft_m_rot_y(f32 a) { sftmat r = sft_m_identity(); const f32 c = cosf(a), s = sinf(a); r.m[0][0] = c; r.m[0][2] = s; r.m[2][0] = -s; r.m[2][2] = c; return r; }
SFT_FUNC sftmat sft_m_rot_z(f32 a) { sftmat r = sft_m_identity(); const f32 c = cosf(a), s = sinf(a); r.m[0][0] = c; r.m[0][1] = s; r.m[1][0] = -s; r.m[1][1] = c; return r; }
SFT_FUNC sftmat sft_m_translate(f32 x, f32 y, f32 z) { sftmat r = sft_m_identity(); r.m[3][0] = x; r.m[3][1] = y; r.m[3][2] = z; return r; }
SFT_FUNC sftmat sft_m_scale(f32 x, f32 y, f32 z) { sftmat r = sft_m_identity(); r.m[0][0] = x; r.m[1][1] = y; r.m[2][2] = z; return r; }
SFT_FUNC sftmat sft_m_proj(f32 fov_deg, f32 aspect, f32 near_z, f32 far_z) {
    const f32 fov = 1.f / tanf(fov_deg * 0.5f / 180.f * (f32)SFT_PI);
    sftmat r; memset(&r, 0, sizeof(r));
    r.m[0][0] = fov / aspect; r.m[1][1] = fov; r.m[2][2] = far_z / (far_z - near_z);
    r.m[3][2] = (-far_z * near_z) / (far_z - near_z); r.m[2][3] = 1.f; r.m[3][3] = 0.f;
    return r;
}
SFT_FUNC sftmat sft_m_mul(sftmat a, sftmat b) {   /* left-to-right sums, no contraction (sofren2.c:1668) */
    sftmat r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j] + a.m[i][3] * b.m[3][j];
    return r;
}
SFT_FUNC sftmat sft_m_qinv(sftmat m) {
    sftmat r;
    r.m[0][0] = m.m[0][0]; r.m[0][1] = m.m[1][0]; r.m[0][2] = m.m[2][0]; r.m[0][3] = 0.f;
    r.m[1][0] = m.m[0][1]; r.m[1][1] = m.m[1][1]; r.m[1][2] = m.m[2][1]; r.m[1][3] = 0.f;
    r.m[2][0] = m.m[0][2]; r.m[2][1] = m.m[1][2]; r.m[2][2] = m.m[2][2]; r.m[2][3] = 0.f;
    for (int a = 0; a < 3; a++) r.m[3][a] = -(m.m[3][0] * r.m[0][a] + m.m[3][1] * r.m[1][a] + m.m[3][2] * r.m[2][a]);
    r.m[3][3] = 1.f;
    return r;
}
SFT_FUNC sftmat sft_m_view_look_at(sftvec pos, sftvec target, sftvec up) {
    const sftvec fwd = sft_v_norm(sft_v_sub(target, pos));
    if (fabsf(fwd.x) < SFT_EPSILON && fabsf(fwd.z) < SFT_EPSILON) { up.x = 0.f; up.y = 0.f; up.z = -1.f; }
    up = sft_v_norm(sft_v_sub(up, sft_v_mul(fwd, sft_v_dot(up, fwd))));
    const sftvec right = sft_v_cross(up, fwd);
    sftmat r;
    r.m[0][0] = right.x; r.m[0][1] = up.x; r.m[0][2] = fwd.x; r.m[0][3] = 0.f;
    r.m[1][0] = right.y; r.m[1][1] = up.y; r.m[1][2] = fwd.y; r.m[1][3] = 0.f;
    r.m[2][0] = right.z; r.m[2][1] = up.z; r.m[2][2] = fwd.z; r.m[2][3] = 0.f;
    r.m[3][0] = -sft_v_dot(pos, right); r.m[3][1] = -sft_v_dot(pos, up); r.m[3][2] = -sft_v_dot(pos, fwd); r.m[3][3] = 1.f;
    return r;
}
SFT_FUNC sftmat sft_m_from_quat(sftquat q) {
    sftmat m = sft_m_identity();
    const f32 x2 = q.x + q.x, y2 = q.y + q.y, z2 = q.z + q.z;
    const f32 xx = q.x * x2, xy = q.x * y2, xz = q.x * z2, yy = q.y * y2, yz = q.y * z2, zz = q.z * z2;
    const f32 wx = q.w * x2, wy = q.w * y2, wz = q.w * z2;
    m.m[0][0] = 1.f - (yy + zz); m.m[0][1] = xy + wz; m.m[0][2] = xz - wy;
    m.m[1][0] = xy - wz; m.m[1][1] = 1.f - (xx + zz); m.m[1][2] = yz + wx;
    m.m[2][0] = xz + wy; m.m[2][1] = yz - wx; m.m[2][2] = 1.f - (xx + yy);
    return m;
}
SFT_FUNC sftquat sft_q_mul(sftquat a, sftquat b) {
    sftquat r;
    r.x = a.x * b.w + a.y * b.z - a.z * b.y + a.w * b.x;
    r.y = -a.x * b.z + a.y * b.w + a.z * b.x + a.w * b.y;
    r.z = a.x * b.y - a.y * b.x + a.z * b.w + a.w * b.z;
    r.w = -a.x * b.x - a.y * b.y - a.z * b.z + a.w * b.w;
    return r;
}
SFT_FUNC sftquat sft_q_norm(sftquat q) {
    const f32 l2 = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
    if (l2 != 0.f) { const f32 il = 1.f / sqrtf(l2); q.x *= il; q.y *= il; q.z *= il; q.w *= il; }
    return q;
}
SFT_FUNC sftquat sft_q_slerp(sftquat a, sftquat b, f32 t) {
    f32 dot = a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
    if (dot < 0.f) { b.x = -b.x; b.y = -b.y; b.z = -b.z; b.w = -b.w; dot = -dot; }
    if (dot > 0.9995f) {
        sftquat r = { a.x + t * (b.x - a.x), a.y + t * (b.y - a.y), a.z + t * (b.z - a.z), a.w + t * (b.w - a.w) };
        return sft_q_norm(r);
    }
    const f32 th0 = acosf(dot), th = th0 * t, st = sinf(th), is0 = 1.f / sinf(th0);
    const f32 s0 = cosf(th) - dot * st * is0, s1 = st * is0;
    sftquat r = { a.x * s0 + b.x * s1, a.y * s0 + b.y * s1, a.z * s0 + b.z * s1, a.w * s0 + b.w * s1 };
    return sft_q_norm(r);
}

/* the remaining scalar helpers of the public math set (sofren2.c:1556-1600, 1657-1800, 1894) */
SFT_FUNC sftmat sft_m_model_look_at(sftvec pos, sftvec target, sftvec up) {
    const sftvec fwd = sft_v_norm(sft_v_sub(target, pos));
    up = sft_v_norm(sft_v_sub(up, sft_v_mul(fwd, sft_v_dot(up, fwd))));
    const sftvec right = sft_v_cross(up, fwd);
    sftmat r;
    r.m[0][0] = right.x; r.m[0][1] = right.y; r.m[0][2] = right.z; r.m[0][3] = 0.f;
    r.m[1][0] = up.x; r.m[1][1] = up.y; r.m[1][2] = up.z; r.m[1][3] = 0.f;
    r.m[2][0] = fwd.x; r.m[2][1] = fwd.y; r.m[2][2] = fwd.z; r.m[2][3] = 0.f;
    r.m[3][0] = pos.x; r.m[3][1] = pos.y; r.m[3][2] = pos.z; r.m[3][3] = 1.f;
    return r;
}
SFT_FUNC sftmat sft_m_ortho(f32 left, f32 right, f32 bottom, f32 top, f32 near_z, f32 far_z) {
    sftmat r;
    memset(&r, 0, sizeof(r));
    r.m[0][0] = 2.f / (right - left); r.m[1][1] = 2.f / (top - bottom); r.m[2][2] = 1.f / (far_z - near_z);
    r.m[3][0] = -(right + left) / (right - left); r.m[3][1] = -(top + bottom) / (top - bottom);
    r.m[3][2] = -near_z / (far_z - near_z); r.m[3][3] = 1.f;
    return r;
}
SFT_FUNC sftvec sft_m_mul_vec(sftmat m, sftvec v) {
    sftvec r = { v.x * m.m[0][0] + v.y * m.m[1][0] + v.z * m.m[2][0], v.x * m.m[0][1] + v.y * m.m[1][1] + v.z * m.m[2][1],
                 v.x * m.m[0][2] + v.y * m.m[1][2] + v.z * m.m[2][2] };
    return r;
}
SFT_FUNC sftvec sft_m_mul_quat(sftmat m, sftquat v) {
    sftvec r = { v.x * m.m[0][0] + v.y * m.m[1][0] + v.z * m.m[2][0] + v.w * m.m[3][0],
                 v.x * m.m[0][1] + v.y * m.m[1][1] + v.z * m.m[2][1] + v.w * m.m[3][1],
                 v.x * m.m[0][2] + v.y * m.m[1][2] + v.z * m.m[2][2] + v.w * m.m[3][2] };
    return r;
}
/* translation from row 3, scale from the basis rows' lengths, rotation as x-y-z Euler angles
 * (a rotation about y near +-90 degrees puts all of x's and z's share into x) */
SFT_FUNC void sft_m_decompose(sftmat m, sftvec* pos, sftvec* rot, sftvec* scale) {
    if (pos) { pos->x = m.m[3][0]; pos->y = m.m[3][1]; pos->z = m.m[3][2]; }
    f32 sx = sqrtf(m.m[0][0] * m.m[0][0] + m.m[0][1] * m.m[0][1] + m.m[0][2] * m.m[0][2]);
    f32 sy = sqrtf(m.m[1][0] * m.m[1][0] + m.m[1][1] * m.m[1][1] + m.m[1][2] * m.m[1][2]);
    f32 sz = sqrtf(m.m[2][0] * m.m[2][0] + m.m[2][1] * m.m[2][1] + m.m[2][2] * m.m[2][2]);
    if (scale) { scale->x = sx; scale->y = sy; scale->z = sz; }
    if (!rot) return;
    if (sx < SFT_EPSILON) sx = 1.f;
    if (sy < SFT_EPSILON) sy = 1.f;
    if (sz < SFT_EPSILON) sz = 1.f;
    const f32 r00 = m.m[0][0] / sx, r01 = m.m[0][1] / sx, r02 = m.m[0][2] / sx;
    const f32 r11 = m.m[1][1] / sy, r12 = m.m[1][2] / sy, r21 = m.m[2][1] / sz, r22 = m.m[2][2] / sz;
    rot->y = -asinf(r02 < -1.f ? -1.f : (r02 > 1.f ? 1.f : r02));
    if (cosf(rot->y) > SFT_EPSILON) { rot->x = atan2f(r12, r22); rot->z = atan2f(r01, r00); }
    else { rot->x = atan2f(-r21, r11); rot->z = 0.f; }
}
SFT_FUNC sftquat sft_q_invert(sftquat q) {
    sftquat r = q;
    const f32 l2 = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
    if (0.f != l2) { const f32 il = 1.f / l2; r.x *= -il; r.y *= -il; r.z *= -il; r.w *= il; }
    return r;
}
SFT_FUNC sftvec sft_v_face_normal(sftvec a, sftvec b, sftvec c) { return sft_v_norm(sft_v_cross(sft_v_sub(b, a), sft_v_sub(c, a))); }
SFT_FUNC sftvec sft_v_perpendicular(sftvec v) {
    f32 mn = fabsf(v.x);
    sftvec ax = { 1.f, 0.f, 0.f };
    if (fabsf(v.y) < mn) { mn = fabsf(v.y); ax.x = 0.f; ax.y = 1.f; ax.z = 0.f; }
    if (fabsf(v.z) < mn) { ax.x = 0.f; ax.y = 0.f; ax.z = 1.f; }
    sftvec r = { v.y * ax.z - v.z * ax.y, v.z * ax.x - v.x * ax.z, v.x * ax.y - v.y * ax.x };
    return r;
}
SFT_FUNC sftvec sft_v_rotate_by_quat(sftvec v, sftquat q) {
    sftvec r;
    r.x = v.x * (q.x * q.x + q.w * q.w - q.y * q.y - q.z * q.z) + v.y * (2 * q.x * q.y - 2 * q.w * q.z) + v.z * (2 * q.x * q.z + 2 * q.w * q.y);
    r.y = v.x * (2 * q.w * q.z + 2 * q.x * q.y) + v.y * (q.w * q.w - q.x * q.x + q.y * q.y - q.z * q.z) + v.z * (-2 * q.w * q.x + 2 * q.y * q.z);
    r.z = v.x * (-2 * q.w * q.y + 2 * q.x * q.z) + v.y * (2 * q.w * q.x + 2 * q.y * q.z) + v.z * (q.w * q.w - q.x * q.x - q.y * q.y + q.z * q.z);
    return r;
}

/* ---------------------------------------------------------------- arenas (sofren2.c:9456-9564) */
SFT_FUNC void sft_arena_init(sft_arena* arena, u64 reserve_size) {
    arena->max_size = reserve_size; arena->committed_size = reserve_size; arena->offset = 0; arena->commit_lock = 0;
    arena->base = (u8*)mmap(NULL, reserve_size, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
    if (arena->base == (u8*)MAP_FAILED) SFT__FATAL("mmap reserve of %llu bytes failed\n", (unsigned long long)reserve_size);
}
SFT_FUNC void* sft_arena_alloc(sft_arena* arena, u64 size) {
    if (!arena) return NULL;
    const u64 a = (arena->offset + 63ull) & ~63ull;
    if (a + size > arena->max_size) SFT__FATAL("arena out of memory (%llu of %llu)\n", (unsigned long long)(a + size), (unsigned long long)arena->max_size);
    arena->offset = a + size;
    return arena->base + a;
}
SFT_FUNC void sft_arena_commit_if_needed(sft_arena* arena, u64 required_bytes) { (void)arena; (void)required_bytes; }
SFT_FUNC void sft_arena_frame_begin(sft_arena* arena) { arena->offset = 0; }

/* ---------------------------------------------------------------- BVH build (sofren2.c:2895-3062)
 * The TLAS is rebuilt every frame on the host exactly as the reference does, so the proxy
 * occlusion traversal visits the same nodes.  A model's BLAS is built by the same steps on the
 * device at upload (sftg_blas.cu). */
static void sft__sort_items(sft__item* it, i32 count, int axis) {
    if (count <= 1) return;
    const f32 pivot = it[count / 2].c[axis];
    i32 i = 0, j = count - 1;
    while (i <= j) {
        while (it[i].c[axis] < pivot) i++;
        while (it[j].c[axis] > pivot) j--;
        if (i <= j) { const sft__item t = it[i]; it[i] = it[j]; it[j] = t; i++; j--; }
    }
    if (j > 0) sft__sort_items(it, j + 1, axis);
    if (i < count) sft__sort_items(it + i, count - i, axis);
}
static void sft__split8(sft__item* it, u32 start, u32 count, u32 depth, u32* st, u32* cn, u32* ng) {
    if (!count) return;
    if (depth == 3 || count == 1) { st[*ng] = start; cn[*ng] = count; (*ng)++; return; }
    f32 lo[3] = { 1e30f, 1e30f, 1e30f }, hi[3] = { -1e30f, -1e30f, -1e30f };
    for (u32 i = 0; i < count; i++)
        for (int a = 0; a < 3; a++) {
            if (it[start + i].c[a] < lo[a]) lo[a] = it[start + i].c[a];
            if (it[start + i].c[a] > hi[a]) hi[a] = it[start + i].c[a];
        }
    const f32 dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    const int axis = (dy > dx && dy > dz) ? 1 : (dz > dx && dz > dy) ? 2 : 0;
    sft__sort_items(it + start, (i32)count, axis);
    const u32 mid = count / 2;
    sft__split8(it, start, mid, depth + 1, st, cn, ng);
    sft__split8(it, start + mid, count - mid, depth + 1, st, cn, ng);
}
static u32 sft__bvh_build(sft__item* it, u32 count, sft__node* nodes, u32* ncount, f32* out_lo, f32* out_hi) {
    const u32 ni = (*ncount)++;
    sft__node* n = &nodes[ni];
    memset(n, 0, sizeof(*n));
    for (int i = 0; i < 8; i++) { for (int a = 0; a < 3; a++) { n->mn[a][i] = 1e30f; n->mx[a][i] = -1e30f; } n->child[i] = 0xFFFFFFFFu; }
    f32 lo[3] = { 1e30f, 1e30f, 1e30f }, hi[3] = { -1e30f, -1e30f, -1e30f };
    if (count <= 8) {
        n->leaf = 1; n->count = (u8)count;
        for (u32 i = 0; i < count; i++) {
            for (int a = 0; a < 3; a++) {
                n->mn[a][i] = it[i].mn[a]; n->mx[a][i] = it[i].mx[a];
                if (it[i].mn[a] < lo[a]) lo[a] = it[i].mn[a];
                if (it[i].mx[a] > hi[a]) hi[a] = it[i].mx[a];
            }
            n->child[i] = 0x80000000u | it[i].id;
        }
    } else {
        u32 st[8] = { 0 }, cn[8] = { 0 }, ng = 0;
        sft__split8(it, 0, count, 0, st, cn, &ng);
        n->count = (u8)ng;
        for (u32 c = 0; c < ng; c++) {
            f32 clo[3], chi[3];
            const u32 ci = sft__bvh_build(it + st[c], cn[c], nodes, ncount, clo, chi);
            n = &nodes[ni];
            n->child[c] = ci;
            for (int a = 0; a < 3; a++) {
                n->mn[a][c] = clo[a]; n->mx[a][c] = chi[a];
                if (clo[a] < lo[a]) lo[a] = clo[a];
                if (chi[a] > hi[a]) hi[a] = chi[a];
            }
        }
    }
    if (out_lo) { memcpy(out_lo, lo, 12); memcpy(out_hi, hi, 12); }
    return ni;
}

/* ---------------------------------------------------------------- lifecycle */
static void sft__check(int rc, const char* what) {
    if (rc) SFT__FATAL("%s failed (%d): %s\n", what, rc, sft__s && sft__s->gpu ? sftg_last_error(sft__s->gpu) : "no GPU context");
}

SFT_FUNC void sft_init(i32 width, i32 height, i32 requested_threads) {
    (void)requested_threads;   /* host work is a single thread; the GPU replaces the worker pool */
    sft__s = (struct sft__state*)calloc(1, sizeof(*sft__s));
    if (!sft__s) SFT__FATAL("out of memory\n");
    /* extension: SFT_CUDA_DEVICE selects the GPU (one process per GPU in multi-GPU jobs) */
    const char* dev_env = getenv("SFT_CUDA_DEVICE");
    const int rc = sftg_create(dev_env ? atoi(dev_env) : 0, &sft__s->gpu);
    if (rc) SFT__FATAL("no usable CUDA device (sftg_create returned %d)\n", rc);
    sft__s->width = width; sft__s->height = height; sft__s->samples = SFT_AA_SAMPLES;
    sft__s->lightmap_brightness = 1.5f;
    sft__s->clear_color = 0xFF222222u;
    sft__s->tex_free = -1; sft__s->mat_free = -1;
    /* 256x256 checkerboard default material, as in sft_init (sofren2.c:8060-8086) */
    u32* px = (u32*)malloc(256 * 256 * 4);
    for (i32 y = 0, i = 0; y < 256; y++) for (i32 x = 0; x < 256; x++, i++) px[i] = (((x / 32) % 2) ^ ((y / 32) % 2)) ? 0xFFAFFFAFu : 0xFF555555u;
    const sft_tex_handle checker = sft_texture_create(256, 256, px);
    free(px);
    sft__s->base_mat = sft_material_create(checker, 0xFFFFFFFFu, 2.f);
    sft__s->checker_tex = checker;
    /* dmesh index templates (sofren2.c:8089-8122): 16 quads (32 triangles) or 21 triangles of a
     * 64-vertex meshlet in the 8-lane batch layout; unused triangles stay (0, 0, 0) */
    for (u32 tri = 0; tri < 128; tri++) {
        const u32 off = (tri / 8) * 32, lane = tri % 8;
        if (tri < 32) {
            const u8 bv = (u8)((tri / 2) * 4);
            sft__s->dmesh_quad_inds[off + lane] = bv;
            sft__s->dmesh_quad_inds[off + 8 + lane] = (tri % 2 == 0) ? (u8)(bv + 1) : (u8)(bv + 2);
            sft__s->dmesh_quad_inds[off + 16 + lane] = (tri % 2 == 0) ? (u8)(bv + 2) : (u8)(bv + 3);
        }
        if (tri < 21) {
            const u8 bv = (u8)(tri * 3);
            sft__s->dmesh_tri_inds[off + lane] = bv;
            sft__s->dmesh_tri_inds[off + 8 + lane] = (u8)(bv + 1);
            sft__s->dmesh_tri_inds[off + 16 + lane] = (u8)(bv + 2);
        }
    }
    SFT__LOG("initialized GPU renderer %dx%d, %d sample(s)\n", width, height, sft__s->samples);
}

SFT_FUNC void sft_release(void) {
    if (!sft__s) return;
    for (u32 l = 1; l < SFTG_MAX_LANES; l++) if (sft__s->lane[l].n) sft_batch_wait(l);
    sftg_destroy(sft__s->gpu);
    for (i32 i = 0; i < sft__s->tex_cap; i++) free(sft__s->tex[i].level0);
    free(sft__s->tex); free(sft__s->mat_gen); free(sft__s->mat_next);
    free(sft__s->point); free(sft__s->dir); free(sft__s->bones); free(sft__s->proxies);
    for (u32 i = 0; i < sft__s->n_batch; i++) free(sft__s->batch_mem[i]);
    free(sft__s->batch_fd); free(sft__s->batch_color); free(sft__s->batch_pitch); free(sft__s->batch_mem);
    free(sft__s);
    sft__s = NULL;
}

SFT_FUNC void sft_resize(i32 width, i32 height) { if (sft__s) { sft__s->width = width; sft__s->height = height; } }
SFT_FUNC void sft_set_msaa_samples(i32 samples) { if (sft__s && (samples == 1 || samples == 2 || samples == 4)) sft__s->samples = samples; }
SFT_FUNC const char* sft_get_last_error(void) { return sft__s && sft__s->gpu ? sftg_last_error(sft__s->gpu) : ""; }
SFT_FUNC void sft_set_debug_capture(void* d) { if (sft__s) sft__s->debug = (sftg_debug_out*)d; }
SFT_FUNC void sft_get_frame_timings(f32* out5) { if (sft__s) sftg_last_timings(sft__s->gpu, out5); }
SFT_FUNC i32 sft_get_launch_count(void) { return sft__s ? sftg_last_launch_count(sft__s->gpu) : 0; }
SFT_FUNC void* sft_get_cuda_stream(void) { return sft__s ? sftg_stream(sft__s->gpu) : NULL; }

SFT_FUNC void sft_frame_begin(void) { }
/* ---------------------------------------------------------------- dynamic meshes (sofren2.c:8480-8951)
 * Geometry pushed between sft_dmesh_begin and sft_dmesh_end is packed into 64-vertex meshlets
 * with fixed index templates, exactly as the reference does in its scratch arena; at the end it
 * is uploaded as a transient model (sftg_model_upload_transient) and drawn as an instance this
 * frame.  Meshes and transient models are released at sft_frame_end. */
struct sft_dmesh {
    enum sft_dmesh_type type;
    sft_mat_handle material;
    u32 max_meshlets, curr_meshlet, curr_vert, max_verts_per_chunk;
    f32* attr;                 /* [meshlet][10][64]: x y z nx ny nz u v lu lv */
    f32* cull;                 /* [meshlet][8]: sphere centre, radius, cone axis, cutoff */
    u8* inds;                  /* [meshlet][512] */
    struct sft_dmesh* next;
};
struct sft__transient { sft_model* model; struct sft__transient* next; };

static void sft__dmesh_release_frame(void) {
    struct sft__state* s = sft__s;
    for (struct sft_dmesh* d = s->dmesh_list; d;) { struct sft_dmesh* n = d->next; free(d->attr); free(d->cull); free(d->inds); free(d); d = n; }
    s->dmesh_list = NULL;
    for (struct sft__transient* t = s->transient_list; t;) {
        struct sft__transient* n = t->next;
        free(t->model->mesh_first); free(t->model->mesh_meshlets); free(t->model); free(t);
        t = n;
    }
    if (s->transient_list) sftg_transient_reset(s->gpu);
    s->transient_list = NULL;
}

SFT_FUNC sft_dmesh* sft_dmesh_begin(enum sft_dmesh_type type, sft_mat_handle material, u32 max_prims) {
    if (0 == max_prims) return NULL;
    const u32 max_verts = (SFT_DMESH_QUADS == type) ? 64 : 63;
    const u32 total_verts = max_prims * ((SFT_DMESH_QUADS == type) ? 4 : 3);
    const u32 max_meshlets = (((total_verts + max_verts - 1) / max_verts) + 8 - 1) & ~(u32)(8 - 1);
    sft_dmesh* dm = (sft_dmesh*)calloc(1, sizeof(sft_dmesh));
    dm->type = type; dm->material = material;
    dm->max_meshlets = max_meshlets; dm->max_verts_per_chunk = max_verts;
    dm->attr = (f32*)calloc((size_t)max_meshlets * 640, 4);
    dm->cull = (f32*)calloc((size_t)max_meshlets * 8, 4);
    dm->inds = (u8*)calloc((size_t)max_meshlets * 512, 1);
    dm->next = sft__s->dmesh_list;
    sft__s->dmesh_list = dm;
    return dm;
}

/* sft__dmesh_finalize_chunk (2816-2879) */
static void sft__dmesh_finalize(sft_dmesh* dm) {
    if (0 == dm->curr_vert || dm->curr_meshlet >= dm->max_meshlets) return;
    f32* a = dm->attr + (size_t)dm->curr_meshlet * 640;
    for (u32 i = dm->curr_vert; i < 64; i++)   /* trailing vertices collapse onto vertex 0 */
        for (u32 k = 0; k < 10; k++) a[k * 64 + i] = a[k * 64];
    f32 mn[3] = { 1e30f, 1e30f, 1e30f }, mx[3] = { -1e30f, -1e30f, -1e30f };
    for (u32 i = 0; i < dm->curr_vert; i++)
        for (u32 k = 0; k < 3; k++) {
            const f32 v = a[k * 64 + i];
            if (v < mn[k]) mn[k] = v;
            if (v > mx[k]) mx[k] = v;
        }
    const f32 cx = (mn[0] + mx[0]) * 0.5f, cy = (mn[1] + mx[1]) * 0.5f, cz = (mn[2] + mx[2]) * 0.5f;
    const f32 dx = mx[0] - cx, dy = mx[1] - cy, dz = mx[2] - cz;
    f32* c = dm->cull + (size_t)dm->curr_meshlet * 8;
    c[0] = cx; c[1] = cy; c[2] = cz; c[3] = sqrtf(dx * dx + dy * dy + dz * dz);
    c[4] = 0.f; c[5] = 0.f; c[6] = 1.f; c[7] = 2.f;   /* cone test always passes */
    memcpy(dm->inds + (size_t)dm->curr_meshlet * 512, SFT_DMESH_QUADS == dm->type ? sft__s->dmesh_quad_inds : sft__s->dmesh_tri_inds, 512);
    dm->curr_meshlet++;
    dm->curr_vert = 0;
}

SFT_FUNC void sft_dmesh_push_quad_4n(sft_dmesh* dm, sftvec p0, sftvec p1, sftvec p2, sftvec p3, f32 u0, f32 v0, f32 u1, f32 v1,
                                     sftvec n0, sftvec n1, sftvec n2, sftvec n3) {
    if (dm->curr_vert >= dm->max_verts_per_chunk) sft__dmesh_finalize(dm);
    if (dm->curr_meshlet >= dm->max_meshlets) return;
    f32* a = dm->attr + (size_t)dm->curr_meshlet * 640;
    const u32 v = dm->curr_vert;
    const sftvec P[4] = { p0, p1, p2, p3 }, N[4] = { n0, n1, n2, n3 };
    const f32 U[4] = { u0, u1, u1, u0 }, V[4] = { v0, v0, v1, v1 };
    for (u32 k = 0; k < 4; k++) {
        a[v + k] = P[k].x; a[64 + v + k] = P[k].y; a[128 + v + k] = P[k].z;
        a[192 + v + k] = N[k].x; a[256 + v + k] = N[k].y; a[320 + v + k] = N[k].z;
        a[384 + v + k] = U[k]; a[448 + v + k] = V[k]; a[512 + v + k] = 0.f; a[576 + v + k] = 0.f;
    }
    dm->curr_vert += 4;
}

SFT_FUNC void sft_dmesh_push_quad(sft_dmesh* dm, sftvec p0, sftvec p1, sftvec p2, sftvec p3, f32 u0, f32 v0, f32 u1, f32 v1, sftvec normal) {
    sft_dmesh_push_quad_4n(dm, p0, p1, p2, p3, u0, v0, u1, v1, normal, normal, normal, normal);
}

SFT_FUNC void sft_dmesh_push_tri(sft_dmesh* dm, sftvec p0, sftvec p1, sftvec p2, f32 u0, f32 v0, f32 u1, f32 v1, f32 u2, f32 v2, sftvec normal) {
    if (dm->curr_vert >= dm->max_verts_per_chunk) sft__dmesh_finalize(dm);
    if (dm->curr_meshlet >= dm->max_meshlets) return;
    f32* a = dm->attr + (size_t)dm->curr_meshlet * 640;
    const u32 v = dm->curr_vert;
    const sftvec P[3] = { p0, p1, p2 };
    const f32 U[3] = { u0, u1, u2 }, V[3] = { v0, v1, v2 };
    for (u32 k = 0; k < 3; k++) {
        a[v + k] = P[k].x; a[64 + v + k] = P[k].y; a[128 + v + k] = P[k].z;
        a[192 + v + k] = normal.x; a[256 + v + k] = normal.y; a[320 + v + k] = normal.z;
        a[384 + v + k] = U[k]; a[448 + v + k] = V[k]; a[512 + v + k] = 0.f; a[576 + v + k] = 0.f;
    }
    dm->curr_vert += 3;
}

SFT_FUNC u8 sft_dmesh_alloc_quads(sft_dmesh* dm, u32 count, sft_dmesh_qb* out) {
    u32 room = (dm->max_verts_per_chunk - dm->curr_vert) / 4;
    if (0 == room) { sft__dmesh_finalize(dm); room = dm->max_verts_per_chunk / 4; }
    if (dm->curr_meshlet >= dm->max_meshlets) return 0;
    const u32 n = count < room ? count : room;
    f32* a = dm->attr + (size_t)dm->curr_meshlet * 640;
    out->x = a; out->y = a + 64; out->z = a + 128; out->nx = a + 192; out->ny = a + 256; out->nz = a + 320;
    out->u = a + 384; out->v = a + 448;
    out->vert_offset = dm->curr_vert;
    out->allocated_count = n;
    dm->curr_vert += n * 4;
    return 1;
}

SFT_FUNC void sft_dmesh_end(sft_dmesh* dm, const sftmat* opt_transform) {
    if (!dm) return;
    if (dm->curr_vert > 0) sft__dmesh_finalize(dm);
    if (0 == dm->curr_meshlet) return;
    sftg_mesh_desc md;
    memset(&md, 0, sizeof(md));
    md.meshlet_count = dm->curr_meshlet; md.attr = dm->attr; md.inds = dm->inds; md.cull = dm->cull;
    md.material = (dm->material == SFT_INVALID_HANDLE) ? -1 : (i32)SFT_MAT_INDEX(dm->material);
    md.lightmap_texture = -1;
    sftg_model_desc d;
    memset(&d, 0, sizeof(d));
    d.mesh_count = 1; d.meshes = &md;
    sft_model* m = (sft_model*)calloc(1, sizeof(sft_model));
    m->skeleton_id = -1; m->mesh_count = 1; m->total_meshlets = dm->curr_meshlet;
    m->mesh_first = (u32*)calloc(2, 4); m->mesh_meshlets = (u32*)calloc(2, 4); m->mesh_meshlets[0] = dm->curr_meshlet;
    if (sftg_model_upload_transient(sft__s->gpu, &d, &m->device_id)) {
        fprintf(stderr, "sofren2-gb300: dynamic mesh upload failed: %s\n", sftg_last_error(sft__s->gpu));
        free(m->mesh_first); free(m->mesh_meshlets); free(m);
        return;
    }
    struct sft__transient* t = (struct sft__transient*)calloc(1, sizeof(*t));
    t->model = m; t->next = sft__s->transient_list; sft__s->transient_list = t;
    sft_instance inst;
    memset(&inst, 0, sizeof(inst));
    inst.model = m;
    inst.transform = opt_transform ? *opt_transform : sft_m_identity();
    sft_draw_instance(&inst);
}


SFT_FUNC void sft_draw_cube(sft_dmesh* dm) {   /* 8480-8506 */
    sft_dmesh_push_quad(dm, SFT_V(-0.5f, -0.5f, -0.5f), SFT_V(-0.5f, 0.5f, -0.5f), SFT_V(0.5f, 0.5f, -0.5f), SFT_V(0.5f, -0.5f, -0.5f), 0.f, 0.f, 1.f, 1.f, SFT_V(0.f, 0.f, -1.f));
    sft_dmesh_push_quad(dm, SFT_V(0.5f, -0.5f, -0.5f), SFT_V(0.5f, 0.5f, -0.5f), SFT_V(0.5f, 0.5f, 0.5f), SFT_V(0.5f, -0.5f, 0.5f), 0.f, 0.f, 1.f, 1.f, SFT_V(1.f, 0.f, 0.f));
    sft_dmesh_push_quad(dm, SFT_V(0.5f, -0.5f, 0.5f), SFT_V(0.5f, 0.5f, 0.5f), SFT_V(-0.5f, 0.5f, 0.5f), SFT_V(-0.5f, -0.5f, 0.5f), 0.f, 0.f, 1.f, 1.f, SFT_V(0.f, 0.f, 1.f));
    sft_dmesh_push_quad(dm, SFT_V(-0.5f, -0.5f, 0.5f), SFT_V(-0.5f, 0.5f, 0.5f), SFT_V(-0.5f, 0.5f, -0.5f), SFT_V(-0.5f, -0.5f, -0.5f), 0.f, 0.f, 1.f, 1.f, SFT_V(-1.f, 0.f, 0.f));
    sft_dmesh_push_quad(dm, SFT_V(-0.5f, 0.5f, -0.5f), SFT_V(-0.5f, 0.5f, 0.5f), SFT_V(0.5f, 0.5f, 0.5f), SFT_V(0.5f, 0.5f, -0.5f), 0.f, 0.f, 1.f, 1.f, SFT_V(0.f, 1.f, 0.f));
    sft_dmesh_push_quad(dm, SFT_V(0.5f, -0.5f, 0.5f), SFT_V(-0.5f, -0.5f, 0.5f), SFT_V(-0.5f, -0.5f, -0.5f), SFT_V(0.5f, -0.5f, -0.5f), 0.f, 0.f, 1.f, 1.f, SFT_V(0.f, -1.f, 0.f));
}

SFT_FUNC void sft_draw_cube_inv(sft_dmesh* dm) {   /* 8508-8529 */
    sft_dmesh_push_quad(dm, SFT_V(0.5f, 0.5f, -0.5f), SFT_V(-0.5f, 0.5f, -0.5f), SFT_V(-0.5f, -0.5f, -0.5f), SFT_V(0.5f, -0.5f, -0.5f), 0.f, 0.f, 1.f, 1.f, SFT_V(0.f, 0.f, 1.f));
    sft_dmesh_push_quad(dm, SFT_V(0.5f, 0.5f, 0.5f), SFT_V(0.5f, 0.5f, -0.5f), SFT_V(0.5f, -0.5f, -0.5f), SFT_V(0.5f, -0.5f, 0.5f), 0.f, 0.f, 1.f, 1.f, SFT_V(-1.f, 0.f, 0.f));
    sft_dmesh_push_quad(dm, SFT_V(-0.5f, 0.5f, 0.5f), SFT_V(0.5f, 0.5f, 0.5f), SFT_V(0.5f, -0.5f, 0.5f), SFT_V(-0.5f, -0.5f, 0.5f), 0.f, 0.f, 1.f, 1.f, SFT_V(0.f, 0.f, -1.f));
    sft_dmesh_push_quad(dm, SFT_V(-0.5f, 0.5f, -0.5f), SFT_V(-0.5f, 0.5f, 0.5f), SFT_V(-0.5f, -0.5f, 0.5f), SFT_V(-0.5f, -0.5f, -0.5f), 0.f, 0.f, 1.f, 1.f, SFT_V(1.f, 0.f, 0.f));
    sft_dmesh_push_quad(dm, SFT_V(0.5f, 0.5f, 0.5f), SFT_V(-0.5f, 0.5f, 0.5f), SFT_V(-0.5f, 0.5f, -0.5f), SFT_V(0.5f, 0.5f, -0.5f), 0.f, 0.f, 1.f, 1.f, SFT_V(0.f, -1.f, 0.f));
    sft_dmesh_push_quad(dm, SFT_V(-0.5f, -0.5f, -0.5f), SFT_V(-0.5f, -0.5f, 0.5f), SFT_V(0.5f, -0.5f, 0.5f), SFT_V(0.5f, -0.5f, -0.5f), 0.f, 0.f, 1.f, 1.f, SFT_V(0.f, 1.f, 0.f));
}

SFT_FUNC void sft_draw_sphere(sft_dmesh* dm, i32 rings, i32 slices) {   /* 8531-8577: rings of quads, rotated incrementally */
    const f32 ring_angle = SFT_PI / (rings + 1);
    const f32 slice_angle = 2.f * SFT_PI / slices;
    const f32 cr = cosf(ring_angle), sr = sinf(ring_angle), cs = cosf(slice_angle), ss = sinf(slice_angle);
    sftvec v[4] = { { 0.f, 0.f, 0.f }, { 0.f, 0.f, 0.f }, { 0.f, 1.f, 0.f }, { sr, cr, 0.f } };
    for (i32 i = 0; i <= rings; i++) {
        for (i32 j = 0; j < slices; j++) {
            v[0] = v[2]; v[1] = v[3];
            v[2] = SFT_V(cs * v[2].x - ss * v[2].z, v[2].y, ss * v[2].x + cs * v[2].z);
            v[3] = SFT_V(cs * v[3].x - ss * v[3].z, v[3].y, ss * v[3].x + cs * v[3].z);
            sft_dmesh_push_quad_4n(dm, v[0], v[2], v[3], v[1], 0.f, 0.f, 1.f, 1.f,
                                   sft_v_norm(v[0]), sft_v_norm(v[2]), sft_v_norm(v[3]), sft_v_norm(v[1]));
        }
        v[2] = v[3];
        v[3] = SFT_V(cr * v[3].x + sr * v[3].y, -sr * v[3].x + cr * v[3].y, v[3].z);
    }
}

/* one vertex of a capsule cap ring (8600-8630) */
static sftvec sft__cap_vertex(sftvec c, sftvec b0, sftvec b1, sftvec b2, f32 r, f32 sa, f32 ra, i32 j, i32 i) {
    const f32 rs = sinf(sa * (j)) * cosf(ra * (i)), rc = cosf(sa * (j)) * cosf(ra * (i)), s0 = sinf(ra * (i));
    return SFT_V(c.x + (s0 * b0.x + rs * b1.x + rc * b2.x) * r, c.y + (s0 * b0.y + rs * b1.y + rc * b2.y) * r,
                 c.z + (s0 * b0.z + rs * b1.z + rc * b2.z) * r);
}

SFT_FUNC void sft_draw_capsule(sft_dmesh* dm, sftvec start_pos, sftvec end_pos, f32 radius, i32 slices, i32 rings) {   /* 8579-8668 */
    if (slices < 3) slices = 3;
    sftvec dir = sft_v_sub(end_pos, start_pos);
    const u8 sphere_case = (0.f == dir.x && 0.f == dir.y && 0.f == dir.z);
    if (sphere_case) dir = SFT_V(0.f, 1.f, 0.f);
    sftvec b0 = sft_v_norm(dir);
    const sftvec b1 = sft_v_norm(sft_v_perpendicular(dir));
    const sftvec b2 = sft_v_norm(sft_v_cross(b1, dir));
    sftvec cc = end_pos;
    const f32 sa = 2.f * SFT_PI / slices, ra = 0.5f * SFT_PI / rings;
    for (i32 c = 0; c < 2; c++) {
        for (i32 i = 0; i < rings; i++)
            for (i32 j = 0; j < slices; j++) {
                const sftvec w1 = sft__cap_vertex(cc, b0, b1, b2, radius, sa, ra, j + 0, i + 0);
                const sftvec w2 = sft__cap_vertex(cc, b0, b1, b2, radius, sa, ra, j + 1, i + 0);
                const sftvec w3 = sft__cap_vertex(cc, b0, b1, b2, radius, sa, ra, j + 0, i + 1);
                const sftvec w4 = sft__cap_vertex(cc, b0, b1, b2, radius, sa, ra, j + 1, i + 1);
                const sftvec fc = sft_v_mul(sft_v_add(sft_v_add(w1, w2), sft_v_add(w3, w4)), 0.25f);
                const sftvec fn = sft_v_norm(sft_v_sub(fc, cc));
                if (0 == c) sft_dmesh_push_quad(dm, w3, w1, w2, w4, 0.f, 0.f, 1.f, 1.f, fn);
                else sft_dmesh_push_quad(dm, w3, w4, w2, w1, 0.f, 0.f, 1.f, 1.f, fn);
            }
        cc = start_pos;
        b0 = sft_v_mul(b0, -1.f);
    }
    if (!sphere_case)
        for (i32 j = 0; j < slices; j++) {
            const f32 rs1 = sinf(sa * (j + 0)) * radius, rc1 = cosf(sa * (j + 0)) * radius;
            const f32 rs2 = sinf(sa * (j + 1)) * radius, rc2 = cosf(sa * (j + 1)) * radius;
            const sftvec w1 = SFT_V(start_pos.x + rs1 * b1.x + rc1 * b2.x, start_pos.y + rs1 * b1.y + rc1 * b2.y, start_pos.z + rs1 * b1.z + rc1 * b2.z);
            const sftvec w2 = SFT_V(start_pos.x + rs2 * b1.x + rc2 * b2.x, start_pos.y + rs2 * b1.y + rc2 * b2.y, start_pos.z + rs2 * b1.z + rc2 * b2.z);
            const sftvec w3 = SFT_V(end_pos.x + rs1 * b1.x + rc1 * b2.x, end_pos.y + rs1 * b1.y + rc1 * b2.y, end_pos.z + rs1 * b1.z + rc1 * b2.z);
            const sftvec w4 = SFT_V(end_pos.x + rs2 * b1.x + rc2 * b2.x, end_pos.y + rs2 * b1.y + rc2 * b2.y, end_pos.z + rs2 * b1.z + rc2 * b2.z);
            sft_dmesh_push_quad(dm, w3, w1, w2, w4, 0.f, 0.f, 1.f, 1.f, sft_v_face_normal(w3, w1, w2));
        }
}

SFT_FUNC void sft_draw_cylinder(sft_dmesh* dm, sftvec start_pos, sftvec end_pos, f32 start_radius, f32 end_radius, i32 sides) {   /* 8672-8718 */
    if (sides < 3) sides = 3;
    const sftvec dir = sft_v_sub(end_pos, start_pos);
    if (0 == dir.x && 0 == dir.y && 0 == dir.z) return;
    const sftvec b1 = sft_v_norm(sft_v_perpendicular(dir));
    const sftvec b2 = sft_v_norm(sft_v_cross(b1, dir));
    const f32 ang = (2.f * SFT_PI) / sides;
    for (i32 i = 0; i < sides; i++) {
        const f32 s1 = sinf(ang * (i + 0)) * start_radius, c1 = cosf(ang * (i + 0)) * start_radius;
        const f32 s2 = sinf(ang * (i + 1)) * start_radius, c2 = cosf(ang * (i + 1)) * start_radius;
        const f32 s3 = sinf(ang * (i + 0)) * end_radius, c3 = cosf(ang * (i + 0)) * end_radius;
        const f32 s4 = sinf(ang * (i + 1)) * end_radius, c4 = cosf(ang * (i + 1)) * end_radius;
        const sftvec w1 = SFT_V(start_pos.x + s1 * b1.x + c1 * b2.x, start_pos.y + s1 * b1.y + c1 * b2.y, start_pos.z + s1 * b1.z + c1 * b2.z);
        const sftvec w2 = SFT_V(start_pos.x + s2 * b1.x + c2 * b2.x, start_pos.y + s2 * b1.y + c2 * b2.y, start_pos.z + s2 * b1.z + c2 * b2.z);
        const sftvec w3 = SFT_V(end_pos.x + s3 * b1.x + c3 * b2.x, end_pos.y + s3 * b1.y + c3 * b2.y, end_pos.z + s3 * b1.z + c3 * b2.z);
        const sftvec w4 = SFT_V(end_pos.x + s4 * b1.x + c4 * b2.x, end_pos.y + s4 * b1.y + c4 * b2.y, end_pos.z + s4 * b1.z + c4 * b2.z);
        if (start_radius > 0) sft_dmesh_push_quad(dm, start_pos, w2, w1, w1, 0.f, 0.f, 1.f, 1.f, sft_v_face_normal(start_pos, w2, w1));
        sft_dmesh_push_quad(dm, w3, w1, w2, w4, 0.f, 0.f, 1.f, 1.f, sft_v_face_normal(w3, w1, w2));
        if (end_radius > 0) sft_dmesh_push_quad(dm, end_pos, w3, w4, w4, 0.f, 0.f, 1.f, 1.f, sft_v_face_normal(end_pos, w3, w4));
    }
}

SFT_FUNC void sft_frame_end(void) {
    sft__s->n_inst_claimed = 0; sft__s->n_inst = 0; sft__s->total_ss = 0;
    sft__s->n_point = 0; sft__s->n_dir = 0; sft__s->n_prox = 0; sft__s->n_bones = 0; sft__s->n_transient = 0;
    if (!sft__s->batching) sft__dmesh_release_frame();   /* a batch keeps them until it is submitted */
}

/* ---------------------------------------------------------------- frame setup */
SFT_FUNC void sft_set_camera(sftvec cam_pos, sftmat view, sftmat proj) {   /* sofren2.c:8345-8376 */
    sft__s->cam = cam_pos; sft__s->view = view; sft__s->proj = proj;
    sft__s->view_proj = sft_m_mul(view, proj);
    const sftmat* vp = &sft__s->view_proj;
    f32 pl[6][4];
    for (int i = 0; i < 4; i++) {
        pl[0][i] = vp->m[i][3] + vp->m[i][0]; pl[1][i] = vp->m[i][3] - vp->m[i][0];
        pl[2][i] = vp->m[i][3] + vp->m[i][1]; pl[3][i] = vp->m[i][3] - vp->m[i][1];
        pl[4][i] = vp->m[i][3] + vp->m[i][2]; pl[5][i] = vp->m[i][3] - vp->m[i][2];
    }
    for (int p = 0; p < 6; p++) {
        const f32 len = sqrtf(pl[p][0] * pl[p][0] + pl[p][1] * pl[p][1] + pl[p][2] * pl[p][2]);
        const f32 il = (len < SFT_EPSILON) ? SFT_EPSILON : 1.f / len;
        for (int a = 0; a < 3; a++) sft__s->fn[p][a] = pl[p][a] * il;
        sft__s->fd[p] = pl[p][3] * il;
    }
}
SFT_FUNC void sft_set_debug_mode(enum sft_debug_mode mode) {
    if ((int)mode < 0 || mode >= SFT_DEBUG_COUNT) { fprintf(stderr, "sofren2-gb300: invalid debug mode %d\n", (int)mode); return; }
    sft__s->debug_mode = mode;
}
SFT_FUNC const char* sft_get_debug_name(enum sft_debug_mode mode) {
    switch (mode) {
        case SFT_DEBUG_NONE: return "None";
        case SFT_DEBUG_WIREFRAME: return "Wireframe";
        case SFT_DEBUG_TILES: return "Tiles";
        case SFT_DEBUG_DEPTH: return "Depth";
        case SFT_DEBUG_LIGHT_COUNT: return "Light Count";
        case SFT_DEBUG_CHECKERBOARD: return "Checkerboard";
        default: return "INVALID MODE";
    }
}
SFT_FUNC void sft_set_clear(u8 enabled) { sft__s->clear = enabled; }
SFT_FUNC void sft_set_clear_color(u32 color) { sft__s->clear_color = color; }
SFT_FUNC void sft_set_color_buffer(u32* buf, i32 pitch_in_bytes) { sft__s->color = buf; sft__s->pitch = pitch_in_bytes; }

/* ---------------------------------------------------------------- lights (sofren2.c:9109-9149) */
SFT_FUNC void sft_set_ambient_light(f32 r, f32 g, f32 b) { sft__s->ambient.x = r; sft__s->ambient.y = g; sft__s->ambient.z = b; }
SFT_FUNC void sft_draw_directional_light(sftvec dir, f32 r, f32 g, f32 b, f32 intensity) {
    if (sft__s->n_dir == sft__s->cap_dir) { sft__s->cap_dir = sft__s->cap_dir ? sft__s->cap_dir * 2 : 16; sft__s->dir = (f32*)realloc(sft__s->dir, sft__s->cap_dir * 24); }
    f32* d = sft__s->dir + 6 * sft__s->n_dir++;
    const sftvec n = sft_v_norm(dir);
    d[0] = n.x; d[1] = n.y; d[2] = n.z; d[3] = r * intensity; d[4] = g * intensity; d[5] = b * intensity;
}
SFT_FUNC void sft_draw_point_light(sftvec pos, f32 r, f32 g, f32 b, f32 intensity, f32 radius, u32 light_id) {
    (void)light_id;
    if (sft__s->n_point == sft__s->cap_point) { sft__s->cap_point = sft__s->cap_point ? sft__s->cap_point * 2 : 16; sft__s->point = (f32*)realloc(sft__s->point, sft__s->cap_point * 32); }
    f32* p = sft__s->point + 8 * sft__s->n_point++;
    p[0] = pos.x; p[1] = pos.y; p[2] = pos.z; p[3] = r * intensity; p[4] = g * intensity; p[5] = b * intensity;
    p[6] = radius; p[7] = 1.f / (radius * radius);
}
SFT_FUNC void sft_set_shadows_enabled(u8 enabled) { sft__s->shadows = enabled; }
SFT_FUNC void sft_set_lightmap_brightness(f32 b) { sft__s->lightmap_brightness = b; }

/* ---------------------------------------------------------------- textures (sofren2.c:9181-9391) */
static i32 sft__ilog2(u32 v) { i32 r = 0; while (v >>= 1) r++; return r; }

SFT_FUNC sft_tex_handle sft_texture_create(i32 width, i32 height, const u32* pixels) {
    if (width <= 0 || height <= 0 || !pixels) return SFT_INVALID_HANDLE;
    const u8 is_pot = (0 == (width & (width - 1))) && (0 == (height & (height - 1)));
    i32 cw = width, ch = height, levels = 0; u64 total = 0;
    while (levels < 14) {
        total += (u64)(((cw + 3) & ~3) * ((ch + 3) & ~3));
        levels++;
        if (cw == 1 && ch == 1) break;
        cw = cw > 1 ? cw / 2 : 1; ch = ch > 1 ? ch / 2 : 1;
    }
    u32* texels = (u32*)calloc(total + 16, 4);
    sftg_texture_desc d; memset(&d, 0, sizeof(d));
    d.width = width; d.height = height; d.levels = levels; d.is_pot = is_pot;
    const u32* src = pixels; u32* tmp = NULL; u32 cur = 0;
    cw = width; ch = height;
    for (i32 l = 0; l < levels; l++) {
        if (l > 0) {   /* 4x4 tent filter with 1-2-2-1 integer weights and clamped taps (9261-9290) */
            const i32 nw = cw > 1 ? cw / 2 : 1, nh = ch > 1 ? ch / 2 : 1;
            u32* dst = (u32*)malloc((size_t)nw * nh * 4);
            for (i32 y = 0; y < nh; y++)
                for (i32 x = 0; x < nw; x++) {
                    u32 r = 0, g = 0, b = 0, a = 0, ws = 0;
                    for (i32 ky = -1; ky <= 2; ky++) {
                        const i32 sy = (y * 2 + ky) < 0 ? 0 : ((y * 2 + ky) > ch - 1 ? ch - 1 : (y * 2 + ky));
                        const u32 wy = (ky == -1 || ky == 2) ? 1 : 2;
                        for (i32 kx = -1; kx <= 2; kx++) {
                            const i32 sx = (x * 2 + kx) < 0 ? 0 : ((x * 2 + kx) > cw - 1 ? cw - 1 : (x * 2 + kx));
                            const u32 w = ((kx == -1 || kx == 2) ? 1 : 2) * wy;
                            const u32 c = src[sy * cw + sx];
                            r += ((c >> 16) & 255) * w; g += ((c >> 8) & 255) * w; b += (c & 255) * w; a += ((c >> 24) & 255) * w;
                            ws += w;
                        }
                    }
                    dst[y * nw + x] = ((a / ws) << 24) | ((r / ws) << 16) | ((g / ws) << 8) | (b / ws);
                }
            free(tmp); tmp = dst; src = dst; cw = nw; ch = nh;
        }
        const i32 pw = (cw + 3) & ~3, ph = (ch + 3) & ~3, bw = pw / 4;
        d.level_offset[l] = cur; d.blocks_w[l] = bw; d.stride_shift[l] = is_pot ? sft__ilog2((u32)bw) : 0;
        for (i32 y = 0; y < ch; y++)
            for (i32 x = 0; x < cw; x++)
                texels[cur + (u32)(((y / 4) * bw + x / 4) * 16 + (y % 4) * 4 + (x % 4))] = src[y * cw + x];
        cur += (u32)(pw * ph);
    }
    free(tmp);
    i32 dev = -1;
    sft__check(sftg_texture_upload(sft__s->gpu, texels, total, &d, &dev), "texture upload");
    free(texels);
    /* slot in the generational pool (sofren2.c:4457-4480) */
    if (sft__s->tex_free == -1) {
        const i32 oc = sft__s->tex_cap, nc = oc ? oc * 2 : 1024;
        sft__s->tex = (sft__tex*)realloc(sft__s->tex, (size_t)nc * sizeof(sft__tex));
        for (i32 i = oc; i < nc; i++) { memset(&sft__s->tex[i], 0, sizeof(sft__tex)); sft__s->tex[i].generation = 1; sft__s->tex[i].next_free = i + 1; }
        sft__s->tex[nc - 1].next_free = -1;
        sft__s->tex_free = oc; sft__s->tex_cap = nc;
    }
    const i32 ti = sft__s->tex_free;
    sft__tex* t = &sft__s->tex[ti];
    sft__s->tex_free = t->next_free;
    t->device_index = dev; t->w = width; t->h = height; t->levels = levels; t->is_pot = is_pot; t->live = 1;
    t->level0 = (u32*)malloc((size_t)width * height * 4);
    memcpy(t->level0, pixels, (size_t)width * height * 4);
    return (t->generation << SFT_HANDLE_GEN_SHIFT) | (u32)ti;
}
SFT_FUNC sft_tex_handle sft_texture_create_solid(u32 color) { return sft_texture_create(1, 1, &color); }
SFT_FUNC i32 sft_texture_get_width(sft_tex_handle tex) { return tex == SFT_INVALID_HANDLE ? 0 : sft__s->tex[SFT_HANDLE_INDEX(tex)].w; }
SFT_FUNC i32 sft_texture_get_height(sft_tex_handle tex) { return tex == SFT_INVALID_HANDLE ? 0 : sft__s->tex[SFT_HANDLE_INDEX(tex)].h; }
SFT_FUNC u32* sft_texture_get_linear_pixels(sft_tex_handle tex) {
    if (tex == SFT_INVALID_HANDLE) return NULL;
    const sft__tex* t = &sft__s->tex[SFT_HANDLE_INDEX(tex)];
    u32* r = (u32*)malloc((size_t)t->w * t->h * 4);
    memcpy(r, t->level0, (size_t)t->w * t->h * 4);
    return r;
}
SFT_FUNC void sft_texture_release(sft_tex_handle tex) {
    if (tex == SFT_INVALID_HANDLE) return;
    const u32 ind = SFT_HANDLE_INDEX(tex), gen = tex >> SFT_HANDLE_GEN_SHIFT;
    if (ind >= (u32)sft__s->tex_cap || sft__s->tex[ind].generation != gen) return;
    sft__tex* t = &sft__s->tex[ind];
    free(t->level0); t->level0 = NULL; t->live = 0;
    t->generation++;
    t->next_free = sft__s->tex_free; sft__s->tex_free = (i32)ind;
}

/* ---------------------------------------------------------------- materials (sofren2.c:9393-9454) */
static i32 sft__tex_device(sft_tex_handle h) {
    if (h == SFT_INVALID_HANDLE) return -1;
    const u32 i = SFT_HANDLE_INDEX(h);
    return (i < (u32)sft__s->tex_cap && sft__s->tex[i].live) ? sft__s->tex[i].device_index : -1;
}
SFT_FUNC sft_mat_handle sft_material_create(sft_tex_handle tex, u32 base_color, f32 shininess) {
    if (sft__s->mat_free == -1) {
        const i32 oc = sft__s->mat_cap, nc = oc ? oc * 2 : 32;
        sft__s->mat_gen = (u32*)realloc(sft__s->mat_gen, (size_t)nc * 4);
        sft__s->mat_next = (i32*)realloc(sft__s->mat_next, (size_t)nc * 4);
        for (i32 i = oc; i < nc; i++) { sft__s->mat_gen[i] = 1; sft__s->mat_next[i] = i + 1; }
        sft__s->mat_next[nc - 1] = -1;
        sft__s->mat_free = oc; sft__s->mat_cap = nc;
    }
    const i32 ind = sft__s->mat_free;
    sft__s->mat_free = sft__s->mat_next[ind];
    sft__check(sftg_material_set(sft__s->gpu, ind, sft__tex_device(tex), base_color, shininess), "material upload");
    return (sft__s->mat_gen[ind] << SFT_MAT_GEN_SHIFT) | (u32)ind;
}
SFT_FUNC sft_mat_handle sft_material_clone(sft_mat_handle base_mat) {
    /* transient per-frame materials are not yet resident on the device: clone into a static slot */
    (void)base_mat;
    fprintf(stderr, "sofren2-gb300: sft_material_clone is not supported by the GPU runtime\n");
    return SFT_INVALID_HANDLE;
}
SFT_FUNC void sft_material_release(sft_mat_handle mat) {
    if (mat == SFT_INVALID_HANDLE || SFT_MAT_IS_TRANSIENT(mat)) return;
    const u32 ind = SFT_MAT_INDEX(mat), gen = (mat & SFT_MAT_GEN_MASK) >> SFT_MAT_GEN_SHIFT;
    if (ind >= (u32)sft__s->mat_cap || sft__s->mat_gen[ind] != gen) return;
    sft__s->mat_gen[ind]++;
    sft__s->mat_next[ind] = sft__s->mat_free; sft__s->mat_free = (i32)ind;
}

/* ---------------------------------------------------------------- models */
static sft_model* sft__model_create(const sft_mesh_data* meshes, u32 mesh_count, const sft_shadow_proxy* proxies, u32 proxy_count,
                                    u32 bone_count, const sft_tex_handle* lightmaps, u32 lightmap_count, const void* blas_nodes,
                                    u32 blas_count, u32 blas_root);

SFT_FUNC sft_model* sft_model_create(const sft_mesh_data* meshes, u32 mesh_count, const sft_shadow_proxy* proxies,
                                     u32 proxy_count, u32 bone_count, const sft_tex_handle* lightmaps, u32 lightmap_count,
                                     sft_arena* arena) {
    (void)arena;
    return sft__model_create(meshes, mesh_count, proxies, proxy_count, bone_count, lightmaps, lightmap_count, NULL, 0, 0);
}

/* a model from meshlet arrays; the BLAS is built (blas_nodes NULL) or taken as given */
static sft_model* sft__model_create(const sft_mesh_data* meshes, u32 mesh_count, const sft_shadow_proxy* proxies, u32 proxy_count,
                                    u32 bone_count, const sft_tex_handle* lightmaps, u32 lightmap_count, const void* blas_nodes,
                                    u32 blas_count, u32 blas_root) {
    sft_model* m = (sft_model*)calloc(1, sizeof(sft_model));
    m->mesh_count = mesh_count; m->bone_count = bone_count; m->skeleton_id = -1;
    m->mesh_first = (u32*)calloc(mesh_count + 1, 4); m->mesh_meshlets = (u32*)calloc(mesh_count + 1, 4);
    sftg_mesh_desc* md = (sftg_mesh_desc*)calloc(mesh_count + 1, sizeof(sftg_mesh_desc));
    u32 total = 0;
    for (u32 k = 0; k < mesh_count; k++) {
        const sft_mesh_data* s = &meshes[k];
        m->mesh_first[k] = total; m->mesh_meshlets[k] = s->meshlet_count;
        md[k].meshlet_count = s->meshlet_count; md[k].attr = s->attr; md[k].inds = s->inds; md[k].cull = s->cull;
        md[k].joints = s->joints; md[k].weights = s->weights; md[k].culling_bones = s->culling_bones;
        md[k].material = (s->material == SFT_INVALID_HANDLE) ? -1 : (i32)SFT_MAT_INDEX(s->material);
        md[k].lightmap_texture = (s->lightmap_page != 0xFFFFFFFFu && s->lightmap_page < lightmap_count) ? sft__tex_device(lightmaps[s->lightmap_page]) : -1;
        total += s->meshlet_count;
    }
    m->total_meshlets = total;
    m->proxy_count = proxy_count;
    m->proxies = (sft_shadow_proxy*)calloc(proxy_count + 1, sizeof(sft_shadow_proxy));
    if (proxy_count) memcpy(m->proxies, proxies, proxy_count * sizeof(sft_shadow_proxy));
    /* BLAS over every non-padding triangle, in meshlet / batch / lane order (sofren2.c:3526-3617):
     * taken from the caller (a QSF2 file carries its BLAS) or built on the device at upload */
    if (blas_nodes && blas_count) {
        m->blas = (sft__node*)calloc(blas_count + 1, sizeof(sft__node));
        memcpy(m->blas, blas_nodes, (size_t)blas_count * sizeof(sft__node));
        m->blas_count = blas_count; m->blas_root = blas_root;
    }
    sftg_model_desc d; memset(&d, 0, sizeof(d));
    d.mesh_count = mesh_count; d.meshes = md; d.bone_count = bone_count;
    d.blas_nodes = m->blas; d.blas_count = m->blas_count; d.blas_root = m->blas_root;
    d.build_blas = m->blas ? 0u : 1u;
    sft__check(sftg_model_upload(sft__s->gpu, &d, &m->device_id), "model upload");
    free(md);
    sft__node root;
    memset(&root, 0, sizeof(root));
    if (!m->blas) {   /* node images stay on the device; sft_model_get_blas reads them back */
        sft__check(sftg_model_blas(sft__s->gpu, m->device_id, 0, 0, NULL, &m->blas_count, &m->blas_root), "BLAS query");
        if (m->blas_count) sft__check(sftg_model_blas(sft__s->gpu, m->device_id, m->blas_root, 1, &root, NULL, NULL), "BLAS root read");
    } else if (m->blas_count) {
        root = m->blas[m->blas_root];
    }
    if (m->blas_count) {   /* the model's box from the BLAS root slots, for the TLAS */
        for (int a = 0; a < 3; a++) { m->root_min[a] = 1e30f; m->root_max[a] = -1e30f; }
        for (u32 c = 0; c < root.count; c++)
            for (int a = 0; a < 3; a++) {
                if (root.mn[a][c] < m->root_min[a]) m->root_min[a] = root.mn[a][c];
                if (root.mx[a][c] > m->root_max[a]) m->root_max[a] = root.mx[a][c];
            }
    }
    return m;
}
/* sft_model_load_qsf (sofren2.c:7816-7967): a QSF2 file's textures (each becomes a white
 * material of shininess 2), lightmap pages, meshes (meshlet positions and attributes, flat
 * triangle indices swizzled into the 8-lane batch layout, bounding spheres and cones) and its
 * prebuilt BLAS, uploaded as one resident model.  NULL (with a message) when the file cannot be
 * read.  The arena is not used: model data lives in the device pools. */
SFT_FUNC sft_model* sft_model_load_qsf(const char* path, sft_arena* arena) {
    (void)arena;
    FILE* f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "sofren2-gb300: failed to open '%s'\n", path); return NULL; }
#define SFT__RD(p, n) (fread((p), 1, (n), f) == (size_t)(n))
    char magic[4]; u32 version = 0; u64 game_off = 0;
    if (!SFT__RD(magic, 4) || memcmp(magic, "QSF2", 4) || !SFT__RD(&version, 4) || version != 2 || !SFT__RD(&game_off, 8)) {
        fclose(f); fprintf(stderr, "sofren2-gb300: '%s' is not a QSF2 version 2 file\n", path); return NULL;
    }
    u32 tex_count = 0;
    int ok = SFT__RD(&tex_count, 4);
    sft_mat_handle* mats = (sft_mat_handle*)calloc(tex_count + 1, sizeof(sft_mat_handle));
    for (u32 i = 0; ok && i < tex_count; i++) {
        u32 wh[2];
        ok = SFT__RD(wh, 8) && wh[0] && wh[1] && (u64)wh[0] * wh[1] < (1ull << 28);
        if (!ok) break;
        u32* px = (u32*)malloc((size_t)wh[0] * wh[1] * 4);
        ok = SFT__RD(px, (size_t)wh[0] * wh[1] * 4);
        if (ok) mats[i] = sft_material_create(sft_texture_create((i32)wh[0], (i32)wh[1], px), 0xFFFFFFFFu, 2.f);
        free(px);
    }
    u32 lm_count = 0;
    ok = ok && SFT__RD(&lm_count, 4);
    sft_tex_handle* lms = (sft_tex_handle*)calloc(lm_count + 1, sizeof(sft_tex_handle));
    for (u32 i = 0; ok && i < lm_count; i++) {
        u32 wh[2];
        ok = SFT__RD(wh, 8) && wh[0] && wh[1] && (u64)wh[0] * wh[1] < (1ull << 28);
        if (!ok) break;
        u32* px = (u32*)malloc((size_t)wh[0] * wh[1] * 4);
        ok = SFT__RD(px, (size_t)wh[0] * wh[1] * 4);
        if (ok) lms[i] = sft_texture_create((i32)wh[0], (i32)wh[1], px);
        free(px);
    }
    u32 hdr[4] = { 0, 0, 0, 0 };   /* mesh count, total meshlets, BLAS nodes, BLAS root */
    ok = ok && SFT__RD(hdr, 16) && hdr[0] < (1u << 16) && hdr[1] < (1u << 24);
    sft_mesh_data* md = (sft_mesh_data*)calloc(hdr[0] + 1, sizeof(sft_mesh_data));
    for (u32 k = 0; ok && k < hdr[0]; k++) {
        u32 mh[4];   /* meshlet count, model meshlet offset, texture index, lightmap page */
        ok = SFT__RD(mh, 16) && mh[0] < (1u << 24);
        if (!ok) break;
        const u32 mc = mh[0];
        f32* attr = (f32*)calloc((size_t)mc * 640 + 1, 4);
        u8* inds = (u8*)calloc((size_t)mc * 512 + 1, 1);
        f32* cull = (f32*)calloc((size_t)mc * 8 + 1, 4);
        f32* tmp = (f32*)malloc(((size_t)mc * 448 + 1) * 4);
        u8* flat = (u8*)malloc((size_t)mc * 384 + 1);
        ok = SFT__RD(tmp, (size_t)mc * 768);
        for (u32 j = 0; ok && j < mc; j++) memcpy(attr + (size_t)j * 640, tmp + (size_t)j * 192, 768);   /* x y z */
        ok = ok && SFT__RD(tmp, (size_t)mc * 1792);
        for (u32 j = 0; ok && j < mc; j++) memcpy(attr + (size_t)j * 640 + 192, tmp + (size_t)j * 448, 1792);   /* nx..lv */
        ok = ok && SFT__RD(flat, (size_t)mc * 384);
        for (u32 j = 0; ok && j < mc; j++)
            for (u32 tri = 0; tri < 128; tri++) {
                const u32 off = (tri / 8) * 32, lane = tri % 8;
                for (u32 c = 0; c < 3; c++) inds[(size_t)j * 512 + off + c * 8 + lane] = flat[(size_t)j * 384 + tri * 3 + c];
            }
        /* sphere centre x y z, radius; box min / max (unused); cone axis x y z, cutoff */
        for (u32 a = 0; ok && a < 14; a++) {
            ok = SFT__RD(tmp, (size_t)mc * 4);
            const int dst = a < 4 ? (int)a : (a >= 10 ? (int)a - 6 : -1);
            if (ok && dst >= 0) for (u32 j = 0; j < mc; j++) cull[(size_t)j * 8 + dst] = tmp[j];
        }
        free(tmp); free(flat);
        md[k].meshlet_count = mc; md[k].attr = attr; md[k].inds = inds; md[k].cull = cull;
        md[k].material = mh[2] < tex_count ? mats[mh[2]] : sft__s->base_mat;
        md[k].lightmap_page = mh[3];
    }
    u16* mesh_of = (u16*)malloc(((size_t)hdr[1] + 1) * 2);
    ok = ok && SFT__RD(mesh_of, (size_t)hdr[1] * 2);
    void* blas = malloc((size_t)hdr[2] * 256 + 1);
    ok = ok && SFT__RD(blas, (size_t)hdr[2] * 256);
    fclose(f);
#undef SFT__RD
    /* the BLAS must stay inside the model: inner children are nodes, leaf payloads are
     * (meshlet << 7 | triangle) of this model's meshlets */
    if (ok && hdr[2]) {
        u32 sum = 0;
        for (u32 k = 0; k < hdr[0]; k++) sum += md[k].meshlet_count;
        ok = sum == hdr[1] && hdr[3] < hdr[2];
        const sft__node* nodes = (const sft__node*)blas;
        for (u32 i = 0; ok && i < hdr[2]; i++) {
            ok = nodes[i].count <= 8;
            for (u32 c = 0; ok && c < nodes[i].count; c++) {
                const u32 ch = nodes[i].child[c];
                if (ch == 0xFFFFFFFFu) continue;
                ok = nodes[i].leaf ? ((ch & 0x7FFFFFFFu) >> 7) < hdr[1] : ch < hdr[2];
            }
        }
    }
    sft_model* m = NULL;
    if (ok) m = sft__model_create(md, hdr[0], NULL, 0, 0, lms, lm_count, hdr[2] ? blas : NULL, hdr[2], hdr[3]);
    else fprintf(stderr, "sofren2-gb300: '%s' is truncated or malformed\n", path);
    for (u32 k = 0; k < hdr[0]; k++) { free((void*)md[k].attr); free((void*)md[k].inds); free((void*)md[k].cull); }
    free(md); free(mesh_of); free(blas); free(mats); free(lms);
    return m;
}

SFT_FUNC u32 sft_model_get_meshlet_count(const sft_model* model) { return model ? model->total_meshlets : 0; }
SFT_FUNC const void* sft_model_get_blas(const sft_model* model, u32* out_count, u32* out_root) {
    if (out_count) *out_count = model ? model->blas_count : 0;
    if (out_root) *out_root = model ? model->blas_root : 0;
    if (model && !model->blas && model->blas_count) {   /* built on the device: read once, keep */
        sft_model* mm = (sft_model*)model;
        mm->blas = (sft__node*)calloc((size_t)model->blas_count + 1, sizeof(sft__node));
        if (sftg_model_blas(sft__s->gpu, model->device_id, 0, model->blas_count, mm->blas, NULL, NULL)) { free(mm->blas); mm->blas = NULL; }
    }
    return model ? model->blas : NULL;
}

/* ---------------------------------------------------------------- load-time builders
 * The meshlet builder and the shadow-proxy fitter of the reference's GLB loader, restated on
 * the host; every float expression keeps the reference's operation order, so a model built from
 * the same triangles (and the same rand() state) gets the reference's meshlets and proxies bit
 * for bit. */
#define SFT__CONE_LIMIT (-0.173648f)   /* a candidate's normal may turn at most 100 degrees from the cone axis (sofren2.c:152) */

typedef struct { sftvec c; f32 r; } sft__sphere;

/* spheres through 2, 3 and 4 points (sofren2.c:2180-2243) */
static sft__sphere sft__sphere2(sftvec a, sftvec b) {
    sft__sphere s;
    s.c = sft_v_mul(sft_v_add(a, b), 0.5f);
    s.r = sft_v_length(sft_v_sub(a, b)) * 0.5f;
    return s;
}
static sft__sphere sft__sphere3(sftvec p0, sftvec p1, sftvec p2) {
    const sftvec a = sft_v_sub(p1, p0), b = sft_v_sub(p2, p0), axb = sft_v_cross(a, b);
    const f32 den = 2.f * sft_v_length2(axb);
    if (den < SFT_EPSILON) return sft__sphere2(p0, p1);        /* degenerate: the first two points */
    const sftvec num = sft_v_cross(sft_v_sub(sft_v_mul(b, sft_v_length2(a)), sft_v_mul(a, sft_v_length2(b))), axb);
    sft__sphere s;
    s.c = sft_v_add(p0, sft_v_div(num, den));
    s.r = sft_v_length(sft_v_sub(s.c, p0));
    return s;
}
static sft__sphere sft__sphere4(sftvec p0, sftvec p1, sftvec p2, sftvec p3) {
    const sftvec r1 = sft_v_sub(p1, p0), r2 = sft_v_sub(p2, p0), r3 = sft_v_sub(p3, p0);
    const f32 q1 = sft_v_length2(r1), q2 = sft_v_length2(r2), q3 = sft_v_length2(r3);
    /* 2x2 minors of the rows r1, r2, r3 */
    const f32 m23yz = r2.y * r3.z - r3.y * r2.z, m23xz = r2.x * r3.z - r3.x * r2.z, m23xy = r2.x * r3.y - r3.x * r2.y;
    const f32 m13yz = r1.y * r3.z - r3.y * r1.z, m13xz = r1.x * r3.z - r3.x * r1.z, m13xy = r1.x * r3.y - r3.x * r1.y;
    const f32 m12yz = r1.y * r2.z - r2.y * r1.z, m12xz = r1.x * r2.z - r2.x * r1.z, m12xy = r1.x * r2.y - r2.x * r1.y;
    const f32 det = r1.x * m23yz - r1.y * m23xz + r1.z * m23xy;
    if (fabsf(det) < SFT_EPSILON) return sft__sphere3(p0, p1, p2);   /* coplanar: the first three points */
    const f32 f = 0.5f / det;
    sftvec o;
    o.x = f * (m23yz * q1 - m13yz * q2 + m12yz * q3);
    o.y = f * (-m23xz * q1 + m13xz * q2 - m12xz * q3);
    o.z = f * (m23xy * q1 - m13xy * q2 + m12xy * q3);
    sft__sphere s;
    s.c = sft_v_add(p0, o);
    s.r = sft_v_length(o);
    return s;
}
static sft__sphere sft__sphere_support(const sftvec* sup, i32 n) {
    sft__sphere s;
    memset(&s, 0, sizeof(s));
    if (n == 1) s.c = sup[0];
    else if (n == 2) s = sft__sphere2(sup[0], sup[1]);
    else if (n == 3) s = sft__sphere3(sup[0], sup[1], sup[2]);
    else if (n == 4) s = sft__sphere4(sup[0], sup[1], sup[2], sup[3]);
    return s;
}
/* Welzl's minimal enclosing sphere (sofren2.c:2255-2278): a point drawn with rand() leaves the
 * set, the sphere of the rest is found, and the point joins the support set if it lies outside
 * (squared distance above r^2 + SFT_EPSILON).  pts is reordered. */
static sft__sphere sft__welzl(sftvec* pts, i32 n, sftvec* sup, i32 ns) {
    if (n == 0 || ns == 4) return sft__sphere_support(sup, ns);
    const i32 k = rand() % n;
    const sftvec p = pts[k];
    pts[k] = pts[n - 1];
    pts[n - 1] = p;
    const sft__sphere s = sft__welzl(pts, n - 1, sup, ns);
    if (sft_v_length2(sft_v_sub(p, s.c)) <= s.r * s.r + SFT_EPSILON) return s;
    sup[ns] = p;
    return sft__welzl(pts, n - 1, sup, ns + 1);
}

/* one meshlet under construction (sofren2.c:1235-1246) */
typedef struct {
    i32 gv[SFT_VERTS_PER_MESHLET];   /* local vertex -> mesh vertex */
    u32 nv;
    u8 tri[128 * 3];                  /* local indices */
    u32 nt;
    sftvec axis;                      /* running normal cone axis, renormalised after every triangle */
} sft__mlet;

/* how well a triangle fits the meshlet (sofren2.c:2325-2362): -1 when it does not (full, normal
 * beyond the cone limit, more than 64 vertices), else vertices shared + half the cone alignment */
static f32 sft__mlet_score(const sft__mlet* b, i32 v0, i32 v1, i32 v2, sftvec n) {
    if (b->nt >= 128) return -1.f;
    if (b->nt > 0 && sft_v_dot(b->axis, n) < SFT__CONE_LIMIT) return -1.f;
    u32 fresh = 3, shared = 0;
    for (u32 i = 0; i < b->nv; i++)
        if (b->gv[i] == v0 || b->gv[i] == v1 || b->gv[i] == v2) { fresh--; shared++; }
    if (b->nv + fresh > SFT_VERTS_PER_MESHLET) return -1.f;
    f32 score = (f32)shared;
    if (b->nt > 0) score += sft_v_dot(b->axis, n) * 0.5f;
    return score;
}
/* sofren2.c:2364-2402 */
static void sft__mlet_add(sft__mlet* b, i32 v0, i32 v1, i32 v2, sftvec n) {
    const i32 g[3] = { v0, v1, v2 };
    for (int k = 0; k < 3; k++) {
        i32 l = -1;
        for (u32 i = 0; i < b->nv; i++) if (b->gv[i] == g[k]) { l = (i32)i; break; }
        if (l < 0) { l = (i32)b->nv; b->gv[b->nv++] = g[k]; }
        b->tri[b->nt * 3 + k] = (u8)l;
    }
    b->axis = sft_v_norm(sft_v_add(b->axis, n));
    b->nt++;
}
static sftvec sft__raw_pos(const sft_raw_mesh* m, i32 v) { sftvec p = { m->pos[v * 3], m->pos[v * 3 + 1], m->pos[v * 3 + 2] }; return p; }
static sftvec sft__raw_tri_normal(const sft_raw_mesh* m, i32 t) {
    const i32* ix = m->indices + (size_t)t * 3;
    return sft_v_face_normal(sft__raw_pos(m, ix[0]), sft__raw_pos(m, ix[1]), sft__raw_pos(m, ix[2]));
}

/* writes meshlet `mi` of the output arrays (sofren2.c:6918-7045 and the cone of 7631-7651) */
static void sft__mlet_emit(const sft__mlet* b, const sft_raw_mesh* m, u32 bone_count, i32* scratch, u32 mi, f32* attr, u8* inds,
                           f32* cull, u16* joints, u8* weights, i32* culling_bones) {
    u8* I = inds + (size_t)mi * 512;
    for (u32 t = 0; t < 128; t++) {   /* batches of 8 triangles: v0 x8, v1 x8, v2 x8, 8 zero bytes */
        const u32 bt = t >> 3, l = t & 7;
        const int live = t < b->nt;
        for (int k = 0; k < 3; k++) I[bt * 32 + k * 8 + l] = live ? b->tri[t * 3 + k] : 0;
        I[bt * 32 + 24 + l] = 0;
    }
    f32* A = attr + (size_t)mi * 640;
    const int skinned = m->joints && m->weights;
    if (skinned && scratch) memset(scratch, 0, (size_t)bone_count * sizeof(i32));
    i32 best = 0, best_w = 0;
    sftvec pts[SFT_VERTS_PER_MESHLET];
    for (u32 i = 0; i < SFT_VERTS_PER_MESHLET; i++) {
        const int live = i < b->nv;
        const i32 g = live ? b->gv[i] : 0;
        A[0 * 64 + i] = live ? m->pos[g * 3 + 0] : 0.f;
        A[1 * 64 + i] = live ? m->pos[g * 3 + 1] : 0.f;
        A[2 * 64 + i] = live ? m->pos[g * 3 + 2] : 0.f;
        A[3 * 64 + i] = live ? m->nrm[g * 3 + 0] : 0.f;
        A[4 * 64 + i] = live ? m->nrm[g * 3 + 1] : 0.f;
        A[5 * 64 + i] = live ? m->nrm[g * 3 + 2] : 0.f;
        A[6 * 64 + i] = live ? m->uv[g * 2 + 0] : 0.f;
        A[7 * 64 + i] = live ? m->uv[g * 2 + 1] : 0.f;
        A[8 * 64 + i] = 0.f;   /* no lightmap coordinates from this path */
        A[9 * 64 + i] = 0.f;
        if (skinned) {
            for (int k = 0; k < 4; k++) {
                const u16 j = live ? m->joints[g * 4 + k] : 0;
                const u8 w = live ? m->weights[g * 4 + k] : 0;
                if (joints) joints[(size_t)mi * 256 + k * 64 + i] = j;
                if (weights) weights[(size_t)mi * 256 + k * 64 + i] = w;
                /* the joint carrying the most weight over the meshlet's vertices, first to lead wins */
                if (live && j < bone_count && scratch) {
                    scratch[j] += w;
                    if (scratch[j] > best_w) { best_w = scratch[j]; best = j; }
                }
            }
        }
        if (live) pts[i] = sft__raw_pos(m, g);
    }
    if (culling_bones) culling_bones[mi] = skinned ? best : -1;
    sft__sphere sph;
    memset(&sph, 0, sizeof(sph));
    if (b->nv > 0) { sftvec sup[4]; sph = sft__welzl(pts, (i32)b->nv, sup, 0); }
    /* normal cone: the widest angle between the axis and a triangle's normal, plus a margin */
    const sftvec axis = sft_v_norm(b->axis);
    f32 min_dot = 1.f;
    for (u32 t = 0; t < b->nt; t++) {
        sftvec p[3];
        for (int k = 0; k < 3; k++) { const u32 v = b->tri[t * 3 + k]; p[k].x = A[v]; p[k].y = A[64 + v]; p[k].z = A[128 + v]; }
        const f32 d = sft_v_dot(sft_v_face_normal(p[0], p[1], p[2]), axis);
        if (d < min_dot) min_dot = d;
    }
    const f32 sin_a = (min_dot < 0.f) ? 1.f : sqrtf(1.f - min_dot * min_dot);
    f32* C = cull + (size_t)mi * 8;
    C[0] = sph.c.x; C[1] = sph.c.y; C[2] = sph.c.z; C[3] = sph.r;
    C[4] = axis.x; C[5] = axis.y; C[6] = axis.z; C[7] = sin_a + 0.02f;
}

SFT_FUNC u32 sft_mesh_build_meshlets(const sft_raw_mesh* m, u32 bone_count, u32 cap, f32* attr, u8* inds, f32* cull,
                                     u16* joints, u8* weights, i32* culling_bones) {
    if (!m || !m->triangle_count || !m->indices || !m->pos || !m->nrm || !m->uv) return 0;
    const i32 nt = (i32)m->triangle_count, nv = (i32)m->vertex_count;
    for (i32 k = 0; k < nt * 3; k++) if (m->indices[k] < 0 || m->indices[k] >= nv) return 0;   /* an index outside the vertices */
    /* triangles around each vertex, in triangle order (sofren2.c:7467-7492) */
    i32* first = (i32*)calloc((size_t)nv + 1, sizeof(i32));
    i32* around = (i32*)malloc((size_t)nt * 3 * sizeof(i32));
    i32* head = (i32*)malloc(((size_t)nv + 1) * sizeof(i32));
    u8* used = (u8*)calloc((size_t)nt, 1);
    u8* queued = (u8*)calloc((size_t)nt, 1);
    i32* front = (i32*)malloc((size_t)nt * sizeof(i32));
    i32* scratch = (i32*)calloc((size_t)bone_count + 1, sizeof(i32));
    for (i32 k = 0; k < nt * 3; k++) first[m->indices[k]]++;
    for (i32 v = 0, acc = 0; v <= nv; v++) { const i32 c = v < nv ? first[v] : 0; first[v] = acc; acc += c; }
    memcpy(head, first, ((size_t)nv + 1) * sizeof(i32));
    for (i32 t = 0; t < nt; t++)
        for (int k = 0; k < 3; k++) around[head[m->indices[t * 3 + k]]++] = t;

    u32 count = 0;
    i32 left = nt, seed_from = 0;
    sft__mlet b;
    while (left > 0) {
        b.nv = 0; b.nt = 0; b.axis.x = b.axis.y = b.axis.z = 0.f;
        i32 fh = 0, ft = 0;   /* frontier: triangles next to the meshlet, [fh, ft) still open */
        while (b.nv < SFT_VERTS_PER_MESHLET && b.nt < 128 && left > 0) {
            i32 pick_slot = -1, pick;
            sftvec pick_n;
            if (fh == ft) {   /* empty frontier: the first unused triangle in index order seeds (or joins) */
                pick = -1;
                for (i32 t = seed_from; t < nt; t++) if (!used[t]) { pick = seed_from = t; break; }
                if (pick < 0) break;
                pick_n = sft__raw_tri_normal(m, pick);
                const i32* ix = m->indices + (size_t)pick * 3;
                if (b.nt > 0 && sft__mlet_score(&b, ix[0], ix[1], ix[2], pick_n) < 0.f) break;
            } else {          /* the open frontier triangle with the best score, first of equals */
                f32 best = -1.f;
                for (i32 k = fh; k < ft; k++) {
                    const i32 t = front[k];
                    if (used[t]) continue;
                    const i32* ix = m->indices + (size_t)t * 3;
                    const sftvec n = sft__raw_tri_normal(m, t);
                    const f32 s = sft__mlet_score(&b, ix[0], ix[1], ix[2], n);
                    if (s > best) { best = s; pick_slot = k; pick_n = n; }
                }
                if (pick_slot < 0) { fh = ft = 0; continue; }   /* nothing fits: restart from a seed (flags stay set) */
                pick = front[pick_slot];
            }
            const i32* ix = m->indices + (size_t)pick * 3;
            sft__mlet_add(&b, ix[0], ix[1], ix[2], pick_n);
            used[pick] = 1;
            left--;
            if (pick_slot >= 0) front[pick_slot] = front[fh++];
            for (int k = 0; k < 3; k++)
                for (i32 a = first[ix[k]]; a < first[ix[k] + 1]; a++) {
                    const i32 t = around[a];
                    if (!used[t] && !queued[t]) { front[ft++] = t; queued[t] = 1; }
                }
        }
        for (i32 k = fh; k < ft; k++) queued[front[k]] = 0;
        if (count < cap && attr && inds && cull)
            sft__mlet_emit(&b, m, bone_count, scratch, count, attr, inds, cull, joints, weights, culling_bones);
        else { sftvec pts[SFT_VERTS_PER_MESHLET], sup[4]; for (u32 i = 0; i < b.nv; i++) pts[i] = sft__raw_pos(m, b.gv[i]); if (b.nv) sft__welzl(pts, (i32)b.nv, sup, 0); }
        count++;
    }
    free(first); free(around); free(head); free(used); free(queued); free(front); free(scratch);
    return count;
}

/* ---- shadow proxies (sofren2.c:3064-3524) */

/* a capsule around a point set (sofren2.c:3064-3135): the principal axis by ten power steps on
 * the covariance, the extent along it, a radius between the mean (x1.8) and the largest (x0.95)
 * distance to the axis segment, and ends pushed out by 0.625 r to seal joints */
static sft_shadow_proxy sft__capsule_fit(const sftvec* v, i32 n) {
    sft_shadow_proxy out;
    memset(&out, 0, sizeof(out));
    if (n == 0) return out;
    sftvec c = { 0.f, 0.f, 0.f };
    for (i32 i = 0; i < n; i++) c = sft_v_add(c, v[i]);
    c = sft_v_mul(c, 1.f / n);
    f32 cov[3][3];
    memset(cov, 0, sizeof(cov));
    for (i32 k = 0; k < n; k++) {
        const sftvec d = sft_v_sub(v[k], c);
        const f32 a[3] = { d.x, d.y, d.z };
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) cov[i][j] += a[i] * a[j];
    }
    for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) cov[i][j] /= n;
    sftvec axis = sft_v_normf(1.f, 1.f, 1.f);
    for (int it = 0; it < 10; it++) {
        sftvec nx;
        nx.x = cov[0][0] * axis.x + cov[0][1] * axis.y + cov[0][2] * axis.z;
        nx.y = cov[1][0] * axis.x + cov[1][1] * axis.y + cov[1][2] * axis.z;
        nx.z = cov[2][0] * axis.x + cov[2][1] * axis.y + cov[2][2] * axis.z;
        const f32 len = sft_v_length(nx);
        if (len < SFT_EPSILON) break;
        axis = sft_v_mul(nx, 1.f / len);
    }
    f32 t0 = 1e9f, t1 = -1e9f;
    for (i32 i = 0; i < n; i++) {
        const f32 t = sft_v_dot(sft_v_sub(v[i], c), axis);
        if (t < t0) t0 = t;
        if (t > t1) t1 = t;
    }
    const sftvec ra = sft_v_add(c, sft_v_mul(axis, t0)), ab = sft_v_sub(sft_v_add(c, sft_v_mul(axis, t1)), ra);
    const f32 len2 = sft_v_length2(ab);
    f32 sum_r = 0.f, max_r = 0.f;
    for (i32 i = 0; i < n; i++) {
        f32 t = 0.f;
        if (!(len2 < SFT_EPSILON)) {
            t = sft_v_dot(sft_v_sub(v[i], ra), ab) / len2;
            t = t < 0.f ? 0.f : (t > 1.f ? 1.f : t);
        }
        const f32 r = sqrtf(sft_v_length2(sft_v_sub(v[i], sft_v_add(ra, sft_v_mul(ab, t)))));
        sum_r += r;
        if (r > max_r) max_r = r;
    }
    const f32 ra_ = (sum_r / n) * 1.8f, rb_ = max_r * 0.95f;
    const f32 r = ra_ < rb_ ? ra_ : rb_;
    f32 s0 = t0 - r * 0.625f, s1 = t1 + r * 0.625f;
    if (s0 > s1) s0 = s1 = (t0 + t1) * 0.5f;
    out.posa = sft_v_add(c, sft_v_mul(axis, s0));
    out.posb = sft_v_add(c, sft_v_mul(axis, s1));
    out.radius = r;
    return out;
}

typedef struct { const sft_mesh_data* meshes; u32 mesh_count; const sft__node* nodes; u32 node_count; } sft__pmodel;

/* mesh and local meshlet of a model meshlet index */
static const sft_mesh_data* sft__pm_meshlet(const sft__pmodel* pm, u32 g, u32* local) {
    for (u32 k = 0; k < pm->mesh_count; k++) {
        if (g < pm->meshes[k].meshlet_count) { *local = g; return &pm->meshes[k]; }
        g -= pm->meshes[k].meshlet_count;
    }
    return NULL;
}
/* the triangle corners under a BLAS node, depth first in slot order (sofren2.c:3144-3197) */
static void sft__pm_gather(const sft__pmodel* pm, u32 node, sftvec** v, i32* cap, i32* n, int depth) {
    if (node >= pm->node_count || depth > 64) return;
    const sft__node* nd = &pm->nodes[node];
    for (u32 c = 0; c < nd->count && c < 8; c++) {
        const u32 ch = nd->child[c];
        if (ch == 0xFFFFFFFFu) continue;
        if (!nd->leaf) { sft__pm_gather(pm, ch, v, cap, n, depth + 1); continue; }
        const u32 pay = ch & 0x7FFFFFFFu, tri = pay & 127u;
        u32 lm;
        const sft_mesh_data* md = sft__pm_meshlet(pm, pay >> 7, &lm);
        if (!md) continue;
        const u8* I = md->inds + (size_t)lm * 512;
        const f32* A = md->attr + (size_t)lm * 640;
        const u32 bt = tri >> 3, l = tri & 7;
        if (*n + 3 > *cap) { *cap = *cap ? *cap * 2 + 3 : 1024; *v = (sftvec*)realloc(*v, (size_t)*cap * sizeof(sftvec)); }
        for (int k = 0; k < 3; k++) {
            const u8 q = I[bt * 32 + k * 8 + l];
            sftvec p = { A[q], A[64 + q], A[128 + q] };
            (*v)[(*n)++] = p;
        }
    }
}
/* static model (sofren2.c:3209-3268): starting from the root, the non-leaf node of the largest
 * child-box volume is replaced by its children until `budget` nodes; one capsule per node */
static u32 sft__proxies_bvh(const sft__pmodel* pm, u32 root, i32 budget, sft_shadow_proxy* out, u32 cap) {
    u32* act = (u32*)malloc((size_t)budget * sizeof(u32));
    i32 n = 1;
    act[0] = root;
    while (n < budget) {
        i32 big = -1;
        f32 big_vol = -1.f;
        for (i32 i = 0; i < n; i++) {
            if (act[i] >= pm->node_count) continue;
            const sft__node* nd = &pm->nodes[act[i]];
            if (nd->leaf) continue;
            f32 mn[3] = { 1e30f, 1e30f, 1e30f }, mx[3] = { -1e30f, -1e30f, -1e30f };
            for (u32 c = 0; c < nd->count && c < 8; c++)
                for (int a = 0; a < 3; a++) {
                    if (nd->mn[a][c] < mn[a]) mn[a] = nd->mn[a][c];
                    if (nd->mx[a][c] > mx[a]) mx[a] = nd->mx[a][c];
                }
            const f32 vol = (mx[0] - mn[0]) * (mx[1] - mn[1]) * (mx[2] - mn[2]);
            if (vol > big_vol) { big_vol = vol; big = i; }
        }
        if (big < 0) break;
        const sft__node* sp = &pm->nodes[act[big]];
        act[big] = sp->child[0];
        for (u32 c = 1; c < sp->count && c < 8 && n < budget; c++)
            if (sp->child[c] != 0xFFFFFFFFu) act[n++] = sp->child[c];
    }
    for (i32 i = 0; i < n && (u32)i < cap; i++) {
        sftvec* v = NULL;
        i32 vc = 0, vn = 0;
        sft__pm_gather(pm, act[i], &v, &vc, &vn, 0);
        out[i] = sft__capsule_fit(v, vn);
        out[i].bone_ind = 0xFFFFFFFFu;   /* not bound to a joint */
        free(v);
    }
    free(act);
    return (u32)n;
}

static u16 sft__cluster_of(const u16* map, u16 b) { while (map[b] != b) b = map[b]; return b; }

/* skinned model (sofren2.c:3270-3505) */
static u32 sft__proxies_bones(const sft__pmodel* pm, const sft_raw_bone* bones, u32 nb, i32 budget, sft_shadow_proxy* out, u32 cap) {
    typedef struct { f32 area; sftvec csum; i32 tris; } clus;
    u16* map = (u16*)malloc((size_t)nb * sizeof(u16));
    clus* cl = (clus*)calloc(nb, sizeof(clus));
    for (u32 i = 0; i < nb; i++) map[i] = (u16)i;
    /* each live triangle votes, with its area and centre, for the joint of the largest single
     * weight over its corners (first of equals) */
    for (u32 k = 0; k < pm->mesh_count; k++) {
        const sft_mesh_data* md = &pm->meshes[k];
        if (!md->joints || !md->weights) continue;
        for (u32 ml = 0; ml < md->meshlet_count; ml++) {
            const u8* I = md->inds + (size_t)ml * 512;
            const f32* A = md->attr + (size_t)ml * 640;
            const u16* J = md->joints + (size_t)ml * 256;
            const u8* W = md->weights + (size_t)ml * 256;
            for (u32 t = 0; t < 128; t++) {
                const u32 bt = t >> 3, l = t & 7;
                const u8 q[3] = { I[bt * 32 + l], I[bt * 32 + 8 + l], I[bt * 32 + 16 + l] };
                if (q[0] == q[1] && q[1] == q[2]) continue;   /* padding */
                i32 bone = 0;
                f32 wmax = -1.f;
                for (int c = 0; c < 3; c++)
                    for (int s = 0; s < 4; s++)
                        if ((f32)W[s * 64 + q[c]] > wmax) { wmax = W[s * 64 + q[c]]; bone = J[s * 64 + q[c]]; }
                if ((u32)bone >= nb) continue;
                sftvec p[3];
                for (int c = 0; c < 3; c++) { p[c].x = A[q[c]]; p[c].y = A[64 + q[c]]; p[c].z = A[128 + q[c]]; }
                const f32 area = sft_v_length(sft_v_cross(sft_v_sub(p[1], p[0]), sft_v_sub(p[2], p[0]))) * 0.5f;
                const sftvec ctr = sft_v_mul(sft_v_add(p[0], sft_v_add(p[1], p[2])), 0.333333f);
                cl[bone].area += area;
                cl[bone].csum = sft_v_add(cl[bone].csum, ctr);
                cl[bone].tris += 1;
            }
        }
    }
    i32 active = 0;
    for (u32 i = 0; i < nb; i++) if (cl[i].tris > 0) active++;
    /* merge the smallest-area cluster into its parent's cluster (a root into the largest other
     * cluster) until the budget holds */
    while (active > budget && active > 1) {
        i32 small = -1;
        f32 amin = 1e30f;
        for (u32 i = 0; i < nb; i++) if (cl[i].tris > 0 && cl[i].area < amin) { amin = cl[i].area; small = (i32)i; }
        if (small < 0) break;
        i32 target = -1;
        const i32 parent = bones[small].parent_ind;
        if (parent != -1) target = (parent >= 0 && (u32)parent < nb) ? sft__cluster_of(map, (u16)parent) : -1;
        else {
            f32 amax = -1.f;
            for (u32 i = 0; i < nb; i++) if ((i32)i != small && cl[i].area > amax) { amax = cl[i].area; target = (i32)i; }
        }
        if (target < 0 || target == small) break;
        map[small] = (u16)target;
        cl[target].area += cl[small].area;
        cl[target].csum = sft_v_add(cl[target].csum, cl[small].csum);
        cl[target].tris += cl[small].tris;
        cl[small].tris = 0;
        active--;
    }
    /* every skinned vertex slot with weight goes to the cluster of its heaviest joint */
    sftvec** cv = (sftvec**)calloc(nb, sizeof(sftvec*));
    i32* ccap = (i32*)calloc(nb, sizeof(i32));
    i32* cn = (i32*)calloc(nb, sizeof(i32));
    for (u32 k = 0; k < pm->mesh_count; k++) {
        const sft_mesh_data* md = &pm->meshes[k];
        if (!md->joints || !md->weights) continue;
        for (u32 ml = 0; ml < md->meshlet_count; ml++) {
            const f32* A = md->attr + (size_t)ml * 640;
            const u16* J = md->joints + (size_t)ml * 256;
            const u8* W = md->weights + (size_t)ml * 256;
            for (u32 v = 0; v < SFT_VERTS_PER_MESHLET; v++) {
                u8 wmax = W[v];
                u16 bone = J[v];
                for (int s = 1; s < 4; s++) if (W[s * 64 + v] > wmax) { wmax = W[s * 64 + v]; bone = J[s * 64 + v]; }
                if (wmax == 0 || bone >= nb) continue;
                const u16 c = sft__cluster_of(map, bone);
                if (cn[c] >= ccap[c]) { ccap[c] = ccap[c] ? ccap[c] * 2 : 1024; cv[c] = (sftvec*)realloc(cv[c], (size_t)ccap[c] * sizeof(sftvec)); }
                sftvec p = { A[v], A[64 + v], A[128 + v] };
                cv[c][cn[c]++] = p;
            }
        }
    }
    /* capsules anchored at the joint, along joint -> centroid of the cluster's triangle centres;
     * radius between the mean (x2.2) and the largest (x0.9) distance to the axis */
    u32 w = 0;
    for (u32 i = 0; i < nb; i++) {
        if (cl[i].tris > 0 && cn[i] > 0 && w < cap) {
            const sftvec ctr = sft_v_mul(cl[i].csum, 1.f / cl[i].tris), anc = bones[i].bind_pos;
            sftvec axis = sft_v_sub(ctr, anc);
            const f32 al = sft_v_length(axis);
            if (al > SFT_EPSILON) axis = sft_v_mul(axis, 1.f / al);
            else { axis.x = 0.f; axis.y = 1.f; axis.z = 0.f; }
            f32 t0 = 1e9f, t1 = -1e9f, sum_r = 0.f, max_r = 0.f;
            for (i32 k = 0; k < cn[i]; k++) {
                const f32 t = sft_v_dot(sft_v_sub(cv[i][k], anc), axis);
                if (t < t0) t0 = t;
                if (t > t1) t1 = t;
                const f32 r = sqrtf(sft_v_length2(sft_v_sub(cv[i][k], sft_v_add(anc, sft_v_mul(axis, t)))));
                sum_r += r;
                if (r > max_r) max_r = r;
            }
            const f32 ra_ = (sum_r / cn[i]) * 2.2f, rb_ = max_r * 0.9f;
            const f32 r = ra_ < rb_ ? ra_ : rb_;
            const f32 e0 = t0 - r * 0.25f, e1 = t1 + r * 0.25f;
            f32 s0 = 0.f < e0 ? 0.f : e0, s1 = 0.f > e1 ? 0.f : e1;
            if (s0 > s1) s0 = s1 = (s0 + s1) * 0.5f;
            out[w].posa = sft_v_add(anc, sft_v_mul(axis, s0));
            out[w].posb = sft_v_add(anc, sft_v_mul(axis, s1));
            out[w].radius = r;
            out[w].bone_ind = i;
            w++;
        }
        free(cv[i]);
    }
    /* the reference counts every active cluster; a cluster without vertices leaves a zero proxy */
    for (u32 i = w; i < (u32)active && i < cap; i++) memset(&out[i], 0, sizeof(out[i]));
    free(cv); free(ccap); free(cn); free(map); free(cl);
    return (u32)active;
}

SFT_FUNC u32 sft_model_fit_shadow_proxies(const sft_mesh_data* meshes, u32 mesh_count, const void* blas_nodes, u32 blas_count,
                                          u32 blas_root, const sft_raw_bone* bones, u32 bone_count, i32 budget,
                                          sft_shadow_proxy* out, u32 cap) {
    if (budget <= 0 || !blas_nodes || blas_count == 0 || !meshes) return 0;
    sft__pmodel pm = { meshes, mesh_count, (const sft__node*)blas_nodes, blas_count };
    if (bone_count > 0 && bones) return sft__proxies_bones(&pm, bones, bone_count, budget, out, out ? cap : 0);
    return sft__proxies_bvh(&pm, blas_root, budget, out, out ? cap : 0);
}

SFT_FUNC sft_model* sft_model_build(const sft_raw_mesh* meshes, u32 mesh_count, const sft_raw_bone* bones, u32 bone_count,
                                    i32 shadow_proxy_budget, sft_arena* arena) {
    (void)arena;
    if (!meshes || !mesh_count) return NULL;
    sft_mesh_data* md = (sft_mesh_data*)calloc(mesh_count, sizeof(sft_mesh_data));
    sft_model* m = NULL;
    int ok = 1;
    for (u32 k = 0; k < mesh_count && ok; k++) {
        const sft_raw_mesh* r = &meshes[k];
        const int skinned = r->joints && r->weights;
        /* at most one meshlet per triangle: build straight into arrays of that size */
        const u32 cap = r->triangle_count ? r->triangle_count : 1;
        f32* attr = (f32*)calloc((size_t)cap * 640, sizeof(f32));
        u8* inds = (u8*)calloc((size_t)cap * 512, 1);
        f32* cull = (f32*)calloc((size_t)cap * 8, sizeof(f32));
        u16* jn = skinned ? (u16*)calloc((size_t)cap * 256, sizeof(u16)) : NULL;
        u8* wt = skinned ? (u8*)calloc((size_t)cap * 256, 1) : NULL;
        i32* cb = skinned ? (i32*)calloc(cap, sizeof(i32)) : NULL;
        const u32 n = sft_mesh_build_meshlets(r, bone_count, cap, attr, inds, cull, jn, wt, cb);
        if (n == 0 && r->triangle_count) ok = 0;
        md[k].meshlet_count = n; md[k].attr = attr; md[k].inds = inds; md[k].cull = cull;
        md[k].joints = jn; md[k].weights = wt; md[k].culling_bones = cb;
        md[k].material = r->material; md[k].lightmap_page = 0xFFFFFFFFu;
    }
    if (ok) m = sft__model_create(md, mesh_count, NULL, 0, bone_count, NULL, 0, NULL, 0, 0);
    if (m && shadow_proxy_budget > 0) {
        u32 nodes = 0, root = 0;
        const void* blas = sft_model_get_blas(m, &nodes, &root);
        if (blas && nodes) {
            const u32 np = sft_model_fit_shadow_proxies(md, mesh_count, blas, nodes, root, bones, bone_count, shadow_proxy_budget, NULL, 0);
            sft_shadow_proxy* px = (sft_shadow_proxy*)calloc((size_t)np + 1, sizeof(sft_shadow_proxy));
            sft_model_fit_shadow_proxies(md, mesh_count, blas, nodes, root, bones, bone_count, shadow_proxy_budget, px, np);
            free(m->proxies);
            m->proxies = px; m->proxy_count = np;
        }
    }
    for (u32 k = 0; k < mesh_count; k++) {
        free((void*)md[k].attr); free((void*)md[k].inds); free((void*)md[k].cull);
        free((void*)md[k].joints); free((void*)md[k].weights); free((void*)md[k].culling_bones);
    }
    free(md);
    return m;
}

/* ---------------------------------------------------------------- draw (sofren2.c:8410-8478) */
SFT_FUNC void sft_draw_instance(const sft_instance* in) {
    const i32 slot = sft__s->n_inst_claimed++;
    if (slot >= SFT_MAX_INSTANCES_PER_FRAME) return;    /* same silent drop as the reference */
    const sft_model* md = in->model;
    sftg_instance_desc* d = &sft__s->inst[slot];
    d->model = md->device_id;
    memcpy(d->transform, in->transform.m, 64);
    d->bones = NULL; d->bone_count = 0;
    sft__s->inst_model[slot] = md;
    if (in->posed_bone_matrices && md->bone_count) {
        if (sft__s->n_bones + md->bone_count > sft__s->cap_bones) {
            while (sft__s->n_bones + md->bone_count > sft__s->cap_bones) sft__s->cap_bones = sft__s->cap_bones ? sft__s->cap_bones * 2 : 256;
            sft__s->bones = (f32*)realloc(sft__s->bones, (size_t)sft__s->cap_bones * 64);
        }
        sft__s->inst_bone_off[slot] = sft__s->n_bones;
        memcpy(sft__s->bones + 16 * (size_t)sft__s->n_bones, in->posed_bone_matrices, (size_t)md->bone_count * 64);
        d->bone_count = md->bone_count;
        sft__s->n_bones += md->bone_count;
    }
    sft__s->n_inst = (u32)slot + 1;
    sft__s->total_ss += md->total_meshlets;
    /* world-space shadow proxies (8426-8455) */
    if (sft__s->shadows && md->proxy_count > 0) {
        if (sft__s->n_prox + md->proxy_count > sft__s->cap_prox) {
            while (sft__s->n_prox + md->proxy_count > sft__s->cap_prox) sft__s->cap_prox = sft__s->cap_prox ? sft__s->cap_prox * 2 : 64;
            sft__s->proxies = (f32*)realloc(sft__s->proxies, (size_t)sft__s->cap_prox * 32);
        }
        for (u32 i = 0; i < md->proxy_count; i++) {
            const sft_shadow_proxy* lp = &md->proxies[i];
            sftmat m = in->transform;
            if (lp->bone_ind != 0xFFFFFFFFu && in->posed_bone_matrices) m = sft_m_mul(in->posed_bone_matrices[lp->bone_ind], in->transform);
            f32* w = sft__s->proxies + 8 * (size_t)sft__s->n_prox++;
            w[0] = lp->posa.x * m.m[0][0] + lp->posa.y * m.m[1][0] + lp->posa.z * m.m[2][0] + m.m[3][0];
            w[1] = lp->posa.x * m.m[0][1] + lp->posa.y * m.m[1][1] + lp->posa.z * m.m[2][1] + m.m[3][1];
            w[2] = lp->posa.x * m.m[0][2] + lp->posa.y * m.m[1][2] + lp->posa.z * m.m[2][2] + m.m[3][2];
            w[3] = lp->posb.x * m.m[0][0] + lp->posb.y * m.m[1][0] + lp->posb.z * m.m[2][0] + m.m[3][0];
            w[4] = lp->posb.x * m.m[0][1] + lp->posb.y * m.m[1][1] + lp->posb.z * m.m[2][1] + m.m[3][1];
            w[5] = lp->posb.x * m.m[0][2] + lp->posb.y * m.m[1][2] + lp->posb.z * m.m[2][2] + m.m[3][2];
            const f32 sx = sqrtf(m.m[0][0] * m.m[0][0] + m.m[0][1] * m.m[0][1] + m.m[0][2] * m.m[0][2]);
            w[6] = lp->radius * sx; w[7] = 0.f;
        }
    }
}

/* copies one frame description and everything it points at into one allocation */
static void sft__batch_record(const sftg_frame_desc* fd, u32* color, i32 pitch) {
    struct sft__state* s = sft__s;
    if (s->n_batch == s->cap_batch) {
        s->cap_batch = s->cap_batch ? s->cap_batch * 2 : 16;
        s->batch_fd = (sftg_frame_desc*)realloc(s->batch_fd, s->cap_batch * sizeof(sftg_frame_desc));
        s->batch_color = (u32**)realloc(s->batch_color, s->cap_batch * sizeof(u32*));
        s->batch_pitch = (i32*)realloc(s->batch_pitch, s->cap_batch * sizeof(i32));
        s->batch_mem = (void**)realloc(s->batch_mem, s->cap_batch * sizeof(void*));
    }
    size_t nbones = 0;
    for (u32 i = 0; i < fd->n_instances; i++) nbones += fd->instances[i].bone_count;
    const size_t b_inst = (size_t)fd->n_instances * sizeof(sftg_instance_desc), b_bones = nbones * 64;
    const size_t b_pl = (size_t)fd->n_point * 32, b_dl = (size_t)fd->n_dir * 24, b_px = (size_t)fd->n_proxies * 32;
    const size_t b_tl = (size_t)fd->tlas_count * sizeof(sft__node);
    char* m = (char*)malloc(b_inst + b_bones + b_pl + b_dl + b_px + b_tl + 64);
    char* q = m;
    sftg_frame_desc c = *fd;
    sftg_instance_desc* inst = (sftg_instance_desc*)q; q += b_inst;
    f32* bones = (f32*)q; q += b_bones;
    for (u32 i = 0; i < fd->n_instances; i++) {
        inst[i] = fd->instances[i];
        if (fd->instances[i].bone_count) {
            memcpy(bones, fd->instances[i].bones, (size_t)fd->instances[i].bone_count * 64);
            inst[i].bones = bones;
            bones += 16 * (size_t)fd->instances[i].bone_count;
        }
    }
    c.instances = inst;
    if (b_pl) { memcpy(q, fd->point_lights, b_pl); c.point_lights = (const f32*)q; q += b_pl; }
    if (b_dl) { memcpy(q, fd->dir_lights, b_dl); c.dir_lights = (const f32*)q; q += b_dl; }
    if (b_px) { memcpy(q, fd->proxies, b_px); c.proxies = (const f32*)q; q += b_px; }
    if (b_tl) { memcpy(q, fd->tlas_nodes, b_tl); c.tlas_nodes = q; q += b_tl; }
    s->batch_fd[s->n_batch] = c;
    s->batch_color[s->n_batch] = color;
    s->batch_pitch[s->n_batch] = pitch;
    s->batch_mem[s->n_batch] = m;
    s->n_batch++;
}

SFT_FUNC void sft_present(void) {
    struct sft__state* s = sft__s;
    /* TLAS over instance bounds, rebuilt per frame (sofren2.c:3619-3703) */
    sft__node* tlas = NULL; u32 tlas_count = 0, tlas_root = 0;
    if (s->n_inst) {
        sft__item* it = (sft__item*)calloc(s->n_inst, sizeof(sft__item));
        u32 valid = 0;
        for (u32 i = 0; i < s->n_inst; i++) {
            const sft_model* md = s->inst_model[i];
            if (!md->blas_count) continue;
            const f32* T = s->inst[i].transform;
            f32 lo[3] = { 1e30f, 1e30f, 1e30f }, hi[3] = { -1e30f, -1e30f, -1e30f };
            for (int k = 0; k < 8; k++) {
                const f32 cx = (k & 1) ? md->root_max[0] : md->root_min[0];
                const f32 cy = (k & 2) ? md->root_max[1] : md->root_min[1];
                const f32 cz = (k & 4) ? md->root_max[2] : md->root_min[2];
                for (int a = 0; a < 3; a++) {
                    const f32 t = cx * T[a] + cy * T[4 + a] + cz * T[8 + a] + T[12 + a];
                    if (t < lo[a]) lo[a] = t;
                    if (t > hi[a]) hi[a] = t;
                }
            }
            it[i].id = i;
            for (int a = 0; a < 3; a++) { it[i].mn[a] = lo[a]; it[i].mx[a] = hi[a]; it[i].c[a] = (lo[a] + hi[a]) * 0.5f; }
            valid++;
        }
        tlas = (sft__node*)calloc((size_t)valid * 2 + 1, sizeof(sft__node));
        tlas_root = sft__bvh_build(it, valid, tlas, &tlas_count, NULL, NULL);
        free(it);
    }
    for (u32 i = 0; i < s->n_inst; i++)
        s->inst[i].bones = s->inst[i].bone_count ? s->bones + 16 * (size_t)s->inst_bone_off[i] : NULL;
    sftg_frame_desc fd; memset(&fd, 0, sizeof(fd));
    fd.width = s->width; fd.height = s->height; fd.samples = s->samples;
    fd.cam_pos[0] = s->cam.x; fd.cam_pos[1] = s->cam.y; fd.cam_pos[2] = s->cam.z;
    memcpy(fd.view_proj, s->view_proj.m, 64);
    memcpy(fd.frustum_n, s->fn, sizeof(fd.frustum_n)); memcpy(fd.frustum_d, s->fd, sizeof(fd.frustum_d));
    fd.ambient[0] = s->ambient.x; fd.ambient[1] = s->ambient.y; fd.ambient[2] = s->ambient.z;
    fd.lightmap_brightness = s->lightmap_brightness;
    fd.clear = s->clear; fd.clear_color = s->clear_color; fd.shadows = s->shadows; fd.debug_mode = (u32)s->debug_mode;
    fd.debug_texture = sft__tex_device(s->checker_tex);
    fd.n_point = s->n_point; fd.point_lights = s->point;
    fd.n_dir = s->n_dir; fd.dir_lights = s->dir;
    fd.n_instances = s->n_inst; fd.instances = s->inst;
    fd.n_proxies = s->n_prox; fd.proxies = s->proxies;
    fd.tlas_nodes = tlas; fd.tlas_count = tlas_count; fd.tlas_root = tlas_root;
    if (s->batching) {   /* record a self-contained copy; sft_frame_end may reuse every array */
        sft__batch_record(&fd, s->color, s->pitch);
        free(tlas);
        return;
    }
    const int rc = sftg_frame_render(s->gpu, &fd, s->color, s->pitch, s->debug);
    free(tlas);
    if (rc) fprintf(stderr, "sofren2-gb300: sft_present failed (%d): %s\n", rc, sftg_last_error(s->gpu));
}

SFT_FUNC void sft_batch_begin(void) {
    struct sft__state* s = sft__s;
    for (u32 i = 0; i < s->n_batch; i++) free(s->batch_mem[i]);
    s->n_batch = 0;
    s->batching = 1;
}

SFT_FUNC const void* sft_batch_peek(u32 i) { return sft__s && i < sft__s->n_batch ? (const void*)&sft__s->batch_fd[i] : NULL; }
SFT_FUNC void* sft_get_gpu_context(void) { return sft__s ? (void*)sft__s->gpu : NULL; }

SFT_FUNC i32 sft_batch_autotune(i32 reps) {
    struct sft__state* s = sft__s;
    s->batching = 0;
    const int rc = s->n_batch ? sftg_autotune(s->gpu, s->batch_fd, s->n_batch, reps, NULL) : 0;
    for (u32 i = 0; i < s->n_batch; i++) free(s->batch_mem[i]);
    s->n_batch = 0;
    if (rc) fprintf(stderr, "sofren2-gb300: sft_batch_autotune failed (%d): %s\n", rc, sftg_last_error(s->gpu));
    return rc;
}

SFT_FUNC i32 sft_batch_submit(void) {
    struct sft__state* s = sft__s;
    s->batching = 0;
    if (!s->n_batch) return 0;
    u8 any_host = 0;
    for (u32 i = 0; i < s->n_batch; i++) any_host |= s->batch_color[i] != NULL;
    const int rc = sftg_frames_render(s->gpu, s->batch_fd, s->n_batch, any_host ? s->batch_color : NULL, s->batch_pitch, NULL);
    for (u32 i = 0; i < s->n_batch; i++) free(s->batch_mem[i]);
    s->n_batch = 0;
    sft__dmesh_release_frame();
    if (rc) fprintf(stderr, "sofren2-gb300: sft_batch_submit failed (%d): %s\n", rc, sftg_last_error(s->gpu));
    return rc;
}

static void sft__lane_free(u32 lane) {
    struct sft__state* s = sft__s;
    for (u32 i = 0; i < s->lane[lane].n; i++) free(s->lane[lane].mem[i]);
    free(s->lane[lane].fd); free(s->lane[lane].color); free(s->lane[lane].pitch); free(s->lane[lane].mem);
    memset(&s->lane[lane], 0, sizeof(s->lane[lane]));
}

SFT_FUNC i32 sft_batch_wait(u32 lane) {
    struct sft__state* s = sft__s;
    if (!s || lane == 0 || lane >= SFTG_MAX_LANES) return SFTG_E_ARG;
    if (!s->lane[lane].n) return 0;
    const int rc = sftg_lane_wait(s->gpu, lane);
    sft__lane_free(lane);
    if (rc) fprintf(stderr, "sofren2-gb300: sft_batch_wait failed (%d): %s\n", rc, sftg_last_error(s->gpu));
    return rc;
}

SFT_FUNC i32 sft_batch_submit_async(u32 lane) {
    struct sft__state* s = sft__s;
    s->batching = 0;
    if (lane == 0 || lane >= SFTG_MAX_LANES) return SFTG_E_ARG;
    if (s->lane[lane].n) { const i32 w = sft_batch_wait(lane); if (w) return w; }
    if (!s->n_batch) return 0;
    /* the recorded frames move to the lane and stay there until sft_batch_wait */
    s->lane[lane].fd = s->batch_fd; s->lane[lane].color = s->batch_color; s->lane[lane].pitch = s->batch_pitch;
    s->lane[lane].mem = s->batch_mem; s->lane[lane].n = s->n_batch;
    s->batch_fd = NULL; s->batch_color = NULL; s->batch_pitch = NULL; s->batch_mem = NULL;
    s->n_batch = 0; s->cap_batch = 0;
    u8 any_host = 0;
    for (u32 i = 0; i < s->lane[lane].n; i++) any_host |= s->lane[lane].color[i] != NULL;
    const int rc = sftg_frames_submit(s->gpu, lane, s->lane[lane].fd, s->lane[lane].n, any_host ? s->lane[lane].color : NULL,
                                      s->lane[lane].pitch);
    if (rc) {
        fprintf(stderr, "sofren2-gb300: sft_batch_submit_async failed (%d): %s\n", rc, sftg_last_error(s->gpu));
        sft__lane_free(lane);
    }
    return rc;
}

SFT_FUNC i32 sft_batch_done(u32 lane) {
    if (!sft__s || lane >= SFTG_MAX_LANES) return SFTG_E_ARG;
    return sft__s->lane[lane].n ? sftg_lane_done(sft__s->gpu, lane) : 1;
}

SFT_FUNC i32 sft_model_set_skeleton(sft_model* model, const sftg_bone_desc* bones, u32 bone_count,
                                    const sftg_animation_desc* anims, u32 anim_count) {
    if (!model || bone_count != model->bone_count) return SFTG_E_ARG;
    int32_t id = -1;
    const int rc = sftg_skeleton_upload(sft__s->gpu, bones, bone_count, anims, anim_count, &id);
    if (rc) { fprintf(stderr, "sofren2-gb300: skeleton upload failed (%d): %s\n", rc, sftg_last_error(sft__s->gpu)); return rc; }
    model->skeleton_id = id;
    return 0;
}

/* sft_raycast_instance (sofren2.c:3733-3837) through sftg_raycast: the instance's model and
 * transform with the ray; a NULL instance or model, or a model without a BLAS, gives no hit at
 * max_dist as in the reference */
SFT_FUNC void sft_raycast_batch(const sft_instance* const* insts, const sftvec* origins, const sftvec* dirs, const f32* max_dists,
                                u32 n, sft_ray_hit* out) {
    if (!n) return;
    sftg_ray* rays = (sftg_ray*)calloc(n, sizeof(sftg_ray));
    sftg_ray_hit* hits = (sftg_ray_hit*)calloc(n, sizeof(sftg_ray_hit));
    for (u32 k = 0; k < n; k++) {
        const sft_instance* in = insts[k];
        if (in) memcpy(rays[k].transform, &in->transform, 64);
        rays[k].origin[0] = origins[k].x; rays[k].origin[1] = origins[k].y; rays[k].origin[2] = origins[k].z;
        rays[k].dir[0] = dirs[k].x; rays[k].dir[1] = dirs[k].y; rays[k].dir[2] = dirs[k].z;
        rays[k].max_dist = max_dists[k];
        rays[k].model = in && in->model && in->model->blas_count ? in->model->device_id : -1;
    }
    sft__check(sftg_raycast(sft__s->gpu, rays, n, hits), "sftg_raycast");
    for (u32 k = 0; k < n; k++) {
        memset(&out[k], 0, sizeof(out[k]));
        out[k].hit = (u8)hits[k].hit;
        out[k].distance = hits[k].distance;
        out[k].pos = SFT_V(hits[k].pos[0], hits[k].pos[1], hits[k].pos[2]);
        out[k].normal = SFT_V(hits[k].normal[0], hits[k].normal[1], hits[k].normal[2]);
    }
    free(rays); free(hits);
}

SFT_FUNC sft_ray_hit sft_raycast_instance(const sft_instance* inst, sftvec origin, sftvec dir, f32 max_dist) {
    sft_ray_hit h;
    sft_raycast_batch(&inst, &origin, &dir, &max_dist, 1, &h);
    return h;
}

/* sft_pose_update (sofren2.c:8952-9108): the animation sampled at `time` (wrapped by the clip's
 * duration), evaluated on the GPU (sftg_pose_eval) into pose->global_matrices and
 * pose->posed_bone_matrices.  Nothing happens for a model without animations or an animation
 * index out of range, as in the reference. */
SFT_FUNC void sft_pose_update(sft_pose* pose, i32 anim_id, f32 time) {
    if (!pose || !pose->model || pose->model->skeleton_id < 0 || !pose->model->bone_count) return;
    sftg_pose_request r;
    r.skeleton = pose->model->skeleton_id; r.animation = anim_id; r.time = time;
    const int rc = sftg_pose_eval(sft__s->gpu, &r, 1, (float*)pose->posed_bone_matrices, (float*)pose->global_matrices);
    if (rc) fprintf(stderr, "sofren2-gb300: sft_pose_update failed (%d): %s\n", rc, sftg_last_error(sft__s->gpu));
}

SFT_FUNC sft_pose* sft_pose_create(const sft_model* model, sft_arena* arena) {
    sft_pose* p = (sft_pose*)(arena ? sft_arena_alloc(arena, sizeof(sft_pose)) : calloc(1, sizeof(sft_pose)));
    const u32 n = model ? model->bone_count : 0;
    p->model = model;
    p->global_matrices = (sftmat*)(arena ? sft_arena_alloc(arena, (n + 1) * sizeof(sftmat)) : calloc(n + 1, sizeof(sftmat)));
    p->posed_bone_matrices = (sftmat*)(arena ? sft_arena_alloc(arena, (n + 1) * sizeof(sftmat)) : calloc(n + 1, sizeof(sftmat)));
    for (u32 i = 0; i < n; i++) p->global_matrices[i] = p->posed_bone_matrices[i] = sft_m_identity();
    return p;
}

#ifdef __cplusplus
}
#endif

#endif /* SFT_IMPL */
#endif /* SOFREN2_GB300_H */
