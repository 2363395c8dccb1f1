/*
 * Test infrastructure: runs the unmodified sofren2 reference (sofren2.c, compiled from
 * where it lies, see oracle/Makefile) on an SFTS scene blob, headless, with one worker
 * thread, and dumps what the render path produced:
 *
 *   color      u32[h*w]          ARGB8888 from sft_present (sofren2.c:8139)
 *   tile_counts/tile_payloads    per-tile payload lists, walked from the chunk pool
 *                                (sofren2.c:4619-4647, 6787-6809) in list order
 *   depth/vid  per tile          the tile visibility buffer, captured by replaying the
 *                                reference's own sft__rast_simd_batch (sofren2.c:5148) over
 *                                that list exactly as sft__worker_phase_rasterize does
 *   ss_cache                     sft_state->ss_cache (sofren2.c:1464), culled meshlets left 0xFF
 *   clip                         the clipped-triangle pool (sofren2.c:1271) and its count
 *   light_vis                    per world proxy, per light (sofren2.c:8163-8280)
 *   blas                         every model's BLAS nodes (sofren2.c:3526)
 *   present_ns                   wall time of sft_present
 *
 * usage: ref_harness <scene.sfts> <out.dump> [frame_index=-1 (all)] [threads=1] [repeat=1]
 * SFT_DEBUG_MODE=<n> in the environment selects a debug view (sft_set_debug_mode).
 * Timing runs: SFT_TIMES=<path> appends, per repetition, the wall time of the whole frame (lights,
 * camera, draws, sft_present; u64 ns) to that file, SFT_TIME_BUDGET_MS=<ms> stops repeating once
 * that much time has passed (after 3 repetitions), and SFT_NO_DUMP=1 writes no dump.  The same
 * source builds the reference's NEON path on aarch64 (SFT_SIMD_WIDTH 4), where the index swizzle
 * of the blob's 8-lane batches is converted to 4-lane batches.
 * The MSAA sample count is fixed at compile time (SFT_USE_AA / SFT_AA_SAMPLES), as in the reference.
 */
#define _GNU_SOURCE
#define SFT_IMPL
#define SFT_NO_DEBUG
#if defined(__aarch64__) && defined(SFT_NEON_BUILD_SHIM)
/* The reference's NEON path (sofren2.c:387-519) needs two repairs to run, made here without
 * touching its source.  arm_neon.h is included first, so these macros leave its own definitions
 * alone and apply only to the reference's calls.
 *  - It does not compile with GCC 13.  Its vector-type mismatches (vshrq_n_u32 on int32x4_t,
 *    sofren2.c:497) pass with -flax-vector-conversions (oracle/Makefile); sofren2.c:473 widens
 *    8 bytes to a uint16x8_t and hands that to vmovl_u16, which takes the 4-lane uint16x4_t: the
 *    4-lane loader needs the low four, which the call gets here.
 *  - sft_vf_fmsub(a, b, c) must be a*b - c (the AVX2 path's _mm256_fmsub_ps, sofren2.c:294, and
 *    the scalar path, 550); the NEON path maps it to vfmsq_f32(c, a, b) = c - a*b (sofren2.c:425).
 *    With the sign flipped every triangle fails the area test (4837) and the frame stays empty.
 *    The negation gives a*b - c with the same single rounding (round to nearest is symmetric). */
#include <arm_neon.h>
#define vmovl_u16(x) vmovl_u16(vget_low_u16(x))
#define vfmsq_f32(c, a, b) vnegq_f32(vfmsq_f32((c), (a), (b)))
#endif
#include "sofren2.c"
#include "sfts_blob.h"
#include <time.h>

static uint64_t now_ns(void) {
    struct timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts);
    return (uint64_t)ts.tv_sec * 1000000000ull + (uint64_t)ts.tv_nsec;
}

static void* aalloc(size_t bytes) {
    size_t n = (bytes + 63) & ~(size_t)63;
    void* p = aligned_alloc(64, n ? n : 64);
    memset(p, 0, n ? n : 64);
    return p;
}

static sft_model* build_model(const sfts_scene* sc, const sfts_model* src, const sft_mat_handle* mats,
                              const sft_tex_handle* texs, sft_arena* arena) {
    sft_model* m = (sft_model*)calloc(1, sizeof(sft_model));
    m->mesh_count = src->n_meshes;
    m->meshes = (sft_mesh*)calloc(src->n_meshes + 1, sizeof(sft_mesh));
    u32 total = 0;
    for (u32 k = 0; k < src->n_meshes; k++) total += src->meshes[k].meshlet_count;
    m->total_meshlets = total;
    m->meshlet_mesh_inds = (u16*)aalloc((total + 8) * sizeof(u16));
    u32 off = 0;
    for (u32 k = 0; k < src->n_meshes; k++) {
        const sfts_mesh* sm = &src->meshes[k];
        sft_mesh* ms = &m->meshes[k];
        const u32 n = sm->meshlet_count;
        const u32 pad = ((n + 7) & ~7u) + 8;
        ms->meshlet_count = n;
        ms->model_meshlet_offset = off;
        ms->meshlets = (struct sft_meshlet*)aalloc(pad * sizeof(struct sft_meshlet));
        ms->meshlet_attribs = (struct sft_meshlet_attribs*)aalloc(pad * sizeof(struct sft_meshlet_attribs));
        ms->inds = (struct sft_meshlet_inds*)aalloc(pad * sizeof(struct sft_meshlet_inds));
        ms->meshlet_skins = sm->has_skin ? (struct sft_meshlet_skin*)aalloc(pad * sizeof(struct sft_meshlet_skin)) : NULL;
        f32** fields[8] = { &ms->bounds_center_x, &ms->bounds_center_y, &ms->bounds_center_z, &ms->bounds_radius,
                            &ms->cone_axis_x, &ms->cone_axis_y, &ms->cone_axis_z, &ms->cone_cutoff };
        for (int q = 0; q < 8; q++) *fields[q] = (f32*)aalloc(pad * sizeof(f32));
        ms->culling_bone_inds = sm->has_skin ? (i32*)aalloc(pad * sizeof(i32)) : NULL;
        for (u32 j = 0; j < n; j++) {
            const sfts_meshlet* sl = &sm->meshlets[j];
            memcpy(ms->meshlets[j].x, sl->attr + 0 * 64, 256);
            memcpy(ms->meshlets[j].y, sl->attr + 1 * 64, 256);
            memcpy(ms->meshlets[j].z, sl->attr + 2 * 64, 256);
            memcpy(ms->meshlet_attribs[j].nx, sl->attr + 3 * 64, 256);
            memcpy(ms->meshlet_attribs[j].ny, sl->attr + 4 * 64, 256);
            memcpy(ms->meshlet_attribs[j].nz, sl->attr + 5 * 64, 256);
            memcpy(ms->meshlet_attribs[j].u, sl->attr + 6 * 64, 256);
            memcpy(ms->meshlet_attribs[j].v, sl->attr + 7 * 64, 256);
            memcpy(ms->meshlet_attribs[j].lu, sl->attr + 8 * 64, 256);
            memcpy(ms->meshlet_attribs[j].lv, sl->attr + 9 * 64, 256);
            if (sm->has_skin) {
                memcpy(ms->meshlet_skins[j].j0, sl->joints + 0 * 64, 128);
                memcpy(ms->meshlet_skins[j].j1, sl->joints + 1 * 64, 128);
                memcpy(ms->meshlet_skins[j].j2, sl->joints + 2 * 64, 128);
                memcpy(ms->meshlet_skins[j].j3, sl->joints + 3 * 64, 128);
                memcpy(ms->meshlet_skins[j].w0, sl->weights + 0 * 64, 64);
                memcpy(ms->meshlet_skins[j].w1, sl->weights + 1 * 64, 64);
                memcpy(ms->meshlet_skins[j].w2, sl->weights + 2 * 64, 64);
                memcpy(ms->meshlet_skins[j].w3, sl->weights + 3 * 64, 64);
                ms->culling_bone_inds[j] = sl->culling_bone;
            }
#if SFT_SIMD_WIDTH == 8
            memcpy(ms->inds[j].inds, sl->inds, 512);
#else
            /* the blob holds the AVX2 build's swizzle (batches of 8 triangles: v0 x8, v1 x8, v2 x8,
             * pad x8); the NEON build's batches are SFT_SIMD_WIDTH triangles wide (sofren2.c:2419-2438) */
            for (u32 t = 0; t < 128; t++)
                for (u32 v = 0; v < 4; v++)
                    ms->inds[j].inds[(t / SFT_SIMD_WIDTH) * SFT_SIMD_WIDTH * 4 + v * SFT_SIMD_WIDTH + t % SFT_SIMD_WIDTH] =
                        sl->inds[(t / 8) * 32 + v * 8 + t % 8];
#endif
            for (int q = 0; q < 8; q++) (*fields[q])[j] = sl->cull[q];
            m->meshlet_mesh_inds[off + j] = (u16)k;
        }
        ms->material = (sm->material >= 0) ? mats[sm->material] : SFT_INVALID_HANDLE;
        ms->lightmap_page = sm->lightmap_page;
        off += n;
    }
    m->lightmap_count = src->n_lightmaps;
    m->lightmaps = (sft_tex_handle*)calloc(src->n_lightmaps + 1, sizeof(sft_tex_handle));
    for (u32 i = 0; i < src->n_lightmaps; i++) m->lightmaps[i] = texs[src->lightmaps[i]];
    m->shadow_proxy_count = src->n_proxies;
    m->shadow_proxies = (struct sft_shadow_proxy*)calloc(src->n_proxies + 1, sizeof(struct sft_shadow_proxy));
    for (u32 i = 0; i < src->n_proxies; i++) {
        const sfts_proxy* p = &src->proxies[i];
        m->shadow_proxies[i].posa = SFT_V(p->posa[0], p->posa[1], p->posa[2]);
        m->shadow_proxies[i].posb = SFT_V(p->posb[0], p->posb[1], p->posb[2]);
        m->shadow_proxies[i].radius = p->radius;
        m->shadow_proxies[i].bone_ind = p->bone;
    }
    m->skeleton.bone_count = (i32)src->bone_count;
    m->skeleton.bones = (struct sft_bone*)calloc(src->bone_count + 1, sizeof(struct sft_bone));
    sft__blas_build_model(m, arena);
    (void)sc;
    return m;
}

static void dump_frame(sfts_dump* d, u32 w, u32 h, const u32* color) {
    const i32 cols = sft_state->display.tile_cols, rows = sft_state->display.tile_rows;
    const i32 tiles = cols * rows;
    sfts_dump_section(d, "color", "u32", color, (u64)w * h * 4);

    /* tile payload lists, in chunk-list order */
    i32* counts = (i32*)calloc(tiles, sizeof(i32));
    u64 total = 0;
    for (i32 t = 0; t < tiles; t++) {
        for (i32 ci = sft_state->display.tile_heads[t]; ci != -1; ci = sft_state->display.chunk_pool[ci].next_ind) {
            for (i32 i = 0; i < 31; i++) {
                if (sft_state->display.chunk_pool[ci].payloads[i] == ~0ull) break;
                counts[t]++;
            }
        }
        total += (u64)counts[t];
    }
    u64* payloads = (u64*)malloc((total + 1) * sizeof(u64));
    u64 k = 0;
    for (i32 t = 0; t < tiles; t++)
        for (i32 ci = sft_state->display.tile_heads[t]; ci != -1; ci = sft_state->display.chunk_pool[ci].next_ind)
            for (i32 i = 0; i < 31; i++) {
                const u64 p = sft_state->display.chunk_pool[ci].payloads[i];
                if (p == ~0ull) break;
                payloads[k++] = p;
            }
    sfts_dump_section(d, "tile_counts", "i32", counts, (u64)tiles * 4);
    sfts_dump_section(d, "tile_payloads", "u64", payloads, total * 8);

    /* visibility buffer: replay the reference raster over each tile's list */
    const u64 per_tile = (u64)SFT_TILE_PIXELS * SFT_AA_SAMPLES;
    f32* depth_all = (f32*)malloc(per_tile * tiles * 4);
    u32* vid_all = (u32*)malloc(per_tile * tiles * 4);
    alignas(32) const f32 x_offsets_arr[8] = {0.f, 1.f, 2.f, 3.f, 4.f, 5.f, 6.f, 7.f};
    const vf32 v_x_step = sft_vf_load(x_offsets_arr);
    const vf32 v_zero = sft_vf_setzero();
    alignas(64) static f32 depth_buf[SFT_TILE_PIXELS * SFT_AA_SAMPLES];
    alignas(64) static u32 vid_buf[SFT_TILE_PIXELS * SFT_AA_SAMPLES];
    for (i32 t = 0; t < tiles; t++) {
        const i32 tile_min_x = (t % cols) * SFT_TILE_SIZE, tile_min_y = (t / cols) * SFT_TILE_SIZE;
        memset(depth_buf, 0, sizeof(depth_buf));
        memset(vid_buf, 0xFF, sizeof(vid_buf));
        const vf32 v_tmin_x = sft_vf_set1((f32)tile_min_x);
        const vf32 v_tmax_x = sft_vf_set1((f32)(tile_min_x + SFT_TILE_SIZE - 1));
        const vf32 v_tmin_y = sft_vf_set1((f32)tile_min_y);
        const vf32 v_tmax_y = sft_vf_set1((f32)(tile_min_y + SFT_TILE_SIZE - 1));
        for (i32 ci = sft_state->display.tile_heads[t]; ci != -1; ci = sft_state->display.chunk_pool[ci].next_ind)
            for (i32 i = 0; i < 31; i++) {
                const u64 p = sft_state->display.chunk_pool[ci].payloads[i];
                if (p == ~0ull) break;
                sft__rast_simd_batch(p, depth_buf, vid_buf, tile_min_x, tile_min_y,
                                     v_x_step, v_zero, v_tmin_x, v_tmax_x, v_tmin_y, v_tmax_y);
            }
        memcpy(depth_all + per_tile * t, depth_buf, per_tile * 4);
        memcpy(vid_all + per_tile * t, vid_buf, per_tile * 4);
    }
    sfts_dump_section(d, "depth", "f32", depth_all, per_tile * tiles * 4);
    sfts_dump_section(d, "vid", "u32", vid_all, per_tile * tiles * 4);

    const u64 n_ss = (u64)sft_state->cmd_queue.total_ss_meshlets.count;
    sfts_dump_section(d, "ss_cache", "f32", sft_state->ss_cache, n_ss * sizeof(struct sft_ss_meshlet));
    const i32 n_clip = sft_state->clip_cache.count;
    sfts_dump_section(d, "clip", "f32", sft_state->clip_cache.pool, (u64)(n_clip > 0 ? n_clip : 0) * sizeof(struct sft_clipped_triangle));

    const i32 n_prox = sft_state->shadows.proxy_count.count;
    u8* vis = (u8*)calloc((size_t)(n_prox > 0 ? n_prox : 1) * 64, 1);
    for (i32 p = 0; p < n_prox; p++) memcpy(vis + 64 * p, sft_state->shadows.proxies[p].light_vis, 64);
    sfts_dump_section(d, "light_vis", "u8", vis, (u64)(n_prox > 0 ? n_prox : 0) * 64);
    f32* wprox = (f32*)calloc((size_t)(n_prox > 0 ? n_prox : 1) * 7, sizeof(f32));
    for (i32 p = 0; p < n_prox; p++) {
        const struct sft_world_shadow_proxy* w = &sft_state->shadows.proxies[p];
        f32 v[7] = { w->posa.x, w->posa.y, w->posa.z, w->posb.x, w->posb.y, w->posb.z, w->radius };
        memcpy(wprox + 7 * p, v, sizeof(v));
    }
    sfts_dump_section(d, "world_proxies", "f32", wprox, (u64)(n_prox > 0 ? n_prox : 0) * 28);
    const u32 tlas_n = sft_state->cmd_queue.instance_count.count ? sft_state->cmd_queue.tlas_node_count : 0;
    sfts_dump_section(d, "tlas", "u8", sft_state->cmd_queue.tlas_nodes, (u64)tlas_n * sizeof(struct sft_bvh_node));
    free(counts); free(payloads); free(depth_all); free(vid_all); free(vis); free(wprox);
}

int main(int argc, char** argv) {
    if (argc < 3) { fprintf(stderr, "usage: %s scene.sfts out.dump [frame=-1] [threads=1] [repeat=1]\n", argv[0]); return 2; }
    const int only_frame = argc > 3 ? atoi(argv[3]) : -1;
    const int threads = argc > 4 ? atoi(argv[4]) : 1;
    const int repeat = argc > 5 ? atoi(argv[5]) : 1;
    sfts_scene sc;
    const int rc = sfts_load_file(&sc, argv[1]);
    if (rc) { fprintf(stderr, "cannot parse scene (%d)\n", rc); return 3; }
    if (!sc.n_frames) return 4;

    sft_init((i32)sc.frames[0].width, (i32)sc.frames[0].height, threads);
    if (getenv("SFT_DEBUG_MODE")) sft_set_debug_mode((enum sft_debug_mode)atoi(getenv("SFT_DEBUG_MODE")));
    sft_tex_handle* texs = (sft_tex_handle*)calloc(sc.n_textures + 1, sizeof(sft_tex_handle));
    for (u32 i = 0; i < sc.n_textures; i++) texs[i] = sft_texture_create((i32)sc.textures[i].w, (i32)sc.textures[i].h, sc.textures[i].argb);
    sft_mat_handle* mats = (sft_mat_handle*)calloc(sc.n_materials + 1, sizeof(sft_mat_handle));
    for (u32 i = 0; i < sc.n_materials; i++)
        mats[i] = sft_material_create(sc.materials[i].tex >= 0 ? texs[sc.materials[i].tex] : SFT_INVALID_HANDLE,
                                      sc.materials[i].base_color, sc.materials[i].shininess);
    sft_arena model_arena;
    sft_arena_init(&model_arena, 4ull << 30);
    sft_model** models = (sft_model**)calloc(sc.n_models + 1, sizeof(sft_model*));
    for (u32 i = 0; i < sc.n_models; i++) models[i] = build_model(&sc, &sc.models[i], mats, texs, &model_arena);

    if (getenv("SFT_RAYCAST")) {
        /* ray query mode: sft_raycast_instance for each 96-byte ray record of the file named by
         * SFT_RAYCAST (transform[16], origin[3], dir[3], max_dist, model); writes 32-byte hit
         * records (hit, distance, pos[3], normal[3]) to the output path, and renders nothing */
        FILE* rf = fopen(getenv("SFT_RAYCAST"), "rb");
        FILE* of = fopen(argv[2], "wb");
        if (!rf || !of) return 5;
        struct { f32 T[16]; f32 o[3], dir[3]; f32 max_dist; i32 model; } ray;
        while (fread(&ray, sizeof(ray), 1, rf) == 1) {
            if (ray.model < 0 || (u32)ray.model >= sc.n_models) return 6;
            sft_instance inst;
            memset(&inst, 0, sizeof(inst));
            inst.model = models[ray.model];
            memcpy(&inst.transform, ray.T, 64);
            const sft_ray_hit hit = sft_raycast_instance(&inst, SFT_V(ray.o[0], ray.o[1], ray.o[2]),
                                                         SFT_V(ray.dir[0], ray.dir[1], ray.dir[2]), ray.max_dist);
            u32 out[8] = { 0 };
            out[0] = hit.hit ? 1u : 0u;
            memcpy(&out[1], &hit.distance, 4);
            memcpy(&out[2], &hit.pos, 12);
            memcpy(&out[5], &hit.normal, 12);
            fwrite(out, 4, 8, of);
        }
        fclose(rf); fclose(of);
        return 0;
    }
    sfts_dump d = { fopen(argv[2], "wb") };
    if (!d.f) return 5;
    for (u32 i = 0; i < sc.n_models; i++)
        sfts_dump_section(&d, "blas", "u8", models[i]->blas_nodes, (u64)models[i]->blas_node_count * sizeof(struct sft_bvh_node));
    u32 cur_w = sc.frames[0].width, cur_h = sc.frames[0].height;
    u32* color = NULL;
    for (u32 fi = 0; fi < sc.n_frames; fi++) {
        if (only_frame >= 0 && (u32)only_frame != fi) continue;
        const sfts_frame* f = &sc.frames[fi];
        if (f->width != cur_w || f->height != cur_h) { sft_resize((i32)f->width, (i32)f->height); cur_w = f->width; cur_h = f->height; }
        free(color);
        color = (u32*)aalloc((size_t)f->width * f->height * 4);
        sftmat* bones_store = NULL;
        uint64_t best = ~0ull;
        FILE* times = getenv("SFT_TIMES") ? fopen(getenv("SFT_TIMES"), "ab") : NULL;
        const uint64_t budget_ns = getenv("SFT_TIME_BUDGET_MS") ? (uint64_t)atoll(getenv("SFT_TIME_BUDGET_MS")) * 1000000ull : 0;
        const uint64_t rep_start = now_ns();
        for (int rep = 0; rep < repeat; rep++) {
            if (budget_ns && rep >= 3 && now_ns() - rep_start > budget_ns) break;   /* timing runs only */
            const uint64_t tf0 = now_ns();
            sft_set_ambient_light(f->ambient[0], f->ambient[1], f->ambient[2]);
            for (u32 l = 0; l < f->n_dir; l++)
                sft_draw_directional_light(SFT_V(f->dir[l].dir[0], f->dir[l].dir[1], f->dir[l].dir[2]), f->dir[l].r, f->dir[l].g, f->dir[l].b, f->dir[l].intensity);
            for (u32 l = 0; l < f->n_point; l++)
                sft_draw_point_light(SFT_V(f->point[l].pos[0], f->point[l].pos[1], f->point[l].pos[2]), f->point[l].r, f->point[l].g,
                                     f->point[l].b, f->point[l].intensity, f->point[l].radius, l);
            sft_set_shadows_enabled((u8)f->shadows);
            sft_set_lightmap_brightness(f->lightmap_brightness);
            sft_set_clear((u8)f->clear);
            sft_set_clear_color(f->clear_color);
            sft_set_color_buffer(color, (i32)(f->width * 4));
            sft_frame_begin();
            sftvec cam = SFT_V(f->cam_pos[0], f->cam_pos[1], f->cam_pos[2]);
            sftmat view, projm;
            memcpy(&view, f->view, 64); memcpy(&projm, f->proj, 64);
            sft_set_camera(cam, view, projm);
            u32 nb_total = 0;
            for (u32 k = 0; k < f->n_inst; k++) nb_total += f->inst[k].n_bones;
            free(bones_store);
            bones_store = (sftmat*)aalloc((nb_total + 1) * sizeof(sftmat));
            u32 nb = 0;
            for (u32 k = 0; k < f->n_inst; k++) {
                sft_instance inst;
                memset(&inst, 0, sizeof(inst));
                inst.model = models[f->inst[k].model];
                memcpy(&inst.transform, f->inst[k].transform, 64);
                if (f->inst[k].n_bones) {
                    memcpy(bones_store + nb, f->inst[k].bones, 64u * f->inst[k].n_bones);
                    inst.posed_bone_matrices = bones_store + nb;
                    nb += f->inst[k].n_bones;
                }
                sft_draw_instance(&inst);
            }
            /* mark the screen-space cache so culled meshlets stay recognisable (0xFF) */
            const u64 ss_bytes = (u64)sft_state->cmd_queue.total_ss_meshlets.count * sizeof(struct sft_ss_meshlet);
            if (!getenv("SFT_NO_DUMP")) memset(sft_state->scratch_arena.base, 0xFF, ss_bytes + 64);
            const uint64_t t0 = now_ns();
            sft_present();
            const uint64_t t1 = now_ns();
            if (t1 - t0 < best) best = t1 - t0;
            if (times) { const uint64_t fns = t1 - tf0; fwrite(&fns, 8, 1, times); }
            if (rep + 1 == repeat && !getenv("SFT_NO_DUMP")) {
                dump_frame(&d, f->width, f->height, color);
                const uint64_t ns = best;
                sfts_dump_section(&d, "present_ns", "u64", &ns, 8);
            }
            sft_frame_end();
        }
        if (times) fclose(times);
        free(bones_store);
    }
    fclose(d.f);
    return 0;
}
