/*
 * Test infrastructure: runs the unmodified reference's load-time builders on raw triangle meshes
 * and dumps what they made: the meshlets its GLB loader builds (sofren2.c:7467-7660, with the
 * reference's own sft__builder_reset / _score_candidate / _add_triangle and
 * sft__builder_finalize_attribs, 6918-7045, Welzl spheres 2255-2289), the BLAS
 * (sft__blas_build_model, 3526) and the shadow proxies (sft__generate_shadow_proxies, 3509).
 * The loop that drives the builder lives inside sft_model_load_glb, which needs cgltf; it is
 * restated here step for step around the reference's helpers.  Built by oracle/Makefile from the
 * reference sources where they lie.  The product side is include/sofren2.h's
 * sft_mesh_build_meshlets / sft_model_fit_shadow_proxies; tests/model_build.c reads the same
 * input and writes the same layout.
 *
 * input  "SFTR" u32 version(1) u32 seed i32 proxy_budget u32 n_bones {i32 parent f32 bind[3]}
 *        u32 n_meshes {u32 nv u32 nt u32 skinned f32 pos[nv*3] f32 nrm[nv*3] f32 uv[nv*2]
 *        [u16 joints[nv*4] u8 weights[nv*4]] i32 inds[nt*3]}
 * output per mesh: u32 n f32 attr[n*640] u8 inds[n*512] f32 cull[n*8] [u16 joints[n*256]
 *        u8 weights[n*256] i32 culling_bones[n]]; then u32 n_proxies {f32 posa[3] posb[3] radius
 *        u32 bone}; then u32 blas_count u32 blas_root and the node images (256 B each)
 *
 * usage: build_harness <in.bin> <out.bin>
 *        build_harness_{1x,4x} render <out.bin> <ground.bin> <shapes.bin> <humanoid.bin>
 *        (the frames of oracle/build_scene.h over the three models, colour per frame)
 */
#define _GNU_SOURCE
#define SFT_IMPL
#define SFT_NO_DEBUG
#include "sofren2.c"

/* zeroed and 64-byte aligned, as the reference's arenas give (its SIMD loads need 32) */
static void* zalloc(size_t n) { const size_t m = (n + 63) & ~(size_t)63; void* q = aligned_alloc(64, m ? m : 64); memset(q, 0, m ? m : 64); return q; }

static const unsigned char* rd(const unsigned char** p, size_t n) { const unsigned char* r = *p; *p += n; return r; }
static u32 rd32(const unsigned char** p) { u32 v; memcpy(&v, rd(p, 4), 4); return v; }

/* the reference's build of one input file: meshlets per mesh (their material `mat`), BLAS, proxies */
static sft_model* ref_build(const char* path, sft_mat_handle mat, u32** skinned_out) {
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END); const long fsz = ftell(f); fseek(f, 0, SEEK_SET);
    unsigned char* blob = (unsigned char*)malloc((size_t)fsz + 16);
    if (fread(blob, 1, (size_t)fsz, f) != (size_t)fsz) { fclose(f); return NULL; }
    fclose(f);
    const unsigned char* p = blob;
    if (memcmp(rd(&p, 4), "SFTR", 4) || rd32(&p) != 1) return NULL;
    const u32 seed = rd32(&p);
    const i32 budget = (i32)rd32(&p);
    const u32 nb = rd32(&p);
    sft_model* model = (sft_model*)calloc(1, sizeof(sft_model));
    model->skeleton.bone_count = (i32)nb;
    model->skeleton.bones = (struct sft_bone*)calloc(nb + 1, sizeof(struct sft_bone));
    for (u32 b = 0; b < nb; b++) {
        model->skeleton.bones[b].parent_ind = (i32)rd32(&p);
        f32 bp[3]; memcpy(bp, rd(&p, 12), 12);
        model->skeleton.bones[b].bind_pos = SFT_V(bp[0], bp[1], bp[2]);
    }
    const u32 nm = rd32(&p);
    model->meshes = (sft_mesh*)calloc(nm + 1, sizeof(sft_mesh));
    model->mesh_count = nm;
    u32* skinned_of = (u32*)calloc(nm + 1, 4);
    static sft_arena arena;
    static int arena_ready;
    if (!arena_ready) { sft_arena_init(&arena, 8ull << 30); arena_ready = 1; }
    srand(seed);
    for (u32 mi = 0; mi < nm; mi++) {
        const u32 nv = rd32(&p), nt = rd32(&p), skinned = rd32(&p);
        skinned_of[mi] = skinned;
        const f32* pos = (const f32*)rd(&p, (size_t)nv * 12);
        const f32* nrm = (const f32*)rd(&p, (size_t)nv * 12);
        const f32* uv = (const f32*)rd(&p, (size_t)nv * 8);
        const u16* jn = skinned ? (const u16*)rd(&p, (size_t)nv * 8) : NULL;
        const u8* wt = skinned ? rd(&p, (size_t)nv * 4) : NULL;
        const i32* uni_inds = (const i32*)rd(&p, (size_t)nt * 12);
        /* the loader's SoA vertex streams (sofren2.c:7426-7507) */
        f32 *vx = malloc(nv * 4 + 4), *vy = malloc(nv * 4 + 4), *vz = malloc(nv * 4 + 4), *nx = malloc(nv * 4 + 4), *ny = malloc(nv * 4 + 4),
            *nz = malloc(nv * 4 + 4), *uu = malloc(nv * 4 + 4), *vv = malloc(nv * 4 + 4);
        u16 *j0 = calloc(nv + 1, 2), *j1 = calloc(nv + 1, 2), *j2 = calloc(nv + 1, 2), *j3 = calloc(nv + 1, 2);
        u8 *w0 = calloc(nv + 1, 1), *w1 = calloc(nv + 1, 1), *w2 = calloc(nv + 1, 1), *w3 = calloc(nv + 1, 1);
        for (u32 v = 0; v < nv; v++) {
            vx[v] = pos[v * 3]; vy[v] = pos[v * 3 + 1]; vz[v] = pos[v * 3 + 2];
            nx[v] = nrm[v * 3]; ny[v] = nrm[v * 3 + 1]; nz[v] = nrm[v * 3 + 2];
            uu[v] = uv[v * 2]; vv[v] = uv[v * 2 + 1];
            if (skinned) {
                j0[v] = jn[v * 4]; j1[v] = jn[v * 4 + 1]; j2[v] = jn[v * 4 + 2]; j3[v] = jn[v * 4 + 3];
                w0[v] = wt[v * 4]; w1[v] = wt[v * 4 + 1]; w2[v] = wt[v * 4 + 2]; w3[v] = wt[v * 4 + 3];
            }
        }
        const i32 total_tris = (i32)nt, total_verts = (i32)nv;
        sft_mesh* out_mesh = &model->meshes[mi];
        out_mesh->material = mat;
        out_mesh->lightmap_page = 0xFFFFFFFF;
        /* adjacency (sofren2.c:7467-7492) */
        i32* vertex_offsets = calloc(total_verts + 1, 4);
        i32* adjacency = calloc(total_tris * 3 + 1, 4);
        i32* write_heads = calloc(total_verts + 1, 4);
        for (i32 k = 0; k < total_tris * 3; k++) vertex_offsets[uni_inds[k]] += 1;
        i32 prefix = 0;
        for (i32 k = 0; k < total_verts; k++) { const i32 c = vertex_offsets[k]; vertex_offsets[k] = prefix; prefix += c; }
        vertex_offsets[total_verts] = prefix;
        memcpy(write_heads, vertex_offsets, total_verts * sizeof(i32));
        for (i32 k = 0; k < total_tris; k++)
            for (i32 v = 0; v < 3; v++) adjacency[write_heads[uni_inds[k * 3 + v]]++] = k;
        const i32 max_meshlets = total_tris + 8;
        out_mesh->meshlets = zalloc(max_meshlets * sizeof(struct sft_meshlet));
        out_mesh->meshlet_attribs = zalloc(max_meshlets * sizeof(struct sft_meshlet_attribs));
        out_mesh->inds = zalloc(max_meshlets * sizeof(struct sft_meshlet_inds));
        f32** fields[14] = { &out_mesh->bounds_center_x, &out_mesh->bounds_center_y, &out_mesh->bounds_center_z, &out_mesh->bounds_radius,
                             &out_mesh->bounds_min_x, &out_mesh->bounds_min_y, &out_mesh->bounds_min_z, &out_mesh->bounds_max_x,
                             &out_mesh->bounds_max_y, &out_mesh->bounds_max_z, &out_mesh->cone_axis_x, &out_mesh->cone_axis_y,
                             &out_mesh->cone_axis_z, &out_mesh->cone_cutoff };
        for (int q = 0; q < 14; q++) *fields[q] = zalloc((size_t)max_meshlets * 4);
        out_mesh->meshlet_skins = skinned ? zalloc(max_meshlets * sizeof(struct sft_meshlet_skin)) : NULL;
        out_mesh->culling_bone_inds = skinned ? zalloc((size_t)max_meshlets * 4) : NULL;
        i32* scratch_weights = (i32*)malloc((nb + 1) * sizeof(i32));
        struct sft_raw_geometry raw_data = { .vx = vx, .vy = vy, .vz = vz, .nx = nx, .ny = ny, .nz = nz, .u = uu, .v = vv,
                                             .j0 = j0, .j1 = j1, .j2 = j2, .j3 = j3, .w0 = w0, .w1 = w1, .w2 = w2, .w3 = w3 };
        u8* used_tris = calloc(total_tris + 1, 1);
        u8* in_frontier = calloc(total_tris + 1, 1);
        i32* frontier = calloc(total_tris + 1, 4);
        i32 unmapped_tris = total_tris;
        u32 meshlet_count = 0;
        struct sft_meshlet_builder builder;
        i32 linear_search_head = 0;
        /* the loader's meshlet loop (sofren2.c:7529-7655) */
        while (unmapped_tris > 0) {
            sft__builder_reset(&builder);
            i32 frontier_head = 0, frontier_tail = 0;
            while (builder.vert_count < SFT_VERTS_PER_MESHLET && builder.tri_count < 128 && unmapped_tris > 0) {
                if (frontier_head == frontier_tail) {
                    i32 jump_seed = -1;
                    for (i32 k = linear_search_head; k < total_tris; k++)
                        if (!used_tris[k]) { jump_seed = linear_search_head = k; break; }
                    if (-1 == jump_seed) break;
                    const i32 v0 = uni_inds[jump_seed * 3], v1 = uni_inds[jump_seed * 3 + 1], v2 = uni_inds[jump_seed * 3 + 2];
                    const sftvec normal = sft_v_face_normal(SFT_V(vx[v0], vy[v0], vz[v0]), SFT_V(vx[v1], vy[v1], vz[v1]), SFT_V(vx[v2], vy[v2], vz[v2]));
                    if (builder.tri_count > 0 && sft__builder_score_candidate(&builder, v0, v1, v2, normal) < 0.f) break;
                    sft__builder_add_triangle(&builder, v0, v1, v2, normal);
                    used_tris[jump_seed] = 1;
                    unmapped_tris -= 1;
                    const i32 nvts[3] = { v0, v1, v2 };
                    for (i32 v = 0; v < 3; v++)
                        for (i32 a = vertex_offsets[nvts[v]]; a < vertex_offsets[nvts[v] + 1]; a++) {
                            const i32 t = adjacency[a];
                            if (!used_tris[t] && !in_frontier[t]) { frontier[frontier_tail++] = t; in_frontier[t] = 1; }
                        }
                    continue;
                }
                f32 best_score = -1.f;
                i32 best_tri_ind = -1;
                sftvec best_normal = { 0 };
                for (i32 k = frontier_head; k < frontier_tail; k++) {
                    const i32 c = frontier[k];
                    if (used_tris[c]) continue;
                    const i32 c0 = uni_inds[c * 3], c1 = uni_inds[c * 3 + 1], c2 = uni_inds[c * 3 + 2];
                    const sftvec cn = sft_v_face_normal(SFT_V(vx[c0], vy[c0], vz[c0]), SFT_V(vx[c1], vy[c1], vz[c1]), SFT_V(vx[c2], vy[c2], vz[c2]));
                    const f32 score = sft__builder_score_candidate(&builder, c0, c1, c2, cn);
                    if (score > best_score) { best_score = score; best_tri_ind = k; best_normal = cn; }
                }
                if (-1 == best_tri_ind) { frontier_head = frontier_tail = 0; continue; }
                const i32 bt = frontier[best_tri_ind];
                const i32 b0 = uni_inds[bt * 3], b1 = uni_inds[bt * 3 + 1], b2 = uni_inds[bt * 3 + 2];
                sft__builder_add_triangle(&builder, b0, b1, b2, best_normal);
                used_tris[bt] = 1;
                unmapped_tris -= 1;
                frontier[best_tri_ind] = frontier[frontier_head++];
                const i32 nvts[3] = { b0, b1, b2 };
                for (i32 v = 0; v < 3; v++)
                    for (i32 a = vertex_offsets[nvts[v]]; a < vertex_offsets[nvts[v] + 1]; a++) {
                        const i32 t = adjacency[a];
                        if (!used_tris[t] && !in_frontier[t]) { frontier[frontier_tail++] = t; in_frontier[t] = 1; }
                    }
            }
            for (i32 k = frontier_head; k < frontier_tail; k++) in_frontier[frontier[k]] = 0;
            struct sft_sphere sphere = { 0 };
            struct sft_aabb aabb = { 0 };
            struct sft_meshlet_output out_ptrs = { .verts = &out_mesh->meshlets[meshlet_count], .attribs = &out_mesh->meshlet_attribs[meshlet_count],
                                                   .inds = &out_mesh->inds[meshlet_count],
                                                   .skin = skinned ? &out_mesh->meshlet_skins[meshlet_count] : NULL,
                                                   .culling_bone = skinned ? &out_mesh->culling_bone_inds[meshlet_count] : NULL,
                                                   .sphere = &sphere, .aabb = &aabb };
            sft__builder_finalize_attribs(&builder, &raw_data, nb, scratch_weights, &out_ptrs);
            out_mesh->bounds_center_x[meshlet_count] = sphere.center.x; out_mesh->bounds_center_y[meshlet_count] = sphere.center.y;
            out_mesh->bounds_center_z[meshlet_count] = sphere.center.z; out_mesh->bounds_radius[meshlet_count] = sphere.radius;
            out_mesh->bounds_min_x[meshlet_count] = aabb.min.x; out_mesh->bounds_min_y[meshlet_count] = aabb.min.y;
            out_mesh->bounds_min_z[meshlet_count] = aabb.min.z; out_mesh->bounds_max_x[meshlet_count] = aabb.max.x;
            out_mesh->bounds_max_y[meshlet_count] = aabb.max.y; out_mesh->bounds_max_z[meshlet_count] = aabb.max.z;
            const sftvec true_axis = sft_v_norm(builder.cone_axis);
            f32 min_dot = 1.f;
            const struct sft_meshlet* ml = &out_mesh->meshlets[meshlet_count];
            for (u32 t = 0; t < builder.tri_count; t++) {
                const u8 a0 = builder.local_inds[t * 3], a1 = builder.local_inds[t * 3 + 1], a2 = builder.local_inds[t * 3 + 2];
                const sftvec n = sft_v_face_normal(SFT_V(ml->x[a0], ml->y[a0], ml->z[a0]), SFT_V(ml->x[a1], ml->y[a1], ml->z[a1]),
                                                   SFT_V(ml->x[a2], ml->y[a2], ml->z[a2]));
                const f32 d = sft_v_dot(n, true_axis);
                if (d < min_dot) min_dot = d;
            }
            const f32 sin_alpha = (min_dot < 0.f) ? 1.f : sqrtf(1.f - min_dot * min_dot);
            out_mesh->cone_axis_x[meshlet_count] = true_axis.x; out_mesh->cone_axis_y[meshlet_count] = true_axis.y;
            out_mesh->cone_axis_z[meshlet_count] = true_axis.z; out_mesh->cone_cutoff[meshlet_count] = sin_alpha + 0.02f;
            meshlet_count += 1;
        }
        out_mesh->meshlet_count = meshlet_count;
    }
    model->total_meshlets = 0;
    for (u32 i = 0; i < nm; i++) { model->meshes[i].model_meshlet_offset = model->total_meshlets; model->total_meshlets += model->meshes[i].meshlet_count; }
    model->meshlet_mesh_inds = (u16*)zalloc((size_t)(model->total_meshlets + 8) * 2);
    for (u32 i = 0; i < nm; i++)
        for (u32 j = 0; j < model->meshes[i].meshlet_count; j++) model->meshlet_mesh_inds[model->meshes[i].model_meshlet_offset + j] = (u16)i;
    if (model->total_meshlets > 0) sft__blas_build_model(model, &arena);
    sft__generate_shadow_proxies(model, &arena, budget);

    *skinned_out = skinned_of;
    return model;
}

#ifdef BUILD_SCENE_RENDER
#include "build_scene.h"
#endif

int main(int argc, char** argv) {
#ifdef BUILD_SCENE_RENDER
    /* render <out.bin> <ground.bin> <shapes.bin> <humanoid.bin>: the frames of build_scene.h over
     * the three models, built by the reference with the scene's material */
    if (argc >= 6 && !strcmp(argv[1], "render")) {
        const int w = BUILD_SCENE_W, h = BUILD_SCENE_H;
        sft_init(w, h, 1);
        const sft_mat_handle mat = build_scene_material();
        u32* sk;
        sft_model* ms[3];
        for (int k = 0; k < 3; k++) if (!(ms[k] = ref_build(argv[3 + k], mat, &sk))) return 3;
        u32* color = (u32*)calloc((size_t)w * h, 4);
        FILE* out = fopen(argv[2], "wb");
        if (!out) return 5;
        for (int fi = 0; fi < BUILD_SCENE_FRAMES; fi++) {
            build_scene_frame(fi, ms[0], ms[1], ms[2], color, w, h);
            fwrite(color, 4, (size_t)w * h, out);
        }
        fclose(out);
        return 0;
    }
#endif
    if (argc < 3) { fprintf(stderr, "usage: %s in.bin out.bin | render out.bin ground.bin shapes.bin humanoid.bin\n", argv[0]); return 2; }
    u32* skinned_of = NULL;
    sft_model* model = ref_build(argv[1], SFT_INVALID_HANDLE, &skinned_of);
    if (!model) return 3;
    const u32 nm = model->mesh_count;
    FILE* o = fopen(argv[2], "wb");
    if (!o) return 5;
    for (u32 mi = 0; mi < nm; mi++) {
        const sft_mesh* m = &model->meshes[mi];
        const u32 n = m->meshlet_count;
        fwrite(&n, 4, 1, o);
        for (u32 j = 0; j < n; j++) {
            const struct sft_meshlet* v = &m->meshlets[j];
            const struct sft_meshlet_attribs* a = &m->meshlet_attribs[j];
            fwrite(v->x, 4, 64, o); fwrite(v->y, 4, 64, o); fwrite(v->z, 4, 64, o);
            fwrite(a->nx, 4, 64, o); fwrite(a->ny, 4, 64, o); fwrite(a->nz, 4, 64, o);
            fwrite(a->u, 4, 64, o); fwrite(a->v, 4, 64, o); fwrite(a->lu, 4, 64, o); fwrite(a->lv, 4, 64, o);
        }
        for (u32 j = 0; j < n; j++) fwrite(m->inds[j].inds, 1, 512, o);
        for (u32 j = 0; j < n; j++) {
            const f32 c[8] = { m->bounds_center_x[j], m->bounds_center_y[j], m->bounds_center_z[j], m->bounds_radius[j],
                               m->cone_axis_x[j], m->cone_axis_y[j], m->cone_axis_z[j], m->cone_cutoff[j] };
            fwrite(c, 4, 8, o);
        }
        if (skinned_of[mi]) {
            for (u32 j = 0; j < n; j++) {
                const struct sft_meshlet_skin* s = &m->meshlet_skins[j];
                fwrite(s->j0, 2, 64, o); fwrite(s->j1, 2, 64, o); fwrite(s->j2, 2, 64, o); fwrite(s->j3, 2, 64, o);
            }
            for (u32 j = 0; j < n; j++) {
                const struct sft_meshlet_skin* s = &m->meshlet_skins[j];
                fwrite(s->w0, 1, 64, o); fwrite(s->w1, 1, 64, o); fwrite(s->w2, 1, 64, o); fwrite(s->w3, 1, 64, o);
            }
            fwrite(m->culling_bone_inds, 4, n, o);
        }
    }
    const u32 np = model->shadow_proxy_count;
    fwrite(&np, 4, 1, o);
    for (u32 i = 0; i < np; i++) {
        const struct sft_shadow_proxy* q = &model->shadow_proxies[i];
        const f32 v[7] = { q->posa.x, q->posa.y, q->posa.z, q->posb.x, q->posb.y, q->posb.z, q->radius };
        fwrite(v, 4, 7, o); fwrite(&q->bone_ind, 4, 1, o);
    }
    const u32 bc = model->blas_node_count, br = model->blas_root_ind;
    fwrite(&bc, 4, 1, o); fwrite(&br, 4, 1, o);
    if (bc) fwrite(model->blas_nodes, sizeof(struct sft_bvh_node), bc, o);
    fclose(o);
    return 0;
}
