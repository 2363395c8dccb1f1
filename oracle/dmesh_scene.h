/*
 * Test infrastructure: a scene drawn only with the dynamic-mesh API (sft_dmesh_*, sft_draw_cube,
 * _cube_inv, _sphere, _capsule, _cylinder; sofren2.c:8480-8951), written once against the
 * public sft_* API so that the same calls run on the reference (oracle/dmesh_harness.c) and on
 * this library (tests/dmesh_frame.c).  Camera and transforms avoid libm transcendental calls;
 * the shape generators themselves use sinf / cosf as the reference does.
 */
#ifndef SFT_DMESH_SCENE_H
#define SFT_DMESH_SCENE_H

#define DMESH_SCENE_FRAMES 3

static sft_mat_handle dms_mat[4];

static void dmesh_scene_setup(void) {
    static u32 px[64 * 64];
    for (int y = 0; y < 64; y++)
        for (int x = 0; x < 64; x++) {
            const u32 r = (u32)((x * 37 + y * 11) & 255), g = (u32)((x * 5 + y * 29) & 255), b = (u32)(((x ^ y) * 9) & 255);
            px[y * 64 + x] = 0xFF000000u | (r << 16) | (g << 8) | b;
        }
    const sft_tex_handle t = sft_texture_create(64, 64, px);
    dms_mat[0] = sft_material_create(t, 0xFFFFFFFFu, 16.f);
    dms_mat[1] = sft_material_create(SFT_INVALID_HANDLE, 0xFF60A0E0u, 32.f);
    dms_mat[2] = sft_material_create(t, 0xFFFFC080u, -1.5f);   /* emissive */
    dms_mat[3] = sft_material_create(t, 0xFFFFFFFFu, 4.f);
}

static sftmat dms_tr(f32 x, f32 y, f32 z, f32 s) { return sft_m_mul(sft_m_scale(s, s, s), sft_m_translate(x, y, z)); }

static void dmesh_scene_frame(int f, u32* color, int w, int h) {
    sft_set_ambient_light(0.12f, 0.12f, 0.14f);
    sft_draw_directional_light(SFT_V(0.3f, -1.f, 0.4f), 0.9f, 0.85f, 0.8f, 0.6f);
    sft_draw_point_light(SFT_V(-1.5f, 3.f, 1.f), 1.f, 0.8f, 0.6f, 1.2f, 9.f, 0);
    sft_draw_point_light(SFT_V(2.f, 2.5f, 4.f), 0.5f, 0.7f, 1.f, 1.f, 7.f, 1);
    sft_set_shadows_enabled(1);
    sft_set_clear(1);
    sft_set_clear_color(0xFF202830u);
    sft_set_color_buffer(color, w * 4);
    sft_frame_begin();
    const sftvec cam = SFT_V(0.4f * (f32)f - 0.4f, 2.2f, -5.5f);
    sftmat proj;   /* 60 degree vertical fov, near 0.1, far 100, aspect 16:9 */
    memset(&proj, 0, sizeof(proj));
    proj.m[0][0] = 0.97427857f; proj.m[1][1] = 1.7320508f; proj.m[2][2] = 100.f / 99.9f;
    proj.m[3][2] = (-100.f * 0.1f) / 99.9f; proj.m[2][3] = 1.f;
    sft_set_camera(cam, sft_m_view_look_at(cam, SFT_V(0.f, 0.6f, 2.5f), SFT_V(0.f, 1.f, 0.f)), proj);

    sft_dmesh* dm = sft_dmesh_begin(SFT_DMESH_QUADS, dms_mat[0], 6);
    sft_draw_cube(dm);
    const sftmat t0 = dms_tr(-2.2f, 0.5f + 0.1f * (f32)f, 2.f, 1.f);
    sft_dmesh_end(dm, &t0);

    dm = sft_dmesh_begin(SFT_DMESH_QUADS, dms_mat[3], 6);
    sft_draw_cube_inv(dm);
    const sftmat troom = dms_tr(0.f, 2.5f, 3.f, 9.f);
    sft_dmesh_end(dm, &troom);

    dm = sft_dmesh_begin(SFT_DMESH_QUADS, dms_mat[0], 9 * 16);
    sft_draw_sphere(dm, 8, 16);
    const sftmat t1 = dms_tr(0.f, 1.f, 3.f, 1.2f);
    sft_dmesh_end(dm, &t1);

    dm = sft_dmesh_begin(SFT_DMESH_QUADS, dms_mat[1], 2 * 4 * 12 + 12);
    sft_draw_capsule(dm, SFT_V(1.5f, 0.2f, 2.f), SFT_V(2.4f, 1.5f, 3.f), 0.3f, 12, 4);
    sft_dmesh_end(dm, NULL);

    dm = sft_dmesh_begin(SFT_DMESH_QUADS, dms_mat[2], 3 * 10);
    sft_draw_cylinder(dm, SFT_V(-1.f, 0.f, 4.f), SFT_V(-0.6f, 1.8f, 4.3f), 0.4f, 0.2f, 10);
    sft_dmesh_end(dm, NULL);

    /* a ground of quads with four normals, through alloc_quads, and a strip of triangles */
    dm = sft_dmesh_begin(SFT_DMESH_QUADS, dms_mat[3], 100);
    sft_dmesh_qb qb;
    u32 done = 0;
    while (done < 100 && sft_dmesh_alloc_quads(dm, 100 - done, &qb)) {
        for (u32 q = 0; q < qb.allocated_count; q++) {
            const u32 k = done + q, gx = k % 10, gz = k / 10;
            const f32 x0 = -3.f + 0.6f * (f32)gx, z0 = 0.f + 0.6f * (f32)gz;
            const u32 v = qb.vert_offset + 4 * q;
            const f32 X[4] = { x0, x0, x0 + 0.6f, x0 + 0.6f }, Z[4] = { z0, z0 + 0.6f, z0 + 0.6f, z0 };
            for (int c = 0; c < 4; c++) {
                qb.x[v + c] = X[c]; qb.y[v + c] = 0.f; qb.z[v + c] = Z[c];
                qb.nx[v + c] = 0.f; qb.ny[v + c] = 1.f; qb.nz[v + c] = 0.f;
                qb.u[v + c] = X[c] * 0.5f; qb.v[v + c] = Z[c] * 0.5f;
            }
        }
        done += qb.allocated_count;
    }
    sft_dmesh_end(dm, NULL);

    dm = sft_dmesh_begin(SFT_DMESH_TRIANGLES, dms_mat[1], 30);
    for (int k = 0; k < 30; k++) {
        const f32 x = -2.5f + 0.17f * (f32)k, y = 2.f + 0.05f * (f32)(k % 5);
        sft_dmesh_push_tri(dm, SFT_V(x, y, 5.f), SFT_V(x + 0.15f, y + 0.3f, 5.1f), SFT_V(x + 0.3f, y, 5.f),
                           0.f, 0.f, 0.5f, 1.f, 1.f, 0.f, SFT_V(0.f, 0.f, -1.f));
    }
    sft_dmesh_end(dm, NULL);

    dm = sft_dmesh_begin(SFT_DMESH_QUADS, dms_mat[0], 2);   /* more quads than reserved: the rest are dropped */
    for (int k = 0; k < 40; k++)
        sft_dmesh_push_quad_4n(dm, SFT_V(1.f + 0.1f * k, 2.5f, 1.f), SFT_V(1.f + 0.1f * k, 2.8f, 1.f), SFT_V(1.08f + 0.1f * k, 2.8f, 1.f),
                               SFT_V(1.08f + 0.1f * k, 2.5f, 1.f), 0.f, 0.f, 1.f, 1.f, SFT_V(0.f, 0.f, -1.f), SFT_V(0.f, 0.7f, -0.7f),
                               SFT_V(0.7f, 0.f, -0.7f), SFT_V(0.f, 0.f, -1.f));
    sft_dmesh_end(dm, NULL);

    sft_present();
    sft_frame_end();
}

#endif
