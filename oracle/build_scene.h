/*
 * Test infrastructure: frames drawn through the public sft_* API over three models made by the
 * load-time builders from raw triangles (a ground grid, static shapes, a skinned humanoid with
 * its fitted shadow proxies), written once so that the same calls run on the reference
 * (oracle/build_harness.c, whose models come from the reference's own builders) and on this
 * library (tests/model_build_frame.c, models from sft_model_build).  Two humanoids in their bind
 * pose stand on the ground beside the shapes, lit by two shadowing point lights.
 */
#ifndef SFT_BUILD_SCENE_H
#define SFT_BUILD_SCENE_H

#define BUILD_SCENE_FRAMES 2
#define BUILD_SCENE_W 640
#define BUILD_SCENE_H 360

/* a 64x64 texture of hashed 8x8 cells and the material every built mesh uses */
static sft_mat_handle build_scene_material(void) {
    static u32 tex[64 * 64];
    for (int y = 0; y < 64; y++)
        for (int x = 0; x < 64; x++) {
            u32 hsh = (u32)((x >> 3) * 73856093) ^ (u32)((y >> 3) * 19349663);
            hsh ^= hsh >> 13; hsh *= 0x5bd1e995u; hsh ^= hsh >> 15;
            tex[y * 64 + x] = 0xFF000000u | (hsh & 0x00FFFFFFu) | 0x00404040u;
        }
    return sft_material_create(sft_texture_create(64, 64, tex), 0xFFFFFFFFu, 16.f);
}

static void build_scene_frame(int f, sft_model* ground, sft_model* shapes, sft_model* hum, u32* color, int w, int h) {
    static sftmat bind[64];
    for (int b = 0; b < 64; b++) bind[b] = sft_m_identity();
    sft_set_ambient_light(0.12f, 0.12f, 0.14f);
    sft_draw_point_light(SFT_V(-2.f, 4.f, 1.f), 1.f, 0.9f, 0.8f, 1.f, 14.f, 0);
    sft_draw_point_light(SFT_V(3.f, 3.5f, 5.f + (f32)f), 0.6f, 0.7f, 1.f, 1.f, 12.f, 1);
    sft_set_shadows_enabled(1);
    sft_set_clear(1);
    sft_set_clear_color(0xFF1A1E24u);
    sft_set_color_buffer(color, w * 4);
    sft_frame_begin();
    const sftvec cam = SFT_V(0.6f * (f32)f, 2.2f, -3.5f);
    sftmat proj;   /* 60 degree vertical fov, near 0.1, far 100, aspect 16:9 */
    memset(&proj, 0, sizeof(proj));
    proj.m[0][0] = 0.97427857f; proj.m[1][1] = 1.7320508f; proj.m[2][2] = 100.f / 99.9f;
    proj.m[3][2] = (-100.f * 0.1f) / 99.9f; proj.m[2][3] = 1.f;
    sft_set_camera(cam, sft_m_view_look_at(cam, SFT_V(0.f, 1.f, 3.f), SFT_V(0.f, 1.f, 0.f)), proj);
    sft_instance in;
    memset(&in, 0, sizeof(in));
    in.model = ground; in.transform = sft_m_identity();
    sft_draw_instance(&in);
    in.model = shapes; in.transform = sft_m_mul(sft_m_rot_y(0.4f), sft_m_translate(1.5f, 0.f, 4.f));
    sft_draw_instance(&in);
    in.model = hum; in.posed_bone_matrices = bind;
    in.transform = sft_m_translate(-0.8f, 0.f, 2.f);
    sft_draw_instance(&in);
    in.transform = sft_m_mul(sft_m_rot_y(2.5f), sft_m_translate(0.6f, 0.f, 2.8f));
    sft_draw_instance(&in);
    sft_present();
    sft_frame_end();
}

#endif
