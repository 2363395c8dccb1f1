/*
 * Test infrastructure: a scene whose geometry comes from a QSF2 file through
 * sft_model_load_qsf (sofren2.c:7816-7967), written once against the public sft_* API so that
 * the same calls run on the reference (oracle/qsf_harness.c) and on this library
 * (tests/qsf_frame.c).  Two instances of the loaded model (the second turned a quarter and
 * raised), lit by point and directional lights with the model's lightmap page, seen from a
 * camera that moves per frame.
 */
#ifndef SFT_QSF_SCENE_H
#define SFT_QSF_SCENE_H

#define QSF_SCENE_FRAMES 3

static sft_model* qsf_model;

static int qsf_scene_setup(const char* path, sft_arena* arena) {
    qsf_model = sft_model_load_qsf(path, arena);
    return qsf_model != NULL;
}

static void qsf_scene_frame(int f, u32* color, int w, int h) {
    sft_set_ambient_light(0.1f, 0.1f, 0.12f);
    sft_draw_directional_light(SFT_V(0.2f, -1.f, 0.5f), 0.8f, 0.8f, 0.75f, 0.5f);
    sft_draw_point_light(SFT_V(-2.f, 4.f, 6.f), 1.f, 0.8f, 0.6f, 1.f, 30.f, 0);
    sft_draw_point_light(SFT_V(3.f, 5.f, 10.f), 0.5f, 0.7f, 1.f, 1.f, 25.f, 1);
    sft_set_lightmap_brightness(0.8f + 0.1f * (f32)f);
    sft_set_shadows_enabled(1);
    sft_set_clear(1);
    sft_set_clear_color(0xFF101418u);
    sft_set_color_buffer(color, w * 4);
    sft_frame_begin();
    const sftvec cam = SFT_V(0.5f * (f32)f - 0.5f, 1.7f + 0.3f * (f32)f, 0.5f);
    sftmat proj;   /* 60 degree vertical fov, near 0.1, far 100, aspect 16:9 */
    memset(&proj, 0, sizeof(proj));
    proj.m[0][0] = 0.97427857f; proj.m[1][1] = 1.7320508f; proj.m[2][2] = 100.f / 99.9f;
    proj.m[3][2] = (-100.f * 0.1f) / 99.9f; proj.m[2][3] = 1.f;
    sft_set_camera(cam, sft_m_view_look_at(cam, SFT_V(0.f, 3.f, 12.f), SFT_V(0.f, 1.f, 0.f)), proj);
    sft_instance a;
    memset(&a, 0, sizeof(a));
    a.model = qsf_model;
    a.transform = sft_m_identity();
    sft_draw_instance(&a);
    sft_instance b = a;
    memset(&b.transform, 0, sizeof(b.transform));   /* a quarter turn about y, raised and pushed back */
    b.transform.m[0][2] = -1.f; b.transform.m[1][1] = 1.f; b.transform.m[2][0] = 1.f; b.transform.m[3][3] = 1.f;
    b.transform.m[3][0] = -6.f; b.transform.m[3][1] = 0.5f; b.transform.m[3][2] = 30.f;
    sft_draw_instance(&b);
    sft_present();
    sft_frame_end();
}

#endif
