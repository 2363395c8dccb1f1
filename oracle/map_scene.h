/*
 * Test infrastructure: the frame loop of the reference's viewer (main.c:259-426) over a QSF2 map
 * (the reference's own res/simple.qsf and res/simpleb.qsf), written once against the public
 * sft_* API so that the same calls run on the reference (oracle/qsf_harness.c) and on this
 * library (tests/qsf_frame.c).  As main.c: the map and its game lights (the file's game-data
 * section, attenuation doubled on load and halved at draw), ambient 0.35, lightmap brightness
 * 1.5, shadows and clear on, a 70 degree projection (constants precomputed, so that no libm
 * call differs between hosts).  Four cameras: the viewer's start (0, 2, 0) looking along +z and
 * -x, and two looking at lights of the maps.  map_scene_rays then casts a cube map of rays from two points through
 * sft_raycast_instance.
 */
#ifndef SFT_MAP_SCENE_H
#define SFT_MAP_SCENE_H

#define MAP_SCENE_FRAMES 4
#define MAP_RAY_GRID 16
#define MAP_RAYS (2 * 6 * MAP_RAY_GRID * MAP_RAY_GRID)

static sft_model* map_model;
static struct { u32 type; f32 pos[3]; f32 color[3]; f32 intensity; f32 attenuation; } map_lights[64];
static i32 map_light_count;

static int map_scene_setup(const char* path, sft_arena* arena) {
    map_model = sft_model_load_qsf(path, arena);
    if (!map_model) return 0;
    FILE* f = fopen(path, "rb");
    if (!f) return 0;
    u64 off = 0;
    map_light_count = 0;
    if (fseek(f, 8, SEEK_SET) == 0 && fread(&off, 8, 1, f) == 1 && fseek(f, (long)off, SEEK_SET) == 0 &&
        fread(&map_light_count, 4, 1, f) == 1) {
        if (map_light_count < 0) map_light_count = 0;
        if (map_light_count > 63) map_light_count = 63;
        if (fread(map_lights, sizeof(map_lights[0]), (size_t)map_light_count, f) != (size_t)map_light_count) map_light_count = 0;
        for (i32 i = 0; i < map_light_count; i++) map_lights[i].attenuation *= 2.f;
    }
    fclose(f);
    return 1;
}

static void map_scene_frame(int fr, u32* color, int w, int h) {
    sft_set_clear(1);
    sft_set_shadows_enabled(1);
    sft_set_lightmap_brightness(1.5f);
    sft_set_ambient_light(0.35f, 0.35f, 0.35f);
    if (map_light_count) {
        for (i32 i = 0; i < map_light_count; i++)
            sft_draw_point_light(SFT_V(map_lights[i].pos[0], map_lights[i].pos[1], map_lights[i].pos[2]), map_lights[i].color[0],
                                 map_lights[i].color[1], map_lights[i].color[2], 1.f, map_lights[i].attenuation / 2.f, (u32)i + 1);
    } else {
        sft_draw_directional_light(sft_v_norm(SFT_V(1.f, 0.5f, 0.f)), 1.f, 1.f, 1.f, 0.8f);
    }
    sft_set_color_buffer(color, w * 4);
    sft_frame_begin();
    static const f32 at[MAP_SCENE_FRAMES][6] = {   /* camera position, target */
        { 0.f, 2.f, 0.f, 0.f, 2.f, 1.f }, { 0.f, 2.f, 0.f, -1.f, 2.f, 0.f },
        { -3.f, 4.f, 2.f, -3.25f, 6.f, -10.25f }, { -2.f, 3.f, 8.f, 2.75f, 2.75f, 20.25f } };
    const f32* c = at[fr % MAP_SCENE_FRAMES];
    const sftvec cam = SFT_V(c[0], c[1], c[2]), tgt = SFT_V(c[3], c[4], c[5]);
    sftmat proj;   /* sft_m_proj(70, 16/9, 0.1, 1000) */
    memset(&proj, 0, sizeof(proj));
    proj.m[0][0] = 0x1.9b4e7ap-1f * (1600.f / 900.f) / ((f32)w / (f32)h);
    proj.m[1][1] = 0x1.6d9b18p+0f; proj.m[2][2] = 0x1.00068ep+0f; proj.m[3][2] = -0x1.99a416p-4f; proj.m[2][3] = 1.f;
    sft_set_camera(cam, sft_m_view_look_at(cam, tgt, SFT_V(0.f, 1.f, 0.f)), proj);
    sft_instance inst;
    memset(&inst, 0, sizeof(inst));
    inst.model = map_model;
    inst.transform = sft_m_identity();
    sft_draw_instance(&inst);
    sft_present();
    sft_frame_end();
}

/* MAP_RAYS hits, 8 words each (hit, distance, pos[3], normal[3]): from (0, 2, 0) and (-6, 4, 5),
 * a 16x16 grid over each face of a cube around the origin point */
static void map_scene_rays(u32* out) {
    static const f32 org[2][3] = { { 0.f, 2.f, 0.f }, { -6.f, 4.f, 5.f } };
    sft_instance inst;
    memset(&inst, 0, sizeof(inst));
    inst.model = map_model;
    inst.transform = sft_m_identity();
    u32 k = 0;
    for (int o = 0; o < 2; o++)
        for (int face = 0; face < 6; face++)
            for (int j = 0; j < MAP_RAY_GRID; j++)
                for (int i = 0; i < MAP_RAY_GRID; i++, k++) {
                    const f32 a = ((f32)i - 7.5f) / 8.f, b = ((f32)j - 7.5f) / 8.f, s = (face & 1) ? -1.f : 1.f;
                    const sftvec d = face < 2 ? SFT_V(s, a, b) : face < 4 ? SFT_V(a, s, b) : SFT_V(a, b, s);
                    const sft_ray_hit hit = sft_raycast_instance(&inst, SFT_V(org[o][0], org[o][1], org[o][2]), d, 500.f);
                    u32* r = out + (size_t)k * 8;
                    memset(r, 0, 32);
                    r[0] = hit.hit ? 1u : 0u;
                    memcpy(&r[1], &hit.distance, 4);
                    memcpy(&r[2], &hit.pos, 12);
                    memcpy(&r[5], &hit.normal, 12);
                }
}

#endif
