/*
 * sofren2 per-frame render path: CPU ORACLE (test infrastructure only).
 *
 * A portable scalar restatement of the reference's AVX2 path (sofren2.c), used as the
 * oracle that the CUDA implementation is tested against and as the "port" CPU baseline.  It is not part of
 * the shipped library and the library never links or calls it.
 *
 * Parity anchor: the restatement is pinned against the unmodified reference compiled
 * here (oracle/_ref, built by oracle/Makefile) on the committed golden fixtures
 * (tests/golden); tests/test_oracle.py checks it bit-for-bit.
 *
 * What it emulates exactly:
 *   - 8-wide AVX2 lane semantics: _mm256_min_ps/max_ps operand order (a<b?a:b), truncating
 *     conversions with the 0x80000000 "integer indefinite" result, FMA where the reference
 *     uses fmadd/fmsub/fnmadd intrinsics and separate roundings everywhere else
 *     (the reference is pinned with -ffp-contract=off);
 *   - RCPPS/RSQRTPS through tables measured on the reference CPU (x86_approx_tables.h);
 *   - the 4x2 pixel block of the resolve, including block-level skips that change results
 *     (first-lane LOD, the per-proxy block skip before the smooth-max blend).
 * Single-threaded: tile payload order equals the reference's one-worker order.
 *
 * Each function names the reference lines it follows.
 */
#define _GNU_SOURCE
#include "sfts_blob.h"
#include "x86_approx_tables.h"

#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int32_t i32; typedef uint32_t u32; typedef uint64_t u64; typedef uint8_t u8; typedef uint16_t u16;
typedef float f32;

#define EPS 1e-6f
#define TILE 64
#define TILE_PX 4096
#define INVALID 0xFFFFFFFFu

/* ------------------------------------------------------------ lane primitives */
static const u32 RCP_T[2048] = SFT_X86_RCP_TABLE_INIT;
static const u32 RSQ_T[2048] = SFT_X86_RSQRT_TABLE_INIT;

static inline u32 f2u(f32 f) { u32 u; memcpy(&u, &f, 4); return u; }
static inline f32 u2f(u32 u) { f32 f; memcpy(&f, &u, 4); return f; }

/* RCPPS (sofren2.c:289) */
static f32 x86_rcp(f32 xf) {
    const u32 x = f2u(xf), s = x & 0x80000000u, e = (x >> 23) & 0xFF, m = x & 0x7FFFFF;
    if (e == 0xFF) return u2f(m ? (x | 0x00400000u) : s);
    if (e == 0) return u2f(s | 0x7F800000u);
    if (e >= 253) return u2f(s);
    return u2f(s | ((253u - e) << 23) | RCP_T[m >> 12]);
}
/* RSQRTPS (sofren2.c:296) */
static f32 x86_rsqrt(f32 xf) {
    const u32 x = f2u(xf), s = x & 0x80000000u, e = (x >> 23) & 0xFF, m = x & 0x7FFFFF;
    if (e == 0xFF) { if (m) return u2f(x | 0x00400000u); return u2f(s ? 0xFFC00000u : 0u); }
    if (e == 0) return u2f(s | 0x7F800000u);
    if (s) return u2f(0xFFC00000u);
    const u32 t = RSQ_T[(e & 1) * 1024 + (m >> 13)];
    const i32 oe = ((380 - (i32)e) >> 1) + (i32)(t >> 23) - 1;
    return u2f(((u32)oe << 23) | (t & 0x7FFFFF));
}
/* sft_vf_rcp_refined (sofren2.c:633-638): approx * (2 - a*approx) with a fused fnmadd */
static inline f32 rcpr(f32 a) { const f32 r = x86_rcp(a); return r * fmaf(-a, r, 2.f); }
/* NaN bits as the reference leaves them in memory on x86: every NaN of the render path comes from
 * an invalid operation (0 * inf in rcpr's fnmadd for w = +-0), whose SSE/AVX result is the default
 * NaN 0xFFC00000, passed through unchanged by later mul/add/fma.  aarch64 produces 0x7FC00000 for the
 * same operation, so floats stored to compared buffers go through this map on every host. */
static inline f32 x86nan(f32 v) { return v != v ? u2f(0xFFC00000u) : v; }
static inline f32 vmin(f32 a, f32 b) { return a < b ? a : b; }   /* _mm256_min_ps(a, b) */
static inline f32 vmax(f32 a, f32 b) { return a > b ? a : b; }   /* _mm256_max_ps(a, b) */
/* _mm256_cvttps_epi32: truncation, 0x80000000 when out of range or NaN */
static inline i32 cvtt(f32 x) { return (x >= -2147483648.f && x < 2147483648.f) ? (i32)x : INT32_MIN; }
static inline i32 ctz32(u32 m) { return __builtin_ctz(m); }

typedef struct { f32 x, y, z; } vec3;
typedef struct { f32 m[4][4]; } mat4;

static inline f32 vdot(vec3 a, vec3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }  /* sft_vv_dot (1942) */
static inline vec3 vsub(vec3 a, vec3 b) { vec3 r = { a.x - b.x, a.y - b.y, a.z - b.z }; return r; }
static inline vec3 vadd(vec3 a, vec3 b) { vec3 r = { a.x + b.x, a.y + b.y, a.z + b.z }; return r; }
static inline vec3 vscale(vec3 a, f32 s) { vec3 r = { a.x * s, a.y * s, a.z * s }; return r; }
/* sft_vv_transform (1993-2012): z first, then y, then x, fused */
static inline vec3 xform(vec3 v, const mat4* m) {
    vec3 r;
    r.x = fmaf(v.x, m->m[0][0], fmaf(v.y, m->m[1][0], fmaf(v.z, m->m[2][0], m->m[3][0])));
    r.y = fmaf(v.x, m->m[0][1], fmaf(v.y, m->m[1][1], fmaf(v.z, m->m[2][1], m->m[3][1])));
    r.z = fmaf(v.x, m->m[0][2], fmaf(v.y, m->m[1][2], fmaf(v.z, m->m[2][2], m->m[3][2])));
    return r;
}
/* sft_vv_transform_dir (2013-2030) */
static inline vec3 xform_dir(vec3 v, const mat4* m) {
    vec3 r;
    r.x = fmaf(v.x, m->m[0][0], fmaf(v.y, m->m[1][0], v.z * m->m[2][0]));
    r.y = fmaf(v.x, m->m[0][1], fmaf(v.y, m->m[1][1], v.z * m->m[2][1]));
    r.z = fmaf(v.x, m->m[0][2], fmaf(v.y, m->m[1][2], v.z * m->m[2][2]));
    return r;
}
/* sft_vv_norm (1961-1971) */
static inline vec3 vnorm(vec3 v) {
    f32 len = sqrtf(vdot(v, v));
    len = vmax(len, EPS);
    vec3 r = { v.x / len, v.y / len, v.z / len };
    return r;
}
/* sft_vv_norm_fast (1973-1992) */
static inline vec3 vnorm_fast(vec3 v) {
    const f32 sq = vdot(v, v);
    const f32 a = x86_rsqrt(sq);
    const f32 refined = (0.5f * a) * fmaf(-sq, a * a, 3.f);
    vec3 r = { v.x * refined, v.y * refined, v.z * refined };
    return r;
}

/* ------------------------------------------------------------ scalar math (host side, no FMA) */
static inline f32 sdot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }   /* sft_v_dot (1532) */
static inline vec3 snorm(vec3 v) {                                                       /* sft_v_norm (1548) */
    const f32 l = sqrtf(sdot(v, v));
    if (l > EPS) return vscale(v, 1.f / l);
    vec3 z = { 0, 0, 0 }; return z;
}
static inline vec3 scross(vec3 a, vec3 b) {
    vec3 r = { a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x }; return r;
}
static mat4 mmul(const mat4* a, const mat4* b) {                                          /* sft_m_mul (1668) */
    mat4 r;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            r.m[i][j] = a->m[i][0] * b->m[0][j] + a->m[i][1] * b->m[1][j] + a->m[i][2] * b->m[2][j] + a->m[i][3] * b->m[3][j];
    return r;
}

/* ------------------------------------------------------------ textures (sft_texture_create 9181-9310) */
typedef struct {
    i32 w, h, levels, is_pot;
    u32* texels;                 /* all levels, 4x4 block-linear, each padded to 4x4 */
    u32 offs[14]; i32 bw[14], shift[14];
} otex;

static i32 ilog2(u32 v) { return 31 - __builtin_clz(v); }

static void tex_create(otex* t, i32 w, i32 h, const u32* px) {
    memset(t, 0, sizeof(*t));
    t->w = w; t->h = h;
    t->is_pot = (0 == (w & (w - 1))) && (0 == (h & (h - 1)));
    i32 cw = w, ch = h; u64 total = 0; i32 lv = 0;
    while (lv < 14) {
        total += (u64)(((cw + 3) & ~3) * ((ch + 3) & ~3));
        lv++;
        if (cw == 1 && ch == 1) break;
        cw = cw > 1 ? cw / 2 : 1; ch = ch > 1 ? ch / 2 : 1;
    }
    t->levels = lv;
    t->texels = (u32*)calloc(total + 16, 4);
    u32 cur = 0;
    const u32* src = px; u32* tmp = NULL;
    cw = w; ch = h;
    for (i32 l = 0; l < lv; l++) {
        if (l > 0) {   /* 4x4 tent, weights 1-2-2-1, clamped taps, integer division (9261-9290) */
            const i32 nw = cw > 1 ? cw / 2 : 1, nh = ch > 1 ? ch / 2 : 1;
            u32* dst = (u32*)malloc((size_t)nw * nh * 4);
            for (i32 y = 0; y < nh; y++)
                for (i32 x = 0; x < nw; x++) {
                    u32 r = 0, g = 0, b = 0, a = 0, ws = 0;
                    for (i32 ky = -1; ky <= 2; ky++) {
                        i32 sy = y * 2 + ky; sy = sy < 0 ? 0 : (sy > ch - 1 ? ch - 1 : sy);
                        const u32 wy = (ky == -1 || ky == 2) ? 1 : 2;
                        for (i32 kx = -1; kx <= 2; kx++) {
                            i32 sx = x * 2 + kx; sx = sx < 0 ? 0 : (sx > cw - 1 ? cw - 1 : sx);
                            const u32 wgt = ((kx == -1 || kx == 2) ? 1 : 2) * wy;
                            const u32 c = src[sy * cw + sx];
                            r += ((c >> 16) & 255) * wgt; g += ((c >> 8) & 255) * wgt;
                            b += (c & 255) * wgt; a += ((c >> 24) & 255) * wgt; ws += wgt;
                        }
                    }
                    dst[y * nw + x] = ((a / ws) << 24) | ((r / ws) << 16) | ((g / ws) << 8) | (b / ws);
                }
            free(tmp); tmp = dst; src = dst; cw = nw; ch = nh;
        }
        const i32 pw = (cw + 3) & ~3, ph = (ch + 3) & ~3, bw = pw / 4;
        t->offs[l] = cur; t->bw[l] = bw; t->shift[l] = t->is_pot ? ilog2((u32)bw) : 0;
        for (i32 y = 0; y < ch; y++)
            for (i32 x = 0; x < cw; x++)
                t->texels[cur + (u32)(((y / 4) * bw + x / 4) * 16 + (y % 4) * 4 + (x % 4))] = src[y * cw + x];
        cur += (u32)(pw * ph);
    }
    free(tmp);
}

/* sft__sample_tex_bilinear (5543-5660) for one lane */
static void sample_bilinear(const otex* t, i32 lod, f32 cu, f32 cv, f32* r, f32* g, f32* b) {
    if (!t) { *r = *g = *b = 1.f; return; }
    const i32 w = (t->w >> lod) > 1 ? (t->w >> lod) : 1, h = (t->h >> lod) > 1 ? (t->h >> lod) : 1;
    const f32 upx = cu * (f32)w - 0.5f, vpx = cv * (f32)h - 0.5f;
    const f32 uf0 = floorf(upx), vf0 = floorf(vpx);
    const f32 ufr = upx - uf0, vfr = vpx - vf0;
    const i32 u0 = cvtt(uf0), v0 = cvtt(vf0);
    const i32 wm = w - 1, hm = h - 1;
    i32 u0w, v0w, u1, v1;
    if (t->is_pot) { u1 = (u0 + 1) & wm; v1 = (v0 + 1) & hm; u0w = u0 & wm; v0w = v0 & hm; }
    else {   /* the reference has no lower clamp here (reads outside the texture); clamp at 0 */
        u1 = (u0 + 1) < wm ? u0 + 1 : wm; v1 = (v0 + 1) < hm ? v0 + 1 : hm; u0w = u0 < wm ? u0 : wm; v0w = v0 < hm ? v0 : hm;
        u1 = u1 < 0 ? 0 : u1; v1 = v1 < 0 ? 0 : v1; u0w = u0w < 0 ? 0 : u0w; v0w = v0w < 0 ? 0 : v0w;
    }
    const u32* base = t->texels + t->offs[lod];
#define ADDR(ux, vy) (t->is_pot ? ((((((u32)(vy) >> 2) << t->shift[lod]) + ((u32)(ux) >> 2)) << 4) + (((u32)(vy) & 3) << 2) + ((u32)(ux) & 3)) \
                               : ((((((u32)(vy) >> 2) * (u32)t->bw[lod]) + ((u32)(ux) >> 2)) << 4) + (((u32)(vy) & 3) << 2) + ((u32)(ux) & 3)))
    const u32 c00 = base[ADDR(u0w, v0w)], c10 = base[ADDR(u1, v0w)], c01 = base[ADDR(u0w, v1)], c11 = base[ADDR(u1, v1)];
#undef ADDR
    const f32 i255 = 1.f / 255.f;
    f32 out[3];
    for (int k = 0; k < 3; k++) {
        const int sh = 16 - 8 * k;
        const f32 f00 = (f32)((c00 >> sh) & 255) * i255, f10 = (f32)((c10 >> sh) & 255) * i255;
        const f32 f01 = (f32)((c01 >> sh) & 255) * i255, f11 = (f32)((c11 >> sh) & 255) * i255;
        const f32 top = f00 + (f10 - f00) * ufr, bot = f01 + (f11 - f01) * ufr;
        out[k] = top + (bot - top) * vfr;
    }
    *r = out[0]; *g = out[1]; *b = out[2];
}

/* sft__sample_tex_nearest (5662-5729) */
static void sample_nearest(const otex* t, i32 lod, f32 cu, f32 cv, f32* r, f32* g, f32* b) {
    if (!t) { *r = *g = *b = 1.f; return; }
    const i32 w = (t->w >> lod) > 1 ? (t->w >> lod) : 1, h = (t->h >> lod) > 1 ? (t->h >> lod) : 1;
    const i32 u0 = cvtt(floorf(cu * (f32)w)), v0 = cvtt(floorf(cv * (f32)h));
    const i32 wm = w - 1, hm = h - 1;
    i32 uw, vw;
    if (t->is_pot) { uw = u0 & wm; vw = v0 & hm; } else { uw = u0 < wm ? u0 : wm; vw = v0 < hm ? v0 : hm; uw = uw < 0 ? 0 : uw; vw = vw < 0 ? 0 : vw; }
    u32 a;
    if (t->is_pot) a = (((((u32)vw >> 2) << t->shift[lod]) + ((u32)uw >> 2)) << 4) + (((u32)vw & 3) << 2) + ((u32)uw & 3);
    else a = (((((u32)vw >> 2) * (u32)t->bw[lod]) + ((u32)uw >> 2)) << 4) + (((u32)vw & 3) << 2) + ((u32)uw & 3);
    const u32 c = t->texels[t->offs[lod] + a];
    const f32 i255 = 1.f / 255.f;
    *r = (f32)((c >> 16) & 255) * i255; *g = (f32)((c >> 8) & 255) * i255; *b = (f32)(c & 255) * i255;
}

/* ------------------------------------------------------------ scene state */
typedef struct { i32 tex; u32 base; f32 shin; } omat;

typedef struct {
    u32 first_meshlet;  /* model-relative meshlet offset of this mesh */
    const sfts_mesh* src;
} omesh;

typedef struct {
    const sfts_model* src;
    omesh* meshes;
    u32 total;
    u16* mesh_of;       /* model meshlet -> mesh */
    const sfts_meshlet** ml;   /* model meshlet -> data */
    u8* blas; u32 blas_count, blas_root;   /* sft_bvh_node images, 256 B each */
} omodel;

/* sft_bvh_node (sofren2.c:967-983), x86-64 layout */
typedef struct {
    f32 mn[3][8]; f32 mx[3][8];
    u32 child[8]; u8 count; u8 leaf; u8 pad[30];
} onode;

typedef struct { u32 id; f32 mn[3], mx[3]; f32 c[3]; } obuild;   /* sft_blas_build_item */

/* sft__sort_build_items (2895-2924): quicksort with the middle element as pivot */
static void qsort_items(obuild* it, i32 count, int axis) {
    if (count <= 1) return;
    const f32 pivot = it[count / 2].c[axis];
    i32 i = 0, j = count - 1;
    while (i <= j) {
        while (it[i].c[axis] < pivot) i++;
        while (it[j].c[axis] > pivot) j--;
        if (i <= j) { obuild t = it[i]; it[i] = it[j]; it[j] = t; i++; j--; }
    }
    if (j > 0) qsort_items(it, j + 1, axis);
    if (i < count) qsort_items(it + i, count - i, axis);
}

/* sft__partition_to_8 (2926-2965) */
static void part8(obuild* it, u32 start, u32 count, u32 depth, u32* st, u32* cn, u32* ng) {
    if (!count) return;
    if (depth == 3 || count == 1) { st[*ng] = start; cn[*ng] = count; (*ng)++; return; }
    f32 mn[3] = { 1e30f, 1e30f, 1e30f }, mx[3] = { -1e30f, -1e30f, -1e30f };
    for (u32 i = 0; i < count; i++)
        for (int a = 0; a < 3; a++) {
            if (it[start + i].c[a] < mn[a]) mn[a] = it[start + i].c[a];
            if (it[start + i].c[a] > mx[a]) mx[a] = it[start + i].c[a];
        }
    const f32 dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
    const int axis = (dy > dx && dy > dz) ? 1 : (dz > dx && dz > dy) ? 2 : 0;
    qsort_items(it + start, (i32)count, axis);
    const u32 mid = count / 2;
    part8(it, start, mid, depth + 1, st, cn, ng);
    part8(it, start + mid, count - mid, depth + 1, st, cn, ng);
}

/* sft__bvh_build_recursive (2967-3062) */
static u32 bvh_build(obuild* it, u32 count, onode* nodes, u32* ncount, f32* out_mn, f32* out_mx) {
    const u32 ni = (*ncount)++;
    onode* n = &nodes[ni];
    for (int i = 0; i < 8; i++) {
        for (int a = 0; a < 3; a++) { n->mn[a][i] = 1e30f; n->mx[a][i] = -1e30f; }
        n->child[i] = INVALID;
    }
    f32 bmn[3] = { 1e30f, 1e30f, 1e30f }, bmx[3] = { -1e30f, -1e30f, -1e30f };
    if (count <= 8) {
        n->leaf = 1; n->count = (u8)count;
        for (u32 i = 0; i < count; i++) {
            for (int a = 0; a < 3; a++) {
                n->mn[a][i] = it[i].mn[a]; n->mx[a][i] = it[i].mx[a];
                if (it[i].mn[a] < bmn[a]) bmn[a] = it[i].mn[a];
                if (it[i].mx[a] > bmx[a]) bmx[a] = it[i].mx[a];
            }
            n->child[i] = 0x80000000u | it[i].id;
        }
    } else {
        n->leaf = 0;
        u32 st[8] = { 0 }, cn[8] = { 0 }, ng = 0;
        part8(it, 0, count, 0, st, cn, &ng);
        n->count = (u8)ng;
        for (u32 c = 0; c < ng; c++) {
            f32 cmn[3], cmx[3];
            const u32 ci = bvh_build(it + st[c], cn[c], nodes, ncount, cmn, cmx);
            n = &nodes[ni];
            n->child[c] = ci;
            for (int a = 0; a < 3; a++) {
                n->mn[a][c] = cmn[a]; n->mx[a][c] = cmx[a];
                if (cmn[a] < bmn[a]) bmn[a] = cmn[a];
                if (cmx[a] > bmx[a]) bmx[a] = cmx[a];
            }
        }
    }
    if (out_mn) { memcpy(out_mn, bmn, 12); memcpy(out_mx, bmx, 12); }
    return ni;
}

static const u8* tri_inds(const sfts_meshlet* ml, u32 tri, u32* i0, u32* i1, u32* i2) {
    const u32 b = tri / 8, l = tri % 8;
    *i0 = ml->inds[b * 32 + l]; *i1 = ml->inds[b * 32 + 8 + l]; *i2 = ml->inds[b * 32 + 16 + l];
    return ml->inds;
}

/* sft__blas_build_model (3526-3617) */
static void blas_build(omodel* m) {
    u32 total = 0;
    for (u32 g = 0; g < m->total; g++)
        for (u32 t = 0; t < 128; t++) { u32 a, b, c; tri_inds(m->ml[g], t, &a, &b, &c); if (!(a == b && b == c)) total++; }
    if (!total) return;
    obuild* it = (obuild*)malloc(total * sizeof(obuild));
    u32 k = 0;
    for (u32 g = 0; g < m->total; g++) {
        const f32* at = m->ml[g]->attr;
        for (u32 t = 0; t < 128; t++) {
            u32 a, b, c; tri_inds(m->ml[g], t, &a, &b, &c);
            if (a == b && b == c) continue;
            obuild* o = &it[k++];
            for (int ax = 0; ax < 3; ax++) {
                const f32 p0 = at[ax * 64 + a], p1 = at[ax * 64 + b], p2 = at[ax * 64 + c];
                o->mn[ax] = vmin(p0, vmin(p1, p2));   /* SFT_MIN(v0, SFT_MIN(v1, v2)) */
                o->mx[ax] = vmax(p0, vmax(p1, p2));
                o->c[ax] = (o->mn[ax] + o->mx[ax]) * 0.5f;
            }
            o->id = (g << 7) | t;
        }
    }
    onode* nodes = (onode*)calloc(total * 2 + 1, sizeof(onode));
    m->blas_count = 0;
    m->blas_root = bvh_build(it, total, nodes, &m->blas_count, NULL, NULL);
    m->blas = (u8*)nodes;
    free(it);
}

/* ------------------------------------------------------------ frame state */
typedef struct { vec3 posa, posb; f32 radius; u8 vis[64]; } oproxy;
typedef struct { vec3 n[6], an[6]; f32 d[6]; } ofrustum;
typedef struct {
    f32 sx[3], sy[3], iw[3], u[3], v[3], lu[3], lv[3], px[3], py[3], pz[3], nx[3], ny[3], nz[3];
    u32 inst, m;
} oclip;   /* sft_clipped_triangle (1271-1280) */
typedef struct { f32 sx[64], sy[64], iw[64], wx[64], wy[64], wz[64], wnx[64], wny[64], wnz[64]; } oss;  /* 1464-1477 */
typedef struct { u64* p; u32 n, cap; } olist;

typedef struct {
    /* scene */
    const sfts_scene* sc;
    otex* tex; u32 ntex;
    omat* mats;
    omodel* models;
    /* frame */
    i32 W, H, S;
    f32 hw, hh, vpx, vpy;
    i32 cols, rows;
    vec3 cam; mat4 vp;
    ofrustum fr;
    const sfts_frame* f;
    u32* ss_off;
    oss* ss; u32 n_ss;
    oclip* clip; u32 nclip, clipcap;
    olist* tiles;
    oproxy* prox; u32 nprox;
    onode* tlas; u32 tlas_count, tlas_root;
    u32 invalid_packets;
    f32* depth; u32* vid;        /* per tile buffers, S * 4096 each, all tiles */
    u32* color;
    mat4* inst_T; const mat4** inst_bones;
    int debug_mode;              /* enum sft_debug_mode (sofren2.c:59-67) */
    otex checker;                /* the base material's 256x256 checkerboard (sofren2.c:8062-8080) */
    int fp64;                    /* sfto_shadow_fp64: evaluate the capsule shadows in double too */
    double fp64_max, fp64_sum;   /* largest and summed |FP32 - FP64| shadow intensity */
    u64 fp64_n, fp64_big;        /* pixel x light evaluations, and those differing by more than 1e-5 */
} octx;

static void list_push(olist* l, u64 v) {
    if (l->n == l->cap) { l->cap = l->cap ? l->cap * 2 : 64; l->p = (u64*)realloc(l->p, l->cap * 8); }
    l->p[l->n++] = v;
}

/* sft_set_camera (8345-8376) */
static void set_camera(octx* c, const sfts_frame* f) {
    mat4 view, pr; memcpy(&view, f->view, 64); memcpy(&pr, f->proj, 64);
    c->cam.x = f->cam_pos[0]; c->cam.y = f->cam_pos[1]; c->cam.z = f->cam_pos[2];
    c->vp = mmul(&view, &pr);
    f32 pl[6][4];
    for (int i = 0; i < 4; i++) {
        pl[0][i] = c->vp.m[i][3] + c->vp.m[i][0]; pl[1][i] = c->vp.m[i][3] - c->vp.m[i][0];
        pl[2][i] = c->vp.m[i][3] + c->vp.m[i][1]; pl[3][i] = c->vp.m[i][3] - c->vp.m[i][1];
        pl[4][i] = c->vp.m[i][3] + c->vp.m[i][2]; pl[5][i] = c->vp.m[i][3] - c->vp.m[i][2];
    }
    for (int p = 0; p < 6; p++) {
        const f32 len = sqrtf(pl[p][0] * pl[p][0] + pl[p][1] * pl[p][1] + pl[p][2] * pl[p][2]);
        const f32 il = (len < EPS) ? EPS : 1.f / len;
        c->fr.n[p].x = pl[p][0] * il; c->fr.n[p].y = pl[p][1] * il; c->fr.n[p].z = pl[p][2] * il;
        c->fr.an[p].x = fabsf(c->fr.n[p].x); c->fr.an[p].y = fabsf(c->fr.n[p].y); c->fr.an[p].z = fabsf(c->fr.n[p].z);
        c->fr.d[p] = pl[p][3] * il;
    }
}

/* sft__tlas_build (3619-3703) */
static void tlas_build(octx* c) {
    const u32 n = c->f->n_inst;
    c->tlas_count = 0; c->tlas_root = 0;
    if (!n) return;
    obuild* it = (obuild*)calloc(n, sizeof(obuild));
    u32 valid = 0;
    for (u32 i = 0; i < n; i++) {
        const omodel* m = &c->models[c->f->inst[i].model];
        if (!m->blas_count) continue;
        const onode* root = (const onode*)(m->blas + 256u * m->blas_root);
        f32 mn[3] = { 1e30f, 1e30f, 1e30f }, mx[3] = { -1e30f, -1e30f, -1e30f };
        for (u32 k = 0; k < root->count; k++)
            for (int a = 0; a < 3; a++) {
                if (root->mn[a][k] < mn[a]) mn[a] = root->mn[a][k];
                if (root->mx[a][k] > mx[a]) mx[a] = root->mx[a][k];
            }
        const mat4* T = &c->inst_T[i];
        f32 wmn[3] = { 1e30f, 1e30f, 1e30f }, wmx[3] = { -1e30f, -1e30f, -1e30f };
        for (int k = 0; k < 8; k++) {
            const f32 cx = (k & 1) ? mx[0] : mn[0], cy = (k & 2) ? mx[1] : mn[1], cz = (k & 4) ? mx[2] : mn[2];
            f32 t[3];
            for (int a = 0; a < 3; a++) t[a] = cx * T->m[0][a] + cy * T->m[1][a] + cz * T->m[2][a] + T->m[3][a];
            for (int a = 0; a < 3; a++) { if (t[a] < wmn[a]) wmn[a] = t[a]; }
            for (int a = 0; a < 3; a++) { if (t[a] > wmx[a]) wmx[a] = t[a]; }
        }
        it[i].id = i;
        for (int a = 0; a < 3; a++) { it[i].mn[a] = wmn[a]; it[i].mx[a] = wmx[a]; it[i].c[a] = (wmn[a] + wmx[a]) * 0.5f; }
        valid++;
    }
    c->tlas = (onode*)calloc(valid * 2 + 1, sizeof(onode));
    c->tlas_root = bvh_build(it, valid, c->tlas, &c->tlas_count, NULL, NULL);
    free(it);
}

/* sft__frustum_vs_bvh_node (3906-3968): 8-bit mask of children inside all planes */
static u32 frustum_vs_node(const onode* n, const ofrustum* fr) {
    u32 inside = 0xFF;
    f32 cx[8], cy[8], cz[8], ex[8], ey[8], ez[8];
    for (int l = 0; l < 8; l++) {
        cx[l] = (n->mx[0][l] + n->mn[0][l]) * 0.5f; cy[l] = (n->mx[1][l] + n->mn[1][l]) * 0.5f; cz[l] = (n->mx[2][l] + n->mn[2][l]) * 0.5f;
        ex[l] = (n->mx[0][l] - n->mn[0][l]) * 0.5f; ey[l] = (n->mx[1][l] - n->mn[1][l]) * 0.5f; ez[l] = (n->mx[2][l] - n->mn[2][l]) * 0.5f;
    }
    for (int p = 0; p < 6; p++) {
        u32 pm = 0;
        for (int l = 0; l < 8; l++) {
            const f32 r = fmaf(fr->an[p].x, ex[l], fmaf(fr->an[p].y, ey[l], fr->an[p].z * ez[l]));
            const f32 dc = fmaf(fr->n[p].x, cx[l], fmaf(fr->n[p].y, cy[l], fr->n[p].z * cz[l]));
            const f32 dist = dc + fr->d[p];
            if (dist + r >= 0.f) pm |= 1u << l;
        }
        inside &= pm;
        if (!inside) return 0;
    }
    return inside;
}

/* sft_m_view_look_at (1737-1770) */
static mat4 view_look_at(vec3 pos, vec3 target, vec3 up) {
    const vec3 fwd = snorm(vsub(target, pos));
    if (fabsf(fwd.x) < EPS && fabsf(fwd.z) < EPS) { up.x = 0; up.y = 0; up.z = -1; }
    up = snorm(vsub(up, vscale(fwd, sdot(up, fwd))));
    const vec3 right = scross(up, fwd);
    mat4 r;
    r.m[0][0] = right.x; r.m[0][1] = up.x; r.m[0][2] = fwd.x; r.m[0][3] = 0;
    r.m[1][0] = right.y; r.m[1][1] = up.y; r.m[1][2] = fwd.y; r.m[1][3] = 0;
    r.m[2][0] = right.z; r.m[2][1] = up.z; r.m[2][2] = fwd.z; r.m[2][3] = 0;
    r.m[3][0] = -sdot(pos, right); r.m[3][1] = -sdot(pos, up); r.m[3][2] = -sdot(pos, fwd); r.m[3][3] = 1;
    return r;
}

/* sft__build_packet_frustum (3970-4084).  Returns 0 when the reference's result is undefined
 * (a cluster corner behind the light leaves side-plane fields uninitialised, 4044-4048). */
static int packet_frustum(const f32* ox, const f32* oy, const f32* oz, u32 active, vec3 lpos, f32 lrad, ofrustum* out) {
    f32 mn[3] = { 1e9f, 1e9f, 1e9f }, mx[3] = { -1e9f, -1e9f, -1e9f };
    vec3 ctr = { 0, 0, 0 }; i32 nv = 0;
    for (int i = 0; i < 8; i++) {
        if (!(active & (1u << i))) continue;
        if (ox[i] < mn[0]) mn[0] = ox[i];
        if (ox[i] > mx[0]) mx[0] = ox[i];
        if (oy[i] < mn[1]) mn[1] = oy[i];
        if (oy[i] > mx[1]) mx[1] = oy[i];
        if (oz[i] < mn[2]) mn[2] = oz[i];
        if (oz[i] > mx[2]) mx[2] = oz[i];
        ctr.x += ox[i]; ctr.y += oy[i]; ctr.z += oz[i]; nv++;
    }
    if (!nv) return 1;
    ctr.x /= (f32)nv; ctr.y /= (f32)nv; ctr.z /= (f32)nv;
    const vec3 lf0 = snorm(vsub(ctr, lpos));
    vec3 up = { 0, 1, 0 };
    if (fabsf(lf0.y) > 0.99f) { up.x = 1; up.y = 0; }
    const mat4 lv = view_look_at(lpos, ctr, up);
    f32 mnxz = 1e9f, mxxz = -1e9f, mnyz = 1e9f, mxyz = -1e9f;
    int invalid = 0;
    for (int k = 0; k < 8; k++) {
        const f32 x = (k & 1) ? mx[0] : mn[0], y = (k & 2) ? mx[1] : mn[1], z = (k & 4) ? mx[2] : mn[2];
        const f32 cxv = x * lv.m[0][0] + y * lv.m[1][0] + z * lv.m[2][0] + 1.f * lv.m[3][0];
        const f32 cyv = x * lv.m[0][1] + y * lv.m[1][1] + z * lv.m[2][1] + 1.f * lv.m[3][1];
        const f32 czv = x * lv.m[0][2] + y * lv.m[1][2] + z * lv.m[2][2] + 1.f * lv.m[3][2];
        if (czv < EPS) { invalid = 1; break; }
        if (cxv / czv < mnxz) mnxz = cxv / czv;
        if (cxv / czv > mxxz) mxxz = cxv / czv;
        if (cyv / czv < mnyz) mnyz = cyv / czv;
        if (cyv / czv > mxyz) mxyz = cyv / czv;
    }
    const vec3 lr = { lv.m[0][0], lv.m[1][0], lv.m[2][0] };
    const vec3 lu = { lv.m[0][1], lv.m[1][1], lv.m[2][1] };
    const vec3 lf = { lv.m[0][2], lv.m[1][2], lv.m[2][2] };
    if (invalid) {
        /* undefined in the reference; treated here as "side planes never cull" */
        for (int p = 0; p < 4; p++) { out->n[p].x = out->n[p].y = out->n[p].z = 0; out->an[p] = out->n[p]; out->d[p] = 1e30f; }
    } else {
        vec3 nl[4] = { { 1.f, 0.f, -mnxz }, { -1.f, 0.f, mxxz }, { 0.f, 1.f, -mnyz }, { 0.f, -1.f, mxyz } };
        for (int p = 0; p < 4; p++) {
            const vec3 q = snorm(nl[p]);
            const vec3 nw = vadd(vscale(lr, q.x), vadd(vscale(lu, q.y), vscale(lf, q.z)));
            out->n[p] = nw;
            out->d[p] = -sdot(nw, lpos) + 0.1f;
            out->an[p].x = fabsf(nw.x); out->an[p].y = fabsf(nw.y); out->an[p].z = fabsf(nw.z);
        }
    }
    out->n[4] = lf; out->d[4] = -sdot(lf, lpos) + 0.1f;
    out->an[4].x = fabsf(lf.x); out->an[4].y = fabsf(lf.y); out->an[4].z = fabsf(lf.z);
    vec3 nlf = { -lf.x, -lf.y, -lf.z };
    out->n[5] = nlf; out->d[5] = -sdot(nlf, lpos) + lrad;
    out->an[5] = out->an[4];
    return !invalid;
}

/* sft__ray_packet_vs_triangle_any_hit (3840-3904), per lane */
static u32 packet_vs_tri(vec3 v0, vec3 v1, vec3 v2, const vec3* ro, const vec3* rd, const f32* tmax, u32 active) {
    const vec3 e1 = vsub(v1, v0), e2 = vsub(v2, v0);
    u32 mask = 0; f32 a[8];
    vec3 h[8];
    for (int l = 0; l < 8; l++) {
        h[l].x = rd[l].y * e2.z - rd[l].z * e2.y;
        h[l].y = rd[l].z * e2.x - rd[l].x * e2.z;
        h[l].z = rd[l].x * e2.y - rd[l].y * e2.x;
        a[l] = vdot(e1, h[l]);
        if (fabsf(a[l]) > EPS && (active & (1u << l))) mask |= 1u << l;
    }
    if (!mask) return 0;
    f32 fr[8], u[8]; vec3 s[8];
    u32 m2 = 0;
    for (int l = 0; l < 8; l++) {
        fr[l] = rcpr(a[l]);
        s[l] = vsub(ro[l], v0);
        u[l] = fr[l] * vdot(s[l], h[l]);
        if ((mask & (1u << l)) && u[l] >= 0.f && u[l] <= 1.f) m2 |= 1u << l;
    }
    mask = m2;
    if (!mask) return 0;
    f32 v[8]; vec3 q[8]; m2 = 0;
    for (int l = 0; l < 8; l++) {
        q[l].x = s[l].y * e1.z - s[l].z * e1.y;
        q[l].y = s[l].z * e1.x - s[l].x * e1.z;
        q[l].z = s[l].x * e1.y - s[l].y * e1.x;
        v[l] = fr[l] * vdot(rd[l], q[l]);
        if ((mask & (1u << l)) && v[l] >= 0.f && (u[l] + v[l]) <= 1.f) m2 |= 1u << l;
    }
    mask = m2;
    if (!mask) return 0;
    m2 = 0;
    for (int l = 0; l < 8; l++) {
        const f32 t = fr[l] * vdot(e2, q[l]);
        if ((mask & (1u << l)) && t > EPS && t < tmax[l]) m2 |= 1u << l;
    }
    return m2;
}

/* sft_m_qinv (1693-1712) */
static mat4 qinv(const mat4* m) {
    mat4 r;
    r.m[0][0] = m->m[0][0]; r.m[0][1] = m->m[1][0]; r.m[0][2] = m->m[2][0]; r.m[0][3] = 0;
    r.m[1][0] = m->m[0][1]; r.m[1][1] = m->m[1][1]; r.m[1][2] = m->m[2][1]; r.m[1][3] = 0;
    r.m[2][0] = m->m[0][2]; r.m[2][1] = m->m[1][2]; r.m[2][2] = m->m[2][2]; r.m[2][3] = 0;
    for (int a = 0; a < 3; a++) r.m[3][a] = -(m->m[3][0] * r.m[0][a] + m->m[3][1] * r.m[1][a] + m->m[3][2] * r.m[2][a]);
    r.m[3][3] = 1;
    return r;
}

/* sft__trace_shadow_packet (4086-4243), static_only = 1 */
static u32 trace_packet(octx* c, const f32* ox, const f32* oy, const f32* oz, const f32* lx, const f32* ly, const f32* lz,
                        u32 active, vec3 lpos, f32 lrad) {
    if (!active) return 0;
    u32 sat = 0;
    const u32 full = active;
    ofrustum pf;
    if (!packet_frustum(ox, oy, oz, active, lpos, lrad, &pf)) c->invalid_packets++;
    u32 tstack[64]; i32 ttop = 0;
    tstack[ttop++] = c->tlas_root;
    while (ttop > 0) {
        const onode* tn = &c->tlas[tstack[--ttop]];
        u32 th = frustum_vs_node(tn, &pf);
        while (th) {
            const i32 tl = ctz32(th); th &= th - 1;
            if (tn->child[tl] == INVALID) continue;
            if (!tn->leaf) { tstack[ttop++] = tn->child[tl]; continue; }
            const u32 ii = tn->child[tl] & ~0x80000000u;
            const omodel* m = &c->models[c->f->inst[ii].model];
            if (m->src->bone_count > 0) continue;
            if (!m->blas_count) continue;
            const mat4* M = &c->inst_T[ii];
            ofrustum mf;
            for (int p = 0; p < 6; p++) {
                const f32 nx = pf.n[p].x, ny = pf.n[p].y, nz = pf.n[p].z, d = pf.d[p];
                const f32 nmx = nx * M->m[0][0] + ny * M->m[0][1] + nz * M->m[0][2];
                const f32 nmy = nx * M->m[1][0] + ny * M->m[1][1] + nz * M->m[1][2];
                const f32 nmz = nx * M->m[2][0] + ny * M->m[2][1] + nz * M->m[2][2];
                const f32 dot_t = nx * M->m[3][0] + ny * M->m[3][1] + nz * M->m[3][2];
                const f32 dm = dot_t + d;
                const f32 il = 1.f / sqrtf(nmx * nmx + nmy * nmy + nmz * nmz);
                mf.n[p].x = nmx * il; mf.n[p].y = nmy * il; mf.n[p].z = nmz * il;
                mf.d[p] = dm * il;
                mf.an[p].x = fabsf(nmx * il); mf.an[p].y = fabsf(nmy * il); mf.an[p].z = fabsf(nmz * il);
            }
            const mat4 im = qinv(M);
            vec3 lo[8], ld[8]; f32 ltm[8];
            for (int l = 0; l < 8; l++) {
                const vec3 o = { ox[l], oy[l], oz[l] };
                const vec3 e = { ox[l] + lx[l], oy[l] + ly[l], oz[l] + lz[l] };
                lo[l] = xform(o, &im);
                const vec3 le = xform(e, &im);
                const vec3 L = vsub(le, lo[l]);
                ltm[l] = sqrtf(vdot(L, L));
                ld[l] = vnorm_fast(L);
            }
            u32 bstack[64]; i32 btop = 0;
            bstack[btop++] = m->blas_root;
            while (btop > 0) {
                const onode* bn = (const onode*)(m->blas + 256u * bstack[--btop]);
                u32 bh = frustum_vs_node(bn, &mf);
                while (bh) {
                    const i32 bl = ctz32(bh); bh &= bh - 1;
                    if (bn->child[bl] == INVALID) continue;
                    if (!bn->leaf) { bstack[btop++] = bn->child[bl]; continue; }
                    const u32 pay = bn->child[bl] & ~0x80000000u;
                    const u32 g = pay >> 7, t = pay & 0x7F;
                    const sfts_meshlet* ml = m->ml[g];
                    u32 i0, i1, i2; tri_inds(ml, t, &i0, &i1, &i2);
                    const vec3 v0 = { ml->attr[i0], ml->attr[64 + i0], ml->attr[128 + i0] };
                    const vec3 v1 = { ml->attr[i1], ml->attr[64 + i1], ml->attr[128 + i1] };
                    const vec3 v2 = { ml->attr[i2], ml->attr[64 + i2], ml->attr[128 + i2] };
                    const u32 cur = active & ~sat;
                    sat |= packet_vs_tri(v0, v1, v2, lo, ld, ltm, cur);
                    if (sat == full) return sat;
                }
            }
        }
    }
    return sat;
}

/* proxy occlusion pass inside sft_present (8163-8280) */
static void proxy_occlusion(octx* c) {
    const sfts_frame* f = c->f;
    if (!f->shadows || !f->n_point || !c->nprox) return;
    const i32 pc = (i32)c->nprox, lc = f->n_point < 64 ? (i32)f->n_point : 64;
    for (i32 p = 0; p < pc; p++) for (i32 l = 0; l < lc; l++) c->prox[p].vis[l] = 3;
    for (i32 l = 0; l < lc; l++) {
        const vec3 lpos = { f->point[l].pos[0], f->point[l].pos[1], f->point[l].pos[2] };
        const f32 lrad = f->point[l].radius;
        for (i32 pb = 0; pb < pc; pb += 8) {
            vec3 bc = { 0, 0, 0 }; i32 na = 0;
            for (int ln = 0; ln < 8; ln++) {
                if (pb + ln >= pc) continue;
                const oproxy* px = &c->prox[pb + ln];
                bc.x += (px->posa.x + px->posb.x) * 0.5f; bc.y += (px->posa.y + px->posb.y) * 0.5f; bc.z += (px->posa.z + px->posb.z) * 0.5f;
                na++;
            }
            if (na > 0) bc = vscale(bc, 1.f / (f32)na);
            const vec3 ldir = snorm(vsub(lpos, bc));
            /* sft_v_perpendicular (1564-1584) */
            f32 mnv = fabsf(ldir.x); vec3 card = { 1, 0, 0 };
            if (fabsf(ldir.y) < mnv) { mnv = fabsf(ldir.y); card.x = 0; card.y = 1; card.z = 0; }
            if (fabsf(ldir.z) < mnv) { card.x = 0; card.y = 0; card.z = 1; }
            const vec3 perp = { ldir.y * card.z - ldir.z * card.y, ldir.z * card.x - ldir.x * card.z, ldir.x * card.y - ldir.y * card.x };
            const vec3 lright = snorm(perp);
            const vec3 lup = scross(lright, ldir);
            const f32 r = 0.1f;
            const vec3 tg[3] = {
                vadd(lpos, vscale(lup, r)),
                vadd(lpos, vadd(vscale(lright, r * 0.866025f), vscale(lup, -r * 0.5f))),
                vadd(lpos, vadd(vscale(lright, -r * 0.866025f), vscale(lup, -r * 0.5f))),
            };
            for (int ray = 0; ray < 3; ray++) {
                f32 ox[8], oy[8], oz[8], lx[8], ly[8], lz[8]; u32 am = 0;
                for (int ln = 0; ln < 8; ln++) {
                    if (pb + ln < pc) {
                        const oproxy* px = &c->prox[pb + ln];
                        f32 x, y, z;
                        if (ray == 0) { x = px->posa.x; y = px->posa.y; z = px->posa.z; }
                        else if (ray == 1) { x = px->posb.x; y = px->posb.y; z = px->posb.z; }
                        else { x = (px->posa.x + px->posb.x) * 0.5f; y = (px->posa.y + px->posb.y) * 0.5f; z = (px->posa.z + px->posb.z) * 0.5f; }
                        ox[ln] = x; oy[ln] = y; oz[ln] = z;
                        lx[ln] = tg[ray].x - x; ly[ln] = tg[ray].y - y; lz[ln] = tg[ray].z - z;
                        am |= 1u << ln;
                    } else { ox[ln] = oy[ln] = oz[ln] = lx[ln] = ly[ln] = lz[ln] = 0.f; }
                }
                const u32 occ = trace_packet(c, ox, oy, oz, lx, ly, lz, am, lpos, lrad);
                for (int ln = 0; ln < 8; ln++) if (occ & (1u << ln)) c->prox[pb + ln].vis[l] -= 1;
            }
        }
    }
}

/* sft__geom_bin_tiles (4650-4688) */
static void bin_tiles(octx* c, u64 payload, i32 x0, i32 x1, i32 y0, i32 y1) {
    const i32 mxx = c->cols - 1, mxy = c->rows - 1;
    if (x1 < 0 || x0 > mxx || y1 < 0 || y0 > mxy) return;
    x0 = x0 > 0 ? x0 : 0; x1 = x1 < mxx ? x1 : mxx; y0 = y0 > 0 ? y0 : 0; y1 = y1 < mxy ? y1 : mxy;
    for (i32 ty = y0; ty <= y1; ty++) for (i32 tx = x0; tx <= x1; tx++) list_push(&c->tiles[ty * c->cols + tx], payload);
}

typedef struct { f32 tx, ty, tz, w, u, v, lu, lv, px, py, pz, nx, ny, nz; } cvert;   /* sft_clip_vert 1282-1288 */
static cvert lerp_cv(cvert a, cvert b, f32 t) {   /* sft__lerp_clip_vert (4245-4262) */
    cvert r;
    const f32* pa = &a.tx; const f32* pb = &b.tx; f32* pr = &r.tx;
    for (int i = 0; i < 14; i++) pr[i] = pa[i] + t * (pb[i] - pa[i]);
    return r;
}

/* sft__clip_triangle_near_plane (4264-4349) */
static int clip_near(cvert out[2][3], const cvert in[3]) {
    f32 d[3]; int mask = 0;
    for (int i = 0; i < 3; i++) { d[i] = in[i].tz; mask |= (d[i] >= 0.f) << i; }
    switch (mask) {
    case 0: return 0;
    case 7: out[0][0] = in[0]; out[0][1] = in[1]; out[0][2] = in[2]; return 1;
    case 1: case 2: case 4: {
        const int ia = mask >> 1, ib = (ia == 2) ? 0 : ia + 1, ic = (ia == 0) ? 2 : ia - 1;
        const f32 tab = d[ia] / (d[ia] - d[ib]), tac = d[ia] / (d[ia] - d[ic]);
        out[0][0] = in[ia]; out[0][1] = lerp_cv(in[ia], in[ib], tab); out[0][2] = lerp_cv(in[ia], in[ic], tac);
        return 1;
    }
    case 3: case 5: case 6: {
        const int io = (~mask & 7) >> 1, ia = (io == 0) ? 2 : io - 1, ic = (io == 2) ? 0 : io + 1;
        const f32 tab = d[ia] / (d[ia] - d[io]), tcb = d[ic] / (d[ic] - d[io]);
        const cvert nab = lerp_cv(in[ia], in[io], tab), ncb = lerp_cv(in[ic], in[io], tcb);
        out[0][0] = in[ia]; out[0][1] = nab; out[0][2] = in[ic];
        out[1][0] = nab; out[1][1] = ncb; out[1][2] = in[ic];
        return 2;
    }
    }
    return 0;
}

/* the geometry phase for one job (sft__worker_phase_geom 4901-5145 with its batch setup 4775-4884,
 * clipping 4691-4772 and projection 4351-4381) */
static void geom_job(octx* c, u32 ii, u32 mesh_i, u32 start, u32 count) {
    const sfts_instance* in = &c->f->inst[ii];
    const omodel* md = &c->models[in->model];
    const omesh* ms = &md->meshes[mesh_i];
    const sfts_mesh* sm = ms->src;
    const mat4* T = &c->inst_T[ii];
    const mat4* bones = c->inst_bones[ii];
    const f32 hw = c->hw, hh = c->hh;
    const f32 bias_x = hw + c->vpx, scale_y = -hh, bias_y = hh + c->vpy;
    const int skinned_mesh = sm->has_skin && bones;
    for (u32 i = 0; i < count; i += 8) {
        const u32 mi = start + i;
        u32 active = 0;
        for (u32 ln = 0; ln < 8 && i + ln < count; ln++) {
            const sfts_meshlet* ml = &sm->meshlets[mi + ln];
            vec3 ctr = { ml->cull[0], ml->cull[1], ml->cull[2] }, ax = { ml->cull[4], ml->cull[5], ml->cull[6] };
            if (skinned_mesh) {
                const mat4* B = &bones[sm->meshlets[mi].culling_bone];   /* lane 0's bone for the whole group */
                ctr = xform(ctr, B); ax = xform_dir(ax, B);
                ctr = xform(ctr, T); ax = xform_dir(ax, T);
            } else { ctr = xform(ctr, T); ax = xform_dir(ax, T); }
            const f32 sxs = sqrtf(T->m[0][0] * T->m[0][0] + T->m[0][1] * T->m[0][1] + T->m[0][2] * T->m[0][2]);
            const f32 rad = ml->cull[3] * sxs;
            ax = vnorm(ax);
            int inside = 1;
            for (int p = 0; p < 6; p++) {
                const f32 dist = vdot(ctr, c->fr.n[p]) + c->fr.d[p];
                inside &= (dist + rad >= 0.f);
            }
            const vec3 vr = vsub(ctr, c->cam);
            const f32 dd = sqrtf(vdot(vr, vr));
            const f32 dv = vdot(vr, ax);
            const f32 thr = fmaf(dd, ml->cull[7], rad);
            inside &= (dv <= thr);
            if (inside) active |= 1u << ln;
        }
        if (!active) continue;
        for (u32 ln = 0; ln < 8; ln++) {
            if (i + ln >= count) break;
            if (!(active & (1u << ln))) continue;
            const u32 lm = mi + ln, gm = ms->first_meshlet + lm;
            const sfts_meshlet* ml = &sm->meshlets[lm];
            const u32 ssi = c->ss_off[ii] + gm;
            oss* ss = &c->ss[ssi];
            f32 ctx[64], cty[64], ctz[64], cw[64];
            for (int v = 0; v < 64; v++) {
                const vec3 p = { ml->attr[v], ml->attr[64 + v], ml->attr[128 + v] };
                const vec3 n = { ml->attr[192 + v], ml->attr[256 + v], ml->attr[320 + v] };
                vec3 pw, nw;
                if (skinned_mesh) {
                    const f32 inv255 = 1.f / 255.f;
                    vec3 vp[4], vn[4]; f32 wt[4];
                    for (int k = 0; k < 4; k++) {
                        const mat4* M = &bones[ml->joints[k * 64 + v]];
                        wt[k] = (f32)ml->weights[k * 64 + v] * inv255;
                        vp[k] = xform(p, M); vn[k] = xform_dir(n, M);
                    }
                    pw.x = fmaf(vp[0].x, wt[0], fmaf(vp[1].x, wt[1], fmaf(vp[2].x, wt[2], vp[3].x * wt[3])));
                    pw.y = fmaf(vp[0].y, wt[0], fmaf(vp[1].y, wt[1], fmaf(vp[2].y, wt[2], vp[3].y * wt[3])));
                    pw.z = fmaf(vp[0].z, wt[0], fmaf(vp[1].z, wt[1], fmaf(vp[2].z, wt[2], vp[3].z * wt[3])));
                    nw.x = fmaf(vn[0].x, wt[0], fmaf(vn[1].x, wt[1], fmaf(vn[2].x, wt[2], vn[3].x * wt[3])));
                    nw.y = fmaf(vn[0].y, wt[0], fmaf(vn[1].y, wt[1], fmaf(vn[2].y, wt[2], vn[3].y * wt[3])));
                    nw.z = fmaf(vn[0].z, wt[0], fmaf(vn[1].z, wt[1], fmaf(vn[2].z, wt[2], vn[3].z * wt[3])));
                    pw = xform(pw, T); nw = xform_dir(nw, T);
                } else { pw = xform(p, T); nw = xform_dir(n, T); }
                ss->wx[v] = pw.x; ss->wy[v] = pw.y; ss->wz[v] = pw.z;
                ss->wnx[v] = nw.x; ss->wny[v] = nw.y; ss->wnz[v] = nw.z;
                const mat4* V = &c->vp;
                const f32 w = fmaf(pw.x, V->m[0][3], fmaf(pw.y, V->m[1][3], fmaf(pw.z, V->m[2][3], V->m[3][3])));
                const f32 tx = fmaf(pw.x, V->m[0][0], fmaf(pw.y, V->m[1][0], fmaf(pw.z, V->m[2][0], V->m[3][0])));
                const f32 ty = fmaf(pw.x, V->m[0][1], fmaf(pw.y, V->m[1][1], fmaf(pw.z, V->m[2][1], V->m[3][1])));
                const f32 tz = fmaf(pw.x, V->m[0][2], fmaf(pw.y, V->m[1][2], fmaf(pw.z, V->m[2][2], V->m[3][2])));
                const f32 iw = rcpr(w);
                const f32 sx = fmaf(tx, iw * hw, bias_x), sy = fmaf(ty, iw * scale_y, bias_y);
                ctx[v] = tx; cty[v] = ty; ctz[v] = tz; cw[v] = w;
                ss->sx[v] = x86nan(sx); ss->sy[v] = x86nan(sy); ss->iw[v] = x86nan(iw);
            }
            for (u32 batch = 0; batch < 16; batch++) {
                u32 I0[8], I1[8], I2[8];
                u32 valid = 0, inside = 0, outside = 0;
                for (int l = 0; l < 8; l++) {
                    I0[l] = ml->inds[batch * 32 + l]; I1[l] = ml->inds[batch * 32 + 8 + l]; I2[l] = ml->inds[batch * 32 + 16 + l];
                    if ((i32)(I0[l] | I1[l] | I2[l]) > 0) valid |= 1u << l;
                    const int a = ctz[I0[l]] >= 0.f, b = ctz[I1[l]] >= 0.f, d = ctz[I2[l]] >= 0.f;
                    const int oa = ctz[I0[l]] < 0.f, ob = ctz[I1[l]] < 0.f, od = ctz[I2[l]] < 0.f;
                    if (a && b && d) inside |= 1u << l;
                    if (oa && ob && od) outside |= 1u << l;
                }
                if (!valid) continue;
                u32 inter = valid & ~(inside | outside);
                while (inter) {   /* sft__geom_clip_and_bin */
                    const i32 l = ctz32(inter); inter &= inter - 1;
                    const u32 vi[3] = { I0[l], I1[l], I2[l] };
                    cvert tri[3];
                    for (int k = 0; k < 3; k++) {
                        const u32 q = vi[k];
                        cvert* cv = &tri[k];
                        cv->tx = ctx[q]; cv->ty = cty[q]; cv->tz = ctz[q]; cv->w = cw[q];
                        cv->u = ml->attr[384 + q]; cv->v = ml->attr[448 + q]; cv->lu = ml->attr[512 + q]; cv->lv = ml->attr[576 + q];
                        cv->px = ss->wx[q]; cv->py = ss->wy[q]; cv->pz = ss->wz[q];
                        cv->nx = ss->wnx[q]; cv->ny = ss->wny[q]; cv->nz = ss->wnz[q];
                    }
                    cvert out[2][3];
                    const int nc = clip_near(out, tri);
                    for (int k = 0; k < nc; k++) {
                        if (c->nclip == c->clipcap) { c->clipcap = c->clipcap ? c->clipcap * 2 : 256; c->clip = (oclip*)realloc(c->clip, c->clipcap * sizeof(oclip)); }
                        const u32 slot = c->nclip++;
                        oclip* ct = &c->clip[slot];
                        for (int q = 0; q < 3; q++) {
                            const cvert* cv = &out[k][q];
                            const f32 iw = 1.f / cv->w;
                            ct->sx[q] = (cv->tx * iw + 1.f) * hw + c->vpx;
                            ct->sy[q] = (-cv->ty * iw + 1.f) * hh + c->vpy;
                            ct->iw[q] = iw;
                            ct->u[q] = cv->u; ct->v[q] = cv->v; ct->lu[q] = cv->lu; ct->lv[q] = cv->lv;
                            ct->px[q] = cv->px; ct->py[q] = cv->py; ct->pz[q] = cv->pz;
                            ct->nx[q] = cv->nx; ct->ny[q] = cv->ny; ct->nz[q] = cv->nz;
                        }
                        ct->inst = ii; ct->m = gm;
                        const f32 area = (ct->sx[1] - ct->sx[0]) * (ct->sy[2] - ct->sy[0]) - (ct->sy[1] - ct->sy[0]) * (ct->sx[2] - ct->sx[0]);
                        if (area <= 0.1f) continue;
                        const i32 x0 = cvtt(floorf(vmin(ct->sx[0], vmin(ct->sx[1], ct->sx[2]))));
                        const i32 x1 = cvtt(ceilf(vmax(ct->sx[0], vmax(ct->sx[1], ct->sx[2]))));
                        const i32 y0 = cvtt(floorf(vmin(ct->sy[0], vmin(ct->sy[1], ct->sy[2]))));
                        const i32 y1 = cvtt(ceilf(vmax(ct->sy[0], vmax(ct->sy[1], ct->sy[2]))));
                        bin_tiles(c, (u64)slot, x0 >> 6, x1 >> 6, y0 >> 6, y1 >> 6);
                    }
                }
                if (!inside) continue;
                u32 vm = 0; i32 tx0[8], tx1[8], ty0[8], ty1[8];
                for (int l = 0; l < 8; l++) {
                    const f32 sx0 = ss->sx[I0[l]], sy0 = ss->sy[I0[l]], sx1 = ss->sx[I1[l]], sy1 = ss->sy[I1[l]];
                    const f32 sx2 = ss->sx[I2[l]], sy2 = ss->sy[I2[l]];
                    const f32 dx1 = sx1 - sx0, dy1 = sy1 - sy0, dx2 = sx2 - sx0, dy2 = sy2 - sy0;
                    if (!((inside >> l) & 1)) continue;
                    if (!(fmaf(dx1, dy2, -(dy1 * dx2)) > 0.1f)) continue;
                    tx0[l] = cvtt(vmin(sx0, vmin(sx1, sx2))) >> 6; tx1[l] = cvtt(vmax(sx0, vmax(sx1, sx2))) >> 6;
                    ty0[l] = cvtt(vmin(sy0, vmin(sy1, sy2))) >> 6; ty1[l] = cvtt(vmax(sy0, vmax(sy1, sy2))) >> 6;
                    if (tx1[l] >= 0 && tx0[l] <= c->cols - 1 && ty1[l] >= 0 && ty0[l] <= c->rows - 1) vm |= 1u << l;
                }
                if (!vm) continue;
                i32 bx0 = 9999, bx1 = -9999, by0 = 9999, by1 = -9999;
                for (u32 a = vm; a; a &= a - 1) {
                    const i32 l = ctz32(a);
                    if (tx0[l] < bx0) bx0 = tx0[l];
                    if (tx1[l] > bx1) bx1 = tx1[l];
                    if (ty0[l] < by0) by0 = ty0[l];
                    if (ty1[l] > by1) by1 = ty1[l];
                }
                const u64 payload = (u64)ii | ((u64)gm << 24) | ((u64)batch << 48) | ((u64)vm << 56);
                bin_tiles(c, payload, bx0, bx1, by0, by1);
            }
        }
    }
}

static const f32 MS_OX4[4] = { -0.125f, 0.375f, -0.375f, 0.125f }, MS_OY4[4] = { -0.375f, -0.125f, 0.125f, 0.375f };
static const f32 MS_OX2[2] = { -0.25f, 0.25f }, MS_OY2[2] = { -0.25f, 0.25f };
static const f32 MS_O1[1] = { 0.f };

/* fetches the three vertices of a vis id (clipped or regular), as in 5163-5209 / 6199-6278 */
typedef struct { f32 sx[3], sy[3], iw[3], u[3], v[3], lu[3], lv[3], px[3], py[3], pz[3], nx[3], ny[3], nz[3]; u32 inst, m; } otri;
static void fetch_tri(const octx* c, u32 vid, otri* t) {
    if (vid & 0x80000000u) {
        const oclip* ct = &c->clip[vid & 0x7FFFFFFFu];
        memcpy(t, ct, sizeof(f32) * 39); t->inst = ct->inst; t->m = ct->m;
        return;
    }
    const u32 ii = (vid >> 25) & 63, gm = (vid >> 7) & 0x3FFFF, tri = vid & 127;
    const omodel* md = &c->models[c->f->inst[ii].model];
    const sfts_meshlet* ml = md->ml[gm];
    const oss* ss = &c->ss[c->ss_off[ii] + gm];
    u32 q[3]; tri_inds(ml, tri, &q[0], &q[1], &q[2]);
    for (int k = 0; k < 3; k++) {
        const u32 v = q[k];
        t->sx[k] = ss->sx[v]; t->sy[k] = ss->sy[v]; t->iw[k] = ss->iw[v];
        t->u[k] = ml->attr[384 + v]; t->v[k] = ml->attr[448 + v]; t->lu[k] = ml->attr[512 + v]; t->lv[k] = ml->attr[576 + v];
        t->px[k] = ss->wx[v]; t->py[k] = ss->wy[v]; t->pz[k] = ss->wz[v];
        t->nx[k] = ss->wnx[v]; t->ny[k] = ss->wny[v]; t->nz[k] = ss->wnz[v];
    }
    t->inst = ii; t->m = gm;
}

/* sft__rast_simd_batch (5148-5499) for one payload into one tile's buffers */
static void rast_payload(const octx* c, u64 payload, f32* depth, u32* vidb, i32 tmx, i32 tmy) {
    const u32 raw = (u32)(payload >> 56);
    f32 sx[3][8], sy[3][8], iw[3][8];
    u32 active; u32 vid_base; int clipped = 0; u32 batch = 0;
    if (!raw) {
        clipped = 1;
        const oclip* ct = &c->clip[(u32)(payload & 0xFFFFFFFFu)];
        for (int k = 0; k < 3; k++) for (int l = 0; l < 8; l++) { sx[k][l] = ct->sx[k]; sy[k][l] = ct->sy[k]; iw[k][l] = ct->iw[k]; }
        active = 1; vid_base = (u32)(payload & 0xFFFFFFFFu) | 0x80000000u;
    } else {
        const u32 ii = (u32)(payload & 0xFFFFFF), gm = (u32)((payload >> 24) & 0xFFFFFF);
        batch = (u32)((payload >> 48) & 0xFF);
        active = raw;
        const omodel* md = &c->models[c->f->inst[ii].model];
        const sfts_meshlet* ml = md->ml[gm];
        const oss* ss = &c->ss[c->ss_off[ii] + gm];
        for (int l = 0; l < 8; l++) {
            const u32 q[3] = { ml->inds[batch * 32 + l], ml->inds[batch * 32 + 8 + l], ml->inds[batch * 32 + 16 + l] };
            for (int k = 0; k < 3; k++) { sx[k][l] = ss->sx[q[k]]; sy[k][l] = ss->sy[q[k]]; iw[k][l] = ss->iw[q[k]]; }
        }
        vid_base = (ii << 25) | (gm << 7) | (batch * 8);
    }
    const int S = c->S;
    const f32* OX = S == 4 ? MS_OX4 : S == 2 ? MS_OX2 : MS_O1;
    const f32* OY = S == 4 ? MS_OY4 : S == 2 ? MS_OY2 : MS_O1;
    for (u32 act = active; act; act &= act - 1) {
        const i32 l = ctz32(act);
        const f32 sx0 = sx[0][l], sx1 = sx[1][l], sx2 = sx[2][l], sy0 = sy[0][l], sy1 = sy[1][l], sy2 = sy[2][l];
        const f32 iw0 = iw[0][l], iw1 = iw[1][l], iw2 = iw[2][l];
        const f32 A0 = sy0 - sy1, B0 = sx1 - sx0, A1 = sy1 - sy2, B1 = sx2 - sx1, A2 = sy2 - sy0, B2 = sx0 - sx2;
        const f32 m01 = sx0 * sy1, m10 = sy0 * sx1, m12 = sx1 * sy2, m21 = sy1 * sx2, m20 = sx2 * sy0, m02 = sy2 * sx0;
        const f32 C0 = (fmaf(sx0, sy1, -m10) - fmaf(sy0, sx1, -m01)) * 0.5f;
        const f32 C1 = (fmaf(sx1, sy2, -m21) - fmaf(sy1, sx2, -m12)) * 0.5f;
        const f32 C2 = (fmaf(sx2, sy0, -m02) - fmaf(sy2, sx0, -m20)) * 0.5f;
        const f32 dx1 = sx1 - sx0, dx2 = sx2 - sx0, dy1 = sy1 - sy0, dy2 = sy2 - sy0;
        const f32 det = dx1 * dy2 - dx2 * dy1;
        if (!(det > EPS)) continue;
        const f32 idet = rcpr(det);
        const f32 dzdx = ((iw1 - iw0) * dy2 - (iw2 - iw0) * dy1) * idet;
        const f32 dzdy = ((iw2 - iw0) * dx1 - (iw1 - iw0) * dx2) * idet;
        const f32 c0 = fmaf(B0, 0.5f, fmaf(A0, 0.5f, C0)), c1 = fmaf(B1, 0.5f, fmaf(A1, 0.5f, C1)), c2 = fmaf(B2, 0.5f, fmaf(A2, 0.5f, C2));
        const f32 zb = fmaf(0.5f - sy0, dzdy, fmaf(0.5f - sx0, dzdx, iw0));
        const i32 minx = cvtt(vmax(vmin(sx0, vmin(sx1, sx2)), (f32)tmx));
        const i32 maxx = cvtt(vmin(vmax(sx0, vmax(sx1, sx2)), (f32)(tmx + TILE - 1)));
        const i32 miny = cvtt(vmax(vmin(sy0, vmin(sy1, sy2)), (f32)tmy));
        const i32 maxy = cvtt(vmin(vmax(sy0, vmax(sy1, sy2)), (f32)(tmy + TILE - 1)));
        const u32 vid = clipped ? vid_base : vid_base + (u32)l;
        if (minx > maxx || miny > maxy) continue;
        const i32 ax0 = minx & ~7, ax1 = (maxx & ~7) + 8;
        const f32 se0 = c0 + A0 * (f32)ax0 + B0 * (f32)miny;
        const f32 se1 = c1 + A1 * (f32)ax0 + B1 * (f32)miny;
        const f32 se2 = c2 + A2 * (f32)ax0 + B2 * (f32)miny;
        const f32 sz = zb + dzdx * (f32)ax0 + dzdy * (f32)miny;
        const f32 bw = (f32)(ax1 - 1 - ax0), bh = (f32)(maxy - miny);
        const f32 me0 = se0 + (A0 < 0.f ? A0 * bw : 0.f) + (B0 < 0.f ? B0 * bh : 0.f);
        const f32 me1 = se1 + (A1 < 0.f ? A1 * bw : 0.f) + (B1 < 0.f ? B1 * bh : 0.f);
        const f32 me2 = se2 + (A2 < 0.f ? A2 * bw : 0.f) + (B2 < 0.f ? B2 * bh : 0.f);
        f32 pad0 = 0, pad1 = 0, pad2 = 0; int trivial;
        f32 de0[4], de1[4], de2[4], dz[4];
        if (S > 1) {
            pad0 = 0.375f * (fabsf(A0) + fabsf(B0)); pad1 = 0.375f * (fabsf(A1) + fabsf(B1)); pad2 = 0.375f * (fabsf(A2) + fabsf(B2));
            trivial = (me0 >= pad0 && me1 >= pad1 && me2 >= pad2);
            for (int s = 0; s < S; s++) {
                de0[s] = A0 * OX[s] + B0 * OY[s]; de1[s] = A1 * OX[s] + B1 * OY[s]; de2[s] = A2 * OX[s] + B2 * OY[s];
                dz[s] = dzdx * OX[s] + dzdy * OY[s];
            }
        } else trivial = (me0 >= 0.f && me1 >= 0.f && me2 >= 0.f);
        const f32 zchunk = dzdx * 8.f;
        f32 zrow[8];
        for (int k = 0; k < 8; k++) zrow[k] = sz + dzdx * (f32)k;
        if (trivial) {
            for (i32 y = miny; y <= maxy; y++) {
                f32 z[8]; memcpy(z, zrow, 32);
                i32 pi = (y - tmy) * TILE + (ax0 - tmx);
                for (i32 x = ax0; x < ax1; x += 8, pi += 8) {
                    for (int s = 0; s < S; s++)
                        for (int k = 0; k < 8; k++) {
                            const f32 zs = S > 1 ? z[k] + dz[s] : z[k];
                            const u32 si = (u32)(s * TILE_PX + pi + k);
                            if (zs > depth[si]) { depth[si] = zs; vidb[si] = vid; }
                        }
                    for (int k = 0; k < 8; k++) z[k] = z[k] + zchunk;
                }
                for (int k = 0; k < 8; k++) zrow[k] = zrow[k] + dzdy;
            }
        } else {
            const f32 a0c = A0 * 8.f, a1c = A1 * 8.f, a2c = A2 * 8.f;
            f32 e0r[8], e1r[8], e2r[8];
            for (int k = 0; k < 8; k++) { e0r[k] = se0 + A0 * (f32)k; e1r[k] = se1 + A1 * (f32)k; e2r[k] = se2 + A2 * (f32)k; }
            for (i32 y = miny; y <= maxy; y++) {
                f32 e0[8], e1[8], e2[8], z[8];
                memcpy(e0, e0r, 32); memcpy(e1, e1r, 32); memcpy(e2, e2r, 32); memcpy(z, zrow, 32);
                i32 pi = (y - tmy) * TILE + (ax0 - tmx);
                for (i32 x = ax0; x < ax1; x += 8, pi += 8) {
                    if (S > 1) {
                        int might = 0;
                        for (int k = 0; k < 8; k++) might |= (e0[k] >= -pad0 && e1[k] >= -pad1 && e2[k] >= -pad2);
                        if (might)
                            for (int s = 0; s < S; s++)
                                for (int k = 0; k < 8; k++) {
                                    const f32 a = e0[k] + de0[s], b = e1[k] + de1[s], d = e2[k] + de2[s];
                                    if (!(a >= 0.f && b >= 0.f && d >= 0.f)) continue;
                                    const f32 zs = z[k] + dz[s];
                                    const u32 si = (u32)(s * TILE_PX + pi + k);
                                    if (zs > depth[si]) { depth[si] = zs; vidb[si] = vid; }
                                }
                    } else {
                        for (int k = 0; k < 8; k++) {
                            if (!(e0[k] >= 0.f && e1[k] >= 0.f && e2[k] >= 0.f)) continue;
                            const u32 si = (u32)(pi + k);
                            if (z[k] > depth[si]) { depth[si] = z[k]; vidb[si] = vid; }
                        }
                    }
                    for (int k = 0; k < 8; k++) { e0[k] = e0[k] + a0c; e1[k] = e1[k] + a1c; e2[k] = e2[k] + a2c; z[k] = z[k] + zchunk; }
                }
                for (int k = 0; k < 8; k++) { e0r[k] = e0r[k] + B0; e1r[k] = e1r[k] + B1; e2r[k] = e2r[k] + B2; zrow[k] = zrow[k] + dzdy; }
            }
        }
    }
}

typedef struct { vec3 pa, pb, ab, W; f32 abdab, wdw, rb2, pr, pr2, vis_mult; u32 vis; } opc;   /* sft_light_proxy_cache 991-998 (+ the visibility count) */

static const otex* tex_of(const octx* c, u32 tex_index_plus1) { return tex_index_plus1 ? &c->tex[tex_index_plus1 - 1] : NULL; }

/* tile overlays of the debug views, drawn after the tile's resolve (sft__debug_draw_tile_overlay,
 * 5731-5807); depth is the tile's sample-0 depth plane */
static u32 half_blend(u32 bg, u32 ov) { return ((bg & 0xFEFEFEFEu) >> 1) + ((ov & 0xFEFEFEFEu) >> 1); }

static void debug_overlay(octx* c, i32 tmx, i32 tmy, i32 lim_x, i32 lim_y, f32 zmin, f32 zmax, i32 ntl, const f32* depth) {
    const i32 W = c->W;
    if (c->debug_mode == 2) {
        for (i32 y = tmy; y < lim_y; y++)
            for (i32 x = tmx; x < lim_x; x++) {
                u32* p = &c->color[y * W + x];
                if (x == tmx || x == lim_x - 1 || y == tmy || y == lim_y - 1) *p = 0xFF00FF00u;
                else if ((x % 16 == 0) || (y % 16 == 0)) *p = half_blend(*p, 0xFF004400u);
            }
    } else if (c->debug_mode == 3) {
        f32 dd = 0.f;
        if (zmin <= zmax && zmin > EPS) { const f32 near_w = 1.f / zmax, far_w = 1.f / zmin; dd = far_w - near_w; }
        const u32 border = dd > 16.f ? 0xFFFF0000u : 0xFF00FF00u;
        for (i32 y = tmy; y < lim_y; y++)
            for (i32 x = tmx; x < lim_x; x++) {
                u32* p = &c->color[y * W + x];
                if (x == tmx || x == lim_x - 1 || y == tmy || y == lim_y - 1) { *p = border; continue; }
                const f32 iw = depth[(y - tmy) * TILE + (x - tmx)];
                if (iw <= EPS) continue;
                const f32 lz = 1.f / iw;
                const f32 q = lz / 100.f;
                const f32 nz = q < 0.f ? 0.f : (q > 1.f ? 1.f : q);
                const u32 it = (u32)(nz * 255.f);
                *p = 0xFF000000u | (it << 16) | (it << 8) | it;
            }
    } else {
        const u32 heat = ntl == 0 ? 0xFF222288u : (ntl < 4 ? 0xFF00FF00u : 0xFFFF0000u);
        for (i32 y = tmy; y < lim_y; y++)
            for (i32 x = tmx; x < lim_x; x++) c->color[y * W + x] = half_blend(c->color[y * W + x], heat);
    }
}

/* sft__resolve_tile (5809-6753) */
/* FP64 evaluation of the capsule shadow expression (sofren2.c:6522-6571) for one 4x2 block and
 * one light, beside the FP32 one: the same proxies, lane gates, block-level skip and smooth
 * maximum, with every quantity recomputed in double from the pixel positions, the light position
 * and the proxies' endpoints, radii and visibility counts (where the FP32 path uses the table
 * reciprocal, the fast normalisation and 0.3333333f).  Accumulates |FP32 - FP64| of the shadow
 * intensity over the block's pixels. */
static void shadow_check_fp64(octx* c, const vec3* P, vec3 lpos, const opc* pc, u32 npc, u32 gate, u32 lanes, const f32* ms32) {
    double Lr[8][3], d2[8], lrl[8], Ln[8][3], ms[8];
    for (int l = 0; l < 8; l++) {
        Lr[l][0] = (double)lpos.x - P[l].x; Lr[l][1] = (double)lpos.y - P[l].y; Lr[l][2] = (double)lpos.z - P[l].z;
        d2[l] = Lr[l][0] * Lr[l][0] + Lr[l][1] * Lr[l][1] + Lr[l][2] * Lr[l][2];
        lrl[l] = sqrt(d2[l]);
        for (int a = 0; a < 3; a++) Ln[l][a] = lrl[l] > 0.0 ? Lr[l][a] / lrl[l] : 0.0;
        ms[l] = 0.0;
    }
    for (u32 p = 0; p < npc; p++) {
        const opc* q = &pc[p];
        const double pa[3] = { q->pa.x, q->pa.y, q->pa.z }, pb[3] = { q->pb.x, q->pb.y, q->pb.z };
        double ab[3], W[3], abdab = 0.0, wdw = 0.0;
        for (int a = 0; a < 3; a++) { ab[a] = pb[a] - pa[a]; abdab += ab[a] * ab[a]; }
        const double lp[3] = { lpos.x, lpos.y, lpos.z };
        for (int a = 0; a < 3; a++) { W[a] = (pa[a] + pb[a]) * 0.5 - lp[a]; wdw += W[a] * W[a]; }
        const double br = (double)q->pr + sqrt(abdab) * 0.5, rb2 = br * br, pr2 = (double)q->pr * q->pr, vis = q->vis / 3.0;
        u32 ray = 0;
        for (int l = 0; l < 8; l++) {
            const double wdv = -(W[0] * Lr[l][0] + W[1] * Lr[l][1] + W[2] * Lr[l][2]);
            const double cd2 = wdw - wdv * (wdv / d2[l]);
            if (wdv > 0.0 && wdv < d2[l] && cd2 < rb2 && (gate >> l & 1)) ray |= 1u << l;
        }
        if (!ray) continue;
        for (int l = 0; l < 8; l++) {
            double ao[3], abl = 0.0, abao = 0.0, lao = 0.0;
            for (int a = 0; a < 3; a++) { ao[a] = (double)(a == 0 ? P[l].x : a == 1 ? P[l].y : P[l].z) - pa[a]; }
            for (int a = 0; a < 3; a++) { abl += ab[a] * Ln[l][a]; abao += ab[a] * ao[a]; lao += Ln[l][a] * ao[a]; }
            const double den = abdab - abl * abl, sden = den > 1e-6 ? den : 1e-6;
            double t2 = (abao - abl * lao) / sden;
            t2 = t2 < 0.0 ? 0.0 : (t2 > 1.0 ? 1.0 : t2);
            const double t1 = t2 * abl - lao;
            double dist2 = 0.0;
            for (int a = 0; a < 3; a++) {
                const double pr = (double)(a == 0 ? P[l].x : a == 1 ? P[l].y : P[l].z) + Ln[l][a] * t1, pcap = pa[a] + ab[a] * t2;
                dist2 += (pr - pcap) * (pr - pcap);
            }
            double sv = 1.0 - dist2 / pr2;
            if (sv < 0.0 || !(ray >> l & 1) || !(t1 > 1e-6 && t1 < lrl[l])) sv = 0.0;
            sv *= vis;
            const double h = 0.2 - fabs(ms[l] - sv), hp = h > 0.0 ? h : 0.0;
            ms[l] = (ms[l] > sv ? ms[l] : sv) + hp * hp * (0.25 / 0.2);
        }
    }
    for (int l = 0; l < 8; l++) {
        if (!(lanes >> l & 1)) continue;
        const f32 si32 = vmax(0.f, 1.f - ms32[l]);
        const double si64 = 1.0 - ms[l] > 0.0 ? 1.0 - ms[l] : 0.0;
        const double e = fabs((double)si32 - si64);
        if (e > c->fp64_max) c->fp64_max = e;
        c->fp64_sum += e; c->fp64_n++;
        if (e > 1e-5) c->fp64_big++;
    }
}

static void resolve_tile(octx* c, i32 tile, const f32* depth, const u32* vidb, f32* shadow_out) {
    const sfts_frame* f = c->f;
    const i32 tmx = (tile % c->cols) * TILE, tmy = (tile / c->cols) * TILE;
    const i32 sw = (i32)(c->hw * 2.f), sh = (i32)(c->hh * 2.f);
    const i32 pitch = c->W;
    const i32 lim_x = tmx + TILE < sw ? tmx + TILE : sw, lim_y = tmy + TILE < sh ? tmy + TILE : sh;
    const int S = c->S;
    /* D1: tile depth bounds (5820-5853) */
    f32 zmin = 1e9f, zmax = -1e9f;
    for (i32 i = 0; i < TILE_PX * S; i++) {
        const f32 d = depth[i];
        if (d > 0.0001f) { if (d < zmin) zmin = d; if (d > zmax) zmax = d; }
    }
    /* D2: tile light list (5855-5934) */
    u16 tl[16]; i32 ntl = 0;
    const mat4* vp = &c->vp;
    if (zmin <= zmax && f->n_point > 0) {
        for (u32 l = 0; l < f->n_point; l++) {
            const vec3 pos = { f->point[l].pos[0], f->point[l].pos[1], f->point[l].pos[2] };
            const f32 radius = f->point[l].radius;
            const f32 w = pos.x * vp->m[0][3] + pos.y * vp->m[1][3] + pos.z * vp->m[2][3] + vp->m[3][3];
            const f32 lmin = w - radius, lmax = w + radius;
            if (lmax <= EPS) continue;
            const f32 smin = (lmin > EPS) ? lmin : EPS;
            const f32 iwmin = 1.f / lmax, iwmax = 1.f / smin;
            if (iwmax < zmin || iwmin > zmax) continue;
            if (w > radius) {
                const f32 tx = pos.x * vp->m[0][0] + pos.y * vp->m[1][0] + pos.z * vp->m[2][0] + vp->m[3][0];
                const f32 ty = pos.x * vp->m[0][1] + pos.y * vp->m[1][1] + pos.z * vp->m[2][1] + vp->m[3][1];
                const f32 sx = (tx / w + 1.f) * c->hw + c->vpx;
                const f32 sy = (-ty / w + 1.f) * c->hh + c->vpy;
                const f32 psx = sqrtf(vp->m[0][0] * vp->m[0][0] + vp->m[1][0] * vp->m[1][0] + vp->m[2][0] * vp->m[2][0]);
                const f32 psy = sqrtf(vp->m[0][1] * vp->m[0][1] + vp->m[1][1] * vp->m[1][1] + vp->m[2][1] * vp->m[2][1]);
                const f32 safe_w = (w - radius) > EPS ? (w - radius) : EPS;
                const f32 rx = ((radius * psx) + fabsf(tx) * (radius / w)) / safe_w * c->hw;
                const f32 ry = ((radius * psy) + fabsf(ty) * (radius / w)) / safe_w * c->hh;
                if (sx + rx < (f32)tmx || sx - rx > (f32)(tmx + TILE) || sy + ry < (f32)tmy || sy - ry > (f32)(tmy + TILE)) continue;
            }
            tl[ntl++] = (u16)l;
            if (ntl == 16) break;
        }
    }
    /* D3: proxy cache (5936-5990) */
    opc pcache[16][16];
    u8 npc[16] = { 0 };
    if (f->shadows && c->nprox > 0 && ntl > 0) {
        for (i32 i = 0; i < ntl; i++) {
            const sfts_point_light* L = &f->point[tl[i]];
            const vec3 lpos = { L->pos[0], L->pos[1], L->pos[2] };
            u8 pcn = 0;
            for (u32 p = 0; p < c->nprox && pcn < 16; p++) {
                const oproxy* px = &c->prox[p];
                const u8 vs = px->vis[tl[i]];
                if (!vs) continue;
                const vec3 cc = { (px->posa.x + px->posb.x) * 0.5f, (px->posa.y + px->posb.y) * 0.5f, (px->posa.z + px->posb.z) * 0.5f };
                const vec3 ab = vsub(px->posb, px->posa);
                const f32 cl = sqrtf(sdot(ab, ab));
                const f32 br = px->radius + (cl * 0.5f);
                const f32 cr = br + L->radius;
                const vec3 Wv = vsub(cc, lpos);
                const f32 d2 = sdot(Wv, Wv);
                if (d2 <= cr * cr) {
                    opc* q = &pcache[i][pcn];
                    q->pa = px->posa; q->pb = px->posb; q->ab = ab; q->W = Wv;
                    q->abdab = sdot(ab, ab); q->wdw = d2; q->rb2 = br * br; q->pr = px->radius; q->pr2 = px->radius * px->radius;
                    q->vis_mult = (f32)vs * 0.3333333f; q->vis = vs;
                    pcn++;
                }
            }
            npc[i] = pcn;
        }
    }
    static const i32 IX[8] = { 0, 1, 2, 3, 0, 1, 2, 3 }, IY[8] = { 0, 0, 0, 0, 1, 1, 1, 1 };
    const f32 inv_s = 1.f / (f32)S;
    const u32 cc = f->clear_color;
    const f32 clr[3] = { (f32)((cc >> 16) & 0xFF) * (1.f / 255.f), (f32)((cc >> 8) & 0xFF) * (1.f / 255.f), (f32)(cc & 0xFF) * (1.f / 255.f) };
    for (i32 y = tmy; y < lim_y; y += 2) {
        for (i32 x = tmx; x < lim_x; x += 4) {
            u32 inb = 0; f32 pxf[8], pyf[8]; i32 pind[8];
            for (int l = 0; l < 8; l++) {
                const i32 gx = x + IX[l], gy = y + IY[l];
                if (sw > gx && sh > gy) inb |= 1u << l;
                pxf[l] = ((f32)x + 0.5f) + (f32)IX[l];
                pyf[l] = ((f32)y + 0.5f) + (f32)IY[l];
                pind[l] = (gy - tmy) * TILE + (gx - tmx);
            }
            u32 vids[4][8]; u32 asm_[4] = { 0 }; u32 act = 0; i32 ecount[8] = { 0 };
            for (int s = 0; s < S; s++)
                for (int l = 0; l < 8; l++) {
                    vids[s][l] = vidb[s * TILE_PX + pind[l]];
                    const int empty = vids[s][l] == INVALID;
                    if (!empty && (inb >> l & 1)) asm_[s] |= 1u << l;
                    if (empty && (inb >> l & 1)) ecount[l]++;
                }
            for (int s = 0; s < S; s++) act |= asm_[s];
            f32 acc[3][8];
            if (S == 1) {
                if (f->clear) {
                    for (int l = 0; l < 8; l++)
                        if ((inb >> l & 1) && vids[0][l] == INVALID) c->color[(y + IY[l]) * pitch + x + IX[l]] = cc;
                }
            } else {
                if (!act) {
                    if (f->clear) for (int l = 0; l < 8; l++) if (inb >> l & 1) c->color[(y + IY[l]) * pitch + x + IX[l]] = cc;
                    continue;
                }
                f32 ew[8]; int any_e = 0;
                for (int l = 0; l < 8; l++) { ew[l] = (f32)ecount[l] * inv_s; if (ew[l] > 0.f) any_e = 1; }
                for (int l = 0; l < 8; l++) for (int k = 0; k < 3; k++) acc[k][l] = 0.f;
                if (f->clear) { for (int l = 0; l < 8; l++) for (int k = 0; k < 3; k++) acc[k][l] = clr[k] * ew[l]; }
                else if (any_e) {
                    for (int l = 0; l < 8; l++) {
                        const i32 gx = x + IX[l], gy = y + IY[l];
                        f32 bg[3] = { 0, 0, 0 };
                        if (gx < sw && gy < sh) {
                            const u32 q = c->color[gy * pitch + gx];
                            bg[0] = (f32)((q >> 16) & 0xFF) * (1.f / 255.f); bg[1] = (f32)((q >> 8) & 0xFF) * (1.f / 255.f); bg[2] = (f32)(q & 0xFF) * (1.f / 255.f);
                        }
                        for (int k = 0; k < 3; k++) acc[k][l] = bg[k] * ew[l];
                    }
                }
            }
            const u32 block_write = act;
            while (act) {
                u32 target, tri_mask = 0, tri_lanes = 0; i32 hits[8] = { 0 };
                if (S == 1) {
                    const i32 fl = ctz32(act);
                    target = vids[0][fl];
                    for (int l = 0; l < 8; l++) if (vids[0][l] == target && (inb >> l & 1)) tri_mask |= 1u << l;
                    tri_lanes = tri_mask & act;
                    act &= ~tri_lanes;
                } else {
                    int fs = 0; while (!asm_[fs]) fs++;
                    target = vids[fs][ctz32(asm_[fs])];
                    for (int s = 0; s < S; s++) {
                        u32 match = 0;
                        for (int l = 0; l < 8; l++) if (vids[s][l] == target && (inb >> l & 1)) { match |= 1u << l; hits[l]++; }
                        const u32 mm = match & asm_[s];
                        asm_[s] &= ~mm; tri_lanes |= mm; tri_mask |= match;
                    }
                    act = 0; for (int s = 0; s < S; s++) act |= asm_[s];
                }
                otri T; fetch_tri(c, target, &T);
                const omodel* md = &c->models[f->inst[T.inst].model];
                const omesh* ms = &md->meshes[md->mesh_of[T.m]];
                /* D6 barycentrics + perspective interpolation (6282-6347) */
                const f32 dx1 = T.sx[1] - T.sx[0], dx2 = T.sx[2] - T.sx[0], dy1 = T.sy[1] - T.sy[0], dy2 = T.sy[2] - T.sy[0];
                const f32 idet = rcpr(dx1 * dy2 - dx2 * dy1);
                f32 cu[8], cv[8], clu[8], clv[8]; vec3 P[8], N[8], V[8];
                f32 BU[8], BV[8], BW[8];   /* kept for the wireframe view */
                for (int l = 0; l < 8; l++) {
                    const f32 pxs = pxf[l] - T.sx[0], pys = pyf[l] - T.sy[0];
                    const f32 rbu = (pxs * dy2 - pys * dx2) * idet;
                    const f32 rbv = (pys * dx1 - pxs * dy1) * idet;
                    const f32 rbw = (1.f - rbu) - rbv;
                    f32 bu = rbu, bv = rbv, bw = rbw;
                    if (S > 1) {
                        bu = vmax(0.f, rbu); bv = vmax(0.f, rbv); bw = vmax(0.f, rbw);
                        const f32 bs = rcpr(bu + (bv + bw));
                        bu = bu * bs; bv = bv * bs; bw = bw * bs;
                    }
                    BU[l] = bu; BV[l] = bv; BW[l] = bw;
                    const f32 iz = fmaf(bw, T.iw[0], fmaf(bu, T.iw[1], bv * T.iw[2]));
                    const f32 z = rcpr(iz);
                    const f32 w0 = (bw * T.iw[0]) * z, w1 = (bu * T.iw[1]) * z, w2 = (bv * T.iw[2]) * z;
#define INTERP(a) fmaf(w0, (a)[0], fmaf(w1, (a)[1], w2 * (a)[2]))
                    cu[l] = INTERP(T.u); cv[l] = INTERP(T.v); clu[l] = INTERP(T.lu); clv[l] = INTERP(T.lv);
                    P[l].x = INTERP(T.px); P[l].y = INTERP(T.py); P[l].z = INTERP(T.pz);
                    vec3 nn = { INTERP(T.nx), INTERP(T.ny), INTERP(T.nz) };
#undef INTERP
                    N[l] = vnorm_fast(nn);
                    V[l] = vnorm_fast(vsub(c->cam, P[l]));
                }
                /* material (6350-6382) */
                const sfts_mesh* sm = ms->src;
                u32 base = 0xFFFFFFFFu; const otex* tx = NULL; f32 shin = 4.f;
                if (sm->material >= 0) {
                    const omat* mt = &c->mats[sm->material];
                    base = mt->base; shin = mt->shin; tx = mt->tex >= 0 ? &c->tex[mt->tex] : NULL;
                }
                if (c->debug_mode == 5) { tx = &c->checker; base = 0xFFFFFFFFu; }   /* checkerboard view (6373-6376) */
                const f32 i255 = 1.f / 255.f;
                const f32 br_ = (f32)((base >> 16) & 0xFF) * i255, bg_ = (f32)((base >> 8) & 0xFF) * i255, bb_ = (f32)(base & 0xFF) * i255;
                /* D7 LOD (5501-5541) from the first lane holding the triangle */
                i32 lod = 0;
                if (tx) {
                    const i32 fl = ctz32(tri_mask);
                    const f32 ux = (cu[fl] - cu[fl ^ 1]) * (f32)tx->w, vx = (cv[fl] - cv[fl ^ 1]) * (f32)tx->h;
                    const f32 uy = (cu[fl] - cu[fl ^ 4]) * (f32)tx->w, vy = (cv[fl] - cv[fl ^ 4]) * (f32)tx->h;
                    const f32 a1 = fabsf(ux) > fabsf(vx) ? fabsf(ux) : fabsf(vx);
                    const f32 a2 = fabsf(uy) > fabsf(vy) ? fabsf(uy) : fabsf(vy);
                    const f32 rho = a1 > a2 ? a1 : a2;
                    if (rho > 1.f) {
                        const f32 lf = (f32)(31 - __builtin_clz((u32)cvtt(rho)));
                        const f32 bay = -0.375f;   /* bayer[((y & 1) << 1) | (x & 1)], x and y even */
                        lod = (i32)(lf + 0.5f + bay);
                    }
                    lod = lod < 0 ? 0 : (lod > tx->levels - 1 ? tx->levels - 1 : lod);
                }
                const int lm = sm->lightmap_page != 0xFFFFFFFFu;
                const f32 nsh = shin, sscale = ((shin + 8.f) / 8.f) * 0.04f;
                f32 out[3][8];
                for (int l = 0; l < 8; l++) {
                    f32 tr, tg, tb;
                    if (lod > 1) sample_nearest(tx, lod, cu[l], cv[l], &tr, &tg, &tb);
                    else sample_bilinear(tx, lod, cu[l], cv[l], &tr, &tg, &tb);
                    out[0][l] = tr * br_; out[1][l] = tg * bg_; out[2][l] = tb * bb_;
                }
                if (shin < 0.f) {
                    for (int l = 0; l < 8; l++) for (int k = 0; k < 3; k++) out[k][l] = out[k][l] * (-shin);
                } else {
                    f32 dif[3][8], spc[3][8], lms[8];
                    for (int l = 0; l < 8; l++) { spc[0][l] = spc[1][l] = spc[2][l] = 0.f; lms[l] = 1.f; }
                    if (lm) {
                        const otex* lt = tex_of(c, (u32)(md->src->lightmaps[sm->lightmap_page] + 1));
                        for (int l = 0; l < 8; l++) {
                            sample_bilinear(lt, 0, clu[l], clv[l], &dif[0][l], &dif[1][l], &dif[2][l]);
                            for (int k = 0; k < 3; k++) dif[k][l] = dif[k][l] * f->lightmap_brightness;
                        }
                    } else {
                        for (int l = 0; l < 8; l++) { dif[0][l] = f->ambient[0]; dif[1][l] = f->ambient[1]; dif[2][l] = f->ambient[2]; }
                        for (u32 dl = 0; dl < f->n_dir; dl++) {
                            const vec3 Ld = snorm((vec3){ f->dir[dl].dir[0], f->dir[dl].dir[1], f->dir[dl].dir[2] });
                            const f32 col[3] = { f->dir[dl].r * f->dir[dl].intensity, f->dir[dl].g * f->dir[dl].intensity, f->dir[dl].b * f->dir[dl].intensity };
                            for (int l = 0; l < 8; l++) {
                                const f32 ndl = vmax(vdot(N[l], Ld), 0.f);
                                const int lit = ndl > 0.f;
                                for (int k = 0; k < 3; k++) dif[k][l] = fmaf(ndl, col[k], dif[k][l]);
                                if (!lit) continue;
                                const vec3 H = vnorm_fast(vadd(Ld, V[l]));
                                const f32 ndh = vmax(vdot(N[l], H), 0.f);
                                const f32 den = (nsh - nsh * ndh) + ndh;
                                const f32 sp = ndh * rcpr(den);
                                const f32 term = (sp * sscale) * ndl;
                                for (int k = 0; k < 3; k++) spc[k][l] = fmaf(term, col[k], spc[k][l]);
                            }
                        }
                    }
                    /* D10 point lights + capsule shadows (6474-6607) */
                    for (i32 i = 0; i < ntl; i++) {
                        const sfts_point_light* L = &f->point[tl[i]];
                        const vec3 lpos = { L->pos[0], L->pos[1], L->pos[2] };
                        const f32 col[3] = { L->r * L->intensity, L->g * L->intensity, L->b * L->intensity };
                        const f32 ir2 = 1.f / (L->radius * L->radius);
                        vec3 Lr[8], Ln[8]; f32 d2[8], att[8], ndl[8]; u32 alm = 0, lit = 0;
                        for (int l = 0; l < 8; l++) {
                            Lr[l] = vsub(lpos, P[l]);
                            d2[l] = vdot(Lr[l], Lr[l]);
                            f32 a = vmax(0.f, fmaf(-d2[l], ir2, 1.f));
                            att[l] = a * a;
                            if (att[l] > 0.f) alm |= 1u << l;
                        }
                        if (!alm) continue;
                        for (int l = 0; l < 8; l++) {
                            Ln[l] = vnorm_fast(Lr[l]);
                            ndl[l] = vmax(vdot(N[l], Ln[l]), 0.f);
                            if (ndl[l] > 0.f && (alm >> l & 1) && (tri_mask >> l & 1)) lit |= 1u << l;
                        }
                        f32 ms_[8] = { 0 };
                        if (npc[i] > 0) {
                            f32 lrl[8];
                            for (int l = 0; l < 8; l++) lrl[l] = sqrtf(d2[l]);
                            const f32 bk = 0.2f, b4 = 0.25f / 0.2f;
                            for (u32 pi = 0; pi < npc[i]; pi++) {
                                const opc* q = &pcache[i][pi];
                                u32 ray = 0; f32 wdv[8];
                                for (int l = 0; l < 8; l++) {
                                    wdv[l] = 0.f - vdot(q->W, Lr[l]);
                                    const int btw = wdv[l] > 0.f && wdv[l] < d2[l];
                                    const f32 tf = wdv[l] * rcpr(d2[l]);
                                    const f32 cd2 = fmaf(-wdv[l], tf, q->wdw);
                                    const u32 gate = lm ? tri_mask : lit;
                                    if (btw && cd2 < q->rb2 && (gate >> l & 1)) ray |= 1u << l;
                                }
                                if (!ray) continue;   /* block-level skip: changes the smooth max of every lane */
                                for (int l = 0; l < 8; l++) {
                                    const vec3 ao = vsub(P[l], q->pa);
                                    const f32 abl = vdot(q->ab, Ln[l]), abao = vdot(q->ab, ao), lao = vdot(Ln[l], ao);
                                    const f32 den = fmaf(-abl, abl, q->abdab);
                                    const f32 sden = vmax(den, EPS);
                                    f32 t2 = fmaf(-abl, lao, abao) * rcpr(sden);
                                    t2 = vmax(0.f, vmin(t2, 1.f));
                                    const f32 t1 = fmaf(t2, abl, -lao);
                                    const int vc = t1 > EPS && t1 < lrl[l];
                                    const vec3 pr = vadd(P[l], vscale(Ln[l], t1));
                                    const vec3 pc = vadd(q->pa, vscale(q->ab, t2));
                                    const vec3 dd = vsub(pr, pc);
                                    const f32 dist2 = vdot(dd, dd);
                                    f32 sv = vmax(0.f, 1.f - dist2 / q->pr2);
                                    if (!(ray >> l & 1)) sv = 0.f;
                                    if (!vc) sv = 0.f;
                                    sv = sv * q->vis_mult;
                                    const f32 diff = ms_[l] - sv;
                                    const f32 h = vmax(0.f, bk - fabsf(diff));
                                    const f32 badd = (h * h) * b4;
                                    ms_[l] = vmax(ms_[l], sv) + badd;
                                }
                            }
                        }
                        if (c->fp64) shadow_check_fp64(c, P, lpos, pcache[i], npc[i], lm ? tri_mask : lit, tri_lanes, ms_);
                        for (int l = 0; l < 8; l++) {
                            const f32 si = vmax(0.f, 1.f - ms_[l]);
                            if (shadow_out && (tri_lanes >> l & 1) && i < 16) {
                                const i32 gx = x + IX[l], gy = y + IY[l];
                                shadow_out[((size_t)(gy * c->W + gx)) * 16 + (size_t)i] = si;
                            }
                            if (lm) {
                                const f32 drop = (1.f - si) * att[l];
                                lms[l] = lms[l] * (1.f - drop);
                            } else {
                                const f32 di = ndl[l] * att[l];
                                const f32 md_ = (lit >> l & 1) ? (di * si) : 0.f;
                                for (int k = 0; k < 3; k++) dif[k][l] = fmaf(md_, col[k], dif[k][l]);
                                if (!(lit >> l & 1)) continue;
                                const vec3 H = vnorm_fast(vadd(Ln[l], V[l]));
                                const f32 ndh = vmax(vdot(N[l], H), 0.f);
                                const f32 den = (nsh - nsh * ndh) + ndh;
                                const f32 sp = ndh * rcpr(den);
                                const f32 term = ((sp * sscale) * di) * si;
                                for (int k = 0; k < 3; k++) spc[k][l] = fmaf(term, col[k], spc[k][l]);
                            }
                        }
                    }
                    for (int l = 0; l < 8; l++) {
                        if (lm) {
                            const f32 mod = fmaf(lms[l], 1.f - 0.4f, 0.4f);
                            for (int k = 0; k < 3; k++) out[k][l] = out[k][l] * (dif[k][l] * mod);
                        } else {
                            for (int k = 0; k < 3; k++) out[k][l] = fmaf(out[k][l], dif[k][l], spc[k][l]);
                        }
                    }
                }
                if (c->debug_mode == 1) {   /* wireframe view (6645-6671): edges where a barycentric is under its screen-space width */
                    const f32 dbu_dx = (0.f - dy2) * idet, dbu_dy = dx2 * idet;
                    const f32 dbv_dx = dy1 * idet, dbv_dy = (0.f - dx1) * idet;
                    const f32 fw_u = fabsf(dbu_dx) + fabsf(dbu_dy), fw_v = fabsf(dbv_dx) + fabsf(dbv_dy);
                    const f32 dbw_dx = 0.f - (dbu_dx + dbv_dx), dbw_dy = 0.f - (dbu_dy + dbv_dy);
                    const f32 fw_w = fabsf(dbw_dx) + fabsf(dbw_dy);
                    for (int l = 0; l < 8; l++)
                        if (BU[l] < fw_u || BV[l] < fw_v || BW[l] < fw_w) { out[0][l] = 0.f; out[1][l] = 1.f; out[2][l] = 0.f; }
                }
                if (S == 1) {
                    for (u32 a = tri_lanes; a; a &= a - 1) {
                        const i32 l = ctz32(a);
                        u32 px = 0xFF000000u;
                        for (int k = 0; k < 3; k++) {
                            const f32 q = vmax(0.f, vmin(out[k][l], 1.f)) * 255.f;
                            px |= ((u32)cvtt(q)) << (16 - 8 * k);
                        }
                        c->color[(y + IY[l]) * pitch + x + IX[l]] = px;
                    }
                } else {
                    for (int l = 0; l < 8; l++) {
                        const f32 wgt = (tri_mask >> l & 1) ? (f32)hits[l] * inv_s : 0.f;
                        for (int k = 0; k < 3; k++) acc[k][l] = fmaf(vmax(0.f, vmin(out[k][l], 1.f)), wgt, acc[k][l]);
                    }
                }
            }
            if (S > 1) {
                const u32 store = f->clear ? inb : block_write;
                for (u32 a = store; a; a &= a - 1) {
                    const i32 l = ctz32(a);
                    u32 px = 0xFF000000u;
                    for (int k = 0; k < 3; k++) px |= ((u32)cvtt(vmin(acc[k][l], 1.f) * 255.f)) << (16 - 8 * k);
                    c->color[(y + IY[l]) * pitch + x + IX[l]] = px;
                }
            }
        }
    }
    if (c->debug_mode >= 2 && c->debug_mode <= 4) debug_overlay(c, tmx, tmy, lim_x, lim_y, zmin, zmax, ntl, depth);
}

/* ------------------------------------------------------------ driver */
typedef struct {
    octx* c; i32 t0, t1; f32* shadow;
} tile_job;

static void* tile_worker(void* arg) {
    tile_job* j = (tile_job*)arg;
    octx* c = j->c;
    const u64 per = (u64)TILE_PX * c->S;
    for (i32 t = j->t0; t < j->t1; t++) {
        f32* depth = c->depth + per * t; u32* vid = c->vid + per * t;
        for (u64 i = 0; i < per; i++) { depth[i] = 0.f; vid[i] = INVALID; }
        const i32 tmx = (t % c->cols) * TILE, tmy = (t / c->cols) * TILE;
        for (u32 k = 0; k < c->tiles[t].n; k++) rast_payload(c, c->tiles[t].p[k], depth, vid, tmx, tmy);
        resolve_tile(c, t, depth, vid, j->shadow);
    }
    return NULL;
}

typedef struct {
    u64 ns_total, ns_geom, ns_tiles;
    u32 invalid_packets;
} ostats;

/* Renders one frame of the scene at S samples; fills buffers; optionally writes a dump. */
static int render_frame(octx* c, u32 fi, int S, int threads, const char* dump_path, f32* shadow_out, ostats* st) {
    const sfts_scene* sc = c->sc;
    const sfts_frame* f = &sc->frames[fi];
    struct timespec ta, tb, tc;
    clock_gettime(CLOCK_MONOTONIC, &ta);
    c->f = f; c->S = S;
    c->W = (i32)f->width; c->H = (i32)f->height;
    c->hw = (f32)c->W * 0.5f; c->hh = (f32)c->H * 0.5f; c->vpx = 0.f; c->vpy = 0.f;
    c->cols = (c->W + TILE - 1) / TILE; c->rows = (c->H + TILE - 1) / TILE;
    c->invalid_packets = 0;
    set_camera(c, f);
    /* instances (sft_draw_instance 8410-8478) */
    free(c->ss_off); free(c->inst_T); free(c->inst_bones);
    c->ss_off = (u32*)calloc(f->n_inst + 1, 4);
    c->inst_T = (mat4*)calloc(f->n_inst + 1, sizeof(mat4));
    c->inst_bones = (const mat4**)calloc(f->n_inst + 1, sizeof(mat4*));
    u32 total_ss = 0, np = 0;
    for (u32 i = 0; i < f->n_inst; i++) {
        memcpy(&c->inst_T[i], f->inst[i].transform, 64);
        c->inst_bones[i] = f->inst[i].n_bones ? (const mat4*)f->inst[i].bones : NULL;
        c->ss_off[i] = total_ss;
        total_ss += c->models[f->inst[i].model].total;
        if (f->shadows) np += c->models[f->inst[i].model].src->n_proxies;
    }
    free(c->prox);
    c->prox = (oproxy*)calloc(np + 1, sizeof(oproxy)); c->nprox = np;
    np = 0;
    if (f->shadows)
        for (u32 i = 0; i < f->n_inst; i++) {
            const sfts_model* sm = c->models[f->inst[i].model].src;
            for (u32 p = 0; p < sm->n_proxies; p++) {
                const sfts_proxy* lp = &sm->proxies[p];
                mat4 m = c->inst_T[i];
                if (lp->bone != INVALID && c->inst_bones[i]) m = mmul(&c->inst_bones[i][lp->bone], &c->inst_T[i]);
                oproxy* w = &c->prox[np++];
                w->posa.x = lp->posa[0] * m.m[0][0] + lp->posa[1] * m.m[1][0] + lp->posa[2] * m.m[2][0] + m.m[3][0];
                w->posa.y = lp->posa[0] * m.m[0][1] + lp->posa[1] * m.m[1][1] + lp->posa[2] * m.m[2][1] + m.m[3][1];
                w->posa.z = lp->posa[0] * m.m[0][2] + lp->posa[1] * m.m[1][2] + lp->posa[2] * m.m[2][2] + m.m[3][2];
                w->posb.x = lp->posb[0] * m.m[0][0] + lp->posb[1] * m.m[1][0] + lp->posb[2] * m.m[2][0] + m.m[3][0];
                w->posb.y = lp->posb[0] * m.m[0][1] + lp->posb[1] * m.m[1][1] + lp->posb[2] * m.m[2][1] + m.m[3][1];
                w->posb.z = lp->posb[0] * m.m[0][2] + lp->posb[1] * m.m[1][2] + lp->posb[2] * m.m[2][2] + m.m[3][2];
                const f32 sx = sqrtf(m.m[0][0] * m.m[0][0] + m.m[0][1] * m.m[0][1] + m.m[0][2] * m.m[0][2]);
                w->radius = lp->radius * sx;
            }
        }
    free(c->ss);
    c->ss = (oss*)malloc((size_t)(total_ss + 1) * sizeof(oss));
    memset(c->ss, 0xFF, (size_t)(total_ss + 1) * sizeof(oss));
    c->n_ss = total_ss;
    c->nclip = 0;
    const i32 ntiles = c->cols * c->rows;
    if (c->tiles) free(c->tiles);
    c->tiles = (olist*)calloc((size_t)ntiles, sizeof(olist));
    free(c->tlas); c->tlas = NULL;
    tlas_build(c);
    proxy_occlusion(c);
    /* geometry in job order: instance, mesh, groups of up to 8 meshlets */
    for (u32 i = 0; i < f->n_inst; i++) {
        const omodel* md = &c->models[f->inst[i].model];
        for (u32 m = 0; m < md->src->n_meshes; m++) {
            const u32 n = md->src->meshes[m].meshlet_count;
            for (u32 s = 0; s < n; s += 8) geom_job(c, i, m, s, (n - s) < 8 ? (n - s) : 8);
        }
    }
    clock_gettime(CLOCK_MONOTONIC, &tb);
    const u64 per = (u64)TILE_PX * S;
    free(c->depth); free(c->vid); free(c->color);
    c->depth = (f32*)malloc(per * ntiles * 4);
    c->vid = (u32*)malloc(per * ntiles * 4);
    c->color = (u32*)calloc((size_t)c->W * c->H, 4);
    if (threads < 1) threads = 1;
    pthread_t th[64]; tile_job jobs[64];
    if (threads > 64) threads = 64;
    for (int k = 0; k < threads; k++) {
        jobs[k].c = c; jobs[k].t0 = ntiles * k / threads; jobs[k].t1 = ntiles * (k + 1) / threads; jobs[k].shadow = shadow_out;
        if (threads > 1) pthread_create(&th[k], NULL, tile_worker, &jobs[k]); else tile_worker(&jobs[k]);
    }
    if (threads > 1) for (int k = 0; k < threads; k++) pthread_join(th[k], NULL);
    clock_gettime(CLOCK_MONOTONIC, &tc);
    if (st) {
        st->ns_geom = (u64)(tb.tv_sec - ta.tv_sec) * 1000000000ull + (u64)(tb.tv_nsec - ta.tv_nsec);
        st->ns_tiles = (u64)(tc.tv_sec - tb.tv_sec) * 1000000000ull + (u64)(tc.tv_nsec - tb.tv_nsec);
        st->ns_total = st->ns_geom + st->ns_tiles;
        st->invalid_packets = c->invalid_packets;
    }
    if (dump_path) {
        sfts_dump d = { fopen(dump_path, "ab") };
        if (!d.f) return -1;
        sfts_dump_section(&d, "color", "u32", c->color, (u64)c->W * c->H * 4);
        i32* counts = (i32*)calloc((size_t)ntiles, 4); u64 tot = 0;
        for (i32 t = 0; t < ntiles; t++) { counts[t] = (i32)c->tiles[t].n; tot += c->tiles[t].n; }
        u64* pays = (u64*)malloc((tot + 1) * 8); u64 k = 0;
        for (i32 t = 0; t < ntiles; t++) { memcpy(pays + k, c->tiles[t].p, (size_t)c->tiles[t].n * 8); k += c->tiles[t].n; }
        sfts_dump_section(&d, "tile_counts", "i32", counts, (u64)ntiles * 4);
        sfts_dump_section(&d, "tile_payloads", "u64", pays, tot * 8);
        sfts_dump_section(&d, "depth", "f32", c->depth, per * ntiles * 4);
        sfts_dump_section(&d, "vid", "u32", c->vid, per * ntiles * 4);
        sfts_dump_section(&d, "ss_cache", "f32", c->ss, (u64)total_ss * sizeof(oss));
        sfts_dump_section(&d, "clip", "f32", c->clip, (u64)c->nclip * sizeof(oclip));
        u8* vis = (u8*)calloc((size_t)c->nprox + 1, 64);
        f32* wp = (f32*)calloc((size_t)c->nprox + 1, 28);
        for (u32 p = 0; p < c->nprox; p++) {
            memcpy(vis + 64 * p, c->prox[p].vis, 64);
            const f32 v[7] = { c->prox[p].posa.x, c->prox[p].posa.y, c->prox[p].posa.z, c->prox[p].posb.x, c->prox[p].posb.y, c->prox[p].posb.z, c->prox[p].radius };
            memcpy(wp + 7 * p, v, 28);
        }
        sfts_dump_section(&d, "light_vis", "u8", vis, (u64)c->nprox * 64);
        sfts_dump_section(&d, "world_proxies", "f32", wp, (u64)c->nprox * 28);
        sfts_dump_section(&d, "tlas", "u8", c->tlas, (u64)c->tlas_count * 256);
        const u64 ip = c->invalid_packets;
        sfts_dump_section(&d, "invalid_packets", "u64", &ip, 8);
        fclose(d.f);
        free(counts); free(pays); free(vis); free(wp);
    }
    for (i32 t = 0; t < ntiles; t++) free(c->tiles[t].p);
    return 0;
}

static int load_scene(octx* c, const sfts_scene* sc) {
    memset(c, 0, sizeof(*c));
    c->sc = sc;
    /* texture 0 of the reference pool is the checkerboard made in sft_init; scene textures follow */
    c->ntex = sc->n_textures;
    c->tex = (otex*)calloc(sc->n_textures + 1, sizeof(otex));
    for (u32 i = 0; i < sc->n_textures; i++) tex_create(&c->tex[i], (i32)sc->textures[i].w, (i32)sc->textures[i].h, sc->textures[i].argb);
    c->mats = (omat*)calloc(sc->n_materials + 1, sizeof(omat));
    for (u32 i = 0; i < sc->n_materials; i++) { c->mats[i].tex = sc->materials[i].tex; c->mats[i].base = sc->materials[i].base_color; c->mats[i].shin = sc->materials[i].shininess; }
    c->models = (omodel*)calloc(sc->n_models + 1, sizeof(omodel));
    for (u32 i = 0; i < sc->n_models; i++) {
        omodel* m = &c->models[i];
        m->src = &sc->models[i];
        m->meshes = (omesh*)calloc(m->src->n_meshes + 1, sizeof(omesh));
        u32 tot = 0;
        for (u32 k = 0; k < m->src->n_meshes; k++) { m->meshes[k].first_meshlet = tot; m->meshes[k].src = &m->src->meshes[k]; tot += m->src->meshes[k].meshlet_count; }
        m->total = tot;
        m->mesh_of = (u16*)calloc(tot + 1, 2);
        m->ml = (const sfts_meshlet**)calloc(tot + 1, sizeof(void*));
        for (u32 k = 0; k < m->src->n_meshes; k++)
            for (u32 j = 0; j < m->src->meshes[k].meshlet_count; j++) {
                m->mesh_of[m->meshes[k].first_meshlet + j] = (u16)k;
                m->ml[m->meshes[k].first_meshlet + j] = &m->src->meshes[k].meshlets[j];
            }
        blas_build(m);
    }
    {   /* the checkerboard of sft_init (8062-8080): 32x32 squares */
        u32* px = (u32*)malloc(256 * 256 * 4);
        for (i32 y = 0, i = 0; y < 256; y++)
            for (i32 x = 0; x < 256; x++, i++) px[i] = (((x / 32) % 2) ^ ((y / 32) % 2)) ? 0xFFAFFFAFu : 0xFF555555u;
        tex_create(&c->checker, 256, 256, px);
        free(px);
    }
    return 0;
}

/* ------------------------------------------------------------ C entry points for tests */
typedef struct { sfts_scene sc; octx c; } oracle_handle;

void* sfto_open(const uint8_t* blob, uint64_t size) {
    oracle_handle* h = (oracle_handle*)calloc(1, sizeof(oracle_handle));
    uint8_t* copy = (uint8_t*)malloc(size + 16);
    memcpy(copy, blob, size);
    if (sfts_parse(&h->sc, copy, size)) { free(copy); free(h); return NULL; }
    load_scene(&h->c, &h->sc);
    return h;
}

/* Renders `frame` at `samples` (1, 2 or 4) samples.  color (w*h u32) and shadow (w*h*16 f32,
 * per pixel per tile light) may be NULL.  Returns 0 on success. */
int sfto_render(void* hp, uint32_t frame, int samples, int threads, const char* dump_path, uint32_t* color,
                float* shadow, uint64_t* ns_out, uint32_t* invalid_packets) {
    oracle_handle* h = (oracle_handle*)hp;
    if (!h || frame >= h->sc.n_frames || !(samples == 1 || samples == 2 || samples == 4)) return -1;
    ostats st;
    if (dump_path && frame == 0) {
        sfts_dump d = { fopen(dump_path, "wb") };
        if (!d.f) return -2;
        for (u32 i = 0; i < h->sc.n_models; i++) sfts_dump_section(&d, "blas", "u8", h->c.models[i].blas, (u64)h->c.models[i].blas_count * 256);
        fclose(d.f);
    }
    const int rc = render_frame(&h->c, frame, samples, threads, dump_path, shadow, &st);
    if (rc) return rc;
    if (color) memcpy(color, h->c.color, (size_t)h->c.W * h->c.H * 4);
    if (ns_out) *ns_out = st.ns_total;
    if (invalid_packets) *invalid_packets = st.invalid_packets;
    return 0;
}

/* world-space proxy data and light visibility of the last rendered frame */
int sfto_light_vis(void* hp, uint8_t* out, uint32_t cap_proxies) {
    oracle_handle* h = (oracle_handle*)hp;
    const u32 n = h->c.nprox < cap_proxies ? h->c.nprox : cap_proxies;
    for (u32 p = 0; p < n; p++) memcpy(out + 64 * p, h->c.prox[p].vis, 64);
    return (int)h->c.nprox;
}

/* ------------------------------------------------------------ skeletal pose (sft_pose_update, 8952-9108)
 * Pose blob (little endian): "SFTP", bone count, bones {f32 inverse_bind[16], f32 local_bind[16],
 * i32 parent, f32 base_t[3], f32 base_r[4], f32 base_s[3]}, animation count, per animation
 * {f32 duration, u32 samplers, u32 channels, samplers {u32 count, u32 is_step, f32 inputs[count],
 * f32 outputs[count * 4]}, channels {i32 sampler, i32 node, i32 path}}, request count, requests
 * {i32 animation, f32 time}.  Output per request: bones x 16 posed floats, then bones x 16 global. */
typedef struct { f32 inv[16], loc[16]; i32 parent; f32 bt[3], br[4], bs[3]; } opbone;
typedef struct { u32 count, is_step; const f32* in; const f32* out; } opsmp;
typedef struct { i32 sampler, node, path; } opch;
typedef struct { f32 duration; u32 ns, nc; opsmp* smp; opch* ch; } opanim;

static void pmul(const f32* a, const f32* b, f32* r) {   /* sft_m_mul (1668): left-to-right sums */
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            r[i * 4 + j] = a[i * 4 + 0] * b[0 * 4 + j] + a[i * 4 + 1] * b[1 * 4 + j] + a[i * 4 + 2] * b[2 * 4 + j] + a[i * 4 + 3] * b[3 * 4 + j];
}
static void pqnorm(f32* q) {   /* sft_q_norm (1908) */
    const f32 l2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    if (0.f != l2) { const f32 il = 1.f / sqrtf(l2); q[0] *= il; q[1] *= il; q[2] *= il; q[3] *= il; }
}
static void pslerp(const f32* a, const f32* bi, f32 t, f32* r) {   /* sft_q_slerp (1857) */
    f32 b[4] = { bi[0], bi[1], bi[2], bi[3] };
    f32 dot = a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
    if (dot < 0.f) { b[0] = -b[0]; b[1] = -b[1]; b[2] = -b[2]; b[3] = -b[3]; dot = -dot; }
    if (dot > 0.9995f) { for (int k = 0; k < 4; k++) r[k] = a[k] + t * (b[k] - a[k]); pqnorm(r); return; }
    const f32 th0 = acosf(dot), th = th0 * t, st = sinf(th), is0 = 1.f / sinf(th0);
    const f32 s0 = cosf(th) - dot * st * is0, s1 = st * is0;
    for (int k = 0; k < 4; k++) r[k] = a[k] * s0 + b[k] * s1;
    pqnorm(r);
}
static void pquat(const f32* q, f32* m) {   /* sft_m_from_quat (1822) */
    const f32 x2 = q[0] + q[0], y2 = q[1] + q[1], z2 = q[2] + q[2];
    const f32 xx = q[0] * x2, xy = q[0] * y2, xz = q[0] * z2, yy = q[1] * y2, yz = q[1] * z2, zz = q[2] * z2;
    const f32 wx = q[3] * x2, wy = q[3] * y2, wz = q[3] * z2;
    const f32 r[16] = { 1.f - (yy + zz), xy + wz, xz - wy, 0.f, xy - wz, 1.f - (xx + zz), yz + wx, 0.f,
                        xz + wy, yz - wx, 1.f - (xx + yy), 0.f, 0.f, 0.f, 0.f, 1.f };
    memcpy(m, r, 64);
}

static void pose_update(const opbone* bones, i32 nb, const opanim* an, f32 time, f32* posed, f32* global) {
    if (an->duration > EPS) time = fmodf(time, an->duration);
    f32 tp[128][3], tr[128][4], ts[128][3]; u8 mask[128];
    memset(mask, 0, sizeof(mask));
    for (u32 i = 0; i < an->nc; i++) {
        const opch* ch = &an->ch[i];
        const opsmp* sm = &an->smp[ch->sampler];
        if (ch->node < 0 || ch->node >= nb) continue;
        i32 f0 = 0, f1 = 0; f32 t = 0.f;
        if (time <= sm->in[0]) { f0 = f1 = 0; }
        else if (time >= sm->in[sm->count - 1]) { f0 = f1 = (i32)sm->count - 1; }
        else {
            i32 low = 0, high = (i32)sm->count - 1;
            while (low <= high) {
                const i32 mid = low + (high - low) / 2;
                if (time < sm->in[mid]) high = mid - 1;
                else if (time >= sm->in[mid + 1]) low = mid + 1;
                else { f0 = mid; f1 = mid + 1; break; }
            }
            const f32 dt = sm->in[f1] - sm->in[f0];
            t = (dt > 0.0001f) ? (time - sm->in[f0]) / dt : 0.f;
        }
        if (ch->path == 1) {
            if (sm->is_step) memcpy(tr[ch->node], sm->out + f0 * 4, 16);
            else pslerp(sm->out + f0 * 4, sm->out + f1 * 4, t, tr[ch->node]);
            mask[ch->node] |= 2;
        } else {
            f32 v[3];
            for (int k = 0; k < 3; k++) {
                const f32 v0 = sm->out[f0 * 4 + k], v1 = sm->out[f1 * 4 + k];
                v[k] = sm->is_step ? v0 : v0 + (v1 - v0) * t;
            }
            if (ch->path == 0) { memcpy(tp[ch->node], v, 12); mask[ch->node] |= 1; }
            else if (ch->path == 2) { memcpy(ts[ch->node], v, 12); mask[ch->node] |= 4; }
        }
    }
    for (i32 b = 0; b < nb; b++) {
        f32* g = global + b * 16;
        if (mask[b]) {
            const f32* p = (mask[b] & 1) ? tp[b] : bones[b].bt;
            const f32* q = (mask[b] & 2) ? tr[b] : bones[b].br;
            const f32* sc = (mask[b] & 4) ? ts[b] : bones[b].bs;
            const f32 T[16] = { 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, p[0], p[1], p[2], 1 };
            const f32 S[16] = { sc[0], 0, 0, 0, 0, sc[1], 0, 0, 0, 0, sc[2], 0, 0, 0, 0, 1 };
            f32 R[16], RT[16];
            pquat(q, R); pmul(R, T, RT); pmul(S, RT, g);
        } else {
            memcpy(g, bones[b].loc, 64);
        }
    }
    u8 done[128]; memset(done, 0, sizeof(done));
    i32 count = 0;
    while (count < nb)
        for (i32 b = 0; b < nb; b++) {
            if (done[b]) continue;
            const i32 par = bones[b].parent;
            if (par < 0) { done[b] = 1; count++; }
            else if (done[par]) { f32 r[16]; pmul(global + b * 16, global + par * 16, r); memcpy(global + b * 16, r, 64); done[b] = 1; count++; }
        }
    for (i32 b = 0; b < nb; b++) pmul(bones[b].inv, global + b * 16, posed + b * 16);
}

/* Evaluates every request of a pose blob; out receives per request bones x 16 posed floats
 * followed by bones x 16 global floats.  Returns the request count, or a negative error. */
int sfto_pose_eval(const uint8_t* blob, uint64_t size, float* out, uint64_t out_floats) {
    const uint8_t* p = blob; const uint8_t* e = blob + size;
#define TAKE(n) ((size_t)(e - p) >= (size_t)(n) ? (p += (n), p - (n)) : NULL)
    const uint8_t* q = TAKE(8);
    if (!q || memcmp(q, "SFTP", 4)) return -1;
    u32 nb; memcpy(&nb, q + 4, 4);
    if (nb == 0 || nb > 128) return -2;
    const opbone* bones = (const opbone*)TAKE((size_t)nb * sizeof(opbone));
    q = TAKE(4); if (!q || !bones) return -3;
    u32 na; memcpy(&na, q, 4);
    opanim* an = (opanim*)calloc(na + 1, sizeof(opanim));
    for (u32 a = 0; a < na; a++) {
        q = TAKE(12); if (!q) { free(an); return -4; }
        memcpy(&an[a].duration, q, 4); memcpy(&an[a].ns, q + 4, 4); memcpy(&an[a].nc, q + 8, 4);
        an[a].smp = (opsmp*)calloc(an[a].ns + 1, sizeof(opsmp));
        for (u32 k = 0; k < an[a].ns; k++) {
            q = TAKE(8); if (!q) return -5;
            memcpy(&an[a].smp[k].count, q, 4); memcpy(&an[a].smp[k].is_step, q + 4, 4);
            an[a].smp[k].in = (const f32*)TAKE(an[a].smp[k].count * 4);
            an[a].smp[k].out = (const f32*)TAKE(an[a].smp[k].count * 16);
            if (!an[a].smp[k].in || !an[a].smp[k].out || !an[a].smp[k].count) return -6;
        }
        an[a].ch = (opch*)TAKE(an[a].nc * sizeof(opch));
        if (an[a].nc && !an[a].ch) return -7;
    }
    q = TAKE(4); if (!q) return -8;
    u32 nr; memcpy(&nr, q, 4);
    const uint8_t* rq = TAKE((size_t)nr * 8);
    if (!rq || out_floats < (uint64_t)nr * nb * 32) return -9;
    for (u32 r = 0; r < nr; r++) {
        i32 ai; f32 t; memcpy(&ai, rq + 8 * r, 4); memcpy(&t, rq + 8 * r + 4, 4);
        if (ai < 0 || (u32)ai >= na) continue;
        pose_update(bones, (i32)nb, &an[ai], t, out + (size_t)r * nb * 32, out + (size_t)r * nb * 32 + (size_t)nb * 16);
    }
    for (u32 a = 0; a < na; a++) free(an[a].smp);
    free(an);
#undef TAKE
    return (int)nr;
}

/* ------------------------------------------------------------ ray queries
 * sft_raycast_instance (sofren2.c:3733-3837) and sft__intersect_triangle (3705-3731): the ray is
 * taken into model space by sft_m_qinv of the instance transform and sft_m_mul_vec, which adds
 * no translation (the reference's behaviour, kept), the direction is normalised and the distance
 * limit scaled by its length, and the BLAS is walked depth first from a stack (children in slot
 * order, inner children pushed, leaf triangles tested in place).  A hit shortens the limit, so
 * among equal distances the first triangle found wins.  Records: ray = transform[16], origin[3],
 * dir[3], max_dist, model (96 B); hit = hit, distance, pos[3], normal[3] (32 B). */
typedef struct { f32 T[4][4]; f32 o[3], d[3]; f32 max_dist; i32 model; } oray;
typedef struct { u32 hit; f32 dist; f32 pos[3]; f32 nrm[3]; } ohit;

static int ray_tri(vec3 ro, vec3 rd, vec3 v0, vec3 v1, vec3 v2, f32* t) {   /* sft__intersect_triangle */
    const vec3 e1 = vsub(v1, v0), e2 = vsub(v2, v0), p = scross(rd, e2);
    const f32 det = sdot(e1, p);
    if (fabsf(det) < EPS) return 0;
    const f32 inv = 1.f / det;
    const vec3 tv = vsub(ro, v0);
    const f32 u = sdot(tv, p) * inv;
    if (u < 0.f || u > 1.f) return 0;
    const vec3 q = scross(tv, e1);
    const f32 v = sdot(rd, q) * inv;
    if (v < 0.f || u + v > 1.f) return 0;
    *t = sdot(e2, q) * inv;
    return *t > EPS;
}

static vec3 rot3(const f32 m[4][4], vec3 v) {   /* sft_m_mul_vec (1679): rows 0-2 only */
    vec3 r = { v.x * m[0][0] + v.y * m[1][0] + v.z * m[2][0], v.x * m[0][1] + v.y * m[1][1] + v.z * m[2][1],
               v.x * m[0][2] + v.y * m[1][2] + v.z * m[2][2] };
    return r;
}

static f32 ray_inv(f32 d) { return 1.f / (fabsf(d) > EPS ? d : EPS * (f32)(d < 0 ? -1 : 1)); }

static ohit raycast_one(const omodel* m, const oray* r) {
    ohit h;
    memset(&h, 0, sizeof(h));
    h.dist = r->max_dist;
    if (!m->blas_count) return h;
    f32 inv[4][4];   /* sft_m_qinv (1693-1711) */
    for (int i = 0; i < 3; i++) { for (int j = 0; j < 3; j++) inv[i][j] = r->T[j][i]; inv[i][3] = 0.f; }
    for (int j = 0; j < 3; j++) inv[3][j] = -(r->T[3][0] * inv[0][j] + r->T[3][1] * inv[1][j] + r->T[3][2] * inv[2][j]);
    inv[3][3] = 1.f;
    const vec3 o = { r->o[0], r->o[1], r->o[2] }, d = { r->d[0], r->d[1], r->d[2] };
    const vec3 lo = rot3(inv, o);
    vec3 ld = rot3(inv, d);
    const f32 inv_scale = 1.f / sqrtf(ld.x * ld.x + ld.y * ld.y + ld.z * ld.z);
    ld = vscale(ld, inv_scale);
    const f32 ix = ray_inv(ld.x), iy = ray_inv(ld.y), iz = ray_inv(ld.z);
    u32 stack[256];
    i32 sp = 0;
    stack[sp++] = m->blas_root;
    f32 lmax = r->max_dist / inv_scale;
    const onode* nodes = (const onode*)m->blas;
    while (sp > 0) {
        const onode* n = &nodes[stack[--sp]];
        for (u32 c = 0; c < n->count; c++) {
            if (n->child[c] == 0xFFFFFFFFu) continue;
            const f32 tx1 = (n->mn[0][c] - lo.x) * ix, tx2 = (n->mx[0][c] - lo.x) * ix;
            const f32 ty1 = (n->mn[1][c] - lo.y) * iy, ty2 = (n->mx[1][c] - lo.y) * iy;
            const f32 tz1 = (n->mn[2][c] - lo.z) * iz, tz2 = (n->mx[2][c] - lo.z) * iz;
#define RMIN(a, b) ((a) < (b) ? (a) : (b))
#define RMAX(a, b) ((a) > (b) ? (a) : (b))
            const f32 tmin = RMAX(RMAX(RMIN(tx1, tx2), RMIN(ty1, ty2)), RMIN(tz1, tz2));
            const f32 tmax = RMIN(RMIN(RMAX(tx1, tx2), RMAX(ty1, ty2)), RMAX(tz1, tz2));
#undef RMIN
#undef RMAX
            if (!(tmax >= tmin && tmax > 0.f && tmin < lmax)) continue;
            if (!n->leaf) { if (sp < 256) stack[sp++] = n->child[c]; continue; }
            const u32 pay = n->child[c] & ~0x80000000u, mi = pay >> 7, tri = pay & 127u;
            const sfts_meshlet* ml = m->ml[mi];
            const u32 off = (tri / 8) * 32, lane = tri % 8;
            const u8 i0 = ml->inds[off + lane], i1 = ml->inds[off + 8 + lane], i2 = ml->inds[off + 16 + lane];
            const f32* X = ml->attr;
            const vec3 v0 = { X[i0], X[64 + i0], X[128 + i0] }, v1 = { X[i1], X[64 + i1], X[128 + i1] }, v2 = { X[i2], X[64 + i2], X[128 + i2] };
            f32 t;
            if (ray_tri(lo, ld, v0, v1, v2, &t) && t < lmax) {
                lmax = t;
                h.hit = 1;
                h.dist = t * inv_scale;
                const vec3 lh = vadd(lo, vscale(ld, t));
                const vec3 ln = snorm(scross(vsub(v1, v0), vsub(v2, v0)));   /* sft_v_face_normal */
                const vec3 wp = rot3(r->T, lh), wn = snorm(rot3(r->T, ln));
                h.pos[0] = wp.x; h.pos[1] = wp.y; h.pos[2] = wp.z;
                h.nrm[0] = wn.x; h.nrm[1] = wn.y; h.nrm[2] = wn.z;
            }
        }
    }
    return h;
}

/* rays (96 B records) against the scene's models; returns 0, or -1 for a bad model index */
int sfto_raycast(void* hp, const void* rays, uint32_t n, void* hits) {
    oracle_handle* h = (oracle_handle*)hp;
    if (!h) return -1;
    const oray* R = (const oray*)rays;
    ohit* H = (ohit*)hits;
    for (uint32_t k = 0; k < n; k++) {
        if (R[k].model < 0 || (uint32_t)R[k].model >= h->sc.n_models) return -1;
        H[k] = raycast_one(&h->c.models[R[k].model], &R[k]);
    }
    return 0;
}

/* BLAS of model `mi` as sft_bvh_node images (256 B each): copies up to cap nodes into out and
 * returns the node count; *root receives the root index */
int sfto_model_blas(void* hp, uint32_t mi, uint8_t* out, uint32_t cap, uint32_t* root) {
    oracle_handle* h = (oracle_handle*)hp;
    if (!h || mi >= h->sc.n_models) return -1;
    const omodel* m = &h->c.models[mi];
    if (out) memcpy(out, m->blas, (size_t)(m->blas_count < cap ? m->blas_count : cap) * 256);
    if (root) *root = m->blas_root;
    return (int)m->blas_count;
}

/* Builds model `mi`'s BLAS again `reps` times from its meshlets (the timed CPU side of the BLAS
 * builder's measurement); returns the node count of the last build. */
int sfto_blas_rebuild(void* hp, uint32_t mi, uint32_t reps) {
    oracle_handle* h = (oracle_handle*)hp;
    if (!h || mi >= h->sc.n_models) return -1;
    omodel* m = &h->c.models[mi];
    for (uint32_t r = 0; r < reps; r++) {
        free(m->blas); m->blas = NULL; m->blas_count = 0;
        blas_build(m);
    }
    return (int)m->blas_count;
}

/* The capsule shadows of `frame` at `samples` evaluated in double beside the FP32 restatement
 * (one thread): out[0] the largest |FP32 - FP64| shadow intensity, out[1] the mean, out[2] the
 * number of pixel x light evaluations, out[3] how many differ by more than 1e-5. */
int sfto_shadow_fp64(void* hp, uint32_t frame, int samples, double* out) {
    oracle_handle* h = (oracle_handle*)hp;
    if (!h || !out || frame >= h->sc.n_frames || !(samples == 1 || samples == 2 || samples == 4)) return -1;
    h->c.fp64 = 1; h->c.fp64_max = 0.0; h->c.fp64_sum = 0.0; h->c.fp64_n = 0; h->c.fp64_big = 0;
    const int rc = render_frame(&h->c, frame, samples, 1, NULL, NULL, NULL);
    h->c.fp64 = 0;
    out[0] = h->c.fp64_max; out[1] = h->c.fp64_n ? h->c.fp64_sum / (double)h->c.fp64_n : 0.0;
    out[2] = (double)h->c.fp64_n; out[3] = (double)h->c.fp64_big;
    return rc;
}

/* enum sft_debug_mode for the following renders (0 = none) */
int sfto_set_debug_mode(void* hp, int mode) {
    oracle_handle* h = (oracle_handle*)hp;
    if (!h || mode < 0 || mode > 5) return -1;
    h->c.debug_mode = mode;
    return 0;
}

void sfto_close(void* hp) { free(hp); }

#ifdef SFT_ORACLE_MAIN
int main(int argc, char** argv) {
    if (argc < 4) { fprintf(stderr, "usage: %s scene.sfts out.dump samples [threads] [frame]\n", argv[0]); return 2; }
    sfts_scene sc;
    if (sfts_load_file(&sc, argv[1])) { fprintf(stderr, "bad scene\n"); return 3; }
    const int S = atoi(argv[3]);
    const int threads = argc > 4 ? atoi(argv[4]) : 1;
    const int only = argc > 5 ? atoi(argv[5]) : -1;
    octx c; load_scene(&c, &sc);
    {
        sfts_dump d = { fopen(argv[2], "wb") };
        for (u32 i = 0; i < sc.n_models; i++) sfts_dump_section(&d, "blas", "u8", c.models[i].blas, (u64)c.models[i].blas_count * 256);
        fclose(d.f);
    }
    for (u32 fi = 0; fi < sc.n_frames; fi++) {
        if (only >= 0 && (u32)only != fi) continue;
        ostats st;
        if (render_frame(&c, fi, S, threads, argv[2], NULL, &st)) return 4;
        fprintf(stderr, "frame %u: %.3f ms (geom %.3f, tiles %.3f) invalid_packets %u\n", fi, st.ns_total / 1e6, st.ns_geom / 1e6, st.ns_tiles / 1e6, st.invalid_packets);
    }
    return 0;
}
#endif
