/*
 * Per-tile raster and resolve (sft__worker_phase_rasterize, sofren2.c:6756-6813,
 * sft__rast_simd_batch 5148-5499, sft__resolve_tile 5809-6753).
 *
 * k_raster: one to four CTAs per 64x64 tile, each owning a band of its rows (more for tiles with
 * more payloads; every CTA sets up the tile's whole list and keeps the triangles that reach its
 * band, whose rows it walks from the triangle's first row exactly as the one-CTA walk would).
 * The reference walks the tile's list in order and keeps a
 * sample when z > stored z (strict), so a sample ends holding the largest z, and among equal z
 * the earliest triangle.  That final state does not depend on the order triangles are visited,
 * so each sample is a 64-bit shared-memory word (z bits << 32 | ~order) updated with atomicMax,
 * where order = list position * 8 + lane; only z > 0 ever wins (the buffer starts at 0).
 * Coverage and z are replayed bit-exactly: a group of 8 threads takes one triangle, thread l
 * owns pixel column l of every aligned 8-pixel chunk and performs exactly the reference's
 * incremental adds (row start + B per row, + 8A per chunk) and its trivial-accept / AA
 * guard-band choices; the AA chunk skip is a group ballot.  The decoded visibility buffer
 * (depth, vid) goes to global memory, where it stays L2-resident, with the tile's depth range.
 *
 * k_resolve: 1 to 16 CTAs per tile (a tuning knob per sample count), each a share of its 4x2
 * blocks, small shared memory for high occupancy.  A group of 8 threads is one 4x2 block (the reference's AVX2 lanes).  For
 * each distinct triangle in the block (peeled in the reference's order) all 8 lanes shade it,
 * because the reference's LOD uses the first covered lane's screen derivatives (neighbour
 * lanes via shuffles) and its proxy loop skips a proxy for the whole block when no lane is
 * affected (a ballot), which changes the smooth-max shadow of every lane.
 */
#include "sftg_types.h"
#include "sftg_lane.cuh"
#include "sftg_kernels.h"

#define TILE_THREADS 256          /* resolve CTA */
#define RASTER_THREADS 512        /* raster CTA: 64 groups of 8 */
/* A tile is rastered by 1, 2 or 4 CTAs, each owning a band of its rows, by its payload count: the
 * frame's raster time is set by its heaviest tiles, which one CTA would walk alone. */
#define RASTER_BANDS 4            /* raster CTAs launched per tile; those past the tile's band count exit */
#define BANDS2_ABOVE 48           /* payloads above which a tile gets 2 bands */
#define BANDS4_ABOVE 128          /* and 4 (1x and 2x; measured: at 4x two bands are best for every tile) */
/* keys of one sample plane in shared memory: a whole tile, except at 4x, where every tile takes at
 * least 2 bands so that the keys (S x 32 KB per tile) leave room for 2 CTAs per SM */
template <int S> struct raster_plan {
    static constexpr int min_bands = S == 4 ? 2 : 1, plane = SFTG_TILE_PX / min_bands, rows = SFTG_TILE / min_bands;
};
#define SETUP_CAP RASTER_THREADS  /* triangle set-ups per round: one per thread */
#define MIN_SLAB_ROWS 4           /* smallest raster work item (rows); the slab height is a tuning knob */

struct tri_setup {
    float A[3], B[3], se[3];
    float sz, dzdx, dzdy;
    float pad[3];
    int ax0, ax1, miny, maxy;
    uint32_t order;
    int trivial;
};

/* tri_setup as kept in shared memory (56 B): the guard-band pads are recomputed from A and B,
 * the bounds are tile-local bytes (0..64) and the trivial-accept flag rides in order's top bit
 * (order = list position * 8 + lane stays below 2^31) */
struct tri_setup_packed {
    float A[3], B[3], se[3];
    float sz, dzdx, dzdy;
    uint32_t bounds;       /* ax0 | ax1 << 8 | miny << 16 | maxy << 24, tile-local */
    uint32_t order_triv;
};

SFTG_D tri_setup_packed pack_setup(const tri_setup& T, int tmx, int tmy) {
    tri_setup_packed P;
#pragma unroll
    for (int k = 0; k < 3; k++) { P.A[k] = T.A[k]; P.B[k] = T.B[k]; P.se[k] = T.se[k]; }
    P.sz = T.sz; P.dzdx = T.dzdx; P.dzdy = T.dzdy;
    P.bounds = (uint32_t)(T.ax0 - tmx) | ((uint32_t)(T.ax1 - tmx) << 8) | ((uint32_t)(T.miny - tmy) << 16) | ((uint32_t)(T.maxy - tmy) << 24);
    P.order_triv = T.order | (T.trivial ? 0x80000000u : 0u);
    return P;
}

template <int S>
SFTG_D tri_setup unpack_setup(const tri_setup_packed& P, int tmx, int tmy) {
    tri_setup T;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        T.A[k] = P.A[k]; T.B[k] = P.B[k]; T.se[k] = P.se[k];
        T.pad[k] = S > 1 ? 0.375f * (fabsf(P.A[k]) + fabsf(P.B[k])) : 0.f;   /* as in tri_setup_one */
    }
    T.sz = P.sz; T.dzdx = P.dzdx; T.dzdy = P.dzdy;
    T.ax0 = tmx + (int)(P.bounds & 0xFFu); T.ax1 = tmx + (int)((P.bounds >> 8) & 0xFFu);
    T.miny = tmy + (int)((P.bounds >> 16) & 0xFFu); T.maxy = tmy + (int)(P.bounds >> 24);
    T.order = P.order_triv & 0x7FFFFFFFu; T.trivial = (int)(P.order_triv >> 31);
    return T;
}

struct proxy_cache {   /* sft_light_proxy_cache (sofren2.c:991-998) */
    float pa[3], pb[3], ab[3], W[3];
    float abdab, wdw, rb2, pr, pr2, vis_mult;
};

struct tri_verts {
    float sx[3], sy[3], iw[3], u[3], v[3], lu[3], lv[3], px[3], py[3], pz[3], nx[3], ny[3], nz[3];
    uint32_t inst, m;
};

__constant__ float c_ms_ox4[4] = { -0.125f, 0.375f, -0.375f, 0.125f };
__constant__ float c_ms_oy4[4] = { -0.375f, -0.125f, 0.125f, 0.375f };
__constant__ float c_ms_ox2[2] = { -0.25f, 0.25f };
__constant__ float c_ms_oy2[2] = { -0.25f, 0.25f };

template <int S> SFTG_D float ms_ox(int s) { return S == 4 ? c_ms_ox4[s] : (S == 2 ? c_ms_ox2[s] : 0.f); }
template <int S> SFTG_D float ms_oy(int s) { return S == 4 ? c_ms_oy4[s] : (S == 2 ? c_ms_oy2[s] : 0.f); }

/* a tile's depth range (1/w of its samples above 1e-4): the union of its raster bands' ranges */
SFTG_D float2 tile_zrange(const float2* zr, uint32_t gtile) {
    float2 r = zr[(size_t)gtile * RASTER_BANDS];
#pragma unroll
    for (int b = 1; b < RASTER_BANDS; b++) { const float2 q = zr[(size_t)gtile * RASTER_BANDS + b]; r.x = fminf(r.x, q.x); r.y = fmaxf(r.y, q.y); }
    return r;
}

SFTG_D uint64_t zkey(float z, uint32_t order) { return ((uint64_t)__float_as_uint(z) << 32) | (uint64_t)(0xFFFFFFFFu - order); }

/* vertices of one vis id (sofren2.c:5163-5209, 6199-6278) */
SFTG_D void fetch_tri(const sftg_frame* F, const float* ss, const sftg_clip_tri* clips, uint32_t vid, tri_verts& t) {
    if (vid & 0x80000000u) {
        const sftg_clip_tri* c = &clips[vid & 0x7FFFFFFFu];
        const float* src = c->sx; float* dst = t.sx;
#pragma unroll
        for (int i = 0; i < 39; i++) dst[i] = src[i];
        t.inst = c->inst; t.m = c->m;
        return;
    }
    const uint32_t ii = (vid >> 25) & 63, m = (vid >> 7) & 0x3FFFF, tri = vid & 127;
    const sftg_inst* I = &F->inst[ii];
    const uint32_t g = I->meshlet_base + m;
    const uint8_t* ind = F->ml_inds + (size_t)g * 512;
    const float* at = F->ml_attr + (size_t)g * 640;
    const float* Sc = ss + (size_t)(I->ss_offset + m) * SFTG_SS_FLOATS;
    const uint32_t b = tri >> 3, l = tri & 7;
    const uint32_t q[3] = { ind[b * 32 + l], ind[b * 32 + 8 + l], ind[b * 32 + 16 + l] };
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const uint32_t v = q[k];
        const float4 a = ((const float4*)(Sc + SFTG_SS_A))[v], b4 = ((const float4*)(Sc + SFTG_SS_B))[v];
        const float4 c4 = ((const float4*)(Sc + SFTG_SS_C))[v];
        t.sx[k] = a.x; t.sy[k] = a.y; t.iw[k] = a.z;
        t.u[k] = c4.y; t.v[k] = c4.z; t.lu[k] = c4.w; t.lv[k] = Sc[SFTG_SS_D + v];
        t.px[k] = a.w; t.py[k] = b4.x; t.pz[k] = b4.y;
        t.nx[k] = b4.z; t.ny[k] = b4.w; t.nz[k] = c4.x;
    }
    t.inst = ii; t.m = m;
}

/* Grows [mn, mx] by the world position the resolve interpolates on triangle `vid` at pixel
 * centre (pxf, pyf): the same barycentrics, MSAA clamp, perspective weights and interpolation as
 * the shading loop (D6 below), so the box holds exactly the points the proxy tests use. */
template <int S>
SFTG_D void pixel_pos_acc(const sftg_frame* F, const float* ss, const sftg_clip_tri* clips, uint32_t vid, float pxf, float pyf,
                          float* mn, float* mx) {
    float sx[3], sy[3], iw[3], px[3], py[3], pz[3];
    if (vid & 0x80000000u) {
        const sftg_clip_tri* c = &clips[vid & 0x7FFFFFFFu];
#pragma unroll
        for (int k = 0; k < 3; k++) { sx[k] = c->sx[k]; sy[k] = c->sy[k]; iw[k] = c->iw[k]; px[k] = c->px[k]; py[k] = c->py[k]; pz[k] = c->pz[k]; }
    } else {
        const uint32_t ii = (vid >> 25) & 63, m = (vid >> 7) & 0x3FFFF, tri = vid & 127;
        const sftg_inst* I = &F->inst[ii];
        const uint32_t g = I->meshlet_base + m;
        const uint8_t* ind = F->ml_inds + (size_t)g * 512;
        const float* Sc = ss + (size_t)(I->ss_offset + m) * SFTG_SS_FLOATS;
        const uint32_t b = tri >> 3, l = tri & 7;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const uint32_t v = ind[b * 32 + 8 * k + l];
            const float4 a = ((const float4*)(Sc + SFTG_SS_A))[v], b4 = ((const float4*)(Sc + SFTG_SS_B))[v];
            sx[k] = a.x; sy[k] = a.y; iw[k] = a.z; px[k] = a.w; py[k] = b4.x; pz[k] = b4.y;
        }
    }
    const float dx1 = sx[1] - sx[0], dx2 = sx[2] - sx[0], dy1 = sy[1] - sy[0], dy2 = sy[2] - sy[0];
    const float idet = rcpr(dx1 * dy2 - dx2 * dy1);
    const float pxs = pxf - sx[0], pys = pyf - sy[0];
    const float rbu = (pxs * dy2 - pys * dx2) * idet;
    const float rbv = (pys * dx1 - pxs * dy1) * idet;
    const float rbw = (1.f - rbu) - rbv;
    float bu = rbu, bv = rbv, bw = rbw;
    if (S > 1) {
        bu = vmax(0.f, rbu); bv = vmax(0.f, rbv); bw = vmax(0.f, rbw);
        const float bs = rcpr(bu + (bv + bw));
        bu = bu * bs; bv = bv * bs; bw = bw * bs;
    }
    const float iz = fma_(bw, iw[0], fma_(bu, iw[1], bv * iw[2]));
    const float z = rcpr(iz);
    const float w0 = (bw * iw[0]) * z, w1 = (bu * iw[1]) * z, w2 = (bv * iw[2]) * z;
    const float P[3] = { fma_(w0, px[0], fma_(w1, px[1], w2 * px[2])), fma_(w0, py[0], fma_(w1, py[1], w2 * py[2])),
                         fma_(w0, pz[0], fma_(w1, pz[1], w2 * pz[2])) };
#pragma unroll
    for (int a = 0; a < 3; a++) { mn[a] = fminf(mn[a], P[a]); mx[a] = fmaxf(mx[a], P[a]); }
}

/* edge / depth setup of one triangle lane (5211-5311), false when culled or off-tile */
template <int S>
SFTG_D bool tri_setup_one(float sx0, float sy0, float iw0, float sx1, float sy1, float iw1, float sx2, float sy2, float iw2,
                          int tmx, int tmy, uint32_t order, tri_setup& T) {
    const float A0 = sy0 - sy1, B0 = sx1 - sx0, A1 = sy1 - sy2, B1 = sx2 - sx1, A2 = sy2 - sy0, B2 = sx0 - sx2;
    const float m01 = sx0 * sy1, m10 = sy0 * sx1, m12 = sx1 * sy2, m21 = sy1 * sx2, m20 = sx2 * sy0, m02 = sy2 * sx0;
    const float C0 = (fma_(sx0, sy1, -m10) - fma_(sy0, sx1, -m01)) * 0.5f;
    const float C1 = (fma_(sx1, sy2, -m21) - fma_(sy1, sx2, -m12)) * 0.5f;
    const float C2 = (fma_(sx2, sy0, -m02) - fma_(sy2, sx0, -m20)) * 0.5f;
    const float dx1 = sx1 - sx0, dx2 = sx2 - sx0, dy1 = sy1 - sy0, dy2 = sy2 - sy0;
    const float det = dx1 * dy2 - dx2 * dy1;
    if (!(det > 1e-6f)) return false;
    const float idet = rcpr(det);
    const float dzdx = ((iw1 - iw0) * dy2 - (iw2 - iw0) * dy1) * idet;
    const float dzdy = ((iw2 - iw0) * dx1 - (iw1 - iw0) * dx2) * idet;
    const float c0 = fma_(B0, 0.5f, fma_(A0, 0.5f, C0)), c1 = fma_(B1, 0.5f, fma_(A1, 0.5f, C1)), c2 = fma_(B2, 0.5f, fma_(A2, 0.5f, C2));
    const float zb = fma_(0.5f - sy0, dzdy, fma_(0.5f - sx0, dzdx, iw0));
    const int minx = cvtt(vmax(vmin(sx0, vmin(sx1, sx2)), (float)tmx));
    const int maxx = cvtt(vmin(vmax(sx0, vmax(sx1, sx2)), (float)(tmx + SFTG_TILE - 1)));
    const int miny = cvtt(vmax(vmin(sy0, vmin(sy1, sy2)), (float)tmy));
    const int maxy = cvtt(vmin(vmax(sy0, vmax(sy1, sy2)), (float)(tmy + SFTG_TILE - 1)));
    if (minx > maxx || miny > maxy) return false;
    const int ax0 = minx & ~7, ax1 = (maxx & ~7) + 8;
    T.A[0] = A0; T.A[1] = A1; T.A[2] = A2; T.B[0] = B0; T.B[1] = B1; T.B[2] = B2;
    T.se[0] = c0 + A0 * (float)ax0 + B0 * (float)miny;
    T.se[1] = c1 + A1 * (float)ax0 + B1 * (float)miny;
    T.se[2] = c2 + A2 * (float)ax0 + B2 * (float)miny;
    T.sz = zb + dzdx * (float)ax0 + dzdy * (float)miny;
    T.dzdx = dzdx; T.dzdy = dzdy;
    const float bw = (float)(ax1 - 1 - ax0), bh = (float)(maxy - miny);
    const float me0 = T.se[0] + (A0 < 0.f ? A0 * bw : 0.f) + (B0 < 0.f ? B0 * bh : 0.f);
    const float me1 = T.se[1] + (A1 < 0.f ? A1 * bw : 0.f) + (B1 < 0.f ? B1 * bh : 0.f);
    const float me2 = T.se[2] + (A2 < 0.f ? A2 * bw : 0.f) + (B2 < 0.f ? B2 * bh : 0.f);
    if (S > 1) {
        T.pad[0] = 0.375f * (fabsf(A0) + fabsf(B0));
        T.pad[1] = 0.375f * (fabsf(A1) + fabsf(B1));
        T.pad[2] = 0.375f * (fabsf(A2) + fabsf(B2));
        T.trivial = (me0 >= T.pad[0] && me1 >= T.pad[1] && me2 >= T.pad[2]);
    } else {
        T.pad[0] = T.pad[1] = T.pad[2] = 0.f;
        T.trivial = (me0 >= 0.f && me1 >= 0.f && me2 >= 0.f);
    }
    T.ax0 = ax0; T.ax1 = ax1; T.miny = miny; T.maxy = maxy; T.order = order;
    return true;
}

/* the incremental edge walk for pixel column `l` of one triangle (5345-5497) */
template <int S>
SFTG_D void tri_raster(const tri_setup& T, int y0, int y1, int l, uint32_t gmask, int tmx, int ky0, unsigned long long* keys) {
    float de0[S], de1[S], de2[S], dz[S];
#pragma unroll
    for (int s = 0; s < S; s++) {
        const float ox = ms_ox<S>(s), oy = ms_oy<S>(s);
        de0[s] = T.A[0] * ox + T.B[0] * oy; de1[s] = T.A[1] * ox + T.B[1] * oy; de2[s] = T.A[2] * ox + T.B[2] * oy;
        dz[s] = T.dzdx * ox + T.dzdy * oy;
    }
    const float fl = (float)l;
    float e0r = T.se[0] + T.A[0] * fl, e1r = T.se[1] + T.A[1] * fl, e2r = T.se[2] + T.A[2] * fl;
    float zr = T.sz + T.dzdx * fl;
    /* a slab starting below miny replays the per-row adds it skips, so every row start is the
     * same float the reference's sequential walk reaches */
    for (int y = T.miny; y < y0; y++) { e0r = e0r + T.B[0]; e1r = e1r + T.B[1]; e2r = e2r + T.B[2]; zr = zr + T.dzdy; }
    const float a0c = T.A[0] * 8.f, a1c = T.A[1] * 8.f, a2c = T.A[2] * 8.f, zc = T.dzdx * 8.f;
    const float np0 = -T.pad[0], np1 = -T.pad[1], np2 = -T.pad[2];
    const uint32_t order = T.order;
    for (int y = y0; y <= y1; y++) {
        float e0 = e0r, e1 = e1r, e2 = e2r, z = zr;
        int pi = (y - ky0) * SFTG_TILE + (T.ax0 - tmx) + l;   /* keys hold the band's rows from ky0 */
        for (int x = T.ax0; x < T.ax1; x += 8, pi += 8) {
            if (T.trivial) {
#pragma unroll
                for (int s = 0; s < S; s++) {
                    const float zs = (S > 1) ? z + dz[s] : z;
                    if (zs > 0.f) atomicMax(&keys[s * raster_plan<S>::plane + pi], zkey(zs, order));
                }
            } else if (S == 1) {
                if (e0 >= 0.f && e1 >= 0.f && e2 >= 0.f && z > 0.f) atomicMax(&keys[pi], zkey(z, order));
            } else {
                const bool might = (e0 >= np0 && e1 >= np1 && e2 >= np2);
                if (__ballot_sync(gmask, might) & gmask) {
#pragma unroll
                    for (int s = 0; s < S; s++) {
                        const float a = e0 + de0[s], b = e1 + de1[s], c = e2 + de2[s];
                        if (a >= 0.f && b >= 0.f && c >= 0.f) {
                            const float zs = z + dz[s];
                            if (zs > 0.f) atomicMax(&keys[s * raster_plan<S>::plane + pi], zkey(zs, order));
                        }
                    }
                }
            }
            e0 = e0 + a0c; e1 = e1 + a1c; e2 = e2 + a2c; z = z + zc;
        }
        e0r = e0r + T.B[0]; e1r = e1r + T.B[1]; e2r = e2r + T.B[2]; zr = zr + T.dzdy;
    }
}

/* ---------------------------------------------------------------- texture sampling */
SFTG_D uint32_t tex_addr(const sftg_tex& t, int lod, int u, int v) {
    const uint32_t uu = (uint32_t)u, vv = (uint32_t)v;
    if (t.is_pot) return ((((vv >> 2) << t.shift[lod]) + (uu >> 2)) << 4) + ((vv & 3u) << 2) + (uu & 3u);
    return ((((vv >> 2) * (uint32_t)t.bw[lod]) + (uu >> 2)) << 4) + ((vv & 3u) << 2) + (uu & 3u);
}

/* sft__sample_tex_bilinear (5543-5660) */
SFTG_D void sample_bilinear(const sftg_frame* F, int ti, int lod, float cu, float cv, float& r, float& g, float& b) {
    if (ti < 0) { r = g = b = 1.f; return; }
    const sftg_tex& t = F->texs[ti];
    const int w = max(t.w >> lod, 1), h = max(t.h >> lod, 1);
    const float upx = cu * (float)w - 0.5f, vpx = cv * (float)h - 0.5f;
    const float uf0 = floorf(upx), vf0 = floorf(vpx);
    const float ufr = upx - uf0, vfr = vpx - vf0;
    const int u0 = cvtt(uf0), v0 = cvtt(vf0);
    const int wm = w - 1, hm = h - 1;
    int u0w, v0w, u1, v1;
    if (t.is_pot) { u1 = (u0 + 1) & wm; v1 = (v0 + 1) & hm; u0w = u0 & wm; v0w = v0 & hm; }
    else {   /* the reference has no lower clamp here (it reads outside the texture); clamp at 0 */
        u1 = max(0, min(u0 + 1, wm)); v1 = max(0, min(v0 + 1, hm)); u0w = max(0, min(u0, wm)); v0w = max(0, min(v0, hm));
    }
    const uint32_t* base = F->texels + t.offs[lod];
    const uint32_t c00 = __ldg(&base[tex_addr(t, lod, u0w, v0w)]), c10 = __ldg(&base[tex_addr(t, lod, u1, v0w)]);
    const uint32_t c01 = __ldg(&base[tex_addr(t, lod, u0w, v1)]), c11 = __ldg(&base[tex_addr(t, lod, u1, v1)]);
    const float i255 = 1.f / 255.f;
    float out[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int sh = 16 - 8 * k;
        const float f00 = (float)((c00 >> sh) & 255u) * i255, f10 = (float)((c10 >> sh) & 255u) * i255;
        const float f01 = (float)((c01 >> sh) & 255u) * i255, f11 = (float)((c11 >> sh) & 255u) * i255;
        const float top = f00 + (f10 - f00) * ufr, bot = f01 + (f11 - f01) * ufr;
        out[k] = top + (bot - top) * vfr;
    }
    r = out[0]; g = out[1]; b = out[2];
}

/* sft__sample_tex_nearest (5662-5729) */
SFTG_D void sample_nearest(const sftg_frame* F, int ti, int lod, float cu, float cv, float& r, float& g, float& b) {
    if (ti < 0) { r = g = b = 1.f; return; }
    const sftg_tex& t = F->texs[ti];
    const int w = max(t.w >> lod, 1), h = max(t.h >> lod, 1);
    const int u0 = cvtt(floorf(cu * (float)w)), v0 = cvtt(floorf(cv * (float)h));
    const int wm = w - 1, hm = h - 1;
    int uw, vw;
    if (t.is_pot) { uw = u0 & wm; vw = v0 & hm; } else { uw = max(0, min(u0, wm)); vw = max(0, min(v0, hm)); }
    const uint32_t c = __ldg(&F->texels[t.offs[lod] + tex_addr(t, lod, uw, vw)]);
    const float i255 = 1.f / 255.f;
    r = (float)((c >> 16) & 255u) * i255; g = (float)((c >> 8) & 255u) * i255; b = (float)(c & 255u) * i255;
}

/* ---------------------------------------------------------------- raster */
/* One (tile, band) item, run by one CTA: the tile's payload list into a shared-memory visibility
 * buffer (64-bit z/order words) for the band's rows, decoded into the global visibility buffer
 * (float2: depth, vid bits) plus the band's depth range over valid samples (sofren2.c:5820-5853),
 * which the resolve needs for its light culling (a tile's range is the union of its bands'). */
template <int S>
SFTG_D void raster_item(const sftg_tile_args& A, uint32_t tile0, int slab_rows, int fixed_bands, uint32_t item)
{
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned long long* keys = (unsigned long long*)smem;                  /* S planes, a band uses the first band_px of each */
    tri_setup_packed* setups = (tri_setup_packed*)(smem + (size_t)S * raster_plan<S>::plane * 8);
    uint32_t* items = (uint32_t*)(setups + SETUP_CAP);                     /* set-up index << 8 | slab */
    __shared__ uint32_t s_nsetup, s_nbig, s_nsmall, s_next;
    /* work items of a round: long slabs from the front of the array, short ones from the back,
     * and the queue hands out the long ones first, so that a round does not end on one group
     * still walking a long slab (items touch keys only through atomicMax: order is free) */
    const uint32_t items_cap = (uint32_t)SETUP_CAP * (uint32_t)((raster_plan<S>::rows + slab_rows - 1) / slab_rows);
    __shared__ float s_red[2][RASTER_THREADS / 32];
    const uint32_t gtile = A.tile_order[tile0 + item / RASTER_BANDS];   /* batch-wide tile index, heaviest first */
    const int band = (int)(item % RASTER_BANDS);
    const sftg_frame* F = A.frames + A.tile_view[gtile];
    const int tile = (int)(gtile - F->tile_base);
    const float* ss = A.ss + (size_t)F->ss_base * SFTG_SS_FLOATS;
    const sftg_clip_tri* clips = A.clips + (F->total_ss ? A.clip_base[(size_t)F->ss_base * 16] : 0u);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tmx = (tile % F->cols) * SFTG_TILE, tmy = (tile / F->cols) * SFTG_TILE;
    uint32_t count = A.tile_count[gtile];
    if ((uint64_t)A.tile_start[gtile] + count > F->tile_cap) count = 0;   /* overflowed frame, redone by the host */
    const int bands = max(raster_plan<S>::min_bands,
                          fixed_bands ? fixed_bands : ((S < 4 && count > BANDS4_ABOVE) ? 4 : (count > BANDS2_ABOVE ? 2 : 1)));
    if (band >= bands) {   /* not needed for this tile: an empty depth range for the readers' union */
        if (threadIdx.x == 0) A.zrange[(size_t)gtile * RASTER_BANDS + band] = make_float2(1e9f, -1e9f);
        return;
    }
    const int band_rows = SFTG_TILE / bands, band_px = band_rows * SFTG_TILE;
    const int by0 = tmy + band * band_rows, by1 = by0 + band_rows - 1;   /* this CTA's rows */
    const uint64_t* list = A.tile_pay + A.tile_start[gtile];
    float* vis_depth = A.vis_depth;
    uint32_t* vis_id = A.vis_id;

    for (int i = tid; i < S * band_px; i += RASTER_THREADS) keys[(i / band_px) * raster_plan<S>::plane + i % band_px] = 0ull;
    const int grp_lane = tid & 7;
    const uint32_t gmask = 0xFFu << (lane & ~7);
    /* the payloads in equal rounds of at most SETUP_CAP / 8 (a short last round would leave most
     * groups idle at its barrier) */
    const uint32_t rounds = (count + SETUP_CAP / 8 - 1) / (SETUP_CAP / 8);
    const uint32_t per_round = rounds ? (count + rounds - 1) / rounds : 1u;
    for (uint32_t pbase = 0; pbase < count; pbase += per_round) {
        const uint32_t pend = min(count, pbase + per_round);
        if (tid == 0) { s_nsetup = 0; s_nbig = 0; s_nsmall = 0; s_next = 0; }
        __syncthreads();
        {
            const uint32_t p = pbase + (tid >> 3);
            const int l = grp_lane;
            if (p < pend) {
                const uint64_t pay = list[p];
                const uint32_t raw = (uint32_t)(pay >> 56);
                float sx[3], sy[3], iw[3];
                bool active;
                if (!raw) {
                    active = (l == 0);
                    if (active) {
                        const sftg_clip_tri* c = &clips[(uint32_t)(pay & 0xFFFFFFFFu)];
#pragma unroll
                        for (int k = 0; k < 3; k++) { sx[k] = c->sx[k]; sy[k] = c->sy[k]; iw[k] = c->iw[k]; }
                    }
                } else {
                    active = (raw >> l) & 1u;
                    if (active) {
                        const uint32_t ii = (uint32_t)(pay & 0xFFFFFF), m = (uint32_t)((pay >> 24) & 0xFFFFFF), b = (uint32_t)((pay >> 48) & 0xFF);
                        const sftg_inst* I = &F->inst[ii];
                        const uint32_t g = I->meshlet_base + m;
                        const uint8_t* ind = F->ml_inds + (size_t)g * 512;
                        const float* Sc = ss + (size_t)(I->ss_offset + m) * SFTG_SS_FLOATS;
                        const uint32_t q[3] = { ind[b * 32 + l], ind[b * 32 + 8 + l], ind[b * 32 + 16 + l] };
#pragma unroll
                        for (int k = 0; k < 3; k++) { const float4 a = ((const float4*)(Sc + SFTG_SS_A))[q[k]]; sx[k] = a.x; sy[k] = a.y; iw[k] = a.z; }
                    }
                }
                if (active) {
                    tri_setup T;
                    /* the set-up is the whole tile's (bounds clamped to the 64x64 tile, edge values from
                     * its first row); the band keeps the triangles that reach its rows */
                    if (tri_setup_one<S>(sx[0], sy[0], iw[0], sx[1], sy[1], iw[1], sx[2], sy[2], iw[2], tmx, tmy, p * 8 + l, T) &&
                        T.maxy >= by0 && T.miny <= by1) {
                        const uint32_t slot = atomicAdd(&s_nsetup, 1u);
                        setups[slot] = pack_setup(T, tmx, tmy);
                        const int ys = max(T.miny, by0), ye = min(T.maxy, by1);
                        const uint32_t nslab = (uint32_t)(ye - ys) / (uint32_t)slab_rows + 1u;
                        const int rows = min(ye - ys + 1, slab_rows), chunks = (T.ax1 - T.ax0) >> 3;
                        if (S == 4 || rows * chunks >= 16) {   /* measured: the 4x raster keeps arrival order */
                            const uint32_t ib = atomicAdd(&s_nbig, nslab);
                            for (uint32_t k = 0; k < nslab; k++) items[ib + k] = (slot << 8) | k;
                        } else {
                            const uint32_t ib = atomicAdd(&s_nsmall, nslab);
                            for (uint32_t k = 0; k < nslab; k++) items[items_cap - 1u - (ib + k)] = (slot << 8) | k;
                        }
                    }
                }
            }
        }
        __syncthreads();
        const uint32_t nbig = s_nbig, nitem = nbig + s_nsmall;
        while (true) {
            uint32_t idx = 0;
            if (grp_lane == 0) idx = atomicAdd(&s_next, 1u);
            idx = __shfl_sync(gmask, idx, lane & ~7);
            if (idx >= nitem) break;
            const uint32_t it = idx < nbig ? items[idx] : items[items_cap - 1u - (idx - nbig)];
            const tri_setup T = unpack_setup<S>(setups[it >> 8], tmx, tmy);
            const int y0 = max(T.miny, by0) + (int)(it & 0xFFu) * slab_rows;   /* rows before y0 are replayed */
            const int y1 = min(y0 + slab_rows - 1, min(T.maxy, by1));
            tri_raster<S>(T, y0, y1, grp_lane, gmask, tmx, by0, keys);
        }
        __syncthreads();
    }
    __syncthreads();
    /* decode, store, depth range */
    float zmin = 1e9f, zmax = -1e9f;
    float2* tv = A.vis + F->vis_base + (size_t)tile * S * SFTG_TILE_PX;
    for (int i = tid; i < S * band_px; i += RASTER_THREADS) {
        const int sp = i / band_px, pp = i % band_px;
        const unsigned long long k = keys[sp * raster_plan<S>::plane + pp];
        const int ti = sp * SFTG_TILE_PX + band * band_px + pp;              /* the same sample in the tile */
        float d = 0.f; uint32_t vid = SFTG_INVALID;
        if (k) {
            d = __uint_as_float((uint32_t)(k >> 32));
            const uint32_t order = 0xFFFFFFFFu - (uint32_t)k;
            const uint64_t pay = list[order >> 3];
            if ((pay >> 56) == 0) vid = (uint32_t)pay | 0x80000000u;
            else vid = ((uint32_t)(pay & 0xFFFFFF) << 25) | ((uint32_t)((pay >> 24) & 0xFFFFFF) << 7) | ((uint32_t)((pay >> 48) & 0xFF) * 8 + (order & 7));
        }
        tv[ti] = make_float2(d, __uint_as_float(vid));
        if (vis_id) {
            vis_depth[(size_t)tile * S * SFTG_TILE_PX + ti] = d;
            vis_id[(size_t)tile * S * SFTG_TILE_PX + ti] = vid;
        }
        if (d > 0.0001f) { zmin = fminf(zmin, d); zmax = fmaxf(zmax, d); }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) { zmin = fminf(zmin, __shfl_xor_sync(0xFFFFFFFFu, zmin, o)); zmax = fmaxf(zmax, __shfl_xor_sync(0xFFFFFFFFu, zmax, o)); }
    if (lane == 0) { s_red[0][warp] = zmin; s_red[1][warp] = zmax; }
    __syncthreads();
    if (tid == 0) {
        zmin = 1e9f; zmax = -1e9f;
        for (int w = 0; w < RASTER_THREADS / 32; w++) { zmin = fminf(zmin, s_red[0][w]); zmax = fmaxf(zmax, s_red[1][w]); }
        A.zrange[(size_t)gtile * RASTER_BANDS + band] = make_float2(zmin, zmax);   /* combined by the readers */
    }
}

/* one CTA per (tile, band) item */
template <int S>
__global__ void __launch_bounds__(RASTER_THREADS)
k_raster(const sftg_tile_args A, uint32_t tile0, int slab_rows, int fixed_bands)
{
    raster_item<S>(A, tile0, slab_rows, fixed_bands, blockIdx.x);
}

/* Persistent form: as many CTAs as fit on the GPU at once, each taking the next (tile, band) item
 * in launch order (heaviest tiles first) from a counter until all n_items are taken.  The loop
 * ends after at most n_items + grid counter reads: nothing waits on another CTA. */
template <int S>
__global__ void __launch_bounds__(RASTER_THREADS, 2)   /* the 64 registers k_raster gets: 2 CTAs per SM */
k_raster_queue(const sftg_tile_args A, uint32_t tile0, int slab_rows, int fixed_bands, uint32_t n_items, uint32_t* next)
{
    __shared__ uint32_t s_item;
    for (;;) {
        __syncthreads();   /* the previous item is done with shared memory, and s_item has been read */
        if (threadIdx.x == 0) s_item = atomicAdd(next, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= n_items) break;
        raster_item<S>(A, tile0, slab_rows, fixed_bands, item);
    }
}

/* ---------------------------------------------------------------- resolve */
/* D2 (5855-5934), one warp: the first SFTG_MAX_TILE_LIGHTS point lights in index order whose
 * depth range meets the tile's [zmin, zmax] and whose screen rectangle meets the tile.  Their
 * indices go to out[]; returns their count on every lane. */
SFTG_D int tile_light_list(const sftg_frame* F, float zmin, float zmax, int tmx, int tmy, int lane, uint16_t* out)
{
    int n = 0;
    if (zmin <= zmax && F->n_point > 0) {
        const float* vp = F->vp;
        for (uint32_t base = 0; base < F->n_point && n < SFTG_MAX_TILE_LIGHTS; base += 32) {
            const uint32_t l = base + lane;
            bool pass = false;
            if (l < F->n_point) {
                const sftg_point_light L = F->point[l];
                const float w = L.pos[0] * vp[3] + L.pos[1] * vp[7] + L.pos[2] * vp[11] + vp[15];
                const float lmin = w - L.radius, lmax = w + L.radius;
                pass = !(lmax <= 1e-6f);
                if (pass) {
                    const float smin = (lmin > 1e-6f) ? lmin : 1e-6f;
                    const float iwmin = fdiv(1.f, lmax), iwmax = fdiv(1.f, smin);
                    if (iwmax < zmin || iwmin > zmax) pass = false;
                }
                if (pass && w > L.radius) {
                    const float tx = L.pos[0] * vp[0] + L.pos[1] * vp[4] + L.pos[2] * vp[8] + vp[12];
                    const float ty = L.pos[0] * vp[1] + L.pos[1] * vp[5] + L.pos[2] * vp[9] + vp[13];
                    const float sx = (fdiv(tx, w) + 1.f) * F->hw + F->vpx;
                    const float sy = (fdiv(-ty, w) + 1.f) * F->hh + F->vpy;
                    const float psx = fsqrt(vp[0] * vp[0] + vp[4] * vp[4] + vp[8] * vp[8]);
                    const float psy = fsqrt(vp[1] * vp[1] + vp[5] * vp[5] + vp[9] * vp[9]);
                    const float safe_w = (w - L.radius) > 1e-6f ? (w - L.radius) : 1e-6f;
                    const float rx = fdiv((L.radius * psx) + fabsf(tx) * fdiv(L.radius, w), safe_w) * F->hw;
                    const float ry = fdiv((L.radius * psy) + fabsf(ty) * fdiv(L.radius, w), safe_w) * F->hh;
                    if (sx + rx < (float)tmx || sx - rx > (float)(tmx + SFTG_TILE) || sy + ry < (float)tmy || sy - ry > (float)(tmy + SFTG_TILE)) pass = false;
                }
            }
            const uint32_t bal = __ballot_sync(0xFFFFFFFFu, pass);
            const int rank = __popc(bal & ((1u << lane) - 1u));
            if (pass && n + rank < SFTG_MAX_TILE_LIGHTS) out[n + rank] = (uint16_t)l;
            n = min(SFTG_MAX_TILE_LIGHTS, n + __popc(bal));
        }
    }
    return n;
}

/* Per tile, once for all of its resolve CTAs: the light list (D2) and, per listed light, the
 * selected proxies (D3: in index order, those whose light_vis entry is set and whose bounding
 * sphere reaches the light's sphere, the first SFTG_MAX_LIGHT_PROXIES). */
__global__ void __launch_bounds__(TILE_THREADS)
k_tile_lights(const sftg_tile_args A, uint32_t tile0)
{
    __shared__ uint16_t s_lights[SFTG_MAX_TILE_LIGHTS];
    __shared__ int s_nlights;
    const uint32_t gtile = A.tile_order[tile0 + blockIdx.x];
    const sftg_frame* F = A.frames + A.tile_view[gtile];
    const int tile = (int)(gtile - F->tile_base);
    const uint8_t* light_vis = A.light_vis + (size_t)F->prox_base * 64;
    sftg_tile_lights* TL = A.tile_lights + gtile;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tmx = (tile % F->cols) * SFTG_TILE, tmy = (tile / F->cols) * SFTG_TILE;
    const float2 zr = tile_zrange(A.zrange, gtile);
    const float zmin = zr.x, zmax = zr.y;

    if (warp == 0) {   /* D2 */
        const int n = tile_light_list(F, zmin, zmax, tmx, tmy, lane, s_lights);
        if (lane == 0) {
            s_nlights = n;
            A.tile_nlights[gtile] = (uint8_t)n;
            TL->nlights = (uint32_t)n;
        }
    }
    __syncthreads();
    const int ntl = s_nlights;
    if (tid < SFTG_MAX_TILE_LIGHTS) TL->light[tid] = tid < ntl ? s_lights[tid] : (uint16_t)0;
    for (int i = warp; i < SFTG_MAX_TILE_LIGHTS; i += TILE_THREADS / 32) {
        int n = 0;
        if (i < ntl && F->shadows && F->n_proxies > 0) {
            const sftg_point_light L = F->point[s_lights[i]];
            for (uint32_t base = 0; base < F->n_proxies && n < SFTG_MAX_LIGHT_PROXIES; base += 32) {
                const uint32_t p = base + lane;
                bool take = false;
                if (p < F->n_proxies && light_vis[(size_t)p * 64 + s_lights[i]]) {
                    const sftg_proxy px = F->proxies[p];
                    const v3 cc = mk3((px.posa[0] + px.posb[0]) * 0.5f, (px.posa[1] + px.posb[1]) * 0.5f, (px.posa[2] + px.posb[2]) * 0.5f);
                    const v3 ab = mk3(px.posb[0] - px.posa[0], px.posb[1] - px.posa[1], px.posb[2] - px.posa[2]);
                    const float cl = fsqrt(sdot(ab, ab));
                    const float br = px.radius + (cl * 0.5f);
                    const float cr = br + L.radius;
                    const v3 Wv = sub3(cc, mk3(L.pos[0], L.pos[1], L.pos[2]));
                    take = sdot(Wv, Wv) <= cr * cr;
                }
                const uint32_t bal = __ballot_sync(0xFFFFFFFFu, take);
                const int rank = __popc(bal & ((1u << lane) - 1u));
                if (take && n + rank < SFTG_MAX_LIGHT_PROXIES) TL->proxy[i][n + rank] = p;
                n = min(SFTG_MAX_LIGHT_PROXIES, n + __popc(bal));
            }
        }
        if (lane == 0) TL->npc[i] = (uint8_t)n;
    }
}

/* the tile's 4x2 block that a resolve CTA's b-th block is: at 4x the CTAs of a tile take every
 * split-th block, so the costly ones (many triangles, many lights) spread over all of them
 * (measured on the atrium at 4x: the slowest CTA of a tile took twice the mean with contiguous
 * ranges); at 1x and 2x a contiguous range of rows keeps each CTA's surface points close together,
 * which tightens the per-CTA proxy filter */
template <int S>
SFTG_D int block_of(int part, int split, int nblk, int b) { return S == 4 ? b * split + part : part * nblk + b; }
#define TILE_BLOCKS (16 * 32)                 /* 4x2 blocks per 64x64 tile; a CTA resolves 1/split of them */

/* One CTA per quarter tile: tile light list (5855-5934) and proxy cache (5936-5990), then one
 * 8-thread group per 4x2 block for the per-triangle shading and MSAA resolve (6029-6745). */
template <int S>
SFTG_D void resolve_item(const sftg_tile_args& A, uint32_t tile0, int split, bool records, uint32_t item)
{
    __shared__ proxy_cache pcache[SFTG_MAX_TILE_LIGHTS * SFTG_MAX_LIGHT_PROXIES];
    /* the per-lane "between" test's operands of each cached proxy, in pcache's order: W (proxy
     * centre minus light) with |W|^2 as one 16-byte load, and the squared bounding radius */
    __shared__ float4 s_btw[SFTG_MAX_TILE_LIGHTS * SFTG_MAX_LIGHT_PROXIES];
    __shared__ float s_rb2[SFTG_MAX_TILE_LIGHTS * SFTG_MAX_LIGHT_PROXIES];
    __shared__ uint16_t s_lights[SFTG_MAX_TILE_LIGHTS];
    __shared__ sftg_point_light s_pl[SFTG_MAX_TILE_LIGHTS];   /* the tile's lights, in list order */
    __shared__ int s_nlights;
    __shared__ uint8_t s_npc[SFTG_MAX_TILE_LIGHTS];

    const uint32_t gtile = A.tile_order[tile0 + item / (uint32_t)split];   /* batch-wide tile index, heaviest first */
    const int part = (int)(item % (uint32_t)split);
    const int nblk = TILE_BLOCKS / split;
    const sftg_frame* F = A.frames + A.tile_view[gtile];
    const int tile = (int)(gtile - F->tile_base);
    const float* ss = A.ss + (size_t)F->ss_base * SFTG_SS_FLOATS;
    const sftg_clip_tri* clips = A.clips + (F->total_ss ? A.clip_base[(size_t)F->ss_base * 16] : 0u);
    const uint8_t* light_vis = A.light_vis + (size_t)F->prox_base * 64;
    uint32_t* color = F->color_dev;
    const int CP = F->pitch;   /* colour row stride in pixels (the caller's buffer when written directly) */
    float* shadow_out = A.shadow_out;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tmx = (tile % F->cols) * SFTG_TILE, tmy = (tile / F->cols) * SFTG_TILE;
    const float2 zr = tile_zrange(A.zrange, gtile);
    const float zmin = zr.x, zmax = zr.y;
    const float2* vis = A.vis + F->vis_base + (size_t)tile * S * SFTG_TILE_PX;

    const sftg_tile_lights* TL = A.tile_lights + gtile;
    if (records) {   /* D2 and D3's selection come from the tile's record (k_tile_lights) */
        if (tid < SFTG_MAX_TILE_LIGHTS) { s_lights[tid] = TL->light[tid]; s_npc[tid] = TL->npc[tid]; }
        if (tid == 0) s_nlights = (int)TL->nlights;
    } else {
        if (warp == 0) {   /* D2 */
            const int n = tile_light_list(F, zmin, zmax, tmx, tmy, lane, s_lights);
            if (lane == 0) {
                s_nlights = n;
                if (part == 0) A.tile_nlights[gtile] = (uint8_t)n;
            }
        }
    }
    __syncthreads();
    const int ntl = s_nlights;
    if (tid < ntl) s_pl[tid] = F->point[s_lights[tid]];

    /* World box of every surface point this CTA shades (per covered pixel and distinct sample
     * triangle, interpolated as the shading loop does), for the proxy filter below. */
    __shared__ float s_bnd[TILE_THREADS / 32][6];
    const int sw = (int)(F->hw * 2.f), sh = (int)(F->hh * 2.f);
    const int lim_x = min(tmx + SFTG_TILE, sw), lim_y = min(tmy + SFTG_TILE, sh);
    const bool cull_proxies = F->shadows && F->n_proxies > 0 && ntl > 0;
    if (cull_proxies) {
        float mn[3] = { 1e30f, 1e30f, 1e30f }, mx[3] = { -1e30f, -1e30f, -1e30f };
        uint32_t last = SFTG_INVALID;
        const int ix0 = tid & 3, iy0 = (tid >> 2) & 1;
        for (int b = tid >> 3; b < nblk; b += TILE_THREADS / 8) {
            const int blk = block_of<S>(part, split, nblk, b);
            const int gx = tmx + (blk & 15) * 4 + ix0, gy = tmy + (blk >> 4) * 2 + iy0;
            if (gx >= lim_x || gy >= lim_y) continue;
            const int pind = (gy - tmy) * SFTG_TILE + (gx - tmx);
            const float pxf = ((float)(gx - ix0) + 0.5f) + (float)ix0, pyf = ((float)(gy - iy0) + 0.5f) + (float)iy0;
            last = SFTG_INVALID;
#pragma unroll
            for (int s = 0; s < S; s++) {
                const uint32_t vid = __float_as_uint(vis[s * SFTG_TILE_PX + pind].y);
                if (vid != SFTG_INVALID && vid != last) { last = vid; pixel_pos_acc<S>(F, ss, clips, vid, pxf, pyf, mn, mx); }
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1)
#pragma unroll
            for (int a = 0; a < 3; a++) {
                mn[a] = fminf(mn[a], __shfl_xor_sync(0xFFFFFFFFu, mn[a], o));
                mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xFFFFFFFFu, mx[a], o));
            }
        if (lane == 0) { s_bnd[warp][0] = mn[0]; s_bnd[warp][1] = mn[1]; s_bnd[warp][2] = mn[2]; s_bnd[warp][3] = mx[0]; s_bnd[warp][4] = mx[1]; s_bnd[warp][5] = mx[2]; }
    }

    if (records) {
        /* D3's proxy cache (5936-5990): the tile's selected proxies, one thread per (light, slot), the
         * entries computed as the selection computed them */
        for (int t = tid; t < SFTG_MAX_TILE_LIGHTS * SFTG_MAX_LIGHT_PROXIES; t += TILE_THREADS) {
            const int i = t / SFTG_MAX_LIGHT_PROXIES, k = t % SFTG_MAX_LIGHT_PROXIES;
            if (i >= ntl || k >= s_npc[i]) continue;
            const uint32_t p = TL->proxy[i][k];
            const sftg_point_light L = F->point[s_lights[i]];   /* s_pl is read only after the next barrier */
            const sftg_proxy px = F->proxies[p];
            const uint8_t vs = light_vis[(size_t)p * 64 + s_lights[i]];
            const v3 cc = mk3((px.posa[0] + px.posb[0]) * 0.5f, (px.posa[1] + px.posb[1]) * 0.5f, (px.posa[2] + px.posb[2]) * 0.5f);
            const v3 ab = mk3(px.posb[0] - px.posa[0], px.posb[1] - px.posa[1], px.posb[2] - px.posa[2]);
            const float cl = fsqrt(sdot(ab, ab));
            const float br = px.radius + (cl * 0.5f);
            const v3 Wv = sub3(cc, mk3(L.pos[0], L.pos[1], L.pos[2]));
            const float d2 = sdot(Wv, Wv);
            proxy_cache* q = &pcache[t];
            q->pa[0] = px.posa[0]; q->pa[1] = px.posa[1]; q->pa[2] = px.posa[2];
            q->pb[0] = px.posb[0]; q->pb[1] = px.posb[1]; q->pb[2] = px.posb[2];
            q->ab[0] = ab.x; q->ab[1] = ab.y; q->ab[2] = ab.z;
            q->W[0] = Wv.x; q->W[1] = Wv.y; q->W[2] = Wv.z;
            q->abdab = sdot(ab, ab); q->wdw = d2; q->rb2 = br * br; q->pr = px.radius; q->pr2 = px.radius * px.radius;
            q->vis_mult = (float)vs * 0.3333333f;
            s_btw[t] = make_float4(Wv.x, Wv.y, Wv.z, d2);
            s_rb2[t] = q->rb2;
        }
    } else {
        /* D3: per light, the first 16 proxies that see it and can reach it (5936-5990) */
        for (int i = warp; i < SFTG_MAX_TILE_LIGHTS; i += TILE_THREADS / 32) {
            int n = 0;
            if (i < ntl && F->shadows && F->n_proxies > 0) {
                const sftg_point_light L = F->point[s_lights[i]];
                for (uint32_t base = 0; base < F->n_proxies && n < SFTG_MAX_LIGHT_PROXIES; base += 32) {
                    const uint32_t p = base + lane;
                    bool take = false; uint8_t vs = 0;
                    v3 cc, ab, Wv; float br = 0.f, d2 = 0.f;
                    sftg_proxy px;
                    if (p < F->n_proxies) {
                        px = F->proxies[p];
                        vs = light_vis[(size_t)p * 64 + s_lights[i]];
                        if (vs) {
                            cc = mk3((px.posa[0] + px.posb[0]) * 0.5f, (px.posa[1] + px.posb[1]) * 0.5f, (px.posa[2] + px.posb[2]) * 0.5f);
                            ab = mk3(px.posb[0] - px.posa[0], px.posb[1] - px.posa[1], px.posb[2] - px.posa[2]);
                            const float cl = fsqrt(sdot(ab, ab));
                            br = px.radius + (cl * 0.5f);
                            const float cr = br + L.radius;
                            Wv = sub3(cc, mk3(L.pos[0], L.pos[1], L.pos[2]));
                            d2 = sdot(Wv, Wv);
                            take = d2 <= cr * cr;
                        }
                    }
                    const uint32_t bal = __ballot_sync(0xFFFFFFFFu, take);
                    const int rank = __popc(bal & ((1u << lane) - 1u));
                    if (take && n + rank < SFTG_MAX_LIGHT_PROXIES) {
                        proxy_cache* q = &pcache[i * SFTG_MAX_LIGHT_PROXIES + n + rank];
                        q->pa[0] = px.posa[0]; q->pa[1] = px.posa[1]; q->pa[2] = px.posa[2];
                        q->pb[0] = px.posb[0]; q->pb[1] = px.posb[1]; q->pb[2] = px.posb[2];
                        q->ab[0] = ab.x; q->ab[1] = ab.y; q->ab[2] = ab.z;
                        q->W[0] = Wv.x; q->W[1] = Wv.y; q->W[2] = Wv.z;
                        q->abdab = sdot(ab, ab); q->wdw = d2; q->rb2 = br * br; q->pr = px.radius; q->pr2 = px.radius * px.radius;
                        s_btw[i * SFTG_MAX_LIGHT_PROXIES + n + rank] = make_float4(Wv.x, Wv.y, Wv.z, d2);
                        s_rb2[i * SFTG_MAX_LIGHT_PROXIES + n + rank] = q->rb2;
                        q->vis_mult = (float)vs * 0.3333333f;
                    }
                    n = min(SFTG_MAX_LIGHT_PROXIES, n + __popc(bal));
                }
            }
            if (lane == 0) s_npc[i] = (uint8_t)n;
        }
    }
    __syncthreads();

    /* Conservative filter of the cached proxies (order kept).  Every pixel this CTA shades lies
     * in the ball (Bc, Br) around the bounds above.  The per-block skip (6520-6540) drops a
     * proxy unless some lane's segment pixel -> light passes within the proxy's bounding radius
     * of its centre; for pixels in the ball that segment stays within Br of the segment
     * Bc -> light.  So a proxy farther than rb + Br (+ a rounding margin) from that segment is
     * skipped by every block, and removing it here leaves every pixel unchanged. */
    if (cull_proxies) {
        float mn[3], mx[3];
#pragma unroll
        for (int a = 0; a < 3; a++) { mn[a] = s_bnd[0][a]; mx[a] = s_bnd[0][3 + a]; }
        for (int w = 1; w < TILE_THREADS / 32; w++)
#pragma unroll
            for (int a = 0; a < 3; a++) { mn[a] = fminf(mn[a], s_bnd[w][a]); mx[a] = fmaxf(mx[a], s_bnd[w][3 + a]); }
        const bool empty = !(mn[0] <= mx[0] && mn[1] <= mx[1] && mn[2] <= mx[2]);
        const v3 bc = mk3((mn[0] + mx[0]) * 0.5f, (mn[1] + mx[1]) * 0.5f, (mn[2] + mx[2]) * 0.5f);
        const v3 he = mk3((mx[0] - mn[0]) * 0.5f, (mx[1] - mn[1]) * 0.5f, (mx[2] - mn[2]) * 0.5f);
        const float br = sqrtf(he.x * he.x + he.y * he.y + he.z * he.z);
        const bool usable = isfinite(br) && isfinite(bc.x) && isfinite(bc.y) && isfinite(bc.z);
        for (int i = warp; i < ntl; i += TILE_THREADS / 32) {
            const int n = s_npc[i];
            if (n == 0 || (usable == false && !empty)) continue;
            const sftg_point_light L = F->point[s_lights[i]];
            bool keep = false;
            proxy_cache q;
            if (lane < n) {
                q = pcache[i * SFTG_MAX_LIGHT_PROXIES + lane];
                if (!empty) {
                    const v3 Wv = mk3(q.W[0], q.W[1], q.W[2]);
                    const v3 D = mk3(bc.x - L.pos[0], bc.y - L.pos[1], bc.z - L.pos[2]);
                    const float dd = D.x * D.x + D.y * D.y + D.z * D.z;
                    const float t = dd > 0.f ? fminf(fmaxf((Wv.x * D.x + Wv.y * D.y + Wv.z * D.z) / dd, 0.f), 1.f) : 0.f;
                    const v3 E = mk3(Wv.x - t * D.x, Wv.y - t * D.y, Wv.z - t * D.z);
                    const float dist = sqrtf(E.x * E.x + E.y * E.y + E.z * E.z);
                    const float m = 2e-3f * (sqrtf(q.wdw) + sqrtf(dd) + br) + 1e-3f;
                    keep = !(dist > sqrtf(q.rb2) + br + m);
                }
            }
            const uint32_t bal = __ballot_sync(0xFFFFFFFFu, keep);
            __syncwarp();
            if (keep) {
                const int k = i * SFTG_MAX_LIGHT_PROXIES + __popc(bal & ((1u << lane) - 1u));
                pcache[k] = q;
                s_btw[k] = make_float4(q.W[0], q.W[1], q.W[2], q.wdw);
                s_rb2[k] = q.rb2;
            }
            if (lane == 0) s_npc[i] = (uint8_t)__popc(bal);
        }
        __syncthreads();
    }

    /* ---------------- resolve: one 8-thread group per 4x2 block ---------------- */
    const int W = F->width;
    const int grp = tid >> 3, gl = tid & 7, gshift = lane & ~7;
    const uint32_t gmask = 0xFFu << gshift;
    const int ix = gl & 3, iy = gl >> 2;
    const float inv_s = 1.f / (float)S;
    const uint32_t cc = F->clear_color;
    const float clr[3] = { (float)((cc >> 16) & 0xFF) * (1.f / 255.f), (float)((cc >> 8) & 0xFF) * (1.f / 255.f), (float)(cc & 0xFF) * (1.f / 255.f) };
    const v3 cam = mk3(F->cam[0], F->cam[1], F->cam[2]);

    for (int b = grp; b < nblk; b += TILE_THREADS / 8) {
        const int blk = block_of<S>(part, split, nblk, b);
        const int x = tmx + (blk & 15) * 4, y = tmy + (blk >> 4) * 2;
        if (x >= lim_x || y >= lim_y) continue;
        const int gx = x + ix, gy = y + iy;
        const bool inb = (sw > gx) && (sh > gy);
        const int pind = (gy - tmy) * SFTG_TILE + (gx - tmx);
        const float pxf = ((float)x + 0.5f) + (float)ix, pyf = ((float)y + 0.5f) + (float)iy;
        uint32_t vids[S];
        uint32_t asm_[S];
        int ecount = 0;
#pragma unroll
        for (int s = 0; s < S; s++) {
            vids[s] = __float_as_uint(vis[s * SFTG_TILE_PX + pind].y);
            const bool empty = vids[s] == SFTG_INVALID;
            asm_[s] = (__ballot_sync(gmask, !empty && inb) >> gshift) & 0xFFu;
            ecount += (empty && inb);
        }
        uint32_t act = 0;
#pragma unroll
        for (int s = 0; s < S; s++) act |= asm_[s];
        float acc[3] = { 0.f, 0.f, 0.f };
        if (S == 1) {
            if (F->clear && inb && vids[0] == SFTG_INVALID) color[gy * CP + gx] = cc;
        } else {
            if (!act) {
                if (F->clear && inb) color[gy * CP + gx] = cc;
                continue;
            }
            const float ew = (float)ecount * inv_s;
            const bool any_e = (__ballot_sync(gmask, ew > 0.f) & gmask) != 0;
            if (F->clear) { acc[0] = clr[0] * ew; acc[1] = clr[1] * ew; acc[2] = clr[2] * ew; }
            else if (any_e) {
                float bg[3] = { 0.f, 0.f, 0.f };
                if (gx < sw && gy < sh) {
                    const uint32_t q = color[gy * CP + gx];
                    bg[0] = (float)((q >> 16) & 0xFF) * (1.f / 255.f); bg[1] = (float)((q >> 8) & 0xFF) * (1.f / 255.f); bg[2] = (float)(q & 0xFF) * (1.f / 255.f);
                }
                acc[0] = bg[0] * ew; acc[1] = bg[1] * ew; acc[2] = bg[2] * ew;
            }
        }
        const uint32_t block_write = act;
        while (act) {
            uint32_t target, tri_mask = 0, tri_lanes = 0; int hits = 0;
            if (S == 1) {
                const int fl = __ffs(act) - 1;
                target = __shfl_sync(gmask, vids[0], gshift + fl);
                tri_mask = (__ballot_sync(gmask, vids[0] == target && inb) >> gshift) & 0xFFu;
                tri_lanes = tri_mask & act;
                act &= ~tri_lanes;
            } else {
                int fs = 0;
                while (!asm_[fs]) fs++;
                const int fl = __ffs(asm_[fs]) - 1;
                uint32_t vsel = vids[0];
#pragma unroll
                for (int s = 1; s < S; s++) if (s == fs) vsel = vids[s];
                target = __shfl_sync(gmask, vsel, gshift + fl);
#pragma unroll
                for (int s = 0; s < S; s++) {
                    const bool match = vids[s] == target && inb;
                    const uint32_t mb = (__ballot_sync(gmask, match) >> gshift) & 0xFFu;
                    const uint32_t mm = mb & asm_[s];
                    asm_[s] &= ~mm; tri_lanes |= mm; tri_mask |= mb;
                    hits += match;
                }
                act = 0;
#pragma unroll
                for (int s = 0; s < S; s++) act |= asm_[s];
            }
            const bool in_tri = (tri_mask >> gl) & 1u;
            tri_verts T;
            fetch_tri(F, ss, clips, target, T);
            const sftg_inst* I = &F->inst[T.inst];
            const sftg_meshlet_info info = F->ml_info[I->meshlet_base + T.m];
            /* D6 barycentrics and perspective-correct interpolation (6282-6347) */
            const float dx1 = T.sx[1] - T.sx[0], dx2 = T.sx[2] - T.sx[0], dy1 = T.sy[1] - T.sy[0], dy2 = T.sy[2] - T.sy[0];
            const float idet = rcpr(dx1 * dy2 - dx2 * dy1);
            const float pxs = pxf - T.sx[0], pys = pyf - T.sy[0];
            const float rbu = (pxs * dy2 - pys * dx2) * idet;
            const float rbv = (pys * dx1 - pxs * dy1) * idet;
            const float rbw = (1.f - rbu) - rbv;
            float bu = rbu, bv = rbv, bw = rbw;
            if (S > 1) {
                bu = vmax(0.f, rbu); bv = vmax(0.f, rbv); bw = vmax(0.f, rbw);
                const float bs = rcpr(bu + (bv + bw));
                bu = bu * bs; bv = bv * bs; bw = bw * bs;
            }
            const float iz = fma_(bw, T.iw[0], fma_(bu, T.iw[1], bv * T.iw[2]));
            const float z = rcpr(iz);
            const float w0 = (bw * T.iw[0]) * z, w1 = (bu * T.iw[1]) * z, w2 = (bv * T.iw[2]) * z;
#define INTERP(a) fma_(w0, (a)[0], fma_(w1, (a)[1], w2 * (a)[2]))
            const float cu = INTERP(T.u), cv = INTERP(T.v), clu = INTERP(T.lu), clv = INTERP(T.lv);
            const v3 P = mk3(INTERP(T.px), INTERP(T.py), INTERP(T.pz));
            const v3 N = vnorm_fast(mk3(INTERP(T.nx), INTERP(T.ny), INTERP(T.nz)));
#undef INTERP
            const v3 V = vnorm_fast(sub3(cam, P));
            /* material (6350-6382) */
            uint32_t base = 0xFFFFFFFFu; int ti = -1; float shin = 4.f;
            if (info.material >= 0) { const sftg_mat mt = F->mats[info.material]; base = mt.base_color; ti = mt.tex; shin = mt.shininess; }
            if (F->debug_mode == 5) { ti = F->debug_tex; base = 0xFFFFFFFFu; }   /* checkerboard view (6373-6376) */
            const float i255 = 1.f / 255.f;
            const float bcol[3] = { (float)((base >> 16) & 0xFF) * i255, (float)((base >> 8) & 0xFF) * i255, (float)(base & 0xFF) * i255 };
            /* D7 LOD from the first covered lane's derivatives (5501-5541) */
            int lod = 0;
            {
                const int fl = __ffs(tri_mask) - 1;
                const float cu_f = __shfl_sync(gmask, cu, gshift + fl), cv_f = __shfl_sync(gmask, cv, gshift + fl);
                const float cu_x = __shfl_sync(gmask, cu, gshift + (fl ^ 1)), cv_x = __shfl_sync(gmask, cv, gshift + (fl ^ 1));
                const float cu_y = __shfl_sync(gmask, cu, gshift + (fl ^ 4)), cv_y = __shfl_sync(gmask, cv, gshift + (fl ^ 4));
                if (ti >= 0) {
                    const sftg_tex& tx = F->texs[ti];
                    const float ux = (cu_f - cu_x) * (float)tx.w, vx = (cv_f - cv_x) * (float)tx.h;
                    const float uy = (cu_f - cu_y) * (float)tx.w, vy = (cv_f - cv_y) * (float)tx.h;
                    const float a1 = fabsf(ux) > fabsf(vx) ? fabsf(ux) : fabsf(vx);
                    const float a2 = fabsf(uy) > fabsf(vy) ? fabsf(uy) : fabsf(vy);
                    const float rho = a1 > a2 ? a1 : a2;
                    if (rho > 1.f) {
                        const float lf = (float)(31 - __clz((uint32_t)cvtt(rho)));
                        lod = (int)((lf + 0.5f) + (-0.375f));
                    }
                    lod = lod < 0 ? 0 : (lod > tx.levels - 1 ? tx.levels - 1 : lod);
                }
            }
            float out[3];
            {
                float tr, tg, tb;
                if (lod > 1) sample_nearest(F, ti, lod, cu, cv, tr, tg, tb);
                else sample_bilinear(F, ti, lod, cu, cv, tr, tg, tb);
                out[0] = tr * bcol[0]; out[1] = tg * bcol[1]; out[2] = tb * bcol[2];
            }
            const bool lm = info.lightmap_tex >= 0;
            if (shin < 0.f) {
                out[0] = out[0] * (-shin); out[1] = out[1] * (-shin); out[2] = out[2] * (-shin);
            } else {
                const float sscale = ((shin + 8.f) / 8.f) * 0.04f;
                float dif[3], spc[3] = { 0.f, 0.f, 0.f }, lms = 1.f;
                if (lm) {
                    sample_bilinear(F, info.lightmap_tex, 0, clu, clv, dif[0], dif[1], dif[2]);
                    dif[0] = dif[0] * F->lightmap_brightness; dif[1] = dif[1] * F->lightmap_brightness; dif[2] = dif[2] * F->lightmap_brightness;
                } else {
                    dif[0] = F->ambient[0]; dif[1] = F->ambient[1]; dif[2] = F->ambient[2];
                    for (uint32_t dl = 0; dl < F->n_dir; dl++) {
                        const sftg_dir_light D = F->dir[dl];
                        const v3 Ld = mk3(D.dir[0], D.dir[1], D.dir[2]);
                        const float ndl = vmax(vdot(N, Ld), 0.f);
                        dif[0] = fma_(ndl, D.color[0], dif[0]); dif[1] = fma_(ndl, D.color[1], dif[1]); dif[2] = fma_(ndl, D.color[2], dif[2]);
                        if (ndl > 0.f) {
                            const v3 Hh = vnorm_fast(add3(Ld, V));
                            const float ndh = vmax(vdot(N, Hh), 0.f);
                            const float den = (shin - shin * ndh) + ndh;
                            const float sp = ndh * rcpr(den);
                            const float term = (sp * sscale) * ndl;
                            spc[0] = fma_(term, D.color[0], spc[0]); spc[1] = fma_(term, D.color[1], spc[1]); spc[2] = fma_(term, D.color[2], spc[2]);
                        }
                    }
                }
                /* D10 point lights and capsule shadows (6474-6607) */
                /* A lightmapped surface and a light with no cached proxy: msh = 0, si = 1 and the
                 * light multiplies lms by 1 - 0 * att, a no-op unless att is NaN (att is in [0, 1]
                 * or NaN).  The reference's path below reaches that product only when some lane
                 * of the block has att > 0 and some covered lane has a NaN att; such lights are
                 * gathered as bits and applied after the loop (NaN absorbs the other factors, so
                 * order does not matter).  Not used while per-light shadow factors are captured. */
                const bool lm_quick = lm && shadow_out == nullptr;
                uint32_t q_alive = 0, q_nan = 0;
                for (int i = 0; i < ntl; i++) {
                    const sftg_point_light& L = s_pl[i];
                    const v3 Lr = sub3(mk3(L.pos[0], L.pos[1], L.pos[2]), P);
                    const float d2 = vdot(Lr, Lr);
                    float att = vmax(0.f, fma_(-d2, L.inv_radius_sqr, 1.f));
                    att = att * att;
                    const bool alive = att > 0.f;
                    if (lm_quick && s_npc[i] == 0) {
                        q_alive |= (uint32_t)alive << i;
                        q_nan |= (uint32_t)(in_tri && !(att <= 3.402823466e38f)) << i;
                        continue;
                    }
                    if (!(__ballot_sync(gmask, alive) & gmask)) continue;
                    v3 Ln = mk3(0.f, 0.f, 0.f);
                    float ndl = 0.f;
                    bool lit = false;
                    if (!lm) {
                        Ln = vnorm_fast(Lr);
                        ndl = vmax(vdot(N, Ln), 0.f);
                        lit = (ndl > 0.f) && alive && in_tri;
                    }
                    /* every cached proxy's "between" test first (independent, so they overlap),
                     * then the block-level skip as the OR over the block's lanes */
                    const int np = s_npc[i];
                    uint32_t rmask = 0, bmask = 0;
                    const bool want = lm ? in_tri : lit;
                    /* a lane's bit needs `want`: with no lane of the block wanting, every mask is 0 */
                    if (np > 0 && (__ballot_sync(gmask, want) & gmask)) {
                        const float rd2 = rcpr(d2);   /* loop-invariant: the reference recomputes the same value per proxy */
                        const float nd2 = -d2;
                        /* The reference's test with wdv = 0 - dot(W, Lr): wdv > 0 && wdv < d2, then
                         * cd2 = fma(-wdv, wdv * rd2, |W|^2) < rb2.  With v = dot(W, Lr): wdv > 0 is
                         * v < 0 (both false for a zero or NaN v), wdv < d2 is v > -d2, and for such
                         * v, wdv = -v exactly, wdv * rd2 = -(v * rd2) (round to nearest is
                         * symmetric) and cd2 = fma(-v, v * rd2, |W|^2): the same bits. */
#pragma unroll 4
                        for (int pi = 0; pi < np; pi++) {
                            const float4 bt = s_btw[i * SFTG_MAX_LIGHT_PROXIES + pi];
                            const float v = vdot(mk3(bt.x, bt.y, bt.z), Lr);
                            const bool btw = v < 0.f && v > nd2;
                            const float cd2 = fma_(-v, v * rd2, bt.w);
                            rmask |= (uint32_t)(btw && (cd2 < s_rb2[i * SFTG_MAX_LIGHT_PROXIES + pi]) && want) << pi;
                        }
                        bmask = rmask;
                        bmask |= __shfl_xor_sync(gmask, bmask, 1);
                        bmask |= __shfl_xor_sync(gmask, bmask, 2);
                        bmask |= __shfl_xor_sync(gmask, bmask, 4);
                    }
                    if (lm && !bmask) {
                        /* lightmapped and no proxy shadows the block: si = 1, drop = 0 * att and the
                         * light leaves lms unchanged, unless att is not finite on a covered lane */
                        if (!(__ballot_sync(gmask, in_tri && !(att <= 3.402823466e38f)) & gmask)) {
                            if (shadow_out && S == 1 && ((tri_lanes >> gl) & 1u) && i < 16)
                                shadow_out[((size_t)gy * W + gx) * 16 + i] = 1.f;
                            continue;
                        }
                    }
                    if (lm) Ln = vnorm_fast(Lr);
                    float msh = 0.f;
                    if (bmask) {
                        const float lrl = fsqrt(d2);
                        const float bk = 0.2f, b4 = 0.25f / 0.2f;
                        /* the smooth-max blend over the surviving proxies in index order */
                        while (bmask) {
                            const int pi = __ffs(bmask) - 1;
                            bmask &= bmask - 1;
                            const proxy_cache& q = pcache[i * SFTG_MAX_LIGHT_PROXIES + pi];
                            const bool ray = (rmask >> pi) & 1u;
                            const v3 pa = mk3(q.pa[0], q.pa[1], q.pa[2]), ab = mk3(q.ab[0], q.ab[1], q.ab[2]);
                            const v3 ao = sub3(P, pa);
                            const float abl = vdot(ab, Ln), abao = vdot(ab, ao), lao = vdot(Ln, ao);
                            const float den = fma_(-abl, abl, q.abdab);
                            const float sden = vmax(den, 1e-6f);
                            float t2 = fma_(-abl, lao, abao) * rcpr(sden);
                            t2 = vmax(0.f, vmin(t2, 1.f));
                            const float t1 = fma_(t2, abl, -lao);
                            const bool vc = t1 > 1e-6f && t1 < lrl;
                            const v3 pr = add3(P, scl3(Ln, t1));
                            const v3 pc = add3(pa, scl3(ab, t2));
                            const v3 dd = sub3(pr, pc);
                            const float dist2 = vdot(dd, dd);
                            float sv = vmax(0.f, 1.f - fdiv(dist2, q.pr2));
                            if (!ray || !vc) sv = 0.f;
                            sv = sv * q.vis_mult;
                            const float h = vmax(0.f, bk - fabsf(msh - sv));
                            const float badd = (h * h) * b4;
                            msh = vmax(msh, sv) + badd;
                        }
                    }
                    const float si = vmax(0.f, 1.f - msh);
                    if (shadow_out && S == 1 && ((tri_lanes >> gl) & 1u) && i < 16)
                        shadow_out[((size_t)gy * W + gx) * 16 + i] = si;
                    if (lm) {
                        const float drop = (1.f - si) * att;
                        lms = lms * (1.f - drop);
                    } else {
                        const float di = ndl * att;
                        const float md = lit ? (di * si) : 0.f;
                        dif[0] = fma_(md, L.color[0], dif[0]); dif[1] = fma_(md, L.color[1], dif[1]); dif[2] = fma_(md, L.color[2], dif[2]);
                        if (lit) {
                            const v3 Hh = vnorm_fast(add3(Ln, V));
                            const float ndh = vmax(vdot(N, Hh), 0.f);
                            const float den = (shin - shin * ndh) + ndh;
                            const float sp = ndh * rcpr(den);
                            const float term = ((sp * sscale) * di) * si;
                            spc[0] = fma_(term, L.color[0], spc[0]); spc[1] = fma_(term, L.color[1], spc[1]); spc[2] = fma_(term, L.color[2], spc[2]);
                        }
                    }
                }
                if (lm_quick) {   /* uniform over the block's 8 lanes, as the shuffles need */
                    uint32_t ga = q_alive;
                    ga |= __shfl_xor_sync(gmask, ga, 1);
                    ga |= __shfl_xor_sync(gmask, ga, 2);
                    ga |= __shfl_xor_sync(gmask, ga, 4);
                    if (ga & q_nan) lms = __int_as_float(0x7FFFFFFF);
                }
                if (lm) {
                    const float mod = fma_(lms, 1.f - 0.4f, 0.4f);
                    out[0] = out[0] * (dif[0] * mod); out[1] = out[1] * (dif[1] * mod); out[2] = out[2] * (dif[2] * mod);
                } else {
                    out[0] = fma_(out[0], dif[0], spc[0]); out[1] = fma_(out[1], dif[1], spc[1]); out[2] = fma_(out[2], dif[2], spc[2]);
                }
            }
            if (F->debug_mode == 1) {   /* wireframe view (6645-6671): edges where a barycentric is under its screen width */
                const float dbu_dx = (0.f - dy2) * idet, dbu_dy = dx2 * idet;
                const float dbv_dx = dy1 * idet, dbv_dy = (0.f - dx1) * idet;
                const float fw_u = fabsf(dbu_dx) + fabsf(dbu_dy), fw_v = fabsf(dbv_dx) + fabsf(dbv_dy);
                const float dbw_dx = 0.f - (dbu_dx + dbv_dx), dbw_dy = 0.f - (dbu_dy + dbv_dy);
                const float fw_w = fabsf(dbw_dx) + fabsf(dbw_dy);
                if (bu < fw_u || bv < fw_v || bw < fw_w) { out[0] = 0.f; out[1] = 1.f; out[2] = 0.f; }
            }
            if (S == 1) {
                if ((tri_lanes >> gl) & 1u) {
                    uint32_t px = 0xFF000000u;
#pragma unroll
                    for (int k = 0; k < 3; k++) px |= ((uint32_t)cvtt(vmax(0.f, vmin(out[k], 1.f)) * 255.f)) << (16 - 8 * k);
                    color[gy * CP + gx] = px;
                }
            } else {
                const float wgt = in_tri ? (float)hits * inv_s : 0.f;
#pragma unroll
                for (int k = 0; k < 3; k++) acc[k] = fma_(vmax(0.f, vmin(out[k], 1.f)), wgt, acc[k]);
            }
        }
        if (S > 1) {
            const bool store = F->clear ? inb : ((block_write >> gl) & 1u);
            if (store) {
                uint32_t px = 0xFF000000u;
#pragma unroll
                for (int k = 0; k < 3; k++) px |= ((uint32_t)cvtt(vmin(acc[k], 1.f) * 255.f)) << (16 - 8 * k);
                color[gy * CP + gx] = px;
            }
        }
    }
}

/* one CTA per (tile, part) item */
template <int S>
__global__ void __launch_bounds__(TILE_THREADS, S == 1 ? 3 : 4)   /* 64 registers at 2x and 4x, 80 at 1x: measured best */
k_resolve(const sftg_tile_args A, uint32_t tile0, int split, bool records)
{
    resolve_item<S>(A, tile0, split, records, blockIdx.x);
}

/* Persistent form, as k_raster_queue: CTAs take (tile, part) items in launch order from a counter. */
template <int S>
__global__ void __launch_bounds__(TILE_THREADS, S == 1 ? 3 : 4)
k_resolve_queue(const sftg_tile_args A, uint32_t tile0, int split, bool records, uint32_t n_items, uint32_t* next)
{
    __shared__ uint32_t s_item;
    for (;;) {
        __syncthreads();   /* the previous item is done with shared memory, and s_item has been read */
        if (threadIdx.x == 0) s_item = atomicAdd(next, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= n_items) break;
        resolve_item<S>(A, tile0, split, records, item);
    }
}

/* ---------------------------------------------------------------- tile order
 * The reference's workers take tiles in descending payload count (sofren2.c:6815-6857) so the
 * heaviest start first.  Here the same idea keeps the tail of the raster and resolve grids
 * short: tiles are bucketed by floor(log2(count + 1)) inside their sample-count range and the
 * launches walk the buckets heaviest first.  Order affects scheduling only, never results. */
#define ORDER_BUCKETS 32

__device__ __forceinline__ uint32_t order_bucket(const sftg_frame* frames, const uint16_t* tile_view, const uint32_t* tile_count, uint32_t t) {
    const int S = frames[tile_view[t]].samples;
    const uint32_t si = S == 1 ? 0u : (S == 2 ? 1u : 2u);
    const uint32_t key = 31u - (uint32_t)__clz(tile_count[t] + 1u);          /* 0..31, heavier = larger */
    return si * ORDER_BUCKETS + (ORDER_BUCKETS - 1u - key);
}

__global__ void k_order_count(const sftg_frame* __restrict__ frames, const uint16_t* __restrict__ tile_view,
                              const uint32_t* __restrict__ tile_count, uint32_t n_tiles, uint32_t* __restrict__ hist)
{
    __shared__ uint32_t h[3 * ORDER_BUCKETS];
    for (int i = threadIdx.x; i < 3 * ORDER_BUCKETS; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n_tiles) atomicAdd(&h[order_bucket(frames, tile_view, tile_count, t)], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * ORDER_BUCKETS; i += blockDim.x) if (h[i]) atomicAdd(&hist[i], h[i]);
}

__global__ void k_order_scatter(const sftg_frame* __restrict__ frames, const uint16_t* __restrict__ tile_view,
                                const uint32_t* __restrict__ tile_count, uint32_t n_tiles, const uint32_t* __restrict__ hist,
                                uint32_t* __restrict__ cursor, uint32_t* __restrict__ order)
{
    __shared__ uint32_t base[3 * ORDER_BUCKETS];
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int i = 0; i < 3 * ORDER_BUCKETS; i++) { base[i] = run; run += hist[i]; }
    }
    __syncthreads();
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tiles) return;
    const uint32_t b = order_bucket(frames, tile_view, tile_count, t);
    order[base[b] + atomicAdd(&cursor[b], 1u)] = t;
}

/* the same order in one CTA for small tile counts: histogram, bucket starts and scatter in
 * shared memory */
__global__ void __launch_bounds__(1024)
k_order_small(const sftg_frame* __restrict__ frames, const uint16_t* __restrict__ tile_view, const uint32_t* __restrict__ tile_count,
              uint32_t n_tiles, uint32_t* __restrict__ order)
{
    __shared__ uint32_t h[3 * ORDER_BUCKETS], base[3 * ORDER_BUCKETS];
    for (int i = threadIdx.x; i < 3 * ORDER_BUCKETS; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < n_tiles; t += blockDim.x) atomicAdd(&h[order_bucket(frames, tile_view, tile_count, t)], 1u);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (int i = 0; i < 3 * ORDER_BUCKETS; i++) { base[i] = run; run += h[i]; }
    }
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < n_tiles; t += blockDim.x) {
        const uint32_t b = order_bucket(frames, tile_view, tile_count, t);
        order[atomicAdd(&base[b], 1u)] = t;
    }
}

#define ORDER_SMALL 8192u   /* tile counts up to this are ordered by one CTA */

int sftg_launch_tile_order(const sftg_frame* frames, const uint16_t* tile_view, const uint32_t* tile_count, uint32_t n_tiles,
                           uint32_t* scratch, uint32_t* order, cudaStream_t st) {
    if (!n_tiles) return 0;
    if (n_tiles <= ORDER_SMALL) {
        k_order_small<<<1, 1024, 0, st>>>(frames, tile_view, tile_count, n_tiles, order);
        return 1;
    }
    cudaMemsetAsync(scratch, 0, 2 * 3 * ORDER_BUCKETS * sizeof(uint32_t), st);
    const uint32_t g = (n_tiles + 255) / 256;
    k_order_count<<<g, 256, 0, st>>>(frames, tile_view, tile_count, n_tiles, scratch);
    k_order_scatter<<<g, 256, 0, st>>>(frames, tile_view, tile_count, n_tiles, scratch, scratch + 3 * ORDER_BUCKETS, order);
    return 2;
}

/* ---------------------------------------------------------------- debug overlays
 * sft__debug_draw_tile_overlay (5731-5807): tile borders and a 16-pixel grid (view 2), sample-0
 * linear depth with a border coloured by the tile's depth span (view 3), a heat tint from the
 * tile's light count (view 4).  One CTA per tile, after every tile has been resolved; each
 * overlay touches only its own tile, as in the reference where it follows that tile's resolve. */
__device__ __forceinline__ uint32_t half_blend(uint32_t bg, uint32_t ov) { return ((bg & 0xFEFEFEFEu) >> 1) + ((ov & 0xFEFEFEFEu) >> 1); }

__global__ void __launch_bounds__(256) k_debug_overlay(const sftg_tile_args A)
{
    const uint32_t gtile = blockIdx.x;
    const sftg_frame* F = A.frames + A.tile_view[gtile];
    const int mode = F->debug_mode;
    if (mode < 2 || mode > 4) return;
    const int tile = (int)(gtile - F->tile_base);
    const int tmx = (tile % F->cols) * SFTG_TILE, tmy = (tile / F->cols) * SFTG_TILE;
    const int sw = (int)(F->hw * 2.f), sh = (int)(F->hh * 2.f);
    const int lim_x = min(tmx + SFTG_TILE, sw), lim_y = min(tmy + SFTG_TILE, sh);
    uint32_t* color = F->color_dev;
    const float2* depth = A.vis + F->vis_base + (size_t)tile * F->samples * SFTG_TILE_PX;   /* sample 0 plane first */
    const float2 zr = tile_zrange(A.zrange, gtile);
    const int ntl = A.tile_nlights[gtile];
    uint32_t border = 0xFF00FF00u, heat = 0;
    if (mode == 3) {
        float dd = 0.f;
        if (zr.x <= zr.y && zr.x > 1e-6f) { const float near_w = fdiv(1.f, zr.y), far_w = fdiv(1.f, zr.x); dd = far_w - near_w; }
        border = dd > 16.f ? 0xFFFF0000u : 0xFF00FF00u;
    }
    if (mode == 4) heat = ntl == 0 ? 0xFF222288u : (ntl < 4 ? 0xFF00FF00u : 0xFFFF0000u);
    for (int i = threadIdx.x; i < SFTG_TILE_PX; i += blockDim.x) {
        const int x = tmx + (i & (SFTG_TILE - 1)), y = tmy + (i >> 6);
        if (x >= lim_x || y >= lim_y) continue;
        uint32_t* p = &color[(size_t)y * F->pitch + x];
        const bool edge = x == tmx || x == lim_x - 1 || y == tmy || y == lim_y - 1;
        if (mode == 2) {
            if (edge) *p = 0xFF00FF00u;
            else if ((x % 16 == 0) || (y % 16 == 0)) *p = half_blend(*p, 0xFF004400u);
        } else if (mode == 3) {
            if (edge) { *p = border; continue; }
            const float iw = depth[i].x;
            if (iw <= 1e-6f) continue;
            const float lz = fdiv(1.f, iw);
            const float q = fdiv(lz, 100.f);
            const float nz = q < 0.f ? 0.f : (q > 1.f ? 1.f : q);
            const uint32_t it = (uint32_t)(nz * 255.f);
            *p = 0xFF000000u | (it << 16) | (it << 8) | it;
        } else {
            *p = half_blend(*p, heat);
        }
    }
}

void sftg_launch_debug_overlay(uint32_t tiles, cudaStream_t st, const sftg_tile_args& A) {
    if (tiles) k_debug_overlay<<<tiles, 256, 0, st>>>(A);
}

/* ---------------------------------------------------------------- host-side launch helpers */
/* keys, packed set-ups, then the work items of one round: up to SETUP_CAP * (64 / slab_rows) */
static size_t raster_smem(int S, int slab_rows) {
    const size_t plane = S == 4 ? raster_plan<4>::plane : SFTG_TILE_PX, rows = S == 4 ? raster_plan<4>::rows : SFTG_TILE;
    return (size_t)S * plane * 8 + (size_t)SETUP_CAP * sizeof(tri_setup_packed) +
           (size_t)SETUP_CAP * ((rows + slab_rows - 1) / slab_rows) * 4;
}

int sftg_raster_bands(void) { return RASTER_BANDS; }

cudaError_t sftg_tile_configure(int max_dynamic_smem) {
    cudaError_t e = cudaSuccess;
    const int S_[3] = { 1, 2, 4 };
    for (int k = 0; k < 3 && e == cudaSuccess; k++) {
        const int need = (int)raster_smem(S_[k], MIN_SLAB_ROWS);
        const int v = need < max_dynamic_smem ? need : max_dynamic_smem;
        if (S_[k] == 1) e = cudaFuncSetAttribute(k_raster<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
        if (S_[k] == 2) e = cudaFuncSetAttribute(k_raster<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
        if (S_[k] == 4) e = cudaFuncSetAttribute(k_raster<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
        if (e != cudaSuccess) break;
        if (S_[k] == 1) e = cudaFuncSetAttribute(k_raster_queue<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
        if (S_[k] == 2) e = cudaFuncSetAttribute(k_raster_queue<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
        if (S_[k] == 4) e = cudaFuncSetAttribute(k_raster_queue<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
    }
    return e;
}

/* CTAs of a persistent launch: as many as are resident at once on all SMs (at least 1), never more
 * than there are items */
template <class K>
static uint32_t queue_grid(K kernel, int threads, size_t smem, uint32_t n_items) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    const uint64_t g = (uint64_t)(sms > 0 ? sms : 1) * (uint64_t)(per_sm > 0 ? per_sm : 1);
    return (uint32_t)(g < n_items ? g : n_items);
}

void sftg_launch_raster(int S, uint32_t tile0, uint32_t tiles, int slab_rows, int bands, uint32_t* queue, cudaStream_t st,
                        const sftg_tile_args& A) {
    if (!tiles) return;
    const size_t sm = raster_smem(S, slab_rows);
    const uint32_t items = tiles * RASTER_BANDS;
    if (queue) {
        if (S == 1) k_raster_queue<1><<<queue_grid(k_raster_queue<1>, RASTER_THREADS, sm, items), RASTER_THREADS, sm, st>>>(A, tile0, slab_rows, bands, items, queue);
        else if (S == 2) k_raster_queue<2><<<queue_grid(k_raster_queue<2>, RASTER_THREADS, sm, items), RASTER_THREADS, sm, st>>>(A, tile0, slab_rows, bands, items, queue);
        else k_raster_queue<4><<<queue_grid(k_raster_queue<4>, RASTER_THREADS, sm, items), RASTER_THREADS, sm, st>>>(A, tile0, slab_rows, bands, items, queue);
        return;
    }
    if (S == 1) k_raster<1><<<items, RASTER_THREADS, sm, st>>>(A, tile0, slab_rows, bands);
    else if (S == 2) k_raster<2><<<items, RASTER_THREADS, sm, st>>>(A, tile0, slab_rows, bands);
    else k_raster<4><<<items, RASTER_THREADS, sm, st>>>(A, tile0, slab_rows, bands);
}

void sftg_launch_tile_lights(uint32_t tile0, uint32_t tiles, cudaStream_t st, const sftg_tile_args& A) {
    if (tiles) k_tile_lights<<<tiles, TILE_THREADS, 0, st>>>(A, tile0);
}

void sftg_launch_resolve(int S, uint32_t tile0, uint32_t tiles, int split, bool records, uint32_t* queue, cudaStream_t st,
                         const sftg_tile_args& A) {
    if (!tiles) return;
    const uint32_t items = tiles * (uint32_t)split;
    if (queue) {
        if (S == 1) k_resolve_queue<1><<<queue_grid(k_resolve_queue<1>, TILE_THREADS, 0, items), TILE_THREADS, 0, st>>>(A, tile0, split, records, items, queue);
        else if (S == 2) k_resolve_queue<2><<<queue_grid(k_resolve_queue<2>, TILE_THREADS, 0, items), TILE_THREADS, 0, st>>>(A, tile0, split, records, items, queue);
        else k_resolve_queue<4><<<queue_grid(k_resolve_queue<4>, TILE_THREADS, 0, items), TILE_THREADS, 0, st>>>(A, tile0, split, records, items, queue);
        return;
    }
    if (S == 1) k_resolve<1><<<items, TILE_THREADS, 0, st>>>(A, tile0, split, records);
    else if (S == 2) k_resolve<2><<<items, TILE_THREADS, 0, st>>>(A, tile0, split, records);
    else k_resolve<4><<<items, TILE_THREADS, 0, st>>>(A, tile0, split, records);
}
