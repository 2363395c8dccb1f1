/*
 * The per-frame proxy occlusion pass (inside sft_present, sofren2.c:8163-8280), in three phases:
 *   k_occl_tlas      one warp per packet (light, batch of 8 proxies, one of 3 disk rays): ray
 *                    set-up, packet frustum, TLAS walk; each reached static instance becomes a
 *                    (packet, instance) pair
 *   k_occl_blas      one warp per pair: BLAS walk with one child AABB per lane
 *                    (sft__frustum_vs_bvh_node 3906-3968) and the any-hit test on lanes
 *                    (triangle, ray) (3840-3904); blocked rays are OR-ed into the packet
 *   k_occl_finalize  light_vis = 3 - blocked rays per (proxy, light)
 * The reference traces each packet serially and stops once every ray is blocked; the OR of
 * hits it accumulates does not depend on the visiting order, so splitting the walk across
 * warps gives the same light_vis.  Stacks are fixed-size in shared memory; an overflow sets a
 * status bit instead of writing out of bounds.
 */
#include "sftg_types.h"
#include "sftg_lane.cuh"
#include "sftg_kernels.h"

#define OCC_WARPS 4
#define OCC_STACK 64

struct frustum6 { float n[6][3], an[6][3], d[6]; };

/* child mask of one BVH node against a frustum: lane c < 8 tests child c */
SFTG_D uint32_t node_mask(const sftg_bvh_node* nd, const frustum6& fr, int lane) {
    bool in = false;
    if (lane < 8) {
        const float mnx = nd->mn[0][lane], mny = nd->mn[1][lane], mnz = nd->mn[2][lane];
        const float mxx = nd->mx[0][lane], mxy = nd->mx[1][lane], mxz = nd->mx[2][lane];
        const float cx = (mxx + mnx) * 0.5f, cy = (mxy + mny) * 0.5f, cz = (mxz + mnz) * 0.5f;
        const float ex = (mxx - mnx) * 0.5f, ey = (mxy - mny) * 0.5f, ez = (mxz - mnz) * 0.5f;
        in = true;
#pragma unroll
        for (int p = 0; p < 6; p++) {
            const float r = fma_(fr.an[p][0], ex, fma_(fr.an[p][1], ey, fr.an[p][2] * ez));
            const float dc = fma_(fr.n[p][0], cx, fma_(fr.n[p][1], cy, fr.n[p][2] * cz));
            const float dist = dc + fr.d[p];
            in = in && (dist + r >= 0.f);
        }
    }
    return __ballot_sync(0xFFFFFFFFu, in) & 0xFFu;
}

/* sft_m_view_look_at (1737-1770) */
SFTG_D void view_look_at(v3 pos, v3 target, v3 up, float* m) {
    const v3 fwd = snorm(sub3(target, pos));
    if (fabsf(fwd.x) < 1e-6f && fabsf(fwd.z) < 1e-6f) up = mk3(0.f, 0.f, -1.f);
    up = snorm(sub3(up, scl3(fwd, sdot(up, fwd))));
    const v3 right = cross3(up, fwd);
    m[0] = right.x; m[1] = up.x; m[2] = fwd.x; m[3] = 0.f;
    m[4] = right.y; m[5] = up.y; m[6] = fwd.y; m[7] = 0.f;
    m[8] = right.z; m[9] = up.z; m[10] = fwd.z; m[11] = 0.f;
    m[12] = -sdot(pos, right); m[13] = -sdot(pos, up); m[14] = -sdot(pos, fwd); m[15] = 1.f;
}

/* sft__build_packet_frustum (3970-4084); returns false when the reference leaves the side
 * planes undefined (a cluster corner at or behind the light); those planes then never cull. */
SFTG_D bool packet_frustum(const float* ox, const float* oy, const float* oz, uint32_t active, v3 lpos, float lrad, frustum6& f) {
    float mn[3] = { 1e9f, 1e9f, 1e9f }, mx[3] = { -1e9f, -1e9f, -1e9f };
    v3 ctr = mk3(0.f, 0.f, 0.f); int nv = 0;
    for (int i = 0; i < 8; i++) {
        if (!((active >> i) & 1u)) continue;
        if (ox[i] < mn[0]) mn[0] = ox[i];
        if (ox[i] > mx[0]) mx[0] = ox[i];
        if (oy[i] < mn[1]) mn[1] = oy[i];
        if (oy[i] > mx[1]) mx[1] = oy[i];
        if (oz[i] < mn[2]) mn[2] = oz[i];
        if (oz[i] > mx[2]) mx[2] = oz[i];
        ctr.x = ctr.x + ox[i]; ctr.y = ctr.y + oy[i]; ctr.z = ctr.z + oz[i]; nv++;
    }
    if (!nv) return true;
    ctr.x = fdiv(ctr.x, (float)nv); ctr.y = fdiv(ctr.y, (float)nv); ctr.z = fdiv(ctr.z, (float)nv);
    const v3 lf0 = snorm(sub3(ctr, lpos));
    v3 up = mk3(0.f, 1.f, 0.f);
    if (fabsf(lf0.y) > 0.99f) up = mk3(1.f, 0.f, 0.f);
    float lv[16];
    view_look_at(lpos, ctr, up, lv);
    float mnxz = 1e9f, mxxz = -1e9f, mnyz = 1e9f, mxyz = -1e9f;
    bool invalid = false;
    for (int k = 0; k < 8; k++) {
        const float x = (k & 1) ? mx[0] : mn[0], y = (k & 2) ? mx[1] : mn[1], z = (k & 4) ? mx[2] : mn[2];
        const float cxv = x * lv[0] + y * lv[4] + z * lv[8] + 1.f * lv[12];
        const float cyv = x * lv[1] + y * lv[5] + z * lv[9] + 1.f * lv[13];
        const float czv = x * lv[2] + y * lv[6] + z * lv[10] + 1.f * lv[14];
        if (czv < 1e-6f) { invalid = true; break; }
        const float qx = fdiv(cxv, czv), qy = fdiv(cyv, czv);
        if (qx < mnxz) mnxz = qx;
        if (qx > mxxz) mxxz = qx;
        if (qy < mnyz) mnyz = qy;
        if (qy > mxyz) mxyz = qy;
    }
    const v3 lr = mk3(lv[0], lv[4], lv[8]), lu = mk3(lv[1], lv[5], lv[9]), lf = mk3(lv[2], lv[6], lv[10]);
    if (invalid) {
        for (int p = 0; p < 4; p++) { for (int a = 0; a < 3; a++) { f.n[p][a] = 0.f; f.an[p][a] = 0.f; } f.d[p] = 1e30f; }
    } else {
        const v3 nl[4] = { mk3(1.f, 0.f, -mnxz), mk3(-1.f, 0.f, mxxz), mk3(0.f, 1.f, -mnyz), mk3(0.f, -1.f, mxyz) };
        for (int p = 0; p < 4; p++) {
            const v3 q = snorm(nl[p]);
            const v3 nw = add3(scl3(lr, q.x), add3(scl3(lu, q.y), scl3(lf, q.z)));
            f.n[p][0] = nw.x; f.n[p][1] = nw.y; f.n[p][2] = nw.z;
            f.d[p] = -sdot(nw, lpos) + 0.1f;
            f.an[p][0] = fabsf(nw.x); f.an[p][1] = fabsf(nw.y); f.an[p][2] = fabsf(nw.z);
        }
    }
    f.n[4][0] = lf.x; f.n[4][1] = lf.y; f.n[4][2] = lf.z; f.d[4] = -sdot(lf, lpos) + 0.1f;
    f.an[4][0] = fabsf(lf.x); f.an[4][1] = fabsf(lf.y); f.an[4][2] = fabsf(lf.z);
    const v3 nlf = mk3(-lf.x, -lf.y, -lf.z);
    f.n[5][0] = nlf.x; f.n[5][1] = nlf.y; f.n[5][2] = nlf.z; f.d[5] = -sdot(nlf, lpos) + lrad;
    f.an[5][0] = f.an[4][0]; f.an[5][1] = f.an[4][1]; f.an[5][2] = f.an[4][2];
    return !invalid;
}

/* status bits */
#define OCC_STACK_OVERFLOW 1u
#define OCC_UNDEFINED_FRUSTUM 2u
#define OCC_PAIR_OVERFLOW 4u

/* one traced packet: 8 rays from proxy points toward one point of the light disk */
struct sftg_packet {
    frustum6 f;                 /* world-space packet frustum */
    float o[3][8], e[3][8];     /* ray origins and ends (origin + L) */
    uint32_t active;
    uint32_t hits;              /* OR of the rays found blocked */
};

/* Phase A: one warp per packet (light, proxy batch, ray): ray set-up, packet frustum and the
 * TLAS walk (sofren2.c:8178-8269, 4086-4135); every static instance the frustum reaches becomes
 * a (packet, instance) pair for phase B. */
__global__ void __launch_bounds__(OCC_WARPS * 32)
k_occl_tlas(const sftg_frame* __restrict__ frames, const uint16_t* __restrict__ packet_view, uint32_t n_packets,
            sftg_packet* __restrict__ packets, uint2* __restrict__ pairs, uint32_t* __restrict__ n_pairs, uint32_t max_pairs,
            uint32_t* __restrict__ status)
{
    __shared__ uint32_t s_stack[OCC_WARPS][OCC_STACK];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t pk = blockIdx.x * OCC_WARPS + warp;   /* batch-wide packet index */
    if (pk >= n_packets) return;
    const sftg_frame* F = frames + packet_view[pk];
    const uint32_t lpk = pk - F->packet_base;            /* packet index within the view */
    const uint32_t pc = F->n_proxies, nbatch = (pc + 7) / 8;
    const uint32_t ray = lpk % 3, b = (lpk / 3) % nbatch, l = lpk / (3 * nbatch), pb = b * 8;
    const sftg_point_light L = F->point[l];
    const v3 lpos = mk3(L.pos[0], L.pos[1], L.pos[2]);
    /* batch centre and light-disk targets, identical on every lane */
    v3 bc = mk3(0.f, 0.f, 0.f); int na = 0;
    for (int k = 0; k < 8; k++) {
        if (pb + k >= pc) continue;
        const sftg_proxy px = F->proxies[pb + k];
        bc.x = bc.x + (px.posa[0] + px.posb[0]) * 0.5f; bc.y = bc.y + (px.posa[1] + px.posb[1]) * 0.5f; bc.z = bc.z + (px.posa[2] + px.posb[2]) * 0.5f;
        na++;
    }
    if (na > 0) bc = scl3(bc, fdiv(1.f, (float)na));
    const v3 ldir = snorm(sub3(lpos, bc));
    float mnv = fabsf(ldir.x); v3 card = mk3(1.f, 0.f, 0.f);
    if (fabsf(ldir.y) < mnv) { mnv = fabsf(ldir.y); card = mk3(0.f, 1.f, 0.f); }
    if (fabsf(ldir.z) < mnv) card = mk3(0.f, 0.f, 1.f);
    const v3 perp = mk3(ldir.y * card.z - ldir.z * card.y, ldir.z * card.x - ldir.x * card.z, ldir.x * card.y - ldir.y * card.x);
    const v3 lright = snorm(perp);
    const v3 lup = cross3(lright, ldir);
    const float r = 0.1f;
    v3 tg;
    if (ray == 0) tg = add3(lpos, scl3(lup, r));
    else if (ray == 1) tg = add3(lpos, add3(scl3(lright, r * 0.866025f), scl3(lup, -r * 0.5f)));
    else tg = add3(lpos, add3(scl3(lright, -r * 0.866025f), scl3(lup, -r * 0.5f)));
    float ox[8], oy[8], oz[8];
    uint32_t am = 0;
    sftg_packet* P = &packets[pk];
    for (int k = 0; k < 8; k++) {
        float x = 0.f, y = 0.f, z = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
        if (pb + k < pc) {
            const sftg_proxy px = F->proxies[pb + k];
            if (ray == 0) { x = px.posa[0]; y = px.posa[1]; z = px.posa[2]; }
            else if (ray == 1) { x = px.posb[0]; y = px.posb[1]; z = px.posb[2]; }
            else { x = (px.posa[0] + px.posb[0]) * 0.5f; y = (px.posa[1] + px.posb[1]) * 0.5f; z = (px.posa[2] + px.posb[2]) * 0.5f; }
            lx = tg.x - x; ly = tg.y - y; lz = tg.z - z;
            am |= 1u << k;
        }
        ox[k] = x; oy[k] = y; oz[k] = z;
        if (lane == k) {
            P->o[0][k] = x; P->o[1][k] = y; P->o[2][k] = z;
            P->e[0][k] = x + lx; P->e[1][k] = y + ly; P->e[2][k] = z + lz;
        }
    }
    frustum6 pf;
    if (!packet_frustum(ox, oy, oz, am, lpos, L.radius, pf) && lane == 0) atomicOr(status, OCC_UNDEFINED_FRUSTUM);
    if (lane == 0) { P->f = pf; P->active = am; P->hits = 0; }
    if (am == 0 || F->tlas_count == 0) return;
    int top = 1;
    if (lane == 0) s_stack[warp][0] = F->tlas_root;
    __syncwarp();
    /* lane c < 8 handles child c of each node: pushes (inner nodes) and pair emission (leaves)
     * are warp-aggregated; the pairs' order does not matter (hits are OR-ed) */
    while (top > 0) {
        const uint32_t ni = s_stack[warp][--top];
        __syncwarp();
        const sftg_bvh_node* nd = &F->tlas[ni];
        const uint32_t m = node_mask(nd, pf, lane);
        const uint32_t ch = lane < 8 ? nd->child[lane] : SFTG_INVALID;
        const bool mine = lane < 8 && ((m >> lane) & 1u) && ch != SFTG_INVALID;
        if (!nd->leaf) {
            if (__ballot_sync(0xFFFFFFFFu, mine && ch >= F->tlas_count)) { if (lane == 0) atomicOr(status, OCC_STACK_OVERFLOW); return; }
            const uint32_t pm = __ballot_sync(0xFFFFFFFFu, mine);
            if (top + __popc(pm) > OCC_STACK) { if (lane == 0) atomicOr(status, OCC_STACK_OVERFLOW); return; }
            if (mine) s_stack[warp][top + __popc(pm & ((1u << lane) - 1u))] = ch;
            top += __popc(pm);
            __syncwarp();
            continue;
        }
        bool emit = false;
        const uint32_t ii = ch & ~0x80000000u;
        if (mine && ii < F->n_inst) {
            const sftg_model Md = F->models[F->inst[ii].model];
            emit = !(Md.bone_count > 0 || Md.blas_count == 0);   /* static instances only */
        }
        const uint32_t em = __ballot_sync(0xFFFFFFFFu, emit);
        if (!em) continue;
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(n_pairs, (uint32_t)__popc(em));
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (emit) {
            const uint32_t slot = base + __popc(em & ((1u << lane) - 1u));
            if (slot < max_pairs) pairs[slot] = make_uint2(pk, ii);
            else atomicOr(status, OCC_PAIR_OVERFLOW);
        }
    }
}

/* Phase B: a warp per (packet, static instance) pair, in two launches.  The packet frustum and
 * rays are taken into model space, then the BLAS is walked with one child AABB per lane
 * (4137-4238); at a leaf, lanes are (triangle k of 4, ray r of 8) and run the any-hit test
 * (3840-3904).  Hits are OR-ed into the packet, which is what the reference accumulates in any
 * visiting order, so a walk can be split into independent sub-walks: the expand launch walks
 * the top OCC_EXPAND_DEPTH levels of every pair and turns each deeper node that passes the
 * frustum test into an item (pair, node); the walk launch runs every item to the bottom.  Both
 * start from the rays the packet already has blocked, which only skips tests whose outcome is
 * already recorded. */
#define OCC_EXPAND_DEPTH 2
#define OCC_GRID_CTAS (152 * 8)

struct occ_walk {
    frustum6 mf;
    v3 lo, ld;
    float tmax;
    uint32_t full;
};

/* The packet's 8 rays in model space, shared by the warp, for the ray-box prune below. */
struct occ_rays { float ox[8], oy[8], oz[8], ix[8], iy[8], iz[8], tmax[8]; };

/* Optional second cull (sftg_tuning.occl_ray_prune) of the children the frustum test kept: child
 * c (lane & 7) survives if one of the rays still unblocked, (lane >> 3) or (lane >> 3) + 4,
 * passes through its box grown by a margin.  A well-conditioned any-hit test only reports
 * triangles within rounding of the ray, so the result is unchanged; but when a ray grazes a
 * triangle's plane (|a| just above the test's 1e-6 threshold while its true value is rounding
 * noise) the reference's u, v and t are noise and it can report a hit far from the ray, which
 * this cull would skip.  That is why it is off by default. */
SFTG_D uint32_t ray_box_mask(const sftg_bvh_node* nd, const occ_rays& R, uint32_t open_rays, int lane) {
    const int c = lane & 7;
    const float lo[3] = { nd->mn[0][c], nd->mn[1][c], nd->mn[2][c] };
    const float hi[3] = { nd->mx[0][c], nd->mx[1][c], nd->mx[2][c] };
    float blo[3], bhi[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float m = 1e-4f * (fabsf(lo[a]) + fabsf(hi[a]) + (hi[a] - lo[a])) + 1e-5f;
        blo[a] = lo[a] - m; bhi[a] = hi[a] + m;
    }
    bool hit = false;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int r = (lane >> 3) + 4 * h;
        if (!((open_rays >> r) & 1u)) continue;
        const float o[3] = { R.ox[r], R.oy[r], R.oz[r] }, id[3] = { R.ix[r], R.iy[r], R.iz[r] };
        float tn = -3.0e38f, tf = 3.0e38f;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const float t1 = (blo[a] - o[a]) * id[a], t2 = (bhi[a] - o[a]) * id[a];
            tn = fmaxf(tn, fminf(t1, t2)); tf = fminf(tf, fmaxf(t1, t2));
        }
        const float tm = R.tmax[r] * 1.0001f + 1e-4f;
        hit = hit || (tn <= tf && tf >= -1e-4f && tn <= tm);
    }
    const uint32_t b = __ballot_sync(0xFFFFFFFFu, hit);
    return (b | (b >> 8) | (b >> 16) | (b >> 24)) & 0xFFu;
}

/* lanes 0..7 publish their ray; inverse directions with zero components made huge, not infinite */
SFTG_D void occ_rays_publish(const occ_walk& w, occ_rays& R, int lane) {
    if (lane < 8) {
        R.ox[lane] = w.lo.x; R.oy[lane] = w.lo.y; R.oz[lane] = w.lo.z;
        R.ix[lane] = w.ld.x != 0.f ? 1.f / w.ld.x : copysignf(1e30f, w.ld.x);
        R.iy[lane] = w.ld.y != 0.f ? 1.f / w.ld.y : copysignf(1e30f, w.ld.y);
        R.iz[lane] = w.ld.z != 0.f ? 1.f / w.ld.z : copysignf(1e30f, w.ld.z);
        R.tmax[lane] = w.tmax;
    }
    __syncwarp();
}

SFTG_D void occ_pair_setup(const sftg_inst* I, const sftg_packet* P, int lane, occ_walk& w) {
    const frustum6 pf = P->f;
    const float* M = I->T;
    for (int p = 0; p < 6; p++) {
        const float nx = pf.n[p][0], ny = pf.n[p][1], nz = pf.n[p][2], d = pf.d[p];
        const float nmx = nx * M[0] + ny * M[1] + nz * M[2];
        const float nmy = nx * M[4] + ny * M[5] + nz * M[6];
        const float nmz = nx * M[8] + ny * M[9] + nz * M[10];
        const float dot_t = nx * M[12] + ny * M[13] + nz * M[14];
        const float dm = dot_t + d;
        const float il = fdiv(1.f, fsqrt(nmx * nmx + nmy * nmy + nmz * nmz));
        w.mf.n[p][0] = nmx * il; w.mf.n[p][1] = nmy * il; w.mf.n[p][2] = nmz * il;
        w.mf.d[p] = dm * il;
        w.mf.an[p][0] = fabsf(nmx * il); w.mf.an[p][1] = fabsf(nmy * il); w.mf.an[p][2] = fabsf(nmz * il);
    }
    /* sft_m_qinv (1693-1712) */
    float im[16];
    im[0] = M[0]; im[1] = M[4]; im[2] = M[8]; im[3] = 0.f;
    im[4] = M[1]; im[5] = M[5]; im[6] = M[9]; im[7] = 0.f;
    im[8] = M[2]; im[9] = M[6]; im[10] = M[10]; im[11] = 0.f;
    for (int a = 0; a < 3; a++) im[12 + a] = -(M[12] * im[a] + M[13] * im[4 + a] + M[14] * im[8 + a]);
    im[15] = 1.f;
    const int r = lane & 7;
    w.lo = xform(mk3(P->o[0][r], P->o[1][r], P->o[2][r]), im);
    const v3 le = xform(mk3(P->e[0][r], P->e[1][r], P->e[2][r]), im);
    const v3 Lv = sub3(le, w.lo);
    w.tmax = fsqrt(vdot(Lv, Lv));
    w.ld = vnorm_fast(Lv);
    w.full = P->active;
}

/* Walks the BLAS of instance I from `start` (depth `start_depth`).  With EXPAND, a child that
 * would sit at depth OCC_EXPAND_DEPTH is handed out as an item instead of being pushed (or
 * pushed after all when the item list is full).  Returns the rays found blocked. */
template <bool EXPAND>
SFTG_D uint32_t occ_walk_from(const sftg_frame* F, const sftg_inst* I, const sftg_model& Md, const occ_walk& w, uint32_t sat,
                              uint32_t start, uint32_t pair, uint32_t* stack, const occ_rays& R, bool prune, uint2* items,
                              uint32_t* n_items, uint32_t max_items, uint32_t* status, int lane) {
    const int r = lane & 7, kq = lane >> 3;
    const uint32_t full = w.full;
    int top = 1;
    if (lane == 0) stack[0] = start;      /* entry: node | depth << 29 (depth only tracked when expanding) */
    __syncwarp();
    const sftg_bvh_node* blas = F->blas + Md.blas_base;
    uint32_t guard = 0;
    while (top > 0 && sat != full) {
        const uint32_t ent = stack[--top];
        __syncwarp();
        const uint32_t ni = ent & 0x1FFFFFFFu, depth = ent >> 29;
        const sftg_bvh_node* nd = &blas[ni];
        uint32_t m = node_mask(nd, w.mf, lane);
        if (prune && m) m &= ray_box_mask(nd, R, full & ~sat, lane);
        if (!nd->leaf) {
            /* lane c < 8 takes child c: one ballot for the checks, one atomic for the items, one
             * stack write per lane (the stack keeps the children in slot order) */
            const uint32_t ch = lane < 8 ? nd->child[lane] : SFTG_INVALID;
            const bool mine = lane < 8 && ((m >> lane) & 1u) && ch != SFTG_INVALID;
            const uint32_t tm = __ballot_sync(0xFFFFFFFFu, mine);
            guard += (uint32_t)__popc(tm);
            if (__ballot_sync(0xFFFFFFFFu, mine && (ch >= Md.blas_count || ch >= (1u << 29))) || guard > (1u << 24)) {
                if (lane == 0) atomicOr(status, OCC_STACK_OVERFLOW);
                return sat;
            }
            if (!tm) continue;
            uint32_t pm = tm;
            if (EXPAND && depth + 1 >= OCC_EXPAND_DEPTH) {
                uint32_t base = 0;
                if (lane == 0) base = atomicAdd(n_items, (uint32_t)__popc(tm));
                base = __shfl_sync(0xFFFFFFFFu, base, 0);
                const bool placed = mine && base + __popc(tm & ((1u << lane) - 1u)) < max_items;
                if (placed) items[base + __popc(tm & ((1u << lane) - 1u))] = make_uint2(pair, ch);
                pm = tm & ~__ballot_sync(0xFFFFFFFFu, placed);   /* children without an item slot are walked here */
            }
            if (pm) {
                if (top + __popc(pm) > OCC_STACK) {
                    if (lane == 0) atomicOr(status, OCC_STACK_OVERFLOW);
                    return sat;
                }
                if ((pm >> lane) & 1u) stack[top + __popc(pm & ((1u << lane) - 1u))] = ch | (EXPAND ? (depth + 1) << 29 : 0u);
                top += __popc(pm);
                __syncwarp();
            }
            continue;
        }
        while (m && sat != full) {
            /* the next up to 4 triangles of this leaf, lane = (triangle kq, ray r) */
            int c = -1;
            uint32_t mm = m;
            for (int q = 0; q <= kq && mm; q++) { c = __ffs(mm) - 1; mm &= mm - 1; }
            const bool have = (__popc(m) > kq) && c >= 0;
            for (int q = 0; q < 4 && m; q++) m &= m - 1;
            bool hit = false;
            if (have && nd->child[c] != SFTG_INVALID && ((full & ~sat) >> r & 1u)) {
                const uint32_t pay = nd->child[c] & ~0x80000000u;
                const uint32_t g = I->meshlet_base + (pay >> 7), t = pay & 0x7F;
                const uint8_t* ind = F->ml_inds + (size_t)g * 512;
                const float* at = F->ml_attr + (size_t)g * 640;
                const uint32_t tb = t >> 3, tl = t & 7;
                const uint32_t i0 = ind[tb * 32 + tl], i1 = ind[tb * 32 + 8 + tl], i2 = ind[tb * 32 + 16 + tl];
                const v3 v0 = mk3(at[i0], at[64 + i0], at[128 + i0]);
                const v3 v1 = mk3(at[i1], at[64 + i1], at[128 + i1]);
                const v3 v2 = mk3(at[i2], at[64 + i2], at[128 + i2]);
                const v3 e1 = sub3(v1, v0), e2 = sub3(v2, v0);
                const v3 h = cross3(w.ld, e2);
                const float a = vdot(e1, h);
                hit = fabsf(a) > 1e-6f;
                const float fr = rcpr(a);
                const v3 sv = sub3(w.lo, v0);
                const float u = fr * vdot(sv, h);
                hit = hit && u >= 0.f && u <= 1.f;
                const v3 q = cross3(sv, e1);
                const float v = fr * vdot(w.ld, q);
                hit = hit && v >= 0.f && (u + v) <= 1.f;
                const float tt = fr * vdot(e2, q);
                hit = hit && tt > 1e-6f && tt < w.tmax;
            }
            const uint32_t bal = __ballot_sync(0xFFFFFFFFu, hit);
            sat |= (bal | (bal >> 8) | (bal >> 16) | (bal >> 24)) & 0xFFu;
        }
    }
    return sat;
}

SFTG_D uint32_t occ_hits_now(const sftg_packet* P) { return *(volatile const uint32_t*)&P->hits; }

__global__ void __launch_bounds__(OCC_WARPS * 32)
k_occl_blas_expand(const sftg_frame* __restrict__ frames, const uint16_t* __restrict__ packet_view, sftg_packet* __restrict__ packets,
                   const uint2* __restrict__ pairs, const uint32_t* __restrict__ n_pairs, uint32_t max_pairs,
                   uint2* __restrict__ items, uint32_t* __restrict__ n_items, uint32_t max_items, uint32_t* __restrict__ status,
                   int prune)
{
    __shared__ uint32_t s_stack[OCC_WARPS][OCC_STACK];
    __shared__ occ_rays s_rays[OCC_WARPS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t np = min(*n_pairs, max_pairs);
    for (uint32_t item = blockIdx.x * OCC_WARPS + warp; item < np; item += gridDim.x * OCC_WARPS) {
        const uint2 pr = pairs[item];
        const sftg_frame* F = frames + packet_view[pr.x];
        sftg_packet* P = &packets[pr.x];
        const sftg_inst* I = &F->inst[pr.y];
        const sftg_model Md = F->models[I->model];
        occ_walk w;
        occ_pair_setup(I, P, lane, w);
        occ_rays_publish(w, s_rays[warp], lane);
        const uint32_t sat = occ_walk_from<true>(F, I, Md, w, occ_hits_now(P) & w.full, Md.blas_root, item, s_stack[warp],
                                                 s_rays[warp], prune != 0, items, n_items, max_items, status, lane);
        if (lane == 0 && sat) atomicOr(&P->hits, sat);
        __syncwarp();
    }
}

__global__ void __launch_bounds__(OCC_WARPS * 32)
k_occl_blas_walk(const sftg_frame* __restrict__ frames, const uint16_t* __restrict__ packet_view, sftg_packet* __restrict__ packets,
                 const uint2* __restrict__ pairs, const uint2* __restrict__ items, const uint32_t* __restrict__ n_items,
                 uint32_t max_items, uint32_t* __restrict__ status, int prune)
{
    __shared__ uint32_t s_stack[OCC_WARPS][OCC_STACK];
    __shared__ occ_rays s_rays[OCC_WARPS];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t ni = min(*n_items, max_items);
    for (uint32_t it = blockIdx.x * OCC_WARPS + warp; it < ni; it += gridDim.x * OCC_WARPS) {
        const uint2 itm = items[it];
        const uint2 pr = pairs[itm.x];
        const sftg_frame* F = frames + packet_view[pr.x];
        sftg_packet* P = &packets[pr.x];
        const uint32_t known = occ_hits_now(P) & P->active;
        if (known == P->active) continue;            /* every ray already blocked */
        const sftg_inst* I = &F->inst[pr.y];
        const sftg_model Md = F->models[I->model];
        occ_walk w;
        occ_pair_setup(I, P, lane, w);
        occ_rays_publish(w, s_rays[warp], lane);
        const uint32_t sat = occ_walk_from<false>(F, I, Md, w, known, itm.y, 0, s_stack[warp], s_rays[warp], prune != 0, nullptr,
                                                  nullptr, 0, status, lane);
        if (lane == 0 && (sat & ~known)) atomicOr(&P->hits, sat);
        __syncwarp();
    }
}

/* Phase C: light_vis[p][l] = 3 - rays blocked (8169-8276); one thread per (batch-wide proxy,
 * light column); columns at or beyond the view's light count keep the zero they were cleared to. */
__global__ void k_occl_finalize(const sftg_frame* __restrict__ frames, const uint16_t* __restrict__ prox_view, uint32_t n_proxies,
                                const sftg_packet* __restrict__ packets, uint8_t* __restrict__ light_vis)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_proxies * 64) return;
    const uint32_t gp = i >> 6, l = i & 63;
    const sftg_frame* F = frames + prox_view[gp];
    const uint32_t pc = F->n_proxies, lc = min(F->n_point, 64u), nbatch = (pc + 7) / 8;
    if (l >= lc) return;
    const uint32_t p = gp - F->prox_base, b = p / 8, k = p % 8;
    const sftg_packet* P = packets + F->packet_base;
    int blocked = 0;
    for (int ray = 0; ray < 3; ray++) blocked += (P[(l * nbatch + b) * 3 + ray].hits >> k) & 1u;
    light_vis[(size_t)gp * 64 + l] = (uint8_t)(3 - blocked);
}

size_t sftg_packet_bytes() { return sizeof(sftg_packet); }

void sftg_launch_occlusion(const sftg_frame* frames, const uint16_t* packet_view, uint32_t n_packets, const uint16_t* prox_view,
                           uint32_t n_proxies, uint32_t max_inst, void* packets, uint2* pairs, uint32_t* n_pairs,
                           uint32_t max_pairs, uint32_t items_per_pair, uint8_t* light_vis, uint32_t* status, int ray_prune,
                           cudaStream_t st) {
    cudaMemsetAsync(n_pairs, 0, 8, st);   /* pair and item counters */
    if (!n_packets) return;
    k_occl_tlas<<<(n_packets + OCC_WARPS - 1) / OCC_WARPS, OCC_WARPS * 32, 0, st>>>(frames, packet_view, n_packets,
                                                                                   (sftg_packet*)packets, pairs, n_pairs, max_pairs, status);
    /* the item list shares the pair buffer's tail: pairs take [0, max_pairs), items the rest */
    uint2* items = pairs + max_pairs;
    uint32_t* n_items = n_pairs + 1;
    const uint32_t max_items = max_pairs * items_per_pair;
    const uint64_t want = (uint64_t)n_packets * (max_inst ? max_inst : 1);
    const uint32_t mp = want < max_pairs ? (uint32_t)want : max_pairs;
    const uint32_t g1 = (mp + OCC_WARPS - 1) / OCC_WARPS;
    k_occl_blas_expand<<<g1 < OCC_GRID_CTAS ? g1 : OCC_GRID_CTAS, OCC_WARPS * 32, 0, st>>>(frames, packet_view, (sftg_packet*)packets,
                                                                                         pairs, n_pairs, max_pairs, items, n_items,
                                                                                         max_items, status, ray_prune);
    k_occl_blas_walk<<<OCC_GRID_CTAS, OCC_WARPS * 32, 0, st>>>(frames, packet_view, (sftg_packet*)packets, pairs, items, n_items,
                                                               max_items, status, ray_prune);
    k_occl_finalize<<<(n_proxies * 64 + 255) / 256, 256, 0, st>>>(frames, prox_view, n_proxies, (const sftg_packet*)packets, light_vis);
}
