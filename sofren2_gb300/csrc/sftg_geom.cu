/*
 * Geometry, clipping and binning kernels of the sofren2 render path.
 *
 *   k_geometry  one warp per job of up to 8 meshlets (sft__worker_phase_geom, sofren2.c:4901-5145):
 *               lanes 0-7 run the bounding-sphere frustum test and normal-cone test; each
 *               surviving meshlet is skinned (4 joints, bone matrices staged in shared
 *               memory), transformed and projected two vertices per lane, written to the
 *               screen-space cache, then its 128 triangles are set up four batches at a
 *               time (sft__geom_setup_and_bin_batch, 4775-4884): one 8-lane group per batch,
 *               shuffles build the batch's tile rectangle and lane mask.
 *   k_clip      near-plane clipping of straddling triangles (4691-4772, 4264-4381); clip
 *               slots come from an exclusive scan of per-batch clip counts, which numbers
 *               them in the reference's single-worker emission order.
 *   k_coarse    one CTA per super-tile (4 x 4 tiles) lists, in slot order, the meshlets of its
 *               view whose tile rectangle overlaps it; run once to count and once to write.
 *   k_bin       one CTA per tile builds that tile's payload list in the reference's order
 *               (meshlet, batch, clipped triangles before the batch payload) with ordered
 *               warp-aggregated compaction over its super-tile's meshlet list (every meshlet
 *               that touches the tile is on it, in slot order); run once to count and once
 *               to write.
 *   k_scan_*    a three-phase exclusive scan used for clip slots and tile list offsets.
 */
#include "sftg_types.h"
#include "sftg_lane.cuh"
#include "sftg_kernels.h"

#define GEOM_WARPS 4
#define GEOM_BONES 64

/* ----------------------------------------------------------------------------------------- */
__global__ void __launch_bounds__(GEOM_WARPS * 32)
k_geometry(const sftg_frame* __restrict__ frames, const sftg_job* __restrict__ jobs, uint32_t n_jobs, float* __restrict__ ss,
           sftg_batch_rec* __restrict__ recs, uint32_t* __restrict__ clip_cnt, int4* __restrict__ mrect)
{
    __shared__ float s_bones[GEOM_WARPS][GEOM_BONES * 16];
    __shared__ float s_v[GEOM_WARPS][6][64];   /* tx ty tz w sx sy */
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t job_i = blockIdx.x * GEOM_WARPS + warp;
    if (job_i >= n_jobs) return;
    const sftg_job J = jobs[job_i];
    const sftg_frame* F = frames + J.view;
    const sftg_inst* I = &F->inst[J.inst];
    float T[16];
#pragma unroll
    for (int k = 0; k < 16; k++) T[k] = I->T[k];
    const sftg_model Md = F->models[I->model];
    const float* bones_g = (J.skinned && I->bones >= 0) ? F->bones + (size_t)I->bones * 16 : nullptr;
    const int nb = (int)Md.bone_count;
    const bool bones_in_smem = bones_g && nb <= GEOM_BONES;
    if (bones_in_smem) {
        for (int k = lane; k < nb * 16; k += 32) s_bones[warp][k] = bones_g[k];
        __syncwarp();
    }
    const float* bones = bones_in_smem ? s_bones[warp] : bones_g;

    /* ---- cull (lanes 0..7), 4939-4994 ---- */
    bool inside = false;
    const uint32_t g0 = I->meshlet_base + J.first;
    if (lane < (int)J.count) {
        const float* cl = F->ml_cull + (size_t)(g0 + lane) * 8;
        v3 ctr = mk3(cl[0], cl[1], cl[2]), ax = mk3(cl[4], cl[5], cl[6]);
        if (J.skinned) {
            const int cb = F->ml_info[I->meshlet_base + J.group_first].culling_bone;   /* the group's first bone */
            const float* B = bones + (size_t)cb * 16;
            ctr = xform(ctr, B); ax = xform_dir(ax, B);
        }
        ctr = xform(ctr, T); ax = xform_dir(ax, T);
        const float sxs = fsqrt(T[0] * T[0] + T[1] * T[1] + T[2] * T[2]);
        const float rad = cl[3] * sxs;
        ax = vnorm(ax);
        bool in = true;
#pragma unroll
        for (int p = 0; p < 6; p++) {
            const float dist = vdot(ctr, mk3(F->fn[p][0], F->fn[p][1], F->fn[p][2])) + F->fd[p];
            in = in && (dist + rad >= 0.f);
        }
        const v3 vr = sub3(ctr, mk3(F->cam[0], F->cam[1], F->cam[2]));
        const float dd = fsqrt(vdot(vr, vr));
        const float dv = vdot(vr, ax);
        const float thr = fma_(dd, cl[7], rad);
        inside = in && (dv <= thr);
    }
    const uint32_t alive = __ballot_sync(0xFFFFFFFFu, inside) & 0xFFu;

    const float hw = F->hw, hh = F->hh;
    const float bias_x = hw + F->vpx, scale_y = -hh, bias_y = hh + F->vpy;
    const float* VP = F->vp;
    const int cols = F->cols, rows = F->rows;

    for (uint32_t ln = 0; ln < J.count; ln++) {
        const uint32_t m = J.first + ln;             /* model-relative meshlet index */
        const uint32_t g = I->meshlet_base + m;      /* pool index */
        const uint32_t ssi = F->ss_base + I->ss_offset + m;
        if (!((alive >> ln) & 1u)) {
            if (lane < 16) {
                sftg_batch_rec r; r.payload = 0; r.x0 = 1; r.x1 = 0; r.y0 = 1; r.y1 = 0;
                recs[(size_t)ssi * 16 + lane] = r;
                clip_cnt[(size_t)ssi * 16 + lane] = 0;
            }
            if (lane == 0) mrect[ssi] = make_int4(1, 0, 1, 0);
            continue;
        }
        const float* at = F->ml_attr + (size_t)g * 640;
        float* S = ss + (size_t)ssi * SFTG_SS_FLOATS;
        const sftg_meshlet_info info = F->ml_info[g];
        /* ---- vertices: lane and lane + 32 (5015-5124) ---- */
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int v = lane + 32 * h;
            const v3 p = mk3(at[v], at[64 + v], at[128 + v]);
            const v3 n = mk3(at[192 + v], at[256 + v], at[320 + v]);
            v3 pw, nw;
            if (J.skinned) {
                const uint16_t* js = F->skin_j + (size_t)info.skin_slot * 256;
                const uint8_t* ws = F->skin_w + (size_t)info.skin_slot * 256;
                const float inv255 = 1.f / 255.f;
                v3 vp[4], vn[4]; float wt[4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const float* M = bones + (size_t)js[k * 64 + v] * 16;
                    wt[k] = (float)ws[k * 64 + v] * inv255;
                    vp[k] = xform(p, M); vn[k] = xform_dir(n, M);
                }
                pw.x = fma_(vp[0].x, wt[0], fma_(vp[1].x, wt[1], fma_(vp[2].x, wt[2], vp[3].x * wt[3])));
                pw.y = fma_(vp[0].y, wt[0], fma_(vp[1].y, wt[1], fma_(vp[2].y, wt[2], vp[3].y * wt[3])));
                pw.z = fma_(vp[0].z, wt[0], fma_(vp[1].z, wt[1], fma_(vp[2].z, wt[2], vp[3].z * wt[3])));
                nw.x = fma_(vn[0].x, wt[0], fma_(vn[1].x, wt[1], fma_(vn[2].x, wt[2], vn[3].x * wt[3])));
                nw.y = fma_(vn[0].y, wt[0], fma_(vn[1].y, wt[1], fma_(vn[2].y, wt[2], vn[3].y * wt[3])));
                nw.z = fma_(vn[0].z, wt[0], fma_(vn[1].z, wt[1], fma_(vn[2].z, wt[2], vn[3].z * wt[3])));
                pw = xform(pw, T); nw = xform_dir(nw, T);
            } else {
                pw = xform(p, T); nw = xform_dir(n, T);
            }
            const float w = fma_(pw.x, VP[3], fma_(pw.y, VP[7], fma_(pw.z, VP[11], VP[15])));
            const float tx = fma_(pw.x, VP[0], fma_(pw.y, VP[4], fma_(pw.z, VP[8], VP[12])));
            const float ty = fma_(pw.x, VP[1], fma_(pw.y, VP[5], fma_(pw.z, VP[9], VP[13])));
            const float tz = fma_(pw.x, VP[2], fma_(pw.y, VP[6], fma_(pw.z, VP[10], VP[14])));
            const float iw = rcpr(w);
            const float sx = fma_(tx, iw * hw, bias_x), sy = fma_(ty, iw * scale_y, bias_y);
            /* vertex-major record (sftg_types.h, SFTG_SS_*): two float4 and one float per vertex */
            ((float4*)(S + SFTG_SS_A))[v] = make_float4(x86nan(sx), x86nan(sy), x86nan(iw), pw.x);
            ((float4*)(S + SFTG_SS_B))[v] = make_float4(pw.y, pw.z, nw.x, nw.y);
            ((float4*)(S + SFTG_SS_C))[v] = make_float4(nw.z, at[384 + v], at[448 + v], at[512 + v]);
            S[SFTG_SS_D + v] = at[576 + v];
            s_v[warp][0][v] = tx; s_v[warp][1][v] = ty; s_v[warp][2][v] = tz; s_v[warp][3][v] = w;
            s_v[warp][4][v] = sx; s_v[warp][5][v] = sy;
        }
        __syncwarp();
        /* ---- triangle batches: 4 per round, one 8-lane group each (4775-4884) ---- */
        const uint8_t* ind = F->ml_inds + (size_t)g * 512;
        const int grp = lane >> 3, tl = lane & 7;
        const uint32_t gmask = 0xFFu << (grp * 8);
        int4 mr = make_int4(9999, -9999, 9999, -9999);
        for (int round = 0; round < 4; round++) {
            const int b = round * 4 + grp;
            const uint32_t i0 = ind[b * 32 + tl], i1 = ind[b * 32 + 8 + tl], i2 = ind[b * 32 + 16 + tl];
            const bool valid = (int)(i0 | i1 | i2) > 0;
            const float tz0 = s_v[warp][2][i0], tz1 = s_v[warp][2][i1], tz2 = s_v[warp][2][i2];
            const bool ai = (tz0 >= 0.f) && (tz1 >= 0.f) && (tz2 >= 0.f);
            const bool ao = (tz0 < 0.f) && (tz1 < 0.f) && (tz2 < 0.f);
            const bool inter = valid && !(ai || ao);
            uint32_t nclip = inter ? (uint32_t)((tz0 >= 0.f) + (tz1 >= 0.f) + (tz2 >= 0.f)) : 0u;
            const float sx0 = s_v[warp][4][i0], sy0 = s_v[warp][5][i0];
            const float sx1 = s_v[warp][4][i1], sy1 = s_v[warp][5][i1];
            const float sx2 = s_v[warp][4][i2], sy2 = s_v[warp][5][i2];
            const float dx1 = sx1 - sx0, dy1 = sy1 - sy0, dx2 = sx2 - sx0, dy2 = sy2 - sy0;
            const int tx0 = cvtt(vmin(sx0, vmin(sx1, sx2))) >> 6, tx1 = cvtt(vmax(sx0, vmax(sx1, sx2))) >> 6;
            const int ty0 = cvtt(vmin(sy0, vmin(sy1, sy2))) >> 6, ty1 = cvtt(vmax(sy0, vmax(sy1, sy2))) >> 6;
            const bool ok = ai && (fma_(dx1, dy2, -(dy1 * dx2)) > 0.1f) &&
                            tx1 >= 0 && tx0 <= cols - 1 && ty1 >= 0 && ty0 <= rows - 1;
            const uint32_t vm = (__ballot_sync(0xFFFFFFFFu, ok) >> (grp * 8)) & 0xFFu;
            int x0 = ok ? tx0 : 9999, x1 = ok ? tx1 : -9999, y0 = ok ? ty0 : 9999, y1 = ok ? ty1 : -9999;
#pragma unroll
            for (int o = 1; o < 8; o <<= 1) {
                x0 = min(x0, __shfl_xor_sync(0xFFFFFFFFu, x0, o));
                x1 = max(x1, __shfl_xor_sync(0xFFFFFFFFu, x1, o));
                y0 = min(y0, __shfl_xor_sync(0xFFFFFFFFu, y0, o));
                y1 = max(y1, __shfl_xor_sync(0xFFFFFFFFu, y1, o));
                nclip += __shfl_xor_sync(0xFFFFFFFFu, nclip, o);
            }
            (void)gmask;
            if (tl == 0) {
                sftg_batch_rec r;
                if (vm) {
                    r.payload = (uint64_t)J.inst | ((uint64_t)m << 24) | ((uint64_t)b << 48) | ((uint64_t)vm << 56);
                    r.x0 = (int16_t)max(-30000, min(30000, x0)); r.x1 = (int16_t)max(-30000, min(30000, x1));
                    r.y0 = (int16_t)max(-30000, min(30000, y0)); r.y1 = (int16_t)max(-30000, min(30000, y1));
                } else { r.payload = 0; r.x0 = 1; r.x1 = 0; r.y0 = 1; r.y1 = 0; }
                recs[(size_t)ssi * 16 + b] = r;
                clip_cnt[(size_t)ssi * 16 + b] = nclip;
            }
            if (vm) { mr.x = min(mr.x, x0); mr.y = max(mr.y, x1); mr.z = min(mr.z, y0); mr.w = max(mr.w, y1); }
        }
        /* meshlet-level rectangle: union of the batch rectangles */
#pragma unroll
        for (int o = 8; o < 32; o <<= 1) {
            mr.x = min(mr.x, __shfl_xor_sync(0xFFFFFFFFu, mr.x, o));
            mr.y = max(mr.y, __shfl_xor_sync(0xFFFFFFFFu, mr.y, o));
            mr.z = min(mr.z, __shfl_xor_sync(0xFFFFFFFFu, mr.z, o));
            mr.w = max(mr.w, __shfl_xor_sync(0xFFFFFFFFu, mr.w, o));
        }
        if (lane == 0) mrect[ssi] = mr;
        __syncwarp();
    }
}

/* ----------------------------------------------------------------------------------------- */
struct cvert { float tx, ty, tz, w, u, v, lu, lv, px, py, pz, nx, ny, nz; };

SFTG_D cvert lerp_cv(const cvert& a, const cvert& b, float t) {
    cvert r;
    const float* pa = &a.tx; const float* pb = &b.tx; float* pr = &r.tx;
#pragma unroll
    for (int i = 0; i < 14; i++) pr[i] = pa[i] + t * (pb[i] - pa[i]);
    return r;
}

/* Batch records with clip outputs (clipping is rare).  Each warp scans 32 records; the records
 * that clip are taken four at a time, one per 8-lane group, lane tl of the group clipping
 * triangle tl of the batch.  A triangle's clip slots follow those of the batch's earlier
 * triangles (exclusive scan over the group), the reference's order. */
__global__ void k_clip(const sftg_frame* __restrict__ frames, uint32_t n_views, const float* __restrict__ ss,
                       const uint32_t* __restrict__ clip_cnt, const uint32_t* __restrict__ clip_base,
                       sftg_clip_tri* __restrict__ clips, int4* __restrict__ clip_rect, int4* __restrict__ mrect,
                       uint32_t n_records)
{
    const int lane = threadIdx.x & 31, gl = lane & 7, gshift = lane & ~7;
    const uint32_t gmask = 0xFFu << gshift;
    const uint32_t r_lane = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t pending = __ballot_sync(0xFFFFFFFFu, r_lane < n_records && clip_cnt[r_lane] != 0);
    const uint32_t r_base = r_lane - (uint32_t)lane;
    while (pending) {
        /* group g takes the g-th pending record */
        uint32_t pick = pending;
        for (int g = 0; g < (lane >> 3) && pick; g++) pick &= pick - 1;
        const bool have = pick != 0;
        const uint32_t r = r_base + (have ? (uint32_t)(__ffs(pick) - 1) : 0u);
        for (int g = 0; g < 4 && pending; g++) pending &= pending - 1;
        if (!have) continue;   /* whole group: the same pick on its 8 lanes */
        const uint32_t ssi = r / 16, b = r % 16;
        /* the view, then the instance, owning this screen-space slot (both laid out in order) */
        uint32_t v = 0;
        for (uint32_t k = 0; k < n_views; k++) if (frames[k].ss_base <= ssi && frames[k].total_ss) v = k;
        const sftg_frame* F = frames + v;
        const uint32_t lss = ssi - F->ss_base;
        uint32_t ii = 0;
        for (uint32_t k = 0; k < F->n_inst; k++) if (F->inst[k].ss_offset <= lss) ii = k;
        const sftg_inst* I = &F->inst[ii];
        const uint32_t m = lss - I->ss_offset, g = I->meshlet_base + m;
        const float* at = F->ml_attr + (size_t)g * 640;
        const float* S = ss + (size_t)ssi * SFTG_SS_FLOATS;
        const uint8_t* ind = F->ml_inds + (size_t)g * 512;
        const float* VP = F->vp;
        const float hw = F->hw, hh = F->hh;
        const int tl = gl;
        const uint32_t q[3] = { ind[b * 32 + tl], ind[b * 32 + 8 + tl], ind[b * 32 + 16 + tl] };
        cvert in[3];
        cvert out[2][3];
        int nc = 0;
        if ((int)(q[0] | q[1] | q[2]) > 0) {
            for (int k = 0; k < 3; k++) {
                const uint32_t vv = q[k];
                const float4 sa = ((const float4*)(S + SFTG_SS_A))[vv], sb = ((const float4*)(S + SFTG_SS_B))[vv];
                const float wx = sa.w, wy = sb.x, wz = sb.y;
                in[k].w = fma_(wx, VP[3], fma_(wy, VP[7], fma_(wz, VP[11], VP[15])));
                in[k].tx = fma_(wx, VP[0], fma_(wy, VP[4], fma_(wz, VP[8], VP[12])));
                in[k].ty = fma_(wx, VP[1], fma_(wy, VP[5], fma_(wz, VP[9], VP[13])));
                in[k].tz = fma_(wx, VP[2], fma_(wy, VP[6], fma_(wz, VP[10], VP[14])));
                in[k].u = at[384 + vv]; in[k].v = at[448 + vv]; in[k].lu = at[512 + vv]; in[k].lv = at[576 + vv];
                in[k].px = wx; in[k].py = wy; in[k].pz = wz;
                in[k].nx = sb.z; in[k].ny = sb.w; in[k].nz = S[SFTG_SS_C + 4 * vv];
            }
            const bool a = in[0].tz >= 0.f, bb = in[1].tz >= 0.f, c = in[2].tz >= 0.f;
            const bool ai = a && bb && c, ao = (in[0].tz < 0.f) && (in[1].tz < 0.f) && (in[2].tz < 0.f);
            if (!(ai || ao)) {
                /* sft__clip_triangle_near_plane (4264-4349) */
                const int mask = (int)a | ((int)bb << 1) | ((int)c << 2);
                float d[3] = { in[0].tz, in[1].tz, in[2].tz };
                if (mask == 1 || mask == 2 || mask == 4) {
                    const int ia = mask >> 1, ib = (ia == 2) ? 0 : ia + 1, ic = (ia == 0) ? 2 : ia - 1;
                    const float tab = fdiv(d[ia], d[ia] - d[ib]), tac = fdiv(d[ia], d[ia] - d[ic]);
                    out[0][0] = in[ia]; out[0][1] = lerp_cv(in[ia], in[ib], tab); out[0][2] = lerp_cv(in[ia], in[ic], tac);
                    nc = 1;
                } else {
                    const int io = (~mask & 7) >> 1, ia = (io == 0) ? 2 : io - 1, ic = (io == 2) ? 0 : io + 1;
                    const float tab = fdiv(d[ia], d[ia] - d[io]), tcb = fdiv(d[ic], d[ic] - d[io]);
                    const cvert nab = lerp_cv(in[ia], in[io], tab), ncb = lerp_cv(in[ic], in[io], tcb);
                    out[0][0] = in[ia]; out[0][1] = nab; out[0][2] = in[ic];
                    out[1][0] = nab; out[1][1] = ncb; out[1][2] = in[ic];
                    nc = 2;
                }
            }
        }
        /* exclusive scan of the output counts over the group's 8 triangles */
        int incl = nc;
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            const int t = __shfl_up_sync(gmask, incl, o, 8);
            if (gl >= o) incl += t;
        }
        uint32_t slot = clip_base[r] + (uint32_t)(incl - nc);
        int4 mr = make_int4(0x7FFFFFFF, (int)0x80000000, 0x7FFFFFFF, (int)0x80000000);
        bool grew = false;
        for (int k = 0; k < nc; k++, slot++) {
            if (slot >= F->clip_cap) continue;   /* over capacity: the host grows the pool and re-renders */
            sftg_clip_tri ct;
            for (int qv = 0; qv < 3; qv++) {
                const cvert& cv = out[k][qv];
                const float iw = fdiv(1.f, cv.w);
                ct.sx[qv] = (cv.tx * iw + 1.f) * hw + F->vpx;
                ct.sy[qv] = (-cv.ty * iw + 1.f) * hh + F->vpy;
                ct.iw[qv] = iw;
                ct.u[qv] = cv.u; ct.v[qv] = cv.v; ct.lu[qv] = cv.lu; ct.lv[qv] = cv.lv;
                ct.px[qv] = cv.px; ct.py[qv] = cv.py; ct.pz[qv] = cv.pz;
                ct.nx[qv] = cv.nx; ct.ny[qv] = cv.ny; ct.nz[qv] = cv.nz;
            }
            ct.inst = ii; ct.m = m;
            clips[slot] = ct;
            const float area = (ct.sx[1] - ct.sx[0]) * (ct.sy[2] - ct.sy[0]) - (ct.sy[1] - ct.sy[0]) * (ct.sx[2] - ct.sx[0]);
            int4 rc = make_int4(1, 0, 1, 0);
            if (area > 0.1f) {
                const int x0 = cvtt(floorf(vmin(ct.sx[0], vmin(ct.sx[1], ct.sx[2])))) >> 6;
                const int x1 = cvtt(ceilf(vmax(ct.sx[0], vmax(ct.sx[1], ct.sx[2])))) >> 6;
                const int y0 = cvtt(floorf(vmin(ct.sy[0], vmin(ct.sy[1], ct.sy[2])))) >> 6;
                const int y1 = cvtt(ceilf(vmax(ct.sy[0], vmax(ct.sy[1], ct.sy[2])))) >> 6;
                if (!(x1 < 0 || x0 > F->cols - 1 || y1 < 0 || y0 > F->rows - 1)) {
                    rc = make_int4(x0, x1, y0, y1);
                    mr.x = min(mr.x, x0); mr.y = max(mr.y, x1); mr.z = min(mr.z, y0); mr.w = max(mr.w, y1);
                    grew = true;
                }
            }
            clip_rect[slot] = rc;
        }
        /* several triangles and batches of one meshlet may clip: widen its rectangle atomically
         * (min / max commute, so the result does not depend on the order) */
        if (grew) {
            atomicMin(&mrect[ssi].x, mr.x); atomicMax(&mrect[ssi].y, mr.y);
            atomicMin(&mrect[ssi].z, mr.z); atomicMax(&mrect[ssi].w, mr.w);
        }
    }
}

/* ----------------------------------------------------------------------------------------- */
#define BIN_THREADS 256

SFTG_D bool rect_has(int x0, int x1, int y0, int y1, int tx, int ty) { return x0 <= tx && tx <= x1 && y0 <= ty && ty <= y1; }

/* Payloads of one meshlet that land on tile (tx, ty), counted or written in reference order:
 * for each batch, its clipped triangles (slot order) then its batch payload.  Lanes 0..15 =
 * batches; returns the meshlet total (same on all lanes). */
SFTG_D uint32_t bin_meshlet(const sftg_batch_rec* recs, const uint32_t* clip_cnt, const uint32_t* clip_base,
                            const int4* clip_rect, uint32_t clip_cap, uint32_t vclip, uint32_t ssi, int tx, int ty, int lane, uint64_t* out)
{
    uint32_t cnt = 0, nclip = 0, cb = 0;
    sftg_batch_rec r; r.payload = 0;
    if (lane < 16) {
        r = recs[(size_t)ssi * 16 + lane];
        nclip = clip_cnt[(size_t)ssi * 16 + lane];
        if (nclip) {
            cb = clip_base[(size_t)ssi * 16 + lane];
            for (uint32_t k = 0; k < nclip && cb + k < clip_cap; k++) {
                const int4 q = clip_rect[cb + k];
                cnt += rect_has(q.x, q.y, q.z, q.w, tx, ty);
            }
        }
        cnt += (r.payload != 0) && rect_has(r.x0, r.x1, r.y0, r.y1, tx, ty);
    }
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += v;
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    if (out && lane < 16 && cnt) {
        uint64_t* o = out + (incl - cnt);
        for (uint32_t k = 0; k < nclip && cb + k < clip_cap; k++) {
            const int4 q = clip_rect[cb + k];
            if (rect_has(q.x, q.y, q.z, q.w, tx, ty)) *o++ = (uint64_t)(cb + k - vclip);
        }
        if (r.payload != 0 && rect_has(r.x0, r.x1, r.y0, r.y1, tx, ty)) *o = r.payload;
    }
    return total;
}

#define COARSE_THREADS 1024   /* a super-tile scans its view's meshlet slots 1024 at a time */

__global__ void __launch_bounds__(COARSE_THREADS)
k_coarse(const sftg_frame* __restrict__ frames, const uint16_t* __restrict__ stile_view, const int4* __restrict__ mrect,
         uint32_t* __restrict__ stile_count, const uint32_t* __restrict__ stile_start, uint32_t* __restrict__ stile_list)
{
    __shared__ uint32_t s_wsum[COARSE_THREADS / 32];
    const int gst = blockIdx.x;                         /* batch-wide super-tile index */
    const sftg_frame* F = frames + stile_view[gst];
    const int st = gst - (int)F->stile_base;
    const int sx0 = (st % (int)F->scols) * SFTG_STILE, sy0 = (st / (int)F->scols) * SFTG_STILE;
    const int sx1 = sx0 + SFTG_STILE - 1, sy1 = sy0 + SFTG_STILE - 1;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t* out = nullptr;
    if (stile_list) {
        /* over capacity: the host grows the lists and re-renders; write nothing */
        if ((uint64_t)stile_start[gst] + stile_count[gst] > F->stile_cap) return;
        out = stile_list + stile_start[gst];
    }
    uint32_t running = 0;
    for (uint32_t base = 0; base < F->total_ss; base += COARSE_THREADS) {
        const uint32_t s = F->ss_base + base + tid;
        bool hit = false;
        if (base + tid < F->total_ss) {
            const int4 q = mrect[s];   /* inclusive tile rectangle x0, x1, y0, y1; empty when x0 > x1 */
            hit = q.x <= q.y && q.z <= q.w && q.x <= sx1 && q.y >= sx0 && q.z <= sy1 && q.w >= sy0;
        }
        const uint32_t bal = __ballot_sync(0xFFFFFFFFu, hit);
        if (lane == 0) s_wsum[warp] = __popc(bal);
        __syncthreads();
        uint32_t off = 0, tot = 0;
        for (int w = 0; w < COARSE_THREADS / 32; w++) { if (w < warp) off += s_wsum[w]; tot += s_wsum[w]; }
        if (out && hit) out[running + off + __popc(bal & ((1u << lane) - 1u))] = s;
        running += tot;
        __syncthreads();
    }
    if (!stile_list && tid == 0) stile_count[gst] = running;
}

__global__ void __launch_bounds__(BIN_THREADS)
k_bin(const sftg_frame* __restrict__ frames, const uint16_t* __restrict__ tile_view, const sftg_batch_rec* __restrict__ recs,
      const uint32_t* __restrict__ clip_cnt, const uint32_t* __restrict__ clip_base, const int4* __restrict__ clip_rect,
      const int4* __restrict__ mrect, const uint32_t* __restrict__ stile_count, const uint32_t* __restrict__ stile_start,
      const uint32_t* __restrict__ stile_list, uint32_t* __restrict__ tile_count, const uint32_t* __restrict__ tile_start,
      uint64_t* __restrict__ tile_pay)
{
    __shared__ uint32_t s_hits[BIN_THREADS];
    __shared__ uint32_t s_cnt[BIN_THREADS];
    __shared__ uint32_t s_wsum[BIN_THREADS / 32];
    __shared__ uint32_t s_nhits;
    const int gtile = blockIdx.x;                       /* batch-wide tile index */
    const sftg_frame* F = frames + tile_view[gtile];
    const int tile = gtile - (int)F->tile_base;
    const int tx = tile % F->cols, ty = tile / F->cols;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t n_ss = F->total_ss;
    /* clipped payloads carry the view's own slot numbers (slots restart at 0 per frame) */
    const uint32_t vclip = n_ss ? clip_base[(size_t)F->ss_base * 16] : 0u;
    uint64_t* out = nullptr;
    if (tile_pay) {
        /* over capacity: the host grows the buffer and re-renders; write nothing */
        if ((uint64_t)tile_start[gtile] + tile_count[gtile] > F->tile_cap) return;
        out = tile_pay + tile_start[gtile];
    }
    /* the meshlets that can touch this tile: its super-tile's list, in slot order, or every slot
     * of the view when the view has no coarse lists (scols == 0) */
    uint32_t n_cand = n_ss;
    const uint32_t* cand = nullptr;
    if (F->scols) {
        const uint32_t gst = F->stile_base + (uint32_t)((ty / SFTG_STILE) * (int)F->scols + tx / SFTG_STILE);
        n_cand = stile_count[gst];
        if ((uint64_t)stile_start[gst] + n_cand > F->stile_cap) n_cand = 0;   /* lists overflowed: the host re-renders */
        cand = stile_list + stile_start[gst];
    }
    uint32_t running = 0;
    for (uint32_t base = 0; base < n_cand; base += BIN_THREADS) {
        uint32_t s = 0;
        bool hit = false;
        if (base + tid < n_cand) {
            s = cand ? cand[base + tid] : F->ss_base + base + tid;
            const int4 q = mrect[s];
            hit = rect_has(q.x, q.y, q.z, q.w, tx, ty);
        }
        if (!__syncthreads_or(hit)) continue;   /* no meshlet of this chunk touches the tile */
        /* ordered compaction of hit meshlets */
        const uint32_t bal = __ballot_sync(0xFFFFFFFFu, hit);
        if (lane == 0) s_wsum[warp] = __popc(bal);
        __syncthreads();
        uint32_t off = 0, tot = 0;
        for (int w = 0; w < BIN_THREADS / 32; w++) { if (w < warp) off += s_wsum[w]; tot += s_wsum[w]; }
        if (hit) s_hits[off + __popc(bal & ((1u << lane) - 1u))] = s;
        if (tid == 0) s_nhits = tot;
        __syncthreads();
        const uint32_t nh = s_nhits;
        /* per-hit payload counts */
        for (uint32_t h = warp; h < nh; h += BIN_THREADS / 32) {
            const uint32_t c = bin_meshlet(recs, clip_cnt, clip_base, clip_rect, F->clip_cap, vclip, s_hits[h], tx, ty, lane, nullptr);
            if (lane == 0) s_cnt[h] = c;
        }
        __syncthreads();
        if (warp == 0) {   /* exclusive scan of the hit counts (nh <= 256, 8 per lane); total in s_wsum[0] */
            uint32_t v[BIN_THREADS / 32], local = 0;
#pragma unroll
            for (int k = 0; k < BIN_THREADS / 32; k++) {
                const uint32_t h = (uint32_t)lane * (BIN_THREADS / 32) + k;
                v[k] = h < nh ? s_cnt[h] : 0u;
                local += v[k];
            }
            uint32_t incl = local;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) { const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o); if (lane >= o) incl += t; }
            uint32_t acc = incl - local;
#pragma unroll
            for (int k = 0; k < BIN_THREADS / 32; k++) {
                const uint32_t h = (uint32_t)lane * (BIN_THREADS / 32) + k;
                if (h < nh) s_cnt[h] = acc;
                acc += v[k];
            }
            if (lane == 31) s_wsum[0] = incl;
        }
        __syncthreads();
        if (out) {   /* ordered writes */
            for (uint32_t h = warp; h < nh; h += BIN_THREADS / 32)
                bin_meshlet(recs, clip_cnt, clip_base, clip_rect, F->clip_cap, vclip, s_hits[h], tx, ty, lane, out + running + s_cnt[h]);
        }
        running += s_wsum[0];
        __syncthreads();
    }
    if (!out && tid == 0) tile_count[gtile] = running;
}

/* ----------------------------------------------------------------------------------------- */
/* three-phase exclusive scan of u32 (n <= 1024 * 1024 * 4) */
#define SCAN_BLOCK 1024

SFTG_D uint32_t block_excl_scan(uint32_t v, uint32_t* s_w, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) { const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o); if (lane >= o) incl += t; }
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t x = lane < nw ? s_w[lane] : 0, xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) { const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, xi, o); if (lane >= o) xi += t; }
        if (lane < nw) s_w[lane] = xi - x;
        if (lane == 31) s_w[32] = xi;
    }
    __syncthreads();
    const uint32_t r = s_w[warp] + incl - v;
    if (total) *total = s_w[32];
    __syncthreads();
    return r;
}

__global__ void k_scan_reduce(const uint32_t* __restrict__ in, uint32_t n, uint32_t* __restrict__ sums) {
    __shared__ uint32_t s_w[33];
    uint32_t acc = 0;
    const uint32_t base = blockIdx.x * SCAN_BLOCK * 4;
    for (int k = 0; k < 4; k++) { const uint32_t i = base + k * SCAN_BLOCK + threadIdx.x; if (i < n) acc += in[i]; }
    uint32_t tot;
    block_excl_scan(acc, s_w, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_top(uint32_t* __restrict__ sums, uint32_t nb, uint32_t* __restrict__ total_out) {
    __shared__ uint32_t s_w[33];
    uint32_t carry = 0;
    for (uint32_t base = 0; base < nb; base += SCAN_BLOCK) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < nb ? sums[i] : 0;
        uint32_t tot;
        const uint32_t e = block_excl_scan(v, s_w, &tot);
        if (i < nb) sums[i] = e + carry;
        carry += tot;
    }
    if (threadIdx.x == 0 && total_out) *total_out = carry;
}

/* the whole scan in one CTA for small inputs (n <= SFTG_SCAN_SMALL): each thread a run of
 * consecutive elements, one block scan of the run sums */
__global__ void __launch_bounds__(SCAN_BLOCK)
k_scan_small(const uint32_t* __restrict__ in, uint32_t n, uint32_t* __restrict__ out, uint32_t* __restrict__ total_out) {
    __shared__ uint32_t s_w[33];
    const uint32_t per = (n + SCAN_BLOCK - 1) / SCAN_BLOCK;
    const uint32_t i0 = threadIdx.x * per;
    uint32_t acc = 0;
    for (uint32_t k = 0; k < per; k++) { const uint32_t i = i0 + k; if (i < n) acc += in[i]; }
    uint32_t tot;
    uint32_t e = block_excl_scan(acc, s_w, &tot);
    for (uint32_t k = 0; k < per; k++) { const uint32_t i = i0 + k; if (i < n) { const uint32_t x = in[i]; out[i] = e; e += x; } }
    if (threadIdx.x == 0 && total_out) *total_out = tot;
}

__global__ void k_scan_down(const uint32_t* __restrict__ in, uint32_t n, const uint32_t* __restrict__ sums, uint32_t* __restrict__ out) {
    __shared__ uint32_t s_w[33];
    const uint32_t base = blockIdx.x * SCAN_BLOCK * 4;
    const uint32_t i0 = base + threadIdx.x * 4;
    uint32_t v[4], acc = 0;
    for (int k = 0; k < 4; k++) { const uint32_t i = i0 + k; v[k] = i < n ? in[i] : 0; acc += v[k]; }
    uint32_t e = block_excl_scan(acc, s_w, nullptr) + sums[blockIdx.x];
    for (int k = 0; k < 4; k++) { const uint32_t i = i0 + k; if (i < n) out[i] = e; e += v[k]; }
}
