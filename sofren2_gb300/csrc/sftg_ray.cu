/*
 * Ray queries against resident models: sft_raycast_instance (sofren2.c:3733-3837) with
 * sft__intersect_triangle (3705-3731), 8 lanes per ray.
 *
 *   model space  sft_m_qinv of the instance transform, applied by sft_m_mul_vec, which uses rows
 *                0-2 only (no translation; the reference's behaviour, kept); the direction is
 *                normalised and the distance limit divided by its inverse length
 *   walk         depth first from a stack, children in slot order: inner children that pass the
 *                slab test are pushed, leaf triangles are tested in place; a hit shortens the
 *                limit, so among equal distances the first triangle found wins, as in the
 *                reference's walk
 *   result       distance back in world scale, position and normal through rows 0-2 of the
 *                transform, the normal normalised (sft_v_norm)
 * Arithmetic is the reference's scalar C sequence in IEEE single precision: the file is built
 * with -fmad=false, and divisions and square roots are the correctly rounded intrinsics.  The
 * stack holds RAY_STACK entries (an 8-wide BLAS needs 7 per level); a walk that would overflow
 * it, or that meets a node or meshlet index outside its model, stops and marks its record with
 * hit = 2.
 */
#include "sftg_types.h"
#include "sftg_kernels.h"

#define RAY_STACK 128
#define RAY_EPS 1e-6f

struct v3 { float x, y, z; };

__device__ __forceinline__ v3 vsub(v3 a, v3 b) { return { a.x - b.x, a.y - b.y, a.z - b.z }; }
__device__ __forceinline__ float vdot(v3 a, v3 b) { return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z)); }
__device__ __forceinline__ v3 vcross(v3 a, v3 b) {
    return { __fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
             __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)) };
}
__device__ __forceinline__ v3 vscale(v3 a, float s) { return { __fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s) }; }
__device__ __forceinline__ v3 vnorm(v3 v) {   /* sft_v_norm (1548-1551) */
    const float l = __fsqrt_rn(vdot(v, v));
    return l > RAY_EPS ? vscale(v, __fdiv_rn(1.f, l)) : v3{ 0.f, 0.f, 0.f };
}
/* sft_m_mul_vec (1679-1685): v.x * m[0][j] + v.y * m[1][j] + v.z * m[2][j] */
__device__ __forceinline__ v3 rot3(const float* m, v3 v) {
    return { __fadd_rn(__fadd_rn(__fmul_rn(v.x, m[0]), __fmul_rn(v.y, m[4])), __fmul_rn(v.z, m[8])),
             __fadd_rn(__fadd_rn(__fmul_rn(v.x, m[1]), __fmul_rn(v.y, m[5])), __fmul_rn(v.z, m[9])),
             __fadd_rn(__fadd_rn(__fmul_rn(v.x, m[2]), __fmul_rn(v.y, m[6])), __fmul_rn(v.z, m[10])) };
}
__device__ __forceinline__ float inv_axis(float d) {
    return __fdiv_rn(1.f, fabsf(d) > RAY_EPS ? d : __fmul_rn(RAY_EPS, d < 0.f ? -1.f : 1.f));
}
__device__ __forceinline__ float rmin(float a, float b) { return a < b ? a : b; }   /* SFT_MIN */
__device__ __forceinline__ float rmax(float a, float b) { return a > b ? a : b; }   /* SFT_MAX */

/* 8 lanes per ray (4 rays per warp): lane c takes child slot c of a node, so
 * a node's boxes load coalesced and are tested at once.  Inner nodes: the limit does not change
 * while their children are tested, so the passing children are pushed at once, in slot order
 * (the order the sequential walk pushes them).  Leaves: each lane tests its box and intersects
 * its triangle; the results are then taken in slot order against the running limit, exactly as
 * the sequential loop would (a box test that passed with the limit at node entry is re-checked
 * with the current one).  The winning lane computes the hit record. */
#define RAY8_WARPS 4

__global__ void __launch_bounds__(RAY8_WARPS * 32)
k_raycast8(const sftg_ray* __restrict__ rays, uint32_t n, const sftg_model* __restrict__ models, uint32_t n_models,
           const sftg_bvh_node* __restrict__ blas, const float* __restrict__ ml_attr, const uint8_t* __restrict__ ml_inds,
           sftg_ray_hit* __restrict__ hits)
{
    __shared__ uint32_t s_stack[RAY8_WARPS * 4][RAY_STACK];
    const int lane = threadIdx.x & 31, gl = lane & 7, gshift = lane & ~7;
    const uint32_t gmask = 0xFFu << gshift;
    const int grp = (threadIdx.x >> 5) * 4 + (lane >> 3);
    const uint32_t k = blockIdx.x * (RAY8_WARPS * 4) + (uint32_t)grp;
    if (k >= n) return;   /* whole group: every lane of a group has the same k */
    uint32_t* stack = s_stack[grp];
    const sftg_ray& R = rays[k];
    sftg_ray_hit H;
    H.hit = 0; H.distance = R.max_dist;
    H.pos[0] = H.pos[1] = H.pos[2] = 0.f; H.normal[0] = H.normal[1] = H.normal[2] = 0.f;
    if (R.model < 0 || (uint32_t)R.model >= n_models || models[R.model].blas_count == 0) { if (gl == 0) hits[k] = H; return; }
    const sftg_model M = models[R.model];
    float T[16];
#pragma unroll
    for (int q = 0; q < 16; q++) T[q] = R.transform[q];
    const float inv[16] = { T[0], T[4], T[8], 0.f, T[1], T[5], T[9], 0.f, T[2], T[6], T[10], 0.f, 0.f, 0.f, 0.f, 1.f };
    const v3 lo = rot3(inv, v3{ R.origin[0], R.origin[1], R.origin[2] });
    v3 ld = rot3(inv, v3{ R.dir[0], R.dir[1], R.dir[2] });
    const float inv_scale = __fdiv_rn(1.f, __fsqrt_rn(vdot(ld, ld)));
    ld = vscale(ld, inv_scale);
    const float ix = inv_axis(ld.x), iy = inv_axis(ld.y), iz = inv_axis(ld.z);
    float lmax = __fdiv_rn(R.max_dist, inv_scale);
    const sftg_bvh_node* nodes = blas + M.blas_base;
    int top = 1;
    if (gl == 0) stack[0] = M.blas_root;
    __syncwarp(gmask);
    bool overflow = false;
    while (top > 0) {
        const uint32_t ni = stack[--top];
        __syncwarp(gmask);
        if (ni >= M.blas_count) { overflow = true; break; }
        const sftg_bvh_node* nd = nodes + ni;
        const uint32_t cnt = nd->count;
        const bool leaf = nd->leaf != 0;
        const uint32_t ch = nd->child[gl];
        const bool valid = (uint32_t)gl < cnt && ch != 0xFFFFFFFFu;
        const float tx1 = __fmul_rn(__fsub_rn(nd->mn[0][gl], lo.x), ix), tx2 = __fmul_rn(__fsub_rn(nd->mx[0][gl], lo.x), ix);
        const float ty1 = __fmul_rn(__fsub_rn(nd->mn[1][gl], lo.y), iy), ty2 = __fmul_rn(__fsub_rn(nd->mx[1][gl], lo.y), iy);
        const float tz1 = __fmul_rn(__fsub_rn(nd->mn[2][gl], lo.z), iz), tz2 = __fmul_rn(__fsub_rn(nd->mx[2][gl], lo.z), iz);
        const float tmin = rmax(rmax(rmin(tx1, tx2), rmin(ty1, ty2)), rmin(tz1, tz2));
        const float tmax = rmin(rmin(rmax(tx1, tx2), rmax(ty1, ty2)), rmax(tz1, tz2));
        const bool pass = valid && tmax >= tmin && tmax > 0.f && tmin < lmax;
        if (!leaf) {
            const uint32_t pm = (__ballot_sync(gmask, pass) >> gshift) & 0xFFu;
            if (top + __popc(pm) > RAY_STACK) { overflow = true; break; }
            if (pass) stack[top + __popc(pm & ((1u << gl) - 1u))] = ch;
            top += __popc(pm);
            __syncwarp(gmask);
            continue;
        }
        /* leaf: this lane's triangle, intersected whatever the limit */
        bool tri_ok = false, bad = false;
        float t = 0.f;
        v3 e1{ 0.f, 0.f, 0.f }, e2{ 0.f, 0.f, 0.f };
        if (pass) {
            const uint32_t pay = ch & ~0x80000000u, tri = pay & 127u;
            if ((pay >> 7) >= M.total_meshlets) bad = true;
            else {
                const uint32_t g = M.meshlet_base + (pay >> 7);
                const uint8_t* ind = ml_inds + (size_t)g * 512 + (tri >> 3) * 32 + (tri & 7);
                const float* X = ml_attr + (size_t)g * 640;
                const uint32_t i0 = ind[0], i1 = ind[8], i2 = ind[16];
                const v3 v0{ X[i0], X[64 + i0], X[128 + i0] }, v1{ X[i1], X[64 + i1], X[128 + i1] }, v2{ X[i2], X[64 + i2], X[128 + i2] };
                e1 = vsub(v1, v0); e2 = vsub(v2, v0);
                const v3 p = vcross(ld, e2);
                const float det = vdot(e1, p);
                if (!(fabsf(det) < RAY_EPS)) {
                    const float id = __fdiv_rn(1.f, det);
                    const v3 tv = vsub(lo, v0);
                    const float u = __fmul_rn(vdot(tv, p), id);
                    if (!(u < 0.f || u > 1.f)) {
                        const v3 qv = vcross(tv, e1);
                        const float v = __fmul_rn(vdot(ld, qv), id);
                        if (!(v < 0.f || __fadd_rn(u, v) > 1.f)) {
                            t = __fmul_rn(vdot(e2, qv), id);
                            tri_ok = t > RAY_EPS;
                        }
                    }
                }
            }
        }
        if (__ballot_sync(gmask, bad) & gmask) { overflow = true; break; }
        /* slot order against the running limit */
        const uint32_t cand = (__ballot_sync(gmask, pass && tri_ok) >> gshift) & 0xFFu;
        int win = -1;
        for (uint32_t c = cand; c; c &= c - 1) {
            const int s = __ffs(c) - 1;
            const float tmin_s = __shfl_sync(gmask, tmin, gshift + s), t_s = __shfl_sync(gmask, t, gshift + s);
            if (tmin_s < lmax && t_s < lmax) { lmax = t_s; win = s; }
        }
        if (win >= 0) {
            /* the hit record, computed by the winning lane and broadcast */
            float rec[7] = { 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f };
            if (gl == win) {
                rec[0] = __fmul_rn(t, inv_scale);
                const v3 sd = vscale(ld, t);
                const v3 lh{ __fadd_rn(lo.x, sd.x), __fadd_rn(lo.y, sd.y), __fadd_rn(lo.z, sd.z) };
                const v3 ln = vnorm(vcross(e1, e2));   /* sft_v_face_normal */
                const v3 wp = rot3(T, lh), wn = vnorm(rot3(T, ln));
                rec[1] = wp.x; rec[2] = wp.y; rec[3] = wp.z; rec[4] = wn.x; rec[5] = wn.y; rec[6] = wn.z;
            }
#pragma unroll
            for (int q = 0; q < 7; q++) rec[q] = __shfl_sync(gmask, rec[q], gshift + win);
            H.hit = 1; H.distance = rec[0];
            H.pos[0] = rec[1]; H.pos[1] = rec[2]; H.pos[2] = rec[3];
            H.normal[0] = rec[4]; H.normal[1] = rec[5]; H.normal[2] = rec[6];
        }
    }
    if (overflow) H.hit = 2;
    if (gl == 0) hits[k] = H;
}

void sftg_launch_raycast(const sftg_ray* rays, uint32_t n, const sftg_model* models, uint32_t n_models, const sftg_bvh_node* blas,
                         const float* ml_attr, const uint8_t* ml_inds, sftg_ray_hit* hits, cudaStream_t st) {
    if (!n) return;
    k_raycast8<<<(n + RAY8_WARPS * 4 - 1) / (RAY8_WARPS * 4), RAY8_WARPS * 32, 0, st>>>(rays, n, models, n_models, blas, ml_attr, ml_inds, hits);
}
