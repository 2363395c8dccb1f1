/*
 * Skeletal pose evaluation (sft_pose_update, sofren2.c:8952-9108), one warp per request.
 *
 *   channels   lanes take channels in order of their index; each finds its keyframe pair by the
 *              reference's binary search, interpolates (lerp for T and S, sft_q_slerp for R, or
 *              the step value), and the values are stored in channel order, so a later channel
 *              of the same node and path wins as in the reference's sequential loop
 *   locals     per bone S * (R * T) from the animated or rest TRS, else the local bind matrix
 *   hierarchy  parents before children, level by level (host-computed order): global =
 *              local * global[parent], each bone once, as the reference's repeated passes do
 *   posed      inverse bind * global
 * Matrix products follow sft_m_mul (sofren2.c:1668): left-to-right sums of plain products.
 */
#include "sftg_types.h"
#include "sftg_kernels.h"

#define POSE_WARPS 1

struct pose_trs { float p[3], r[4], s[3]; uint32_t mask; };

__device__ __forceinline__ void mmul(const float* a, const float* b, float* r) {
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
            r[i * 4 + j] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(a[i * 4 + 0], b[0 * 4 + j]), __fmul_rn(a[i * 4 + 1], b[1 * 4 + j])),
                                              __fmul_rn(a[i * 4 + 2], b[2 * 4 + j])), __fmul_rn(a[i * 4 + 3], b[3 * 4 + j]));
}

__device__ __forceinline__ void qnorm(float* q) {   /* sft_q_norm */
    const float l2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    if (l2 != 0.f) { const float il = __fdiv_rn(1.f, __fsqrt_rn(l2)); q[0] *= il; q[1] *= il; q[2] *= il; q[3] *= il; }
}

__device__ void slerp(const float* a, const float* b_in, float t, float* out) {   /* sft_q_slerp (1857-1892) */
    float b[4] = { b_in[0], b_in[1], b_in[2], b_in[3] };
    float dot = a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
    if (dot < 0.f) { b[0] = -b[0]; b[1] = -b[1]; b[2] = -b[2]; b[3] = -b[3]; dot = -dot; }
    if (dot > 0.9995f) {
#pragma unroll
        for (int k = 0; k < 4; k++) out[k] = a[k] + t * (b[k] - a[k]);
        qnorm(out);
        return;
    }
    const float th0 = acosf(dot), th = th0 * t, st = sinf(th), is0 = __fdiv_rn(1.f, sinf(th0));
    const float s0 = cosf(th) - dot * st * is0, s1 = st * is0;
#pragma unroll
    for (int k = 0; k < 4; k++) out[k] = a[k] * s0 + b[k] * s1;
    qnorm(out);
}

__device__ void from_quat(const float* q, float* m) {   /* sft_m_from_quat (1822-1850) */
    const float x2 = q[0] + q[0], y2 = q[1] + q[1], z2 = q[2] + q[2];
    const float xx = q[0] * x2, xy = q[0] * y2, xz = q[0] * z2, yy = q[1] * y2, yz = q[1] * z2, zz = q[2] * z2;
    const float wx = q[3] * x2, wy = q[3] * y2, wz = q[3] * z2;
    m[0] = 1.f - (yy + zz); m[1] = xy + wz; m[2] = xz - wy; m[3] = 0.f;
    m[4] = xy - wz; m[5] = 1.f - (xx + zz); m[6] = yz + wx; m[7] = 0.f;
    m[8] = xz + wy; m[9] = yz - wx; m[10] = 1.f - (xx + yy); m[11] = 0.f;
    m[12] = 0.f; m[13] = 0.f; m[14] = 0.f; m[15] = 1.f;
}

__global__ void __launch_bounds__(32)
k_pose(const sftg_pose_tables T, const sftg_pose_request* __restrict__ reqs, const uint32_t* __restrict__ out_off, uint32_t n,
       float* __restrict__ posed, float* __restrict__ global_out)
{
    __shared__ pose_trs s_trs[SFTG_MAX_BONES];
    __shared__ float s_g[SFTG_MAX_BONES][16];
    const uint32_t k = blockIdx.x;
    const int lane = threadIdx.x;
    if (k >= n) return;
    const sftg_pose_request R = reqs[k];
    if (R.skeleton < 0 || (uint32_t)R.skeleton >= T.n_skels) return;
    const sftg_skel_dev sk = T.skels[R.skeleton];
    if (R.animation < 0 || R.animation >= (int)sk.anim_count) return;   /* sft_pose_update returns early */
    const sftg_anim_dev an = T.anims[sk.anim_base + R.animation];
    const int nb = (int)sk.bone_count;
    float time = R.time;
    if (an.duration > 1e-6f) time = fmodf(time, an.duration);
    for (int b = lane; b < nb; b += 32) s_trs[b].mask = 0;
    __syncwarp();
    /* channels, 32 at a time; values stored in channel order */
    for (int c0 = 0; c0 < an.channel_count; c0 += 32) {
        const int c = c0 + lane;
        bool have = false;
        int node = 0, path = 0;
        float val[4] = { 0.f, 0.f, 0.f, 0.f };
        if (c < an.channel_count) {
            const sftg_channel_desc ch = T.channels[an.channel_base + c];
            node = ch.node; path = ch.path;
            if (node >= 0 && node < nb) {
                have = true;
                const sftg_sampler_dev sm = T.samplers[an.sampler_base + ch.sampler];
                const float* in = T.keys + sm.input_base;
                const float* out = T.keys + sm.output_base;
                int f0 = 0, f1 = 0;
                float t = 0.f;
                if (time <= in[0]) {
                    f0 = f1 = 0;
                } else if (time >= in[sm.count - 1]) {
                    f0 = f1 = sm.count - 1;
                } else {
                    int low = 0, high = sm.count - 1;
                    while (low <= high) {
                        const int mid = low + (high - low) / 2;
                        if (time < in[mid]) high = mid - 1;
                        else if (time >= in[mid + 1]) low = mid + 1;
                        else { f0 = mid; f1 = mid + 1; break; }
                    }
                    const float dt = in[f1] - in[f0];
                    t = (dt > 0.0001f) ? __fdiv_rn(time - in[f0], dt) : 0.f;
                }
                if (path == 1) {
                    if (sm.is_step) { for (int q = 0; q < 4; q++) val[q] = out[f0 * 4 + q]; }
                    else slerp(out + f0 * 4, out + f1 * 4, t, val);
                } else {
                    for (int q = 0; q < 3; q++) {
                        const float v0 = out[f0 * 4 + q], v1 = out[f1 * 4 + q];
                        val[q] = sm.is_step ? v0 : v0 + (v1 - v0) * t;
                    }
                }
            }
        }
        for (int w = 0; w < 32; w++) {   /* channel order */
            if (lane == w && have) {
                pose_trs& d = s_trs[node];
                if (path == 1) { d.r[0] = val[0]; d.r[1] = val[1]; d.r[2] = val[2]; d.r[3] = val[3]; d.mask |= 2u; }
                else if (path == 0) { d.p[0] = val[0]; d.p[1] = val[1]; d.p[2] = val[2]; d.mask |= 1u; }
                else if (path == 2) { d.s[0] = val[0]; d.s[1] = val[1]; d.s[2] = val[2]; d.mask |= 4u; }
            }
            __syncwarp();
        }
    }
    /* local matrices */
    for (int b = lane; b < nb; b += 32) {
        const sftg_bone_dev& bd = T.bones[sk.bone_base + b];
        const pose_trs& tr = s_trs[b];
        if (tr.mask) {
            const float* tp = (tr.mask & 1u) ? tr.p : bd.base_t;
            const float* rq = (tr.mask & 2u) ? tr.r : bd.base_r;
            const float* sc = (tr.mask & 4u) ? tr.s : bd.base_s;
            float Tm[16] = { 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, tp[0], tp[1], tp[2], 1 };
            float Sm[16] = { sc[0], 0, 0, 0, 0, sc[1], 0, 0, 0, 0, sc[2], 0, 0, 0, 0, 1 };
            float Rm[16], RT[16];
            from_quat(rq, Rm);
            mmul(Rm, Tm, RT);
            mmul(Sm, RT, s_g[b]);
        } else {
            for (int q = 0; q < 16; q++) s_g[b][q] = bd.local_bind[q];
        }
    }
    __syncwarp();
    /* hierarchy, level by level */
    const uint16_t* order = T.order + sk.order_base;
    const uint16_t* lvl = T.levels + sk.level_base;
    for (uint32_t L = 1; L < sk.level_count; L++) {
        for (int i = (int)lvl[L] + lane; i < (int)lvl[L + 1]; i += 32) {
            const int b = order[i];
            const int p = T.bones[sk.bone_base + b].parent;
            float g[16];
            mmul(s_g[b], s_g[p], g);
            for (int q = 0; q < 16; q++) s_g[b][q] = g[q];
        }
        __syncwarp();
    }
    /* posed = inverse bind * global */
    float* po = posed + (size_t)out_off[k] * 16;
    for (int b = lane; b < nb; b += 32) {
        float pm[16];
        mmul(T.bones[sk.bone_base + b].inverse_bind, s_g[b], pm);
        for (int q = 0; q < 16; q++) po[b * 16 + q] = pm[q];
        if (global_out) for (int q = 0; q < 16; q++) global_out[(size_t)out_off[k] * 16 + b * 16 + q] = s_g[b][q];
    }
}

void sftg_launch_pose(const sftg_pose_tables& T, const sftg_pose_request* reqs, const uint32_t* out_off, uint32_t n, float* posed,
                      float* global, cudaStream_t st) {
    if (n) k_pose<<<n, 32, 0, st>>>(T, reqs, out_off, n, posed, global);
}
