/*
 * Device-side arithmetic with the exact semantics of sofren2's AVX2 lane layer
 * (sofren2.c:263-385, 632-643, 1921-2060).  Compiled with -fmad=false: every a*b+c
 * below is two roundings unless written as fma(), which is where the reference uses
 * _mm256_fmadd_ps / fmsub / fnmadd.
 */
#pragma once
#include <stdint.h>
#include "x86_approx_tables.h"

#define SFTG_D __device__ __forceinline__

/* measured RCPPS / RSQRTPS results (written by oracle/gen_x86_approx_tables.c) */
__device__ const uint32_t g_rcp_tab[2048] = SFT_X86_RCP_TABLE_INIT;
__device__ const uint32_t g_rsq_tab[2048] = SFT_X86_RSQRT_TABLE_INIT;

/* RCPPS.  The common case (1 <= exponent <= 252, either sign) is one range check, the table
 * load and the assembly of sign, exponent 253 - e and the 12-bit measured mantissa; the rest
 * (zeros and denormals -> +-inf, tiny results -> +-0, inf -> +-0, NaN quieted) is the slow path. */
SFTG_D float x86_rcp(float xf) {
    const uint32_t x = __float_as_uint(xf), ax = x & 0x7FFFFFFFu;
    if (ax - 0x00800000u < (253u << 23) - 0x00800000u)
        return __uint_as_float((x & 0x80000000u) | ((253u << 23) - (ax & 0x7F800000u)) | __ldg(&g_rcp_tab[(x >> 12) & 0x7FFu]));
    const uint32_t s = x & 0x80000000u, e = (x >> 23) & 0xFF, m = x & 0x7FFFFF;
    if (e == 0xFF) return __uint_as_float(m ? (x | 0x00400000u) : s);
    if (e == 0) return __uint_as_float(s | 0x7F800000u);
    return __uint_as_float(s);   /* e >= 253 */
}

/* RSQRTPS.  Positive normal inputs take the fast path: index = exponent parity and the top 10
 * mantissa bits, result exponent (380 - e) / 2 plus the entry's adjustment (its bits 23 and up,
 * less one), mantissa from the entry. */
SFTG_D float x86_rsqrt(float xf) {
    const uint32_t x = __float_as_uint(xf);
    if (x - 0x00800000u < 0x7F000000u) {
        const uint32_t e = x >> 23;
        const uint32_t t = __ldg(&g_rsq_tab[((e & 1u) << 10) | ((x >> 13) & 0x3FFu)]);
        return __uint_as_float((((380u - e) >> 1) << 23) + t - (1u << 23));
    }
    const uint32_t s = x & 0x80000000u, e = (x >> 23) & 0xFF, m = x & 0x7FFFFF;
    if (e == 0xFF) { if (m) return __uint_as_float(x | 0x00400000u); return __uint_as_float(s ? 0xFFC00000u : 0u); }
    if (e == 0) return __uint_as_float(s | 0x7F800000u);
    return __uint_as_float(0xFFC00000u);   /* negative normal */
}

/* NaN bits as x86 leaves them in memory.  Every NaN on the render path comes from an invalid
 * operation (0 * inf in rcpr's fnmadd for w = +-0, inf - inf), whose SSE/AVX result is the default
 * NaN 0xFFC00000; later mul/add/fma pass a NaN operand through unchanged.  CUDA arithmetic returns
 * its own canonical NaN instead, so floats stored to buffers that are compared bit for bit go
 * through this map. */
SFTG_D float x86nan(float v) { return v != v ? __uint_as_float(0xFFC00000u) : v; }

SFTG_D float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
/* sft_vf_rcp_refined: approx * (2 - a * approx), the inner term fused (fnmadd) */
SFTG_D float rcpr(float a) { const float r = x86_rcp(a); return __fmul_rn(r, __fmaf_rn(-a, r, 2.f)); }
SFTG_D float vmin(float a, float b) { return a < b ? a : b; }   /* _mm256_min_ps(a, b) */
SFTG_D float vmax(float a, float b) { return a > b ? a : b; }   /* _mm256_max_ps(a, b) */
/* _mm256_cvttps_epi32 / (i32) cast on x86: truncation, INT_MIN when out of range or NaN */
SFTG_D int cvtt(float x) { return (x >= -2147483648.f && x < 2147483648.f) ? __float2int_rz(x) : (int)0x80000000; }
SFTG_D float fdiv(float a, float b) { return __fdiv_rn(a, b); }
SFTG_D float fsqrt(float a) { return __fsqrt_rn(a); }

struct v3 { float x, y, z; };
SFTG_D v3 mk3(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
SFTG_D v3 sub3(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
SFTG_D v3 add3(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
SFTG_D v3 scl3(v3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
/* sft_vv_dot: x*x' + (y*y' + z*z') */
SFTG_D float vdot(v3 a, v3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
/* sft_v_dot (scalar C, left to right) */
SFTG_D float sdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
SFTG_D v3 cross3(v3 a, v3 b) { return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }

/* sft_vv_transform: z first, fused, row-vector matrix m[16] row-major */
SFTG_D v3 xform(v3 v, const float* m) {
    v3 r;
    r.x = fma_(v.x, m[0], fma_(v.y, m[4], fma_(v.z, m[8], m[12])));
    r.y = fma_(v.x, m[1], fma_(v.y, m[5], fma_(v.z, m[9], m[13])));
    r.z = fma_(v.x, m[2], fma_(v.y, m[6], fma_(v.z, m[10], m[14])));
    return r;
}
SFTG_D v3 xform_dir(v3 v, const float* m) {
    v3 r;
    r.x = fma_(v.x, m[0], fma_(v.y, m[4], v.z * m[8]));
    r.y = fma_(v.x, m[1], fma_(v.y, m[5], v.z * m[9]));
    r.z = fma_(v.x, m[2], fma_(v.y, m[6], v.z * m[10]));
    return r;
}
/* sft_vv_norm */
SFTG_D v3 vnorm(v3 v) {
    float len = fsqrt(vdot(v, v));
    len = vmax(len, 1e-6f);
    return mk3(fdiv(v.x, len), fdiv(v.y, len), fdiv(v.z, len));
}
/* sft_vv_norm_fast */
SFTG_D v3 vnorm_fast(v3 v) {
    const float sq = vdot(v, v);
    const float a = x86_rsqrt(sq);
    const float refined = (0.5f * a) * fma_(-sq, a * a, 3.f);
    return scl3(v, refined);
}
/* sft_v_norm (scalar) */
SFTG_D v3 snorm(v3 v) {
    const float l = fsqrt(sdot(v, v));
    if (l > 1e-6f) return scl3(v, fdiv(1.f, l));
    return mk3(0.f, 0.f, 0.f);
}
