/*
 * Measures the x86 RCPPS / RSQRTPS approximation instructions on the host CPU and
 * writes them out as lookup tables, so that CUDA kernels (and any non-x86 host)
 * can reproduce the exact bits the AVX2 renderer computes.
 *
 * The AVX2 path of sofren2 uses `_mm256_rcp_ps` (sofren2.c:289, through
 * `sft_vf_rcp_refined` sofren2.c:633-638) and `_mm256_rsqrt_ps` (sofren2.c:296,
 * through `sft_vv_norm_fast` sofren2.c:1973-1992). Their outputs are
 * implementation-defined (Intel and AMD differ), so the tables are measured, not
 * derived. On the Intel core these tables were taken from:
 *   rcp(x)   = sign | (253 - e) << 23 | RCP[mantissa >> 12]          (1 <= e <= 252)
 *              +-inf for zero/denormal x, +-0 for e >= 253, quiet NaN for NaN
 *   rsqrt(x) = (e odd/even table) | exponent (380 - e) / 2 style       (x > 0 normal)
 *              +-inf for zero/denormal x, NaN for x < 0, 0 for +inf
 * The generator verifies the table form against the instruction for all 2^32
 * inputs before writing anything; it exits non-zero if any input disagrees.
 *
 * Build (x86-64 with AVX2 only):
 *   gcc -O2 -mavx2 gen_x86_approx_tables.c -o gen && ./gen out.h
 */
#include <immintrin.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

static uint32_t RCP[2048];          /* 23-bit mantissa of rcp for mantissa index m>>12 */
static uint32_t RSQ[2][1024];       /* [e & 1][m >> 13] -> mantissa | (exp_adj << 23) */

static uint32_t rcp_model(uint32_t x) {
    const uint32_t s = x & 0x80000000u, e = (x >> 23) & 0xFF, m = x & 0x7FFFFF;
    if (e == 0xFF) return m ? (x | 0x00400000u) : s;            /* NaN quiet, inf -> 0 */
    if (e == 0) return s | 0x7F800000u;                          /* zero/denormal -> inf */
    if (e >= 253) return s;                                      /* result underflows */
    return s | ((253u - e) << 23) | RCP[m >> 12];
}

static uint32_t rsq_model(uint32_t x) {
    const uint32_t s = x & 0x80000000u, e = (x >> 23) & 0xFF, m = x & 0x7FFFFF;
    if (e == 0xFF) { if (m) return x | 0x00400000u; return s ? 0xFFC00000u : 0u; }
    if (e == 0) return s | 0x7F800000u;
    if (s) return 0xFFC00000u;
    const uint32_t t = RSQ[e & 1][m >> 13];
    /* exponent: unbiased ue = e - 127; result ~ 2^(-ue/2); stored adj covers parity */
    const int32_t out_e = (int32_t)((380 - (int32_t)e) >> 1) + (int32_t)(t >> 23) - 1;
    return ((uint32_t)out_e << 23) | (t & 0x7FFFFF);
}

int main(int argc, char** argv) {
    /* rcp table from exponent 127 */
    for (uint32_t i = 0; i < 2048; i++) {
        const uint32_t x = (127u << 23) | (i << 12);
        const uint32_t r = f2u(_mm_cvtss_f32(_mm_rcp_ss(_mm_set1_ps(u2f(x)))));
        RCP[i] = r & 0x7FFFFF;
        if (((r >> 23) & 0xFF) != 126) { fprintf(stderr, "rcp exponent assumption broken at %u\n", i); return 2; }
    }
    /* rsqrt table from exponents 127 (odd) and 128 (even) */
    for (uint32_t p = 0; p < 2; p++) {
        const uint32_t e = p ? 127u : 128u;
        for (uint32_t i = 0; i < 1024; i++) {
            const uint32_t x = (e << 23) | (i << 13);
            const uint32_t r = f2u(_mm_cvtss_f32(_mm_rsqrt_ss(_mm_set1_ps(u2f(x)))));
            const int32_t base_e = (int32_t)((380 - (int32_t)e) >> 1);
            const int32_t adj = (int32_t)((r >> 23) & 0xFF) - base_e + 1;
            if (adj < 0 || adj > 3) { fprintf(stderr, "rsqrt exponent assumption broken\n"); return 2; }
            RSQ[e & 1][i] = ((uint32_t)adj << 23) | (r & 0x7FFFFF);
        }
    }
    /* exhaustive verification, 8 lanes at a time */
    uint64_t bad_rcp = 0, bad_rsq = 0;
    for (uint64_t base = 0; base < (1ull << 32); base += 8) {
        uint32_t in[8];
        for (int l = 0; l < 8; l++) in[l] = (uint32_t)(base + l);
        __m256 v = _mm256_loadu_ps((const float*)in);
        uint32_t r[8], q[8];
        _mm256_storeu_ps((float*)r, _mm256_rcp_ps(v));
        _mm256_storeu_ps((float*)q, _mm256_rsqrt_ps(v));
        for (int l = 0; l < 8; l++) {
            if (r[l] != rcp_model(in[l])) { if (bad_rcp++ < 8) fprintf(stderr, "rcp %08x: hw %08x model %08x\n", in[l], r[l], rcp_model(in[l])); }
            if (q[l] != rsq_model(in[l])) { if (bad_rsq++ < 8) fprintf(stderr, "rsq %08x: hw %08x model %08x\n", in[l], q[l], rsq_model(in[l])); }
        }
    }
    fprintf(stderr, "verified 2^32 inputs: rcp mismatches %llu, rsqrt mismatches %llu\n",
            (unsigned long long)bad_rcp, (unsigned long long)bad_rsq);
    if (bad_rcp || bad_rsq) return 1;

    FILE* f = (argc > 1) ? fopen(argv[1], "w") : stdout;
    if (!f) return 3;
    fprintf(f, "/* Generated by gen_x86_approx_tables.c on an Intel x86-64 host: the exact outputs of\n"
               " * RCPPS (mantissa index = x mantissa >> 12) and RSQRTPS (index = [exponent & 1][mantissa >> 13],\n"
               " * entry = mantissa | exponent_adjust << 23). Verified against the instruction for all 2^32 inputs. */\n");
    fprintf(f, "#pragma once\n#include <stdint.h>\n");
    fprintf(f, "#define SFT_X86_RCP_TABLE_INIT {");
    for (int i = 0; i < 2048; i++) fprintf(f, "%s0x%06xu", (i % 8) ? "," : ",\\\n  " + (i == 0), RCP[i]);
    fprintf(f, "}\n#define SFT_X86_RSQRT_TABLE_INIT {");
    for (int p = 0; p < 2; p++) for (int i = 0; i < 1024; i++)
        fprintf(f, "%s0x%07xu", ((p * 1024 + i) % 8) ? "," : ",\\\n  " + (p == 0 && i == 0), RSQ[p][i]);
    fprintf(f, "}\n");
    if (f != stdout) fclose(f);
    return 0;
}
