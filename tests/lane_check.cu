/*
 * Exhaustive check of the device RCPPS / RSQRTPS emulation (sftg_lane.cuh) over all 2^32 input
 * bit patterns: the fast paths must give exactly what the plain table form gives, the one the
 * measured tables were written for (include/x86_approx_tables.h; on x86 tests/test_abi.py checks
 * that form against the instructions themselves).  Prints the two mismatch counts and the first
 * mismatching input of each.  Run by tests/test_gpu_lane.py.
 */
#include <cstdio>
#include <cstdint>
#include "sftg_lane.cuh"

__device__ uint32_t rcp_plain(uint32_t x) {
    const uint32_t s = x & 0x80000000u, e = (x >> 23) & 0xFF, m = x & 0x7FFFFF;
    if (e == 0xFF) return m ? (x | 0x00400000u) : s;
    if (e == 0) return s | 0x7F800000u;
    if (e >= 253) return s;
    return s | ((253u - e) << 23) | g_rcp_tab[m >> 12];
}
__device__ uint32_t rsq_plain(uint32_t x) {
    const uint32_t s = x & 0x80000000u, e = (x >> 23) & 0xFF, m = x & 0x7FFFFF;
    if (e == 0xFF) { if (m) return x | 0x00400000u; return s ? 0xFFC00000u : 0u; }
    if (e == 0) return s | 0x7F800000u;
    if (s) return 0xFFC00000u;
    const uint32_t t = g_rsq_tab[(e & 1) * 1024 + (m >> 13)];
    const int oe = ((380 - (int)e) >> 1) + (int)(t >> 23) - 1;
    return ((uint32_t)oe << 23) | (t & 0x7FFFFF);
}

__global__ void k_check(uint64_t base, unsigned long long* bad, unsigned int* first) {
    const uint64_t i = base + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >> 32) return;
    const uint32_t x = (uint32_t)i;
    const float f = __uint_as_float(x);
    if (__float_as_uint(x86_rcp(f)) != rcp_plain(x)) { atomicAdd(&bad[0], 1ull); atomicMin(&first[0], x); }
    if (__float_as_uint(x86_rsqrt(f)) != rsq_plain(x)) { atomicAdd(&bad[1], 1ull); atomicMin(&first[1], x); }
}

int main() {
    unsigned long long* bad; unsigned int* first;
    if (cudaMalloc(&bad, 16) != cudaSuccess || cudaMalloc(&first, 8) != cudaSuccess) { printf("alloc failed\n"); return 2; }
    cudaMemset(bad, 0, 16);
    cudaMemset(first, 0xFF, 8);
    const uint64_t per = 1ull << 30;   /* 2^30 inputs per launch, 4 launches */
    for (uint64_t b = 0; b < (1ull << 32); b += per) k_check<<<(unsigned)(per / 256), 256>>>(b, bad, first);
    unsigned long long h[2]; unsigned int f[2];
    if (cudaMemcpy(h, bad, 16, cudaMemcpyDeviceToHost) != cudaSuccess || cudaMemcpy(f, first, 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
        printf("cuda error: %s\n", cudaGetErrorString(cudaGetLastError())); return 3;
    }
    printf("%llu %llu %08x %08x\n", h[0], h[1], f[0], f[1]);
    return (h[0] || h[1]) ? 1 : 0;
}
