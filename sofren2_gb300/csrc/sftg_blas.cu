/*
 * BLAS construction on the device: sft__blas_build_model (sofren2.c:3526-3617) over
 * sft__bvh_build_recursive (2967-3062), sft__partition_to_8 (2926-2965) and
 * sft__sort_build_items (2895-2924), producing the same 256 B node images in the same order.
 *
 *   items      every non-padding triangle of the model in meshlet / batch / lane order, with its
 *              box and centroid (3526-3617); one warp per meshlet, a ballot keeps the order
 *   shape      a node of more than 8 items splits its range by count (halves, quarters, eighths),
 *              so node numbering, ranges and the list of sorted ranges depend on the item count
 *              only; the host lays them out (blas_plan) and the device does every data-dependent
 *              step
 *   sorts      a sorted range at split depth d of a node at depth t sorts at level 3t + d; the
 *              ranges of one level are disjoint and read the order the previous level left.
 *              Each sort is the reference's quicksort (middle element as pivot, Hoare scans),
 *              every partition computed in parallel: with fi = !(key < pivot) and
 *              fj = !(key > pivot), the scans stop at the fi positions from the left and at the fj
 *              positions from the right, and the k-th left stop swaps with the k-th right stop
 *              while it lies at or before it.  Where the scans stop after the last swap follows
 *              from the next stops and the last swapped pair.  A range longer than BLAS_CAP is
 *              partitioned by one CTA in global memory until its pieces fit; pieces and short
 *              ranges are finished by one CTA in shared memory, one warp per piece.
 *   nodes      leaves and inner nodes written bottom-up, depth by depth, each node's box the
 *              union of its slots in slot order
 * Comparisons and the centroid (mn + mx) * 0.5 are IEEE single precision as in the reference.
 * Output is bit-identical to the host builder: every permutation step is the sequential one.
 * Overflow of a device work list (not reachable for consistent sizes) sets an error word that
 * the host reads.
 */
#include "sftg_types.h"
#include "sftg_kernels.h"
#include <vector>
#include <cstring>
#include <algorithm>

#define BLAS_CAP 4096            /* positions one shared-memory CTA sorts */
#define BLAS_BIG_THREADS 1024
#define BLAS_SMALL_THREADS 512
#define BLAS_SMALL_WARPS (BLAS_SMALL_THREADS / 32)
#define BLAS_SEQ 32              /* pieces of at most this many positions: one thread each */
#define BLAS_SEQ_STACK 16        /* pending disjoint pieces of >= 2 positions within BLAS_SEQ */
#define BLAS_SMALL_SMEM (BLAS_CAP * 4 * 2 + BLAS_CAP * 2 * 2 + (BLAS_CAP / 2) * 4 * 3)

struct blas_pnode {              /* a node of the plan */
    uint32_t start, count;       /* item range; a leaf when count <= 8 */
    uint32_t nchild;
    uint32_t child[8];
};

/* ------------------------------------------------------------------------------ items */
__device__ __forceinline__ bool tri_live(const uint8_t* in, uint32_t t) {
    const uint32_t b = t >> 3, l = t & 7;
    return !(in[b * 32 + l] == in[b * 32 + 8 + l] && in[b * 32 + 8 + l] == in[b * 32 + 16 + l]);
}

__global__ void k_blas_count(const uint8_t* __restrict__ inds, uint32_t nm, uint32_t* __restrict__ cnt) {
    const uint32_t g = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (g >= nm) return;
    const uint8_t* in = inds + (size_t)g * 512;
    uint32_t c = 0;
    for (uint32_t k = 0; k < 4; k++) c += __popc(__ballot_sync(0xffffffffu, tri_live(in, k * 32 + lane)));
    if (lane == 0) cnt[g] = c;
}

/* one CTA: exclusive prefix of the per-meshlet counts and the total */
__global__ void __launch_bounds__(1024) k_blas_offsets(const uint32_t* __restrict__ cnt, uint32_t nm, uint32_t* __restrict__ off,
                                                       uint32_t* __restrict__ total) {
    __shared__ uint32_t ws[32];
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t carry = 0;
    for (uint32_t base = 0; base < nm; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < nm ? cnt[i] : 0;
        uint32_t s = v;
        for (int d = 1; d < 32; d <<= 1) { const uint32_t o = __shfl_up_sync(0xffffffffu, s, d); if (lane >= (uint32_t)d) s += o; }
        if (lane == 31) ws[w] = s;
        __syncthreads();
        if (w == 0) {
            uint32_t t = ws[lane];
            for (int d = 1; d < 32; d <<= 1) { const uint32_t o = __shfl_up_sync(0xffffffffu, t, d); if (lane >= (uint32_t)d) t += o; }
            ws[lane] = t;
        }
        __syncthreads();
        const uint32_t incl = s + (w ? ws[w - 1] : 0);
        if (i < nm) off[i] = carry + incl - v;
        carry += ws[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

/* items as SoA: it[a * n + q] = mn[a], it[(3 + a) * n + q] = mx[a], it[(6 + a) * n + q] = c[a] */
__global__ void k_blas_items(const float* __restrict__ attr, const uint8_t* __restrict__ inds, uint32_t nm,
                             const uint32_t* __restrict__ off, uint32_t n, float* __restrict__ it, uint32_t* __restrict__ ids,
                             uint32_t* __restrict__ perm) {
    const uint32_t g = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (g >= nm) return;
    const uint8_t* in = inds + (size_t)g * 512;
    const float* at = attr + (size_t)g * 640;
    uint32_t q = off[g];
    for (uint32_t k = 0; k < 4; k++) {
        const uint32_t t = k * 32 + lane;
        const bool live = tri_live(in, t);
        const uint32_t bal = __ballot_sync(0xffffffffu, live);
        const uint32_t o = q + __popc(bal & ((1u << lane) - 1u));
        if (live && o < n) {
            const uint32_t b = t >> 3, l = t & 7;
            const uint32_t i0 = in[b * 32 + l], i1 = in[b * 32 + 8 + l], i2 = in[b * 32 + 16 + l];
            for (int a = 0; a < 3; a++) {
                const float p0 = at[a * 64 + i0], p1 = at[a * 64 + i1], p2 = at[a * 64 + i2];
                const float m12 = p1 < p2 ? p1 : p2, x12 = p1 > p2 ? p1 : p2;
                const float mn = p0 < m12 ? p0 : m12, mx = p0 > x12 ? p0 : x12;
                it[(size_t)a * n + o] = mn;
                it[(size_t)(3 + a) * n + o] = mx;
                it[(size_t)(6 + a) * n + o] = __fmul_rn(__fadd_rn(mn, mx), 0.5f);
            }
            ids[o] = (g << 7) | t;
            perm[o] = o;
        }
        q += __popc(bal);
    }
}

/* ------------------------------------------------------------------------------ axis */
/* the split axis of sft__partition_to_8: the widest centroid extent, y over x and z only when
 * strictly wider, then z over x and y */
__device__ __forceinline__ int pick_axis(const float* lo, const float* hi) {
    const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return (dy > dx && dy > dz) ? 1 : (dz > dx && dz > dy) ? 2 : 0;
}
/* min / max with the reference's strict comparisons: a NaN never enters, and the extents are
 * the same in any order (equal values differ at most in the sign of zero, which no later
 * comparison sees) */
__device__ __forceinline__ void warp_bounds(float* lo, float* hi) {
    for (int d = 16; d > 0; d >>= 1)
        for (int a = 0; a < 3; a++) {
            const float ol = __shfl_xor_sync(0xffffffffu, lo[a], d), oh = __shfl_xor_sync(0xffffffffu, hi[a], d);
            if (ol < lo[a]) lo[a] = ol;
            if (oh > hi[a]) hi[a] = oh;
        }
}

/* one CTA per long range: its axis and its keys in global memory */
__global__ void __launch_bounds__(BLAS_BIG_THREADS) k_blas_axis(const uint2* __restrict__ ranges, uint32_t nr, const float* __restrict__ it,
                                                               uint32_t n, const uint32_t* __restrict__ perm, float* __restrict__ key) {
    __shared__ float sb[32][6];
    __shared__ int s_axis;
    if (blockIdx.x >= nr) return;
    const uint32_t s = ranges[blockIdx.x].x, m = ranges[blockIdx.x].y;
    float lo[3] = { 1e30f, 1e30f, 1e30f }, hi[3] = { -1e30f, -1e30f, -1e30f };
    for (uint32_t x = threadIdx.x; x < m; x += BLAS_BIG_THREADS) {
        const uint32_t q = perm[s + x];
        for (int a = 0; a < 3; a++) {
            const float c = it[(size_t)(6 + a) * n + q];
            if (c < lo[a]) lo[a] = c;
            if (c > hi[a]) hi[a] = c;
        }
    }
    warp_bounds(lo, hi);
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) for (int a = 0; a < 3; a++) { sb[w][a] = lo[a]; sb[w][3 + a] = hi[a]; }
    __syncthreads();
    if (w == 0) {
        for (int a = 0; a < 3; a++) { lo[a] = sb[lane][a]; hi[a] = sb[lane][3 + a]; }
        warp_bounds(lo, hi);
        if (lane == 0) s_axis = pick_axis(lo, hi);
    }
    __syncthreads();
    const float* c = it + (size_t)(6 + s_axis) * n;
    for (uint32_t x = threadIdx.x; x < m; x += BLAS_BIG_THREADS) key[s + x] = c[perm[s + x]];
}

/* ------------------------------------------------------------------------------ partitions */
/* where the reference's scans stop once its K swaps are done (K >= 1: the pivot itself stops
 * both scans).  l_last / r_last: the last swapped pair; l_next / r_next: the next stops (or
 * -1 / INT_MAX past the ends); positions relative to the range. */
__device__ __forceinline__ void final_ij(int l_last, int r_last, int l_next, int r_next, int& i, int& j) {
    i = l_last + 1; j = r_last - 1;
    if (i <= j) {
        i = l_next < r_last ? l_next : r_last;
        j = r_next > l_last ? r_next : l_last;
    }
}

__device__ __forceinline__ uint32_t block_excl_scan_1024(uint32_t v, uint32_t* ws, uint32_t& total) {
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t s = v;
    for (int d = 1; d < 32; d <<= 1) { const uint32_t o = __shfl_up_sync(0xffffffffu, s, d); if (lane >= (uint32_t)d) s += o; }
    if (lane == 31) ws[w] = s;
    __syncthreads();
    if (w == 0) {
        uint32_t t = ws[lane];
        for (int d = 1; d < 32; d <<= 1) { const uint32_t o = __shfl_up_sync(0xffffffffu, t, d); if (lane >= (uint32_t)d) t += o; }
        ws[lane] = t;
    }
    __syncthreads();
    const uint32_t r = s - v + (w ? ws[w - 1] : 0);
    total = ws[31];
    __syncthreads();
    return r;
}

__device__ __forceinline__ void push_piece(uint32_t s, uint32_t m, uint2* next, uint32_t next_cap, uint2* small, uint32_t small_cap, uint32_t* ctr) {
    if (m > BLAS_CAP) {
        const uint32_t k = atomicAdd(&ctr[0], 1u);
        if (k < next_cap) next[k] = make_uint2(s, m); else atomicOr(&ctr[2], 1u);
    } else {
        const uint32_t k = atomicAdd(&ctr[1], 1u);
        if (k < small_cap) small[k] = make_uint2(s, m); else atomicOr(&ctr[2], 1u);
    }
}

/* one CTA partitions one long piece in global memory; the pieces it leaves go to the next
 * round (still long) or to the shared-memory sorter */
__global__ void __launch_bounds__(BLAS_BIG_THREADS) k_blas_part_big(const uint2* __restrict__ list, uint32_t nl, float* __restrict__ key,
                                                                   uint32_t* __restrict__ perm, uint32_t* __restrict__ Lp,
                                                                   uint32_t* __restrict__ Rp, uint2* next, uint32_t next_cap,
                                                                   uint2* small, uint32_t small_cap, uint32_t* ctr) {
    __shared__ uint32_t ws[32];
    __shared__ uint32_t s_tot[3];
    if (blockIdx.x >= nl) return;
    const uint32_t s = list[blockIdx.x].x, m = list[blockIdx.x].y;
    const float p = key[s + m / 2];
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x < 3) s_tot[threadIdx.x] = 0;
    uint32_t ci = 0, cj = 0;
    for (uint32_t x = threadIdx.x; x < m; x += BLAS_BIG_THREADS) {
        const float k = key[s + x];
        ci += !(k < p); cj += !(k > p);
    }
    __syncthreads();
    for (int d = 16; d > 0; d >>= 1) { ci += __shfl_xor_sync(0xffffffffu, ci, d); cj += __shfl_xor_sync(0xffffffffu, cj, d); }
    if (lane == 0) { atomicAdd(&s_tot[0], ci); atomicAdd(&s_tot[1], cj); }
    __syncthreads();
    const uint32_t CI = s_tot[0], CJ = s_tot[1];
    uint32_t carry_i = 0, carry_j = 0, valid = 0;
    for (uint32_t base = 0; base < m; base += BLAS_BIG_THREADS) {
        const uint32_t x = base + threadIdx.x;
        const bool in = x < m;
        const float k = in ? key[s + x] : 0.f;
        const bool fi = in && !(k < p), fj = in && !(k > p);
        uint32_t tot;
        const uint32_t ex = block_excl_scan_1024((fi ? 1u : 0u) | (fj ? 0x10000u : 0u), ws, tot);
        const uint32_t r = carry_i + (ex & 0xFFFFu), pj = carry_j + (ex >> 16);
        if (fi) { Lp[s + r] = x; valid += (r < CJ - pj); }
        if (fj) Rp[s + (CJ - 1 - pj)] = x;
        carry_i += tot & 0xFFFFu; carry_j += tot >> 16;
    }
    for (int d = 16; d > 0; d >>= 1) valid += __shfl_xor_sync(0xffffffffu, valid, d);
    if (lane == 0) atomicAdd(&s_tot[2], valid);
    __syncthreads();
    const uint32_t K = s_tot[2];
    for (uint32_t r = threadIdx.x; r < K; r += BLAS_BIG_THREADS) {
        const uint32_t a = s + Lp[s + r], b = s + Rp[s + r];
        const float ka = key[a]; key[a] = key[b]; key[b] = ka;
        const uint32_t pa = perm[a]; perm[a] = perm[b]; perm[b] = pa;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int i, j;
        final_ij((int)Lp[s + K - 1], (int)Rp[s + K - 1], K < CI ? (int)Lp[s + K] : 0x7fffffff, K < CJ ? (int)Rp[s + K] : -1, i, j);
        if (j >= 1) push_piece(s, (uint32_t)j + 1, next, next_cap, small, small_cap, ctr);
        if ((int)m - i >= 2) push_piece(s + (uint32_t)i, m - (uint32_t)i, next, next_cap, small, small_cap, ctr);
    }
    (void)w;
}

/* one warp partitions the piece [s, s + m) of the shared-memory arrays */
__device__ __forceinline__ void warp_partition(float* Ks, uint32_t* Ps, uint16_t* Lp, uint16_t* Rp, int s, int m, int lane, int& oi, int& oj) {
    const float p = Ks[s + m / 2];
    const uint32_t lt = (1u << lane) - 1u;
    int CI = 0, CJ = 0;
    for (int base = 0; base < m; base += 32) {
        const int x = base + lane;
        const bool in = x < m;
        const float k = in ? Ks[s + x] : 0.f;
        CI += __popc(__ballot_sync(0xffffffffu, in && !(k < p)));
        CJ += __popc(__ballot_sync(0xffffffffu, in && !(k > p)));
    }
    int ci = 0, cj = 0, valid = 0;
    for (int base = 0; base < m; base += 32) {
        const int x = base + lane;
        const bool in = x < m;
        const float k = in ? Ks[s + x] : 0.f;
        const bool fi = in && !(k < p), fj = in && !(k > p);
        const uint32_t bi = __ballot_sync(0xffffffffu, fi), bj = __ballot_sync(0xffffffffu, fj);
        const int r = ci + __popc(bi & lt), pj = cj + __popc(bj & lt);
        if (fi) { Lp[s + r] = (uint16_t)(s + x); valid += (r < CJ - pj); }
        if (fj) Rp[s + CJ - 1 - pj] = (uint16_t)(s + x);
        ci += __popc(bi); cj += __popc(bj);
    }
    const int K = __reduce_add_sync(0xffffffffu, valid);
    __syncwarp();
    for (int r = lane; r < K; r += 32) {
        const int a = Lp[s + r], b = Rp[s + r];
        const float ka = Ks[a]; Ks[a] = Ks[b]; Ks[b] = ka;
        const uint32_t pa = Ps[a]; Ps[a] = Ps[b]; Ps[b] = pa;
    }
    __syncwarp();
    final_ij((int)Lp[s + K - 1] - s, (int)Rp[s + K - 1] - s, K < CI ? (int)Lp[s + K] - s : 0x7fffffff, K < CJ ? (int)Rp[s + K] - s : -1, oi, oj);
    __syncwarp();
}

/* The reference's quicksort itself on [s, s + m) of the shared-memory arrays, by
 * one thread, the recursion kept as a stack of the pending (disjoint) pieces.  The scans carry
 * bounds that the pivot sentinel already guarantees. */
__device__ __forceinline__ void seq_quicksort(float* Ks, uint32_t* Ps, int s, int m) {
    int st_s[BLAS_SEQ_STACK], st_m[BLAS_SEQ_STACK], sp = 0;
    st_s[sp] = s; st_m[sp] = m; sp++;
    while (sp > 0) {
        sp--;
        const int b = st_s[sp], c = st_m[sp];
        const float p = Ks[b + c / 2];
        int i = 0, j = c - 1;
        while (i <= j) {
            while (i < c && Ks[b + i] < p) i++;
            while (j >= 0 && Ks[b + j] > p) j--;
            if (i <= j) {
                const float kt = Ks[b + i]; Ks[b + i] = Ks[b + j]; Ks[b + j] = kt;
                const uint32_t pt = Ps[b + i]; Ps[b + i] = Ps[b + j]; Ps[b + j] = pt;
                i++; j--;
            }
        }
        if (j > 0 && sp < BLAS_SEQ_STACK) { st_s[sp] = b; st_m[sp] = j + 1; sp++; }
        if (c - i > 1 && sp < BLAS_SEQ_STACK) { st_s[sp] = b + i; st_m[sp] = c - i; sp++; }
    }
}

/* One CTA finishes the quicksorts inside one span of at most BLAS_CAP positions.
 * PLAN: the span holds whole ranges of one level (tasks[z .. z + w)); each warp takes ranges,
 *       picks their axes and writes their keys.  Otherwise the span is one piece of a long
 *       range whose keys are already in global memory.
 * The pieces of a round are disjoint; each warp partitions its pieces and queues the parts of
 * more than BLAS_SEQ positions for the next round; parts of 2 to BLAS_SEQ positions are
 * finished after the rounds, one thread each. */
template <bool PLAN>
__global__ void __launch_bounds__(BLAS_SMALL_THREADS) k_blas_sort_small(const uint4* __restrict__ spans, const uint2* __restrict__ list,
                                                                       uint32_t nspans, const uint2* __restrict__ tasks,
                                                                       const float* __restrict__ it, uint32_t n,
                                                                       const float* __restrict__ key, uint32_t* __restrict__ perm) {
    extern __shared__ __align__(16) unsigned char sm[];
    float* Ks = (float*)sm;
    uint32_t* Ps = (uint32_t*)(Ks + BLAS_CAP);
    uint16_t* Lp = (uint16_t*)(Ps + BLAS_CAP);
    uint16_t* Rp = Lp + BLAS_CAP;
    uint32_t* lst0 = (uint32_t*)(Rp + BLAS_CAP);   /* two lists of BLAS_CAP / 2 pieces */
    uint32_t* seq = lst0 + BLAS_CAP;                /* short pieces, BLAS_CAP / 2 */
    __shared__ int ncnt[3];
    if (blockIdx.x >= nspans) return;
    uint32_t s0, m0;
    if (PLAN) { s0 = spans[blockIdx.x].x; m0 = spans[blockIdx.x].y; }
    else { s0 = list[blockIdx.x].x; m0 = list[blockIdx.x].y; }
    if (m0 > BLAS_CAP) m0 = 0;   /* never planned; nothing is touched */
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint32_t x = threadIdx.x; x < m0; x += BLAS_SMALL_THREADS) Ps[x] = perm[s0 + x];
    if (!PLAN) for (uint32_t x = threadIdx.x; x < m0; x += BLAS_SMALL_THREADS) Ks[x] = key[s0 + x];
    if (threadIdx.x == 0) { ncnt[0] = 0; ncnt[1] = 0; ncnt[2] = 0; }
    __syncthreads();
    if (PLAN) {
        const uint32_t t0 = spans[blockIdx.x].z, nt = spans[blockIdx.x].w;
        for (uint32_t t = w; t < nt; t += BLAS_SMALL_WARPS) {
            const uint2 tk = tasks[t0 + t];
            const uint32_t ts = tk.x - s0, tc = tk.y;
            if (ts + tc > m0 || tc < 2) continue;
            float lo[3] = { 1e30f, 1e30f, 1e30f }, hi[3] = { -1e30f, -1e30f, -1e30f };
            for (uint32_t x = lane; x < tc; x += 32) {
                const uint32_t q = Ps[ts + x];
                for (int a = 0; a < 3; a++) {
                    const float c = it[(size_t)(6 + a) * n + q];
                    if (c < lo[a]) lo[a] = c;
                    if (c > hi[a]) hi[a] = c;
                }
            }
            warp_bounds(lo, hi);
            const float* c = it + (size_t)(6 + pick_axis(lo, hi)) * n;
            for (uint32_t x = lane; x < tc; x += 32) Ks[ts + x] = c[Ps[ts + x]];
            if (lane == 0) {
                const int q = tc > BLAS_SEQ ? 0 : 2;
                const int k = atomicAdd(&ncnt[q], 1);
                if (k < BLAS_CAP / 2) (q ? seq : lst0)[k] = (ts << 16) | tc;
            }
        }
    } else if (threadIdx.x == 0 && m0 >= 2) {
        if (m0 > BLAS_SEQ) { lst0[0] = m0; ncnt[0] = 1; } else { seq[0] = m0; ncnt[2] = 1; }
    }
    int cur = 0;
    for (;;) {
        __syncthreads();
        const int nc = min(ncnt[cur], BLAS_CAP / 2);
        if (nc == 0) break;
        const uint32_t* in_l = lst0 + cur * (BLAS_CAP / 2);
        uint32_t* out_l = lst0 + (cur ^ 1) * (BLAS_CAP / 2);
        if (threadIdx.x == 0) ncnt[cur ^ 1] = 0;
        __syncthreads();
        for (int e = w; e < nc; e += BLAS_SMALL_WARPS) {
            const uint32_t v = in_l[e];
            const int s = (int)(v >> 16), m = (int)(v & 0xFFFFu);
            int i, j;
            warp_partition(Ks, Ps, Lp, Rp, s, m, lane, i, j);
            if (lane == 0) {
                const uint32_t ps[2] = { (uint32_t)s, (uint32_t)(s + i) };
                const int pm[2] = { j + 1, m - i };
                for (int h = 0; h < 2; h++) {
                    if (pm[h] < 2) continue;
                    const int q = pm[h] > BLAS_SEQ ? (cur ^ 1) : 2;
                    const int k = atomicAdd(&ncnt[q], 1);
                    if (k < BLAS_CAP / 2) (q == 2 ? seq : out_l)[k] = (ps[h] << 16) | (uint32_t)pm[h];
                }
            }
        }
        cur ^= 1;
    }
    const int ns = min(ncnt[2], BLAS_CAP / 2);
    for (int k = threadIdx.x; k < ns; k += BLAS_SMALL_THREADS) seq_quicksort(Ks, Ps, (int)(seq[k] >> 16), (int)(seq[k] & 0xFFFFu));
    __syncthreads();
    for (uint32_t x = threadIdx.x; x < m0; x += BLAS_SMALL_THREADS) perm[s0 + x] = Ps[x];
}

/* ------------------------------------------------------------------------------ nodes */
__global__ void k_blas_nodes(const blas_pnode* __restrict__ pn, const uint32_t* __restrict__ idx, uint32_t cnt,
                             const float* __restrict__ it, const uint32_t* __restrict__ ids, const uint32_t* __restrict__ perm,
                             uint32_t n, float* __restrict__ bounds, sftg_bvh_node* __restrict__ out) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    const uint32_t ni = idx[t];
    const blas_pnode P = pn[ni];
    sftg_bvh_node nd;
    memset(&nd, 0, sizeof(nd));
    for (int i = 0; i < 8; i++) { for (int a = 0; a < 3; a++) { nd.mn[a][i] = 1e30f; nd.mx[a][i] = -1e30f; } nd.child[i] = 0xFFFFFFFFu; }
    float lo[3] = { 1e30f, 1e30f, 1e30f }, hi[3] = { -1e30f, -1e30f, -1e30f };
    if (P.count <= 8) {
        nd.leaf = 1; nd.count = (uint8_t)P.count;
        for (uint32_t i = 0; i < P.count; i++) {
            const uint32_t q = perm[P.start + i];
            for (int a = 0; a < 3; a++) {
                const float mn = it[(size_t)a * n + q], mx = it[(size_t)(3 + a) * n + q];
                nd.mn[a][i] = mn; nd.mx[a][i] = mx;
                if (mn < lo[a]) lo[a] = mn;
                if (mx > hi[a]) hi[a] = mx;
            }
            nd.child[i] = 0x80000000u | ids[q];
        }
    } else {
        nd.count = (uint8_t)P.nchild;
        for (uint32_t c = 0; c < P.nchild && c < 8; c++) {
            const uint32_t ci = P.child[c];
            for (int a = 0; a < 3; a++) {
                const float mn = bounds[(size_t)ci * 6 + a], mx = bounds[(size_t)ci * 6 + 3 + a];
                nd.mn[a][c] = mn; nd.mx[a][c] = mx;
                if (mn < lo[a]) lo[a] = mn;
                if (mx > hi[a]) hi[a] = mx;
            }
            nd.child[c] = ci;
        }
    }
    out[ni] = nd;
    for (int a = 0; a < 3; a++) { bounds[(size_t)ni * 6 + a] = lo[a]; bounds[(size_t)ni * 6 + 3 + a] = hi[a]; }
}

/* ------------------------------------------------------------------------------ host */
struct sftg_blas_job {
    cudaStream_t st = nullptr;
    uint32_t nm = 0, n = 0;
    const float* attr = nullptr;
    const uint8_t* inds = nullptr;
    uint32_t* d_cnt = nullptr;      /* [nm] counts, then [nm] offsets, then total */
    uint32_t launches = 0;          /* kernels launched by begin and finish */
    /* plan */
    std::vector<blas_pnode> nodes;
    std::vector<std::vector<uint32_t>> by_depth;
    std::vector<std::vector<uint2>> by_level;
};

static void plan_split(sftg_blas_job& J, uint32_t start, uint32_t count, uint32_t d, uint32_t level, uint32_t* st, uint32_t* cn, uint32_t& ng) {
    if (!count) return;
    if (d == 3 || count == 1) { st[ng] = start; cn[ng] = count; ng++; return; }
    if (J.by_level.size() <= level + d) J.by_level.resize(level + d + 1);
    J.by_level[level + d].push_back(make_uint2(start, count));
    const uint32_t mid = count / 2;
    plan_split(J, start, mid, d + 1, level, st, cn, ng);
    plan_split(J, start + mid, count - mid, d + 1, level, st, cn, ng);
}

static uint32_t plan_node(sftg_blas_job& J, uint32_t start, uint32_t count, uint32_t depth) {
    const uint32_t ni = (uint32_t)J.nodes.size();
    blas_pnode p;
    memset(&p, 0, sizeof(p));
    p.start = start; p.count = count;
    for (int i = 0; i < 8; i++) p.child[i] = 0xFFFFFFFFu;
    J.nodes.push_back(p);
    if (J.by_depth.size() <= depth) J.by_depth.resize(depth + 1);
    J.by_depth[depth].push_back(ni);
    if (count <= 8) return ni;
    uint32_t st[8] = { 0 }, cn[8] = { 0 }, ng = 0;
    plan_split(J, start, count, 0, 3 * depth, st, cn, ng);
    for (uint32_t c = 0; c < ng; c++) {
        const uint32_t ci = plan_node(J, st[c], cn[c], depth + 1);
        J.nodes[ni].child[c] = ci;
    }
    J.nodes[ni].nchild = ng;
    return ni;
}

#define BK(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return e_; } while (0)

cudaError_t sftg_blas_begin(sftg_blas_job** out, const float* attr, const uint8_t* inds, uint32_t nm, cudaStream_t st,
                            uint32_t* n_items, uint32_t* n_nodes) {
    *out = nullptr; *n_items = 0; *n_nodes = 0;
    sftg_blas_job* J = new sftg_blas_job();
    J->st = st; J->nm = nm; J->attr = attr; J->inds = inds;
    *out = J;
    if (!nm) return cudaSuccess;
    BK(cudaMallocAsync((void**)&J->d_cnt, ((size_t)nm * 2 + 1) * 4, st));
    k_blas_count<<<(nm + 7) / 8, 256, 0, st>>>(inds, nm, J->d_cnt);
    k_blas_offsets<<<1, 1024, 0, st>>>(J->d_cnt, nm, J->d_cnt + nm, J->d_cnt + 2 * (size_t)nm);
    BK(cudaGetLastError());
    J->launches += 2;
    uint32_t total = 0;
    BK(cudaMemcpyAsync(&total, J->d_cnt + 2 * (size_t)nm, 4, cudaMemcpyDeviceToHost, st));
    BK(cudaStreamSynchronize(st));
    J->n = total;
    if (total) plan_node(*J, 0, total, 0);
    *n_items = total;
    *n_nodes = (uint32_t)J->nodes.size();
    return cudaSuccess;
}

cudaError_t sftg_blas_finish(sftg_blas_job* J, sftg_bvh_node* dst, uint32_t* status) {
    *status = 0;
    const uint32_t n = J->n, nn = (uint32_t)J->nodes.size();
    if (!n) return cudaSuccess;
    cudaStream_t st = J->st;
    /* tasks of every level, spans of the short ones, and the node plan, in one upload */
    std::vector<uint2> tasks, big;
    std::vector<uint4> spans;
    std::vector<uint32_t> lv_task_off, lv_span_off, lv_span_cnt, lv_big_off, lv_big_cnt;
    /* short ranges are packed into spans of about n / (3 x SMs) positions (three CTAs fit an SM),
     * so that deep levels of many small ranges still fill the GPU */
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t span_target = std::min<uint32_t>(BLAS_CAP, std::max<uint32_t>(256, n / (3u * (uint32_t)std::max(sms, 1))));
    for (size_t L = 0; L < J->by_level.size(); L++) {
        const std::vector<uint2>& T = J->by_level[L];
        lv_task_off.push_back((uint32_t)tasks.size());
        lv_span_off.push_back((uint32_t)spans.size());
        lv_big_off.push_back((uint32_t)big.size());
        const uint32_t t_base = (uint32_t)tasks.size();
        uint32_t k = 0;
        while (k < T.size()) {
            if (T[k].y > BLAS_CAP) { big.push_back(T[k]); k++; continue; }
            const uint32_t s0 = T[k].x;
            uint32_t e = k + 1;
            while (e < T.size() && T[e].y <= BLAS_CAP && T[e].x + T[e].y - s0 <= span_target) e++;
            spans.push_back(make_uint4(s0, T[e - 1].x + T[e - 1].y - s0, t_base + k, e - k));
            k = e;
        }
        tasks.insert(tasks.end(), T.begin(), T.end());
        lv_span_cnt.push_back((uint32_t)spans.size() - lv_span_off.back());
        lv_big_cnt.push_back((uint32_t)big.size() - lv_big_off.back());
    }
    std::vector<uint32_t> depth_idx, depth_off;
    for (size_t d = 0; d < J->by_depth.size(); d++) {
        depth_off.push_back((uint32_t)depth_idx.size());
        depth_idx.insert(depth_idx.end(), J->by_depth[d].begin(), J->by_depth[d].end());
    }
    const uint32_t list_cap = n / BLAS_CAP + 4, small_cap = n / 2 + 4;
    /* device scratch: items, ids, perm, key, Lp, Rp, bounds, lists, counters, plan */
    size_t o = 0;
    auto take = [&](size_t bytes) { const size_t r = o; o += (bytes + 255) & ~(size_t)255; return r; };
    const size_t o_it = take((size_t)n * 36), o_ids = take((size_t)n * 4), o_perm = take((size_t)n * 4), o_key = take((size_t)n * 4);
    const size_t o_lp = take((size_t)n * 4), o_rp = take((size_t)n * 4), o_bnd = take((size_t)nn * 24);
    const size_t o_l0 = take((size_t)list_cap * 8), o_l1 = take((size_t)list_cap * 8), o_sm = take((size_t)small_cap * 8);
    const size_t o_ctr = take(16);
    const size_t o_tasks = take(tasks.size() * 8 + 8), o_spans = take(spans.size() * 16 + 16), o_big = take(big.size() * 8 + 8);
    const size_t o_pn = take((size_t)nn * sizeof(blas_pnode)), o_didx = take(depth_idx.size() * 4 + 4);
    const size_t o_plan = o_tasks, plan_bytes = o - o_tasks;
    char* d = nullptr;
    BK(cudaMallocAsync((void**)&d, o, st));
    std::vector<char> h(plan_bytes);
    memcpy(h.data() + (o_tasks - o_plan), tasks.data(), tasks.size() * 8);
    memcpy(h.data() + (o_spans - o_plan), spans.data(), spans.size() * 16);
    memcpy(h.data() + (o_big - o_plan), big.data(), big.size() * 8);
    memcpy(h.data() + (o_pn - o_plan), J->nodes.data(), (size_t)nn * sizeof(blas_pnode));
    memcpy(h.data() + (o_didx - o_plan), depth_idx.data(), depth_idx.size() * 4);
    cudaError_t err = cudaMemcpyAsync(d + o_plan, h.data(), plan_bytes, cudaMemcpyHostToDevice, st);
    float* it = (float*)(d + o_it);
    uint32_t* ids = (uint32_t*)(d + o_ids);
    uint32_t* perm = (uint32_t*)(d + o_perm);
    float* key = (float*)(d + o_key);
    uint32_t* Lp = (uint32_t*)(d + o_lp);
    uint32_t* Rp = (uint32_t*)(d + o_rp);
    float* bnd = (float*)(d + o_bnd);
    uint2* lists[2] = { (uint2*)(d + o_l0), (uint2*)(d + o_l1) };
    uint2* small = (uint2*)(d + o_sm);
    uint32_t* ctr = (uint32_t*)(d + o_ctr);
    const uint2* d_tasks = (const uint2*)(d + o_tasks);
    const uint4* d_spans = (const uint4*)(d + o_spans);
    const uint2* d_big = (const uint2*)(d + o_big);
    const blas_pnode* d_pn = (const blas_pnode*)(d + o_pn);
    const uint32_t* d_didx = (const uint32_t*)(d + o_didx);
    if (err == cudaSuccess) err = cudaFuncSetAttribute(k_blas_sort_small<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, BLAS_SMALL_SMEM);
    if (err == cudaSuccess) err = cudaFuncSetAttribute(k_blas_sort_small<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, BLAS_SMALL_SMEM);
    if (err == cudaSuccess) err = cudaMemsetAsync(ctr, 0, 16, st);
    if (err == cudaSuccess) {
        k_blas_items<<<(J->nm + 7) / 8, 256, 0, st>>>(J->attr, J->inds, J->nm, J->d_cnt + J->nm, n, it, ids, perm);
        err = cudaGetLastError();
        J->launches++;
    }
    uint32_t* h_ctr = nullptr;
    if (err == cudaSuccess) err = cudaMallocHost((void**)&h_ctr, 16);
    for (size_t L = 0; err == cudaSuccess && L < J->by_level.size(); L++) {
        if (lv_span_cnt[L]) {
            k_blas_sort_small<true><<<lv_span_cnt[L], BLAS_SMALL_THREADS, BLAS_SMALL_SMEM, st>>>(d_spans + lv_span_off[L], nullptr, lv_span_cnt[L],
                                                                                                 d_tasks, it, n, key, perm);
            J->launches++;
        }
        if (lv_big_cnt[L]) {
            k_blas_axis<<<lv_big_cnt[L], BLAS_BIG_THREADS, 0, st>>>(d_big + lv_big_off[L], lv_big_cnt[L], it, n, perm, key);
            J->launches++;
            const uint2* curl = d_big + lv_big_off[L];
            uint32_t ncur = lv_big_cnt[L], flip = 0;
            err = cudaMemsetAsync(ctr, 0, 8, st);
            while (err == cudaSuccess && ncur) {
                if ((err = cudaMemsetAsync(ctr, 0, 4, st)) != cudaSuccess) break;
                k_blas_part_big<<<ncur, BLAS_BIG_THREADS, 0, st>>>(curl, ncur, key, perm, Lp, Rp, lists[flip], list_cap, small, small_cap, ctr);
                J->launches++;
                if ((err = cudaGetLastError()) != cudaSuccess) break;
                if ((err = cudaMemcpyAsync(h_ctr, ctr, 12, cudaMemcpyDeviceToHost, st)) != cudaSuccess) break;
                if ((err = cudaStreamSynchronize(st)) != cudaSuccess) break;
                if (h_ctr[2]) { *status = 1; break; }
                ncur = h_ctr[0] < list_cap ? h_ctr[0] : 0;
                curl = lists[flip]; flip ^= 1;
            }
            if (err != cudaSuccess || *status) break;
            const uint32_t ns = h_ctr[1] < small_cap ? h_ctr[1] : 0;
            if (ns) {
                k_blas_sort_small<false><<<ns, BLAS_SMALL_THREADS, BLAS_SMALL_SMEM, st>>>(nullptr, small, ns, nullptr, it, n, key, perm);
                J->launches++;
            }
        }
        if (err == cudaSuccess) err = cudaGetLastError();
    }
    for (size_t dd = J->by_depth.size(); err == cudaSuccess && !*status && dd-- > 0;) {
        const uint32_t cnt = (uint32_t)J->by_depth[dd].size();
        k_blas_nodes<<<(cnt + 127) / 128, 128, 0, st>>>(d_pn, d_didx + depth_off[dd], cnt, it, ids, perm, n, bnd, dst);
        err = cudaGetLastError();
        J->launches++;
    }
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    if (h_ctr) cudaFreeHost(h_ctr);
    cudaFreeAsync(d, st);
    return err;
}

uint32_t sftg_blas_launches(const sftg_blas_job* J) { return J ? J->launches : 0; }

void sftg_blas_end(sftg_blas_job* J) {
    if (!J) return;
    if (J->d_cnt) cudaFreeAsync(J->d_cnt, J->st);
    delete J;
}
