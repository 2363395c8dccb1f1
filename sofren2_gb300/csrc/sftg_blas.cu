/*
 * BLAS construction on the device: sft__blas_build_model (sofren2.c:3526-3617) over
 * sft__bvh_build_recursive (2967-3062), sft__partition_to_8 (2926-2965) and
 * sft__sort_build_items (2895-2924), producing the same 256 B node images in the same order.
 *
 *   items      every non-padding triangle of the model in meshlet / batch / lane order, with its
 *              box and centroid (3526-3617); one warp per meshlet, a ballot keeps the order
 *   shape      a node of more than 8 items splits its range by count (halves, quarters, eighths),
 *              so node numbering, ranges and the list of sorted ranges depend on the item count
 *              only; the host lays them out (sftg_blas_plan.h) and the device does every data-dependent
 *              step
 *   sorts      a sorted range at split depth d of a node at depth t sorts at level 3t + d; the
 *              ranges of one level are disjoint and read the order the previous level left.
 *              Each sort is the reference's quicksort (middle element as pivot, Hoare scans),
 *              every partition computed in parallel: with fi = !(key < pivot) and
 *              fj = !(key > pivot), the scans stop at the fi positions from the left and at the fj
 *              positions from the right, and the k-th left stop swaps with the k-th right stop
 *              while it lies at or before it.  Where the scans stop after the last swap follows
 *              from the next stops and the last swapped pair.
 *   long       ranges longer than BLAS_CAP: chunks of BLAS_CHUNK positions, partition rounds of
 *              five kernels over all long pieces of a level, round counts kept on the device
 *   short      ranges and pieces of at most BLAS_CAP: one CTA per span in shared memory, one
 *              warp per piece per round, pieces of at most BLAS_SEQ positions finished by one
 *              thread with the sequential quicksort
 *   nodes      leaves and inner nodes written bottom-up, depth by depth, each node's box the
 *              union of its slots in slot order
 * Comparisons and the centroid (mn + mx) * 0.5 are IEEE single precision as in the reference.
 * The node images are byte-identical to the reference's: every permutation step is the
 * sequential one.  Overflow of a device work list (not reachable for consistent sizes) sets an
 * error word that the host reads.
 */
#include "sftg_types.h"
#include "sftg_kernels.h"
#include "sftg_blas_plan.h"
#include <vector>
#include <cstring>
#include <algorithm>

#define BLAS_CAP 4096            /* positions one shared-memory CTA sorts */
#define BLAS_SMALL_THREADS 512
#define BLAS_SMALL_WARPS (BLAS_SMALL_THREADS / 32)
#define BLAS_SEQ 32              /* pieces of at most this many positions: one thread each */
#define BLAS_CTA_PIECE 1024      /* pieces longer than this: partitioned by the whole CTA */
#define BLAS_BIGQ 8              /* pending such pieces (disjoint, so at most 3 within BLAS_CAP) */
#define BLAS_SEQ_STACK 16        /* pending disjoint pieces of >= 2 positions within BLAS_SEQ */
#define BLAS_SMALL_SMEM (BLAS_CAP * 4 * 2 + BLAS_CAP * 2 * 2 + (BLAS_CAP / 2) * 4 * 3)

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

/* Long ranges are cut into chunks of BLAS_CHUNK positions; a chunk is (piece, start within the
 * piece, length), and the chunks of one piece are consecutive in the chunk table. */
#define BLAS_CHUNK 2048
#define BLAS_CHUNK_THREADS 256
#define BLAS_CHUNK_PER_THREAD (BLAS_CHUNK / BLAS_CHUNK_THREADS)

__device__ __forceinline__ void block_bounds_256(float* lo, float* hi, float (*sb)[6]) {
    warp_bounds(lo, hi);
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) for (int a = 0; a < 3; a++) { sb[w][a] = lo[a]; sb[w][3 + a] = hi[a]; }
    __syncthreads();
    if (w == 0) {
        for (int a = 0; a < 3; a++) { lo[a] = lane < BLAS_CHUNK_THREADS / 32 ? sb[lane][a] : 1e30f; hi[a] = lane < BLAS_CHUNK_THREADS / 32 ? sb[lane][3 + a] : -1e30f; }
        warp_bounds(lo, hi);
    }
}

/* centroid bounds of each chunk of the long ranges */
__global__ void __launch_bounds__(BLAS_CHUNK_THREADS) k_blas_chunk_bounds(const uint2* __restrict__ pieces, const uint4* __restrict__ chunks,
                                                                        uint32_t nch, const float* __restrict__ it, uint32_t n,
                                                                        const uint32_t* __restrict__ perm, float* __restrict__ part) {
    __shared__ float sb[BLAS_CHUNK_THREADS / 32][6];
    if (blockIdx.x >= nch) return;
    const uint4 c = chunks[blockIdx.x];
    const uint32_t s = pieces[c.x].x + c.y;
    float lo[3] = { 1e30f, 1e30f, 1e30f }, hi[3] = { -1e30f, -1e30f, -1e30f };
    for (uint32_t x = threadIdx.x; x < c.z; x += BLAS_CHUNK_THREADS) {
        const uint32_t q = perm[s + x];
        for (int a = 0; a < 3; a++) {
            const float v = it[(size_t)(6 + a) * n + q];
            if (v < lo[a]) lo[a] = v;
            if (v > hi[a]) hi[a] = v;
        }
    }
    block_bounds_256(lo, hi, sb);
    if (threadIdx.x == 0) for (int a = 0; a < 3; a++) { part[(size_t)blockIdx.x * 6 + a] = lo[a]; part[(size_t)blockIdx.x * 6 + 3 + a] = hi[a]; }
}

/* one warp per long range: its split axis from the chunk bounds */
__global__ void k_blas_range_axis(const uint2* __restrict__ pchunk, uint32_t np, const float* __restrict__ part, uint8_t* __restrict__ axis) {
    const uint32_t pi = blockIdx.x * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (pi >= np) return;
    const uint2 pc = pchunk[pi];
    float lo[3] = { 1e30f, 1e30f, 1e30f }, hi[3] = { -1e30f, -1e30f, -1e30f };
    for (uint32_t k = lane; k < pc.y; k += 32)
        for (int a = 0; a < 3; a++) {
            const float l = part[(size_t)(pc.x + k) * 6 + a], h = part[(size_t)(pc.x + k) * 6 + 3 + a];
            if (l < lo[a]) lo[a] = l;
            if (h > hi[a]) hi[a] = h;
        }
    warp_bounds(lo, hi);
    if (lane == 0) axis[pi] = (uint8_t)pick_axis(lo, hi);
}

/* the keys of the long ranges: centroids along each range's axis, in the current order */
__global__ void __launch_bounds__(BLAS_CHUNK_THREADS) k_blas_chunk_keys(const uint2* __restrict__ pieces, const uint4* __restrict__ chunks,
                                                                      uint32_t nch, const uint8_t* __restrict__ axis, const float* __restrict__ it,
                                                                      uint32_t n, const uint32_t* __restrict__ perm, float* __restrict__ key) {
    if (blockIdx.x >= nch) return;
    const uint4 c = chunks[blockIdx.x];
    const uint32_t s = pieces[c.x].x + c.y;
    const float* cv = it + (size_t)(6 + axis[c.x]) * n;
    for (uint32_t x = threadIdx.x; x < c.z; x += BLAS_CHUNK_THREADS) key[s + x] = cv[perm[s + x]];
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

__device__ __forceinline__ uint32_t block_excl_scan_256(uint32_t v, uint32_t* ws) {
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t sc = v;
    for (int d = 1; d < 32; d <<= 1) { const uint32_t o = __shfl_up_sync(0xffffffffu, sc, d); if (lane >= (uint32_t)d) sc += o; }
    if (lane == 31) ws[w] = sc;
    __syncthreads();
    uint32_t before = 0;
    for (uint32_t k = 0; k < w; k++) before += ws[k];
    return before + sc - v;
}

/* Partition round over every long piece, step 1: per chunk, how many positions stop the left
 * scan (fi) and the right scan (fj) for the piece's pivot. */
__global__ void __launch_bounds__(BLAS_CHUNK_THREADS) k_blas_part_count(const uint2* __restrict__ pieces, const uint4* __restrict__ chunks,
                                                                      const uint32_t* __restrict__ rs, const float* __restrict__ key,
                                                                      uint2* __restrict__ cc) {
    __shared__ uint32_t s_c[2];
    if (blockIdx.x >= rs[1]) return;
    const uint4 c = chunks[blockIdx.x];
    const uint2 pc = pieces[c.x];
    const float p = key[pc.x + pc.y / 2];
    if (threadIdx.x < 2) s_c[threadIdx.x] = 0;
    __syncthreads();
    uint32_t ci = 0, cj = 0;
    for (uint32_t x = threadIdx.x; x < c.z; x += BLAS_CHUNK_THREADS) {
        const float k = key[pc.x + c.y + x];
        ci += !(k < p); cj += !(k > p);
    }
    for (int d = 16; d > 0; d >>= 1) { ci += __shfl_xor_sync(0xffffffffu, ci, d); cj += __shfl_xor_sync(0xffffffffu, cj, d); }
    if ((threadIdx.x & 31) == 0) { atomicAdd(&s_c[0], ci); atomicAdd(&s_c[1], cj); }
    __syncthreads();
    if (threadIdx.x == 0) cc[blockIdx.x] = make_uint2(s_c[0], s_c[1]);
}

/* step 2, one warp per piece: each chunk's counts before it within the piece, the piece's totals */
__global__ void k_blas_part_prefix(const uint2* __restrict__ pchunk, const uint32_t* __restrict__ rs, const uint2* __restrict__ cc,
                                   uint2* __restrict__ cpre, uint2* __restrict__ ptot, uint32_t* __restrict__ kc) {
    const uint32_t pi = blockIdx.x * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (pi >= rs[0]) return;
    const uint2 pc = pchunk[pi];
    uint32_t ri = 0, rj = 0;
    for (uint32_t base = 0; base < pc.y; base += 32) {
        const uint32_t k = base + lane;
        const uint2 v = k < pc.y ? cc[pc.x + k] : make_uint2(0, 0);
        uint32_t si = v.x, sj = v.y;
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t oi = __shfl_up_sync(0xffffffffu, si, d), oj = __shfl_up_sync(0xffffffffu, sj, d);
            if (lane >= (uint32_t)d) { si += oi; sj += oj; }
        }
        if (k < pc.y) cpre[pc.x + k] = make_uint2(ri + si - v.x, rj + sj - v.y);
        ri += __shfl_sync(0xffffffffu, si, 31); rj += __shfl_sync(0xffffffffu, sj, 31);
    }
    if (lane == 0) { ptot[pi] = make_uint2(ri, rj); kc[pi] = 0; }
}

/* step 3, per chunk: the rank of every stop (left stops counted from the piece's start, right
 * stops from its end), written as position lists Lp / Rp, and how many left stops are swapped */
__global__ void __launch_bounds__(BLAS_CHUNK_THREADS) k_blas_part_rank(const uint2* __restrict__ pieces, const uint4* __restrict__ chunks,
                                                                     const uint32_t* __restrict__ rs, const float* __restrict__ key,
                                                                     const uint2* __restrict__ cpre,
                                                                     const uint2* __restrict__ ptot, uint32_t* __restrict__ Lp,
                                                                     uint32_t* __restrict__ Rp, uint32_t* __restrict__ kc) {
    __shared__ uint32_t ws[BLAS_CHUNK_THREADS / 32];
    __shared__ uint32_t s_valid;
    if (blockIdx.x >= rs[1]) return;
    const uint4 c = chunks[blockIdx.x];
    const uint2 pc = pieces[c.x];
    const uint32_t s = pc.x, CJ = ptot[c.x].y;
    const float p = key[s + pc.y / 2];
    if (threadIdx.x == 0) s_valid = 0;
    const uint32_t x0 = c.y + threadIdx.x * BLAS_CHUNK_PER_THREAD, xe = c.y + c.z;
    uint32_t ni = 0, nj = 0;
    for (int e = 0; e < BLAS_CHUNK_PER_THREAD; e++) {
        const uint32_t x = x0 + e;
        if (x < xe) { const float k = key[s + x]; ni += !(k < p); nj += !(k > p); }
    }
    const uint32_t ex = block_excl_scan_256(ni | (nj << 16), ws);
    uint32_t r = cpre[blockIdx.x].x + (ex & 0xFFFFu), pj = cpre[blockIdx.x].y + (ex >> 16), valid = 0;
    for (int e = 0; e < BLAS_CHUNK_PER_THREAD; e++) {
        const uint32_t x = x0 + e;
        if (x >= xe) break;
        const float k = key[s + x];
        if (!(k < p)) { Lp[s + r] = x; valid += (r < CJ - pj); r++; }
        if (!(k > p)) { Rp[s + (CJ - 1 - pj)] = x; pj++; }
    }
    for (int d = 16; d > 0; d >>= 1) valid += __shfl_xor_sync(0xffffffffu, valid, d);
    if ((threadIdx.x & 31) == 0 && valid) atomicAdd(&s_valid, valid);
    __syncthreads();
    if (threadIdx.x == 0 && s_valid) atomicAdd(&kc[c.x], s_valid);
}

/* step 4: the k-th left stop swaps with the k-th right stop for k < K; chunk c takes the ranks
 * in its own position range */
__global__ void __launch_bounds__(BLAS_CHUNK_THREADS) k_blas_part_swap(const uint2* __restrict__ pieces, const uint4* __restrict__ chunks,
                                                                     const uint32_t* __restrict__ rs, const uint32_t* __restrict__ kc,
                                                                     const uint32_t* __restrict__ Lp, const uint32_t* __restrict__ Rp,
                                                                     float* __restrict__ key, uint32_t* __restrict__ perm) {
    if (blockIdx.x >= rs[1]) return;
    const uint4 c = chunks[blockIdx.x];
    const uint32_t s = pieces[c.x].x, K = kc[c.x];
    const uint32_t re = min(c.y + c.z, K);
    for (uint32_t r = c.y + threadIdx.x; r < re; r += BLAS_CHUNK_THREADS) {
        const uint32_t a = s + Lp[s + r], b = s + Rp[s + r];
        const float ka = key[a]; key[a] = key[b]; key[b] = ka;
        const uint32_t pa = perm[a]; perm[a] = perm[b]; perm[b] = pa;
    }
}

/* step 5, one thread per piece: where the scans end, and the parts left to sort: long parts with
 * their chunks to the next round's tables (counts in rs_next: pieces, chunks), the others to the
 * shared-memory sorter.  ctr: [0] overflow, [1] short pieces.  Each round's counts live on the
 * device, so rounds are launched without waiting for the host. */
__global__ void k_blas_part_children(const uint2* __restrict__ pieces, const uint32_t* __restrict__ rs, const uint2* __restrict__ ptot,
                                     const uint32_t* __restrict__ kc, const uint32_t* __restrict__ Lp, const uint32_t* __restrict__ Rp,
                                     uint2* __restrict__ next, uint2* __restrict__ next_pchunk, uint4* __restrict__ next_chunks,
                                     uint32_t list_cap, uint32_t chunk_cap, uint2* __restrict__ small, uint32_t small_cap,
                                     uint32_t* __restrict__ rs_next, uint32_t* __restrict__ ctr) {
    const uint32_t pi = blockIdx.x * blockDim.x + threadIdx.x;
    if (pi >= rs[0]) return;
    const uint32_t s = pieces[pi].x, m = pieces[pi].y, K = kc[pi], CI = ptot[pi].x, CJ = ptot[pi].y;
    if (K == 0 || K > CI || K > CJ) { atomicOr(&ctr[0], 1u); return; }
    int i, j;
    final_ij((int)Lp[s + K - 1], (int)Rp[s + K - 1], K < CI ? (int)Lp[s + K] : 0x7fffffff, K < CJ ? (int)Rp[s + K] : -1, i, j);
    const uint32_t ps[2] = { s, s + (uint32_t)i };
    const int pm[2] = { j + 1, (int)m - i };
    for (int h = 0; h < 2; h++) {
        if (pm[h] < 2) continue;
        const uint32_t len = (uint32_t)pm[h];
        if (len > BLAS_CAP) {
            const uint32_t k = atomicAdd(&rs_next[0], 1u);
            const uint32_t nc = (len + BLAS_CHUNK - 1) / BLAS_CHUNK;
            const uint32_t base = atomicAdd(&rs_next[1], nc);
            if (k >= list_cap || base + nc > chunk_cap) { atomicOr(&ctr[0], 1u); continue; }
            next[k] = make_uint2(ps[h], len);
            next_pchunk[k] = make_uint2(base, nc);
            for (uint32_t q = 0; q < nc; q++) next_chunks[base + q] = make_uint4(k, q * BLAS_CHUNK, min(BLAS_CHUNK, len - q * BLAS_CHUNK), 0);
        } else {
            const uint32_t k = atomicAdd(&ctr[1], 1u);
            if (k < small_cap) small[k] = make_uint2(ps[h], len); else atomicOr(&ctr[0], 1u);
        }
    }
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

/* The reference's quicksort itself (sofren2.c:2895-2924) on [s, s + m) of the shared-memory arrays, by
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

/* The whole CTA partitions the piece [s, s + m) of the shared-memory arrays (m > BLAS_CTA_PIECE):
 * the same stop ranks as warp_partition, with one block scan over contiguous runs of positions.
 * Returns i, j (relative) in s_ij; every thread takes part. */
__device__ __forceinline__ void cta_partition(float* Ks, uint32_t* Ps, uint16_t* Lp, uint16_t* Rp, int s, int m, uint32_t* ws,
                                              uint32_t* s_tot, int* s_ij) {
    const float p = Ks[s + m / 2];
    const int E = (m + BLAS_SMALL_THREADS - 1) / BLAS_SMALL_THREADS;
    const int x0 = (int)threadIdx.x * E, xe = min(x0 + E, m);
    uint32_t ni = 0, nj = 0;
    for (int x = x0; x < xe; x++) { const float k = Ks[s + x]; ni += !(k < p); nj += !(k > p); }
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t v = ni | (nj << 16);
    uint32_t sc = v;
    for (int d = 1; d < 32; d <<= 1) { const uint32_t o = __shfl_up_sync(0xffffffffu, sc, d); if (lane >= (uint32_t)d) sc += o; }
    if (lane == 31) ws[w] = sc;
    if (threadIdx.x == 0) s_tot[0] = 0;
    __syncthreads();
    uint32_t before = 0, all = 0;
    for (uint32_t k = 0; k < BLAS_SMALL_WARPS; k++) { if (k < w) before += ws[k]; all += ws[k]; }
    const uint32_t ex = before + sc - v;
    const int CI = (int)(all & 0xFFFFu), CJ = (int)(all >> 16);
    int r = (int)(ex & 0xFFFFu), pj = (int)(ex >> 16);
    uint32_t valid = 0;
    for (int x = x0; x < xe; x++) {
        const float k = Ks[s + x];
        if (!(k < p)) { Lp[s + r] = (uint16_t)(s + x); valid += (r < CJ - pj); r++; }
        if (!(k > p)) { Rp[s + CJ - 1 - pj] = (uint16_t)(s + x); pj++; }
    }
    valid = __reduce_add_sync(0xffffffffu, valid);
    if (lane == 0 && valid) atomicAdd(&s_tot[0], valid);
    __syncthreads();
    const int K = (int)s_tot[0];
    for (int q = (int)threadIdx.x; q < K; q += BLAS_SMALL_THREADS) {
        const int a = Lp[s + q], b = Rp[s + q];
        const float ka = Ks[a]; Ks[a] = Ks[b]; Ks[b] = ka;
        const uint32_t pa = Ps[a]; Ps[a] = Ps[b]; Ps[b] = pa;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int i, j;
        final_ij((int)Lp[s + K - 1] - s, (int)Rp[s + K - 1] - s, K < CI ? (int)Lp[s + K] - s : 0x7fffffff, K < CJ ? (int)Rp[s + K] - s : -1, i, j);
        s_ij[0] = i; s_ij[1] = j;
    }
    __syncthreads();
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
    __shared__ float sbnd[BLAS_SMALL_WARPS][6];
    __shared__ int s_axis;
    __shared__ uint32_t bigq[BLAS_BIGQ], ws[BLAS_SMALL_WARPS], s_tot[1];
    __shared__ int nbig, s_ij[2];
    if (blockIdx.x >= nspans) return;
    uint32_t s0, m0;
    if (PLAN) { s0 = spans[blockIdx.x].x; m0 = spans[blockIdx.x].y; }
    else { s0 = list[blockIdx.x].x; m0 = list[blockIdx.x].y; }
    if (m0 > BLAS_CAP) m0 = 0;   /* never planned; nothing is touched */
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint32_t x = threadIdx.x; x < m0; x += BLAS_SMALL_THREADS) Ps[x] = perm[s0 + x];
    if (!PLAN) for (uint32_t x = threadIdx.x; x < m0; x += BLAS_SMALL_THREADS) Ks[x] = key[s0 + x];
    if (threadIdx.x == 0) { ncnt[0] = 0; ncnt[1] = 0; ncnt[2] = 0; nbig = 0; }
    __syncthreads();
    if (PLAN) {
        const uint32_t t0 = spans[blockIdx.x].z, nt = spans[blockIdx.x].w;
        if (nt == 1) {   /* one range: the whole CTA gathers its bounds and keys */
            const uint2 tk = tasks[t0];
            const uint32_t ts = tk.x - s0, tc = tk.y;
            const bool ok = ts + tc <= m0 && tc >= 2;
            float lo[3] = { 1e30f, 1e30f, 1e30f }, hi[3] = { -1e30f, -1e30f, -1e30f };
            if (ok)
                for (uint32_t x = threadIdx.x; x < tc; x += BLAS_SMALL_THREADS) {
                    const uint32_t q = Ps[ts + x];
                    for (int a = 0; a < 3; a++) {
                        const float c = it[(size_t)(6 + a) * n + q];
                        if (c < lo[a]) lo[a] = c;
                        if (c > hi[a]) hi[a] = c;
                    }
                }
            warp_bounds(lo, hi);
            if (lane == 0) for (int a = 0; a < 3; a++) { sbnd[w][a] = lo[a]; sbnd[w][3 + a] = hi[a]; }
            __syncthreads();
            if (w == 0) {
                for (int a = 0; a < 3; a++) {
                    lo[a] = lane < BLAS_SMALL_WARPS ? sbnd[lane][a] : 1e30f;
                    hi[a] = lane < BLAS_SMALL_WARPS ? sbnd[lane][3 + a] : -1e30f;
                }
                warp_bounds(lo, hi);
                if (lane == 0) s_axis = pick_axis(lo, hi);
            }
            __syncthreads();
            if (ok) {
                const float* c = it + (size_t)(6 + s_axis) * n;
                for (uint32_t x = threadIdx.x; x < tc; x += BLAS_SMALL_THREADS) Ks[ts + x] = c[Ps[ts + x]];
                if (threadIdx.x == 0) {
                    if (tc > BLAS_CTA_PIECE) { bigq[0] = (ts << 16) | tc; nbig = 1; }
                    else { const int q = tc > BLAS_SEQ ? 0 : 2; (q ? seq : lst0)[0] = (ts << 16) | tc; ncnt[q] = 1; }
                }
            }
        } else {
            for (uint32_t t = w; t < nt; t += BLAS_SMALL_WARPS) {
                const uint2 tk = tasks[t0 + t];
                const uint32_t ts = tk.x - s0, tc = tk.y;
                if (ts + tc > m0 || tc < 2) continue;
                float lo[3] = { 1e30f, 1e30f, 1e30f }, hi[3] = { -1e30f, -1e30f, -1e30f };
                for (uint32_t b = lane; b < tc; b += 128) {   /* four elements' loads in flight per lane */
                    uint32_t q[4];
                    float v[4][3];
#pragma unroll
                    for (int u = 0; u < 4; u++) q[u] = b + 32u * u < tc ? Ps[ts + b + 32u * u] : 0xFFFFFFFFu;
#pragma unroll
                    for (int u = 0; u < 4; u++)
                        for (int a = 0; a < 3; a++) v[u][a] = q[u] != 0xFFFFFFFFu ? it[(size_t)(6 + a) * n + q[u]] : 0.f;
#pragma unroll
                    for (int u = 0; u < 4; u++)
                        if (q[u] != 0xFFFFFFFFu)
                            for (int a = 0; a < 3; a++) {
                                if (v[u][a] < lo[a]) lo[a] = v[u][a];
                                if (v[u][a] > hi[a]) hi[a] = v[u][a];
                            }
                }
                warp_bounds(lo, hi);
                const float* c = it + (size_t)(6 + pick_axis(lo, hi)) * n;
                for (uint32_t b = lane; b < tc; b += 128) {
                    uint32_t q[4];
                    float v[4];
#pragma unroll
                    for (int u = 0; u < 4; u++) q[u] = b + 32u * u < tc ? Ps[ts + b + 32u * u] : 0xFFFFFFFFu;
#pragma unroll
                    for (int u = 0; u < 4; u++) v[u] = q[u] != 0xFFFFFFFFu ? c[q[u]] : 0.f;
#pragma unroll
                    for (int u = 0; u < 4; u++) if (q[u] != 0xFFFFFFFFu) Ks[ts + b + 32u * u] = v[u];
                }
                if (lane == 0) {
                    if (tc > BLAS_CTA_PIECE) {
                        const int k = atomicAdd(&nbig, 1);
                        if (k < BLAS_BIGQ) bigq[k] = (ts << 16) | tc;
                    } else {
                        const int q = tc > BLAS_SEQ ? 0 : 2;
                        const int k = atomicAdd(&ncnt[q], 1);
                        if (k < BLAS_CAP / 2) (q ? seq : lst0)[k] = (ts << 16) | tc;
                    }
                }
            }
        }
    } else if (threadIdx.x == 0 && m0 >= 2) {
        if (m0 > BLAS_CTA_PIECE) { bigq[0] = m0; nbig = 1; }
        else if (m0 > BLAS_SEQ) { lst0[0] = m0; ncnt[0] = 1; } else { seq[0] = m0; ncnt[2] = 1; }
    }
    /* long pieces first, one at a time by the whole CTA; their parts of at most BLAS_CTA_PIECE
     * positions go to the warp rounds (or straight to the one-thread finish) */
    for (;;) {
        __syncthreads();
        const int nb = min(nbig, BLAS_BIGQ);
        if (nb == 0) break;
        const uint32_t v = bigq[nb - 1];
        __syncthreads();
        if (threadIdx.x == 0) nbig = nb - 1;
        const int s = (int)(v >> 16), m = (int)(v & 0xFFFFu);
        cta_partition(Ks, Ps, Lp, Rp, s, m, ws, s_tot, s_ij);
        if (threadIdx.x == 0) {
            const int i = s_ij[0], j = s_ij[1];
            const uint32_t ps[2] = { (uint32_t)s, (uint32_t)(s + i) };
            const int pm[2] = { j + 1, m - i };
            for (int h = 0; h < 2; h++) {
                if (pm[h] < 2) continue;
                const uint32_t e = (ps[h] << 16) | (uint32_t)pm[h];
                if (pm[h] > BLAS_CTA_PIECE) { if (nbig < BLAS_BIGQ) bigq[nbig++] = e; }
                else if (pm[h] > BLAS_SEQ) { if (ncnt[0] < BLAS_CAP / 2) lst0[ncnt[0]++] = e; }
                else { if (ncnt[2] < BLAS_CAP / 2) seq[ncnt[2]++] = e; }
            }
        }
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
    blas_plan plan;                 /* the tree's shape for n items */
};

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
    blas_plan_build(J->plan, total);
    *n_items = total;
    *n_nodes = (uint32_t)J->plan.nodes.size();
    return cudaSuccess;
}

cudaError_t sftg_blas_finish(sftg_blas_job* J, sftg_bvh_node* dst, uint32_t* status) {
    *status = 0;
    const uint32_t n = J->n, nn = (uint32_t)J->plan.nodes.size();
    if (!n) return cudaSuccess;
    cudaStream_t st = J->st;
    /* tasks of every level, spans of the short ones, and the node plan, in one upload */
    std::vector<blas_range> tasks, big;
    std::vector<uint2> big_pchunk;
    std::vector<uint4> spans, big_chunks;
    std::vector<uint32_t> lv_task_off, lv_span_off, lv_span_cnt, lv_big_off, lv_big_cnt, lv_chunk_off, lv_chunk_cnt, lv_rounds;
    std::vector<uint32_t> lv_rs;   /* per level: the first round's piece and chunk counts */
    /* short ranges are packed into spans of about n / (3 x SMs) positions (three CTAs fit an SM),
     * so that deep levels of many small ranges still fill the GPU */
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t span_target = std::min<uint32_t>(BLAS_CAP, std::max<uint32_t>(256, n / (3u * (uint32_t)std::max(sms, 1))));
    for (size_t L = 0; L < J->plan.by_level.size(); L++) {
        const std::vector<blas_range>& T = J->plan.by_level[L];
        lv_task_off.push_back((uint32_t)tasks.size());
        lv_span_off.push_back((uint32_t)spans.size());
        lv_big_off.push_back((uint32_t)big.size());
        lv_chunk_off.push_back((uint32_t)big_chunks.size());
        const uint32_t t_base = (uint32_t)tasks.size();
        uint32_t k = 0;
        while (k < T.size()) {
            if (T[k].y > BLAS_CAP) {   /* a long range: its chunks, numbered within the level */
                const uint32_t pi = (uint32_t)big.size() - lv_big_off.back(), c0 = (uint32_t)big_chunks.size() - lv_chunk_off.back();
                const uint32_t nc = (T[k].y + BLAS_CHUNK - 1) / BLAS_CHUNK;
                for (uint32_t q = 0; q < nc; q++) big_chunks.push_back(make_uint4(pi, q * BLAS_CHUNK, std::min<uint32_t>(BLAS_CHUNK, T[k].y - q * BLAS_CHUNK), 0));
                big_pchunk.push_back(make_uint2(c0, nc));
                big.push_back(T[k]); k++; continue;
            }
            const uint32_t s0 = T[k].x;
            uint32_t e = k + 1;
            while (e < T.size() && T[e].y <= BLAS_CAP && T[e].x + T[e].y - s0 <= span_target) e++;
            spans.push_back(make_uint4(s0, T[e - 1].x + T[e - 1].y - s0, t_base + k, e - k));
            k = e;
        }
        tasks.insert(tasks.end(), T.begin(), T.end());
        lv_span_cnt.push_back((uint32_t)spans.size() - lv_span_off.back());
        lv_big_cnt.push_back((uint32_t)big.size() - lv_big_off.back());
        lv_chunk_cnt.push_back((uint32_t)big_chunks.size() - lv_chunk_off.back());
        lv_rs.push_back(lv_big_cnt.back()); lv_rs.push_back(lv_chunk_cnt.back());
        /* rounds until the longest range's parts fit if its pivots split evenly, and one more */
        uint32_t longest = 0, r = 1;
        for (const blas_range& t : T) longest = std::max(longest, t.y);
        while (longest > BLAS_CAP) { longest = (longest + 1) / 2; r++; }
        lv_rounds.push_back(r);
    }
    std::vector<uint32_t> depth_idx, depth_off;
    for (size_t d = 0; d < J->plan.by_depth.size(); d++) {
        depth_off.push_back((uint32_t)depth_idx.size());
        depth_idx.insert(depth_idx.end(), J->plan.by_depth[d].begin(), J->plan.by_depth[d].end());
    }
    const uint32_t list_cap = n / BLAS_CAP + 4, small_cap = n / 2 + 4, chunk_cap = n / BLAS_CHUNK + list_cap + 4;
    /* device scratch: items, ids, perm, key, Lp, Rp, bounds, lists, counters, plan */
    size_t o = 0;
    auto take = [&](size_t bytes) { const size_t r = o; o += (bytes + 255) & ~(size_t)255; return r; };
    const size_t o_it = take((size_t)n * 36), o_ids = take((size_t)n * 4), o_perm = take((size_t)n * 4), o_key = take((size_t)n * 4);
    const size_t o_lp = take((size_t)n * 4), o_rp = take((size_t)n * 4), o_bnd = take((size_t)nn * 24);
    const size_t o_l0 = take((size_t)list_cap * 8), o_l1 = take((size_t)list_cap * 8), o_sm = take((size_t)small_cap * 8);
    const size_t o_pc0 = take((size_t)list_cap * 8), o_pc1 = take((size_t)list_cap * 8);
    const size_t o_ch0 = take((size_t)chunk_cap * 16), o_ch1 = take((size_t)chunk_cap * 16);
    const size_t o_cc = take((size_t)chunk_cap * 8), o_cpre = take((size_t)chunk_cap * 8), o_part = take((size_t)chunk_cap * 24);
    const size_t o_ptot = take((size_t)list_cap * 8), o_kc = take((size_t)list_cap * 4), o_axis = take((size_t)list_cap);
    const size_t o_ctr = take(32);   /* round counts A, B; overflow; short pieces */
    const size_t o_tasks = take(tasks.size() * 8 + 8), o_spans = take(spans.size() * 16 + 16), o_big = take(big.size() * 8 + 8);
    const size_t o_bpc = take(big_pchunk.size() * 8 + 8), o_bch = take(big_chunks.size() * 16 + 16), o_lvrs = take(lv_rs.size() * 4 + 8);
    const size_t o_pn = take((size_t)nn * sizeof(blas_pnode)), o_didx = take(depth_idx.size() * 4 + 4);
    const size_t o_plan = o_tasks, plan_bytes = o - o_tasks;
    char* d = nullptr;
    BK(cudaMallocAsync((void**)&d, o, st));
    /* the plan goes up from a page-locked staging buffer kept per host thread; the previous
     * build's copy out of it finished when that build synchronised its stream */
    static thread_local char* stage = nullptr;
    static thread_local size_t stage_cap = 0;
    if (plan_bytes > stage_cap) {
        if (stage) cudaFreeHost(stage);
        stage = nullptr; stage_cap = 0;
        const size_t cap = plan_bytes + plan_bytes / 4;
        if (cudaMallocHost((void**)&stage, cap) != cudaSuccess) { cudaFreeAsync(d, st); return cudaErrorMemoryAllocation; }
        stage_cap = cap;
    }
    char* h = stage;
    memcpy(h + (o_tasks - o_plan), tasks.data(), tasks.size() * 8);
    memcpy(h + (o_spans - o_plan), spans.data(), spans.size() * 16);
    memcpy(h + (o_big - o_plan), big.data(), big.size() * 8);
    memcpy(h + (o_bpc - o_plan), big_pchunk.data(), big_pchunk.size() * 8);
    memcpy(h + (o_bch - o_plan), big_chunks.data(), big_chunks.size() * 16);
    memcpy(h + (o_lvrs - o_plan), lv_rs.data(), lv_rs.size() * 4);
    memcpy(h + (o_pn - o_plan), J->plan.nodes.data(), (size_t)nn * sizeof(blas_pnode));
    memcpy(h + (o_didx - o_plan), depth_idx.data(), depth_idx.size() * 4);
    cudaError_t err = cudaMemcpyAsync(d + o_plan, h, plan_bytes, cudaMemcpyHostToDevice, st);
    float* it = (float*)(d + o_it);
    uint32_t* ids = (uint32_t*)(d + o_ids);
    uint32_t* perm = (uint32_t*)(d + o_perm);
    float* key = (float*)(d + o_key);
    uint32_t* Lp = (uint32_t*)(d + o_lp);
    uint32_t* Rp = (uint32_t*)(d + o_rp);
    float* bnd = (float*)(d + o_bnd);
    uint2* lists[2] = { (uint2*)(d + o_l0), (uint2*)(d + o_l1) };
    uint2* pchs[2] = { (uint2*)(d + o_pc0), (uint2*)(d + o_pc1) };
    uint4* chs[2] = { (uint4*)(d + o_ch0), (uint4*)(d + o_ch1) };
    uint2* cc = (uint2*)(d + o_cc);
    uint2* cpre = (uint2*)(d + o_cpre);
    float* part = (float*)(d + o_part);
    uint2* ptot = (uint2*)(d + o_ptot);
    uint32_t* kc = (uint32_t*)(d + o_kc);
    uint8_t* axis = (uint8_t*)(d + o_axis);
    uint2* small = (uint2*)(d + o_sm);
    uint32_t* ctr = (uint32_t*)(d + o_ctr);
    const uint2* d_tasks = (const uint2*)(d + o_tasks);
    const uint4* d_spans = (const uint4*)(d + o_spans);
    const uint2* d_big = (const uint2*)(d + o_big);
    const uint2* d_bpc = (const uint2*)(d + o_bpc);
    const uint4* d_bch = (const uint4*)(d + o_bch);
    const uint32_t* d_lvrs = (const uint32_t*)(d + o_lvrs);
    uint32_t* rsb = ctr;              /* rsb[0..1], rsb[2..3]: pieces and chunks of a round */
    uint32_t* cst = ctr + 4;          /* cst[0] overflow, cst[1] short pieces */
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
    static thread_local uint32_t* h_ctr = nullptr;   /* pinned read-back of the round state */
    if (err == cudaSuccess && !h_ctr) err = cudaMallocHost((void**)&h_ctr, 32);
    for (size_t L = 0; err == cudaSuccess && L < J->plan.by_level.size(); L++) {
        if (lv_span_cnt[L]) {
            k_blas_sort_small<true><<<lv_span_cnt[L], BLAS_SMALL_THREADS, BLAS_SMALL_SMEM, st>>>(d_spans + lv_span_off[L], nullptr, lv_span_cnt[L],
                                                                                                 d_tasks, it, n, key, perm);
            J->launches++;
        }
        if (lv_big_cnt[L]) {   /* long ranges: axis and keys, then partition rounds until every part fits */
            const uint2* cur_p = d_big + lv_big_off[L];
            const uint2* cur_pc = d_bpc + lv_big_off[L];
            const uint4* cur_c = d_bch + lv_chunk_off[L];
            const uint32_t np = lv_big_cnt[L], nch = lv_chunk_cnt[L];
            k_blas_chunk_bounds<<<nch, BLAS_CHUNK_THREADS, 0, st>>>(cur_p, cur_c, nch, it, n, perm, part);
            k_blas_range_axis<<<(np + 3) / 4, 128, 0, st>>>(cur_pc, np, part, axis);
            k_blas_chunk_keys<<<nch, BLAS_CHUNK_THREADS, 0, st>>>(cur_p, cur_c, nch, axis, it, n, perm, key);
            J->launches += 3;
            err = cudaMemsetAsync(ctr, 0, 32, st);
            const uint32_t* rs_cur = d_lvrs + 2 * L;
            const uint32_t grid_ch = chunk_cap, grid_p4 = (list_cap + 3) / 4, grid_p128 = (list_cap + 127) / 128;
            uint32_t k = 0, rounds = lv_rounds[L];
            while (err == cudaSuccess) {
                for (uint32_t q = 0; q < rounds && err == cudaSuccess; q++, k++) {
                    uint32_t* rs_next = rsb + 2 * (k & 1);
                    if ((err = cudaMemsetAsync(rs_next, 0, 8, st)) != cudaSuccess) break;
                    k_blas_part_count<<<grid_ch, BLAS_CHUNK_THREADS, 0, st>>>(cur_p, cur_c, rs_cur, key, cc);
                    k_blas_part_prefix<<<grid_p4, 128, 0, st>>>(cur_pc, rs_cur, cc, cpre, ptot, kc);
                    k_blas_part_rank<<<grid_ch, BLAS_CHUNK_THREADS, 0, st>>>(cur_p, cur_c, rs_cur, key, cpre, ptot, Lp, Rp, kc);
                    k_blas_part_swap<<<grid_ch, BLAS_CHUNK_THREADS, 0, st>>>(cur_p, cur_c, rs_cur, kc, Lp, Rp, key, perm);
                    k_blas_part_children<<<grid_p128, 128, 0, st>>>(cur_p, rs_cur, ptot, kc, Lp, Rp, lists[k & 1], pchs[k & 1], chs[k & 1],
                                                                    list_cap, chunk_cap, small, small_cap, rs_next, cst);
                    J->launches += 5;
                    err = cudaGetLastError();
                    rs_cur = rs_next; cur_p = lists[k & 1]; cur_pc = pchs[k & 1]; cur_c = chs[k & 1];
                }
                if (err != cudaSuccess) break;
                /* one read-back per level (more only if its ranges split unevenly) */
                if ((err = cudaMemcpyAsync(h_ctr, ctr, 24, cudaMemcpyDeviceToHost, st)) != cudaSuccess) break;
                if ((err = cudaStreamSynchronize(st)) != cudaSuccess) break;
                const uint32_t* hrs = h_ctr + 2 * ((k - 1) & 1);
                if (h_ctr[4] || hrs[0] > list_cap || hrs[1] > chunk_cap) { *status = 1; break; }
                if (hrs[0] == 0) break;
                rounds = 2;
            }
            if (err != cudaSuccess || *status) break;
            const uint32_t ns = h_ctr[5] < small_cap ? h_ctr[5] : 0;
            if (ns) {
                k_blas_sort_small<false><<<ns, BLAS_SMALL_THREADS, BLAS_SMALL_SMEM, st>>>(nullptr, small, ns, nullptr, it, n, key, perm);
                J->launches++;
            }
        }
        if (err == cudaSuccess) err = cudaGetLastError();
    }
    for (size_t dd = J->plan.by_depth.size(); err == cudaSuccess && !*status && dd-- > 0;) {
        const uint32_t cnt = (uint32_t)J->plan.by_depth[dd].size();
        k_blas_nodes<<<(cnt + 127) / 128, 128, 0, st>>>(d_pn, d_didx + depth_off[dd], cnt, it, ids, perm, n, bnd, dst);
        err = cudaGetLastError();
        J->launches++;
    }
    const cudaError_t se = cudaStreamSynchronize(st);   /* also on error: the staged plan is reused */
    if (err == cudaSuccess) err = se;
    cudaFreeAsync(d, st);
    return err;
}

uint32_t sftg_blas_launches(const sftg_blas_job* J) { return J ? J->launches : 0; }

void sftg_blas_end(sftg_blas_job* J) {
    if (!J) return;
    if (J->d_cnt) cudaFreeAsync(J->d_cnt, J->st);
    delete J;
}
