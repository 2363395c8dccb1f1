/*
 * The shape of a BLAS (host code, no CUDA): sft__bvh_build_recursive (sofren2.c:2967-3062) over
 * sft__partition_to_8 (2926-2965) splits a node of more than 8 items by count (halves, quarters,
 * eighths; a part of one item stops early), so for n items the node numbering (depth-first,
 * children in order), every node's item range and the list of ranges sorted at each level follow
 * from n alone.  A range sorted at split depth d of a node at depth t sorts at level 3t + d; the
 * ranges of one level are disjoint and listed in increasing start order.  The device builder
 * (sftg_blas.cu) does the data-dependent steps over this plan.
 */
#pragma once
#include <cstdint>
#include <cstring>
#include <vector>

struct blas_range { uint32_t x, y; };   /* start, count: the layout of the device's uint2 */
static_assert(sizeof(blas_range) == 8, "blas_range must match uint2");

struct blas_pnode {                     /* a node of the plan */
    uint32_t start, count;              /* item range; a leaf when count <= 8 */
    uint32_t nchild;
    uint32_t child[8];
};

struct blas_plan {
    std::vector<blas_pnode> nodes;                  /* in the reference's node order */
    std::vector<std::vector<uint32_t>> by_depth;    /* node indices per node depth */
    std::vector<std::vector<blas_range>> by_level;  /* sorted ranges per sort level */
};

static inline void blas_plan_split(blas_plan& P, uint32_t start, uint32_t count, uint32_t d, uint32_t level, uint32_t* st, uint32_t* cn,
                                   uint32_t& ng) {
    if (!count) return;
    if (d == 3 || count == 1) { st[ng] = start; cn[ng] = count; ng++; return; }
    if (P.by_level.size() <= level + d) P.by_level.resize(level + d + 1);
    P.by_level[level + d].push_back(blas_range{ start, count });
    const uint32_t mid = count / 2;
    blas_plan_split(P, start, mid, d + 1, level, st, cn, ng);
    blas_plan_split(P, start + mid, count - mid, d + 1, level, st, cn, ng);
}

static inline uint32_t blas_plan_node(blas_plan& P, uint32_t start, uint32_t count, uint32_t depth) {
    const uint32_t ni = (uint32_t)P.nodes.size();
    blas_pnode p;
    memset(&p, 0, sizeof(p));
    p.start = start; p.count = count;
    for (int i = 0; i < 8; i++) p.child[i] = 0xFFFFFFFFu;
    P.nodes.push_back(p);
    if (P.by_depth.size() <= depth) P.by_depth.resize(depth + 1);
    P.by_depth[depth].push_back(ni);
    if (count <= 8) return ni;
    uint32_t st[8] = { 0 }, cn[8] = { 0 }, ng = 0;
    blas_plan_split(P, start, count, 0, 3 * depth, st, cn, ng);
    for (uint32_t c = 0; c < ng; c++) {
        const uint32_t ci = blas_plan_node(P, st[c], cn[c], depth + 1);
        P.nodes[ni].child[c] = ci;
    }
    P.nodes[ni].nchild = ng;
    return ni;
}

/* the plan for n items (none for n = 0) */
static inline void blas_plan_build(blas_plan& P, uint32_t n) {
    P.nodes.clear(); P.by_depth.clear(); P.by_level.clear();
    if (!n) return;
    P.nodes.reserve(n / 3 + 16);
    blas_plan_node(P, 0, n, 0);
}
