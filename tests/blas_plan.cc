/* Dumps the BLAS shape plan (sofren2_gb300/csrc/sftg_blas_plan.h) for each item count given on
 * the command line: per count, u32 node count, u32 level count, the nodes (start, count, nchild,
 * child[8], 11 u32 each), then per level u32 range count and the ranges (start, count). */
#include <cstdio>
#include <cstdlib>
#include "sftg_blas_plan.h"

int main(int argc, char** argv) {
    if (argc < 3) { fprintf(stderr, "usage: %s out.bin count...\n", argv[0]); return 2; }
    FILE* f = fopen(argv[1], "wb");
    if (!f) return 3;
    for (int a = 2; a < argc; a++) {
        blas_plan P;
        blas_plan_build(P, (uint32_t)strtoul(argv[a], nullptr, 10));
        const uint32_t nn = (uint32_t)P.nodes.size(), nl = (uint32_t)P.by_level.size();
        fwrite(&nn, 4, 1, f); fwrite(&nl, 4, 1, f);
        for (const blas_pnode& n : P.nodes) fwrite(&n, sizeof(n), 1, f);
        for (const auto& L : P.by_level) {
            const uint32_t c = (uint32_t)L.size();
            fwrite(&c, 4, 1, f);
            fwrite(L.data(), sizeof(blas_range), L.size(), f);
        }
    }
    fclose(f);
    return 0;
}
