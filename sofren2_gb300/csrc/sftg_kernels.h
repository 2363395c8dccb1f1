/* Device-side records exchanged between the render-path kernels, and the kernel entry points. */
#pragma once
#include <stdint.h>
#include "sftg_types.h"

/* one 8-triangle batch of a drawn meshlet after setup (sofren2.c:4775-4884) */
struct __align__(16) sftg_batch_rec {
    uint64_t payload;      /* inst | meshlet << 24 | batch << 48 | lane mask << 56; 0 = nothing binned */
    int16_t x0, x1, y0, y1;/* tile rectangle (inclusive, unclamped) */
};

/* sft_clipped_triangle (sofren2.c:1271-1280), same field order */
struct sftg_clip_tri {
    float sx[3], sy[3], iw[3], u[3], v[3], lu[3], lv[3], px[3], py[3], pz[3], nx[3], ny[3], nz[3];
    uint32_t inst, m;
};

__global__ void k_geometry(const sftg_frame* F, float* ss, sftg_batch_rec* recs, uint32_t* clip_cnt, int4* mrect);
__global__ void k_clip(const sftg_frame* F, const float* ss, const uint32_t* clip_cnt, const uint32_t* clip_base,
                       sftg_clip_tri* clips, int4* clip_rect, int4* mrect, uint32_t n_records);
__global__ void k_bin(const sftg_frame* F, const sftg_batch_rec* recs, const uint32_t* clip_cnt, const uint32_t* clip_base,
                      const int4* clip_rect, const int4* mrect, uint32_t* tile_count, const uint32_t* tile_start, uint64_t* tile_pay);
__global__ void k_scan_reduce(const uint32_t* in, uint32_t n, uint32_t* sums);
__global__ void k_scan_top(uint32_t* sums, uint32_t nb, uint32_t* total_out);
__global__ void k_scan_down(const uint32_t* in, uint32_t n, const uint32_t* sums, uint32_t* out);
size_t sftg_packet_bytes();
void sftg_launch_occlusion(const sftg_frame* F, uint32_t n_point, uint32_t n_proxies, uint32_t n_inst, void* packets, uint2* pairs,
                           uint32_t* n_pairs, uint32_t max_pairs, uint8_t* light_vis, uint32_t* status, cudaStream_t st);
cudaError_t sftg_tile_configure(int max_dynamic_smem);
void sftg_launch_tile(int S, int tiles, cudaStream_t st, const sftg_frame* F, const float* ss, const sftg_clip_tri* clips,
                      const uint32_t* tile_start, const uint32_t* tile_count, const uint64_t* tile_pay, const uint8_t* light_vis,
                      float2* vis, float2* zrange, uint32_t* color, float* vis_depth, uint32_t* vis_id, float* shadow_out,
                      cudaEvent_t between);

#define SFTG_SCAN_ELEMS_PER_BLOCK 4096
