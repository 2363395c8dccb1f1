/*
 * The sftg C ABI: context, device memory and the per-frame launch sequence.
 *
 * Device memory.  Resident assets live in growable device pools (texel heap, texture and
 * material tables, meshlet pool, skin pool, BLAS node pool, model table).  Everything a frame
 * needs beyond that comes from one device bump arena that is reset per frame (the
 * reference's per-frame mmap arenas, sofren2.c:9456-9564); it grows between frames when a
 * frame needs more and never inside one.
 *
 * Frame sequence (sft_present, sofren2.c:8139-8289), replayed as one CUDA graph per layout:
 *   1. one H2D copy of the frame block: constants, instances, bones, jobs, lights, proxies, TLAS
 *   2. k_occl_*           light visibility of every shadow proxy (8163-8280), on a second
 *                         stream beside steps 3-5, joined before the resolve
 *   3. k_geometry         cull, skin, transform, project, batch setup (4901-5145)
 *   4. scan + k_clip      near-plane clipping in emission order (4691-4772)
 *   5. k_bin (count), scan, k_bin (write), tile order   per-tile payload lists (4619-4688)
 *   6. k_raster, k_resolve  per-tile raster into a shared-memory visibility buffer, then
 *                         the resolve, several CTAs per tile (6756-6813)
 *   7. D2H of the colour buffer into the caller's pitch
 */
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <vector>
#include <chrono>

#include "../../include/sftg.h"
#include "sftg_types.h"
#include "sftg_kernels.h"

#define TILE_THREADS 256
#define SETUP_CAP 256

struct dpool {   /* growable device buffer */
    void* ptr = nullptr;
    size_t size = 0, cap = 0;
};

/* One submission slot: its streams, phase events, frame arena, pinned staging, colour pool and
 * the cached graph of its last batch layout.  Lane 0 serves the synchronous calls; lanes 1 and
 * up serve sftg_frames_submit, so that batches on different lanes overlap on the GPU. */
struct sftg_lane {
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;            /* proxy occlusion runs here, beside geometry, binning and raster */
    cudaStream_t stream3 = nullptr;            /* the 1x and 2x tile ranges of raster and resolve, beside the 4x range */
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_geo = nullptr, ev_done = nullptr;
    cudaEvent_t ev_split[2] = { nullptr, nullptr }, ev_merge[2] = { nullptr, nullptr };
    cudaEvent_t ev[6] = { nullptr, nullptr, nullptr, nullptr, nullptr, nullptr };
    void* arena = nullptr;
    size_t arena_cap = 0;
    void* h_stage = nullptr;     /* pinned staging for the frame block */
    size_t h_stage_cap = 0;
    uint32_t* h_status = nullptr;
    uint32_t* d_color = nullptr;
    size_t d_color_cap = 0;
    /* the last batch's launch sequence as an instantiated CUDA graph, replayed while the
     * batch layout (every pointer, count and knob the launches take) stays the same */
    cudaGraphExec_t graph = nullptr;
    uint64_t graph_key = 0;
    uint64_t seen_key = 0;       /* layout of the previous batch: a graph is captured when it repeats */
    int graph_launches = 0;
    float timings[5] = { 0, 0, 0, 0, 0 };
    int launches = 0;
    /* a batch in flight (sftg_frames_submit): what sftg_lane_wait needs to finish it */
    bool busy = false;
    const sftg_frame_desc* fds = nullptr;
    uint32_t nv = 0;
    std::vector<uint32_t*> colors;
    std::vector<int32_t> pitch;
};

struct sftg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;             /* lane 0's stream: uploads and the synchronous calls */
    cudaEvent_t ev_upload = nullptr;           /* orders other lanes after the uploads queued before them */
    sftg_lane lanes[SFTG_MAX_LANES];
    /* the lanes' frame arenas and colour buffers: stream-ordered allocations from this pool, so
     * that a lane outgrowing its buffers frees and allocates on its own stream without
     * synchronising the device (cudaFree would wait for every lane's batch in flight); freed
     * blocks stay reserved in the pool for the next growth */
    cudaMemPool_t lane_pool = nullptr;
    std::vector<void*> retired_stage;          /* outgrown pinned staging: freed at sftg_destroy (cudaFreeHost synchronises) */
    char err[512] = { 0 };
    /* resident */
    dpool texels, texs, mats, ml_attr, ml_inds, ml_cull, ml_info, skin_j, skin_w, blas, models;
    std::vector<sftg_tex> h_texs;
    std::vector<sftg_mat> h_mats;
    std::vector<sftg_model> h_models;
    std::vector<uint32_t> h_model_skinned;   /* per model: has skinned meshes */
    std::vector<std::vector<uint8_t>> h_mesh_skinned;  /* per model, per mesh */
    std::vector<std::vector<uint32_t>> h_mesh_first;   /* per model, per mesh: first meshlet */
    std::vector<std::vector<uint32_t>> h_mesh_count;
    /* per model: its geometry jobs for one instance (inst and view 0, skinned = the mesh has
     * skin), built for job width tmpl_jw and the model's pool base; rebuilt when either changes */
    struct job_tmpl { uint32_t jw = 0, meshlet_base = ~0u, total = ~0u; std::vector<sftg_job> jobs; };
    std::vector<job_tmpl> h_job_tmpl;
    std::vector<sftg_job> tmp_jobs;
    uint32_t n_meshlets = 0, n_skin = 0, n_blas = 0;
    bool tables_dirty = true;
    /* per frame: capacities shared by the lanes (they only grow), the last finished batch's figures */
    uint64_t tile_cap = 1u << 20, clip_cap = 1u << 16, stile_cap = 1u << 18;
    float timings[5] = { 0, 0, 0, 0, 0 };
    int launches = 0;
    uint64_t launch_total = 0;                 /* kernels of every finished batch, on all lanes */
    double blas_ms = 0.0, blas_stream_ms = 0.0; /* last device BLAS build: wall time, upload-stream span */
    uint32_t blas_items = 0, blas_launches = 0; /* and its triangles and kernels */
    cudaEvent_t ev_blas[2] = { nullptr, nullptr };
    bool use_graphs = true;
    sftg_tuning tuning = { { 16, 8, 16 }, { 8, 8, 4 }, 1, 0, { 0, 0, 0 }, { 0, 0, 0 }, 0 };   /* measured best on the single-view workloads */
    /* transient models (one frame's dynamic meshes): pool marks where they start */
    bool tr_live = false, tr_pinned = false;
    uint32_t tr_meshlets = 0, tr_skin = 0, tr_blas = 0;
    size_t tr_models = 0;
    /* skeletons and animations (sftg_skeleton_upload) */
    dpool p_skels, p_bones, p_anims, p_samplers, p_channels, p_keys, p_order, p_levels, p_pose_io;
    dpool p_ray_io;                            /* staging of sftg_raycast */
    std::vector<sftg_skel_dev> h_skels;
    uint32_t n_bones = 0, n_anims = 0, n_samplers = 0, n_channels = 0, n_keys = 0, n_order = 0, n_levels = 0;
};

static int set_err(sftg_ctx* c, int code, const char* fmt, ...) {
    if (c) {
        va_list ap; va_start(ap, fmt);
        vsnprintf(c->err, sizeof(c->err), fmt, ap);
        va_end(ap);
    }
    return code;
}

#define CK(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return set_err(ctx, SFTG_E_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); } while (0)

/* Waits for every lane's work: resident pools are about to move or be overwritten. */
static int wait_lanes(sftg_ctx* ctx) {
    for (int l = 0; l < SFTG_MAX_LANES; l++)
        if (ctx->lanes[l].stream) CK(cudaStreamSynchronize(ctx->lanes[l].stream));
    return 0;
}

static int pool_reserve(sftg_ctx* ctx, dpool& p, size_t bytes) {
    if (bytes <= p.cap) return 0;
    if (int rc = wait_lanes(ctx)) return rc;
    size_t nc = p.cap ? p.cap : 1 << 20;
    while (nc < bytes) nc *= 2;
    void* np = nullptr;
    if (cudaMalloc(&np, nc) != cudaSuccess) return set_err(ctx, SFTG_E_NOMEM, "device pool growth to %zu bytes failed", nc);
    if (p.ptr) {
        CK(cudaMemcpyAsync(np, p.ptr, p.size, cudaMemcpyDeviceToDevice, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
        cudaFree(p.ptr);
    }
    p.ptr = np; p.cap = nc;
    ctx->tables_dirty = true;
    return 0;
}

static int pool_append(sftg_ctx* ctx, dpool& p, const void* src, size_t bytes, size_t* out_offset) {
    const size_t off = (p.size + 255) & ~(size_t)255;
    int rc = pool_reserve(ctx, p, off + bytes);
    if (rc) return rc;
    if (bytes) CK(cudaMemcpyAsync((char*)p.ptr + off, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    p.size = off + bytes;
    if (out_offset) *out_offset = off;
    return 0;
}

extern "C" void sftg_destroy(sftg_ctx* ctx);

static cudaError_t noalloc_scratch_setup(int device);

extern "C" int sftg_create(int device, sftg_ctx** out) {
    if (!out) return SFTG_E_ARG;
    sftg_ctx* ctx = new sftg_ctx();
    ctx->device = device;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= device) { delete ctx; return SFTG_E_CUDA; }
    if (cudaSetDevice(device) != cudaSuccess) { delete ctx; return SFTG_E_CUDA; }
    /* the occlusion stream gets the lowest priority: it only has to finish before the resolve, so
     * the critical-path kernels (geometry, binning, raster) take free SMs first */
    int prio_low = 0, prio_high = 0;
    cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    for (int l = 0; l < SFTG_MAX_LANES; l++) {
        sftg_lane& ln = ctx->lanes[l];
        if (cudaStreamCreateWithPriority(&ln.stream, cudaStreamNonBlocking, prio_high) != cudaSuccess ||
            cudaStreamCreateWithPriority(&ln.stream2, cudaStreamNonBlocking, prio_low) != cudaSuccess ||
            cudaStreamCreateWithPriority(&ln.stream3, cudaStreamNonBlocking, prio_high) != cudaSuccess) { sftg_destroy(ctx); return SFTG_E_CUDA; }
        for (int k = 0; k < 2; k++) {
            cudaEventCreateWithFlags(&ln.ev_split[k], cudaEventDisableTiming);
            cudaEventCreateWithFlags(&ln.ev_merge[k], cudaEventDisableTiming);
        }
        for (int i = 0; i < 6; i++) cudaEventCreate(&ln.ev[i]);
        cudaEventCreateWithFlags(&ln.ev_fork, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&ln.ev_join, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&ln.ev_done, cudaEventDisableTiming);
        cudaEventCreate(&ln.ev_geo);
        if (cudaMallocHost((void**)&ln.h_status, 64) != cudaSuccess) { sftg_destroy(ctx); return SFTG_E_CUDA; }
    }
    ctx->stream = ctx->lanes[0].stream;
    cudaEventCreateWithFlags(&ctx->ev_upload, cudaEventDisableTiming);
    {
        cudaMemPoolProps pp;
        memset(&pp, 0, sizeof(pp));
        pp.allocType = cudaMemAllocationTypePinned;
        pp.location.type = cudaMemLocationTypeDevice;
        pp.location.id = device;
        if (cudaMemPoolCreate(&ctx->lane_pool, &pp) != cudaSuccess) { ctx->lane_pool = nullptr; sftg_destroy(ctx); return SFTG_E_CUDA; }
        uint64_t keep = ~0ull;
        cudaMemPoolSetAttribute(ctx->lane_pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    sftg_tile_configure(227 * 1024);
    if (noalloc_scratch_setup(device) != cudaSuccess) { sftg_destroy(ctx); return SFTG_E_CUDA; }
    { const char* e = getenv("SFTG_NO_GRAPHS"); if (e && *e && *e != '0') ctx->use_graphs = false; }
    *out = ctx;
    return SFTG_OK;
}

extern "C" void sftg_destroy(sftg_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    for (int l = 0; l < SFTG_MAX_LANES; l++) if (ctx->lanes[l].stream) cudaStreamSynchronize(ctx->lanes[l].stream);
    dpool* pools[] = { &ctx->texels, &ctx->texs, &ctx->mats, &ctx->ml_attr, &ctx->ml_inds, &ctx->ml_cull, &ctx->ml_info,
                       &ctx->skin_j, &ctx->skin_w, &ctx->blas, &ctx->models, &ctx->p_skels, &ctx->p_bones, &ctx->p_anims,
                       &ctx->p_samplers, &ctx->p_channels, &ctx->p_keys, &ctx->p_order, &ctx->p_levels, &ctx->p_pose_io, &ctx->p_ray_io };
    for (dpool* p : pools) if (p->ptr) cudaFree(p->ptr);
    for (int l = 0; l < SFTG_MAX_LANES; l++) {
        sftg_lane& ln = ctx->lanes[l];
        if (ln.arena) cudaFree(ln.arena);
        if (ln.d_color) cudaFree(ln.d_color);
        ln.arena = nullptr; ln.d_color = nullptr;
        if (ln.h_stage) cudaFreeHost(ln.h_stage);
        if (ln.h_status) cudaFreeHost(ln.h_status);
        for (int i = 0; i < 6; i++) if (ln.ev[i]) cudaEventDestroy(ln.ev[i]);
        if (ln.graph) cudaGraphExecDestroy(ln.graph);
        if (ln.ev_fork) cudaEventDestroy(ln.ev_fork);
        if (ln.ev_join) cudaEventDestroy(ln.ev_join);
        if (ln.ev_done) cudaEventDestroy(ln.ev_done);
        if (ln.ev_geo) cudaEventDestroy(ln.ev_geo);
        if (ln.stream2) cudaStreamDestroy(ln.stream2);
        if (ln.stream3) cudaStreamDestroy(ln.stream3);
        for (int k = 0; k < 2; k++) {
            if (ln.ev_split[k]) cudaEventDestroy(ln.ev_split[k]);
            if (ln.ev_merge[k]) cudaEventDestroy(ln.ev_merge[k]);
        }
        if (ln.stream) cudaStreamDestroy(ln.stream);
    }
    if (ctx->ev_upload) cudaEventDestroy(ctx->ev_upload);
    for (void* p : ctx->retired_stage) cudaFreeHost(p);
    if (ctx->lane_pool) cudaMemPoolDestroy(ctx->lane_pool);
    for (int k = 0; k < 2; k++) if (ctx->ev_blas[k]) cudaEventDestroy(ctx->ev_blas[k]);
    delete ctx;
}

extern "C" const char* sftg_last_error(const sftg_ctx* ctx) { return ctx ? ctx->err : "no context"; }

extern "C" int sftg_texture_upload(sftg_ctx* ctx, const uint32_t* texels, uint64_t n_texels, const sftg_texture_desc* d, int32_t* out_index) {
    if (!ctx || !texels || !d || !out_index) return SFTG_E_ARG;
    CK(cudaSetDevice(ctx->device));
    size_t off = 0;
    int rc = pool_append(ctx, ctx->texels, texels, n_texels * 4, &off);
    if (rc) return rc;
    sftg_tex t;
    memset(&t, 0, sizeof(t));
    t.w = d->width; t.h = d->height; t.levels = d->levels; t.is_pot = d->is_pot;
    for (int i = 0; i < 14; i++) { t.offs[i] = (uint32_t)(off / 4) + d->level_offset[i]; t.bw[i] = d->blocks_w[i]; t.shift[i] = d->stride_shift[i]; }
    ctx->h_texs.push_back(t);
    ctx->tables_dirty = true;
    *out_index = (int32_t)ctx->h_texs.size() - 1;
    CK(cudaStreamSynchronize(ctx->stream));
    return SFTG_OK;
}

extern "C" int sftg_texture_update_desc(sftg_ctx* ctx, int32_t index, const sftg_texture_desc* d) {
    if (!ctx || index < 0 || (size_t)index >= ctx->h_texs.size()) return SFTG_E_ARG;
    if (!d) { ctx->h_texs[index].w = 0; }
    ctx->tables_dirty = true;
    return SFTG_OK;
}

extern "C" int sftg_material_set(sftg_ctx* ctx, int32_t index, int32_t texture, uint32_t base_color, float shininess) {
    if (!ctx || index < 0) return SFTG_E_ARG;
    if ((size_t)index >= ctx->h_mats.size()) ctx->h_mats.resize(index + 1);
    ctx->h_mats[index].tex = texture;
    ctx->h_mats[index].base_color = base_color;
    ctx->h_mats[index].shininess = shininess;
    ctx->tables_dirty = true;
    return SFTG_OK;
}

static int model_upload(sftg_ctx* ctx, const sftg_model_desc* d, int32_t* out_model, bool transient) {
    if (!ctx || !d || !out_model) return SFTG_E_ARG;
    CK(cudaSetDevice(ctx->device));
    if (transient && !ctx->tr_live) {   /* where the frame's transient models start */
        ctx->tr_live = true; ctx->tr_pinned = false;
        ctx->tr_meshlets = ctx->n_meshlets; ctx->tr_skin = ctx->n_skin; ctx->tr_blas = ctx->n_blas; ctx->tr_models = ctx->h_models.size();
    }
    if (!transient && ctx->tr_live) ctx->tr_pinned = true;   /* a resident model after them: they stay */
    uint32_t total = 0;
    for (uint32_t k = 0; k < d->mesh_count; k++) total += d->meshes[k].meshlet_count;
    std::vector<float> attr((size_t)total * 640), cull((size_t)total * 8);
    std::vector<uint8_t> inds((size_t)total * 512);
    std::vector<sftg_meshlet_info> info(total);
    std::vector<uint16_t> sj; std::vector<uint8_t> sw;
    std::vector<uint8_t> mesh_sk; std::vector<uint32_t> mesh_first, mesh_cnt;
    uint32_t o = 0, nskin = 0;
    for (uint32_t k = 0; k < d->mesh_count; k++) {
        const sftg_mesh_desc& m = d->meshes[k];
        const bool sk = m.joints && m.weights;
        mesh_sk.push_back(sk ? 1 : 0); mesh_first.push_back(o); mesh_cnt.push_back(m.meshlet_count);
        memcpy(&attr[(size_t)o * 640], m.attr, (size_t)m.meshlet_count * 640 * 4);
        memcpy(&inds[(size_t)o * 512], m.inds, (size_t)m.meshlet_count * 512);
        memcpy(&cull[(size_t)o * 8], m.cull, (size_t)m.meshlet_count * 32);
        for (uint32_t j = 0; j < m.meshlet_count; j++) {
            sftg_meshlet_info& in = info[o + j];
            in.material = m.material;
            in.lightmap_tex = m.lightmap_texture;
            in.culling_bone = (sk && m.culling_bones) ? m.culling_bones[j] : -1;
            in.skin_slot = sk ? (int32_t)(ctx->n_skin + nskin + j) : -1;
        }
        if (sk) {
            sj.insert(sj.end(), m.joints, m.joints + (size_t)m.meshlet_count * 256);
            sw.insert(sw.end(), m.weights, m.weights + (size_t)m.meshlet_count * 256);
            nskin += m.meshlet_count;
        }
        o += m.meshlet_count;
    }
    sftg_model md;
    memset(&md, 0, sizeof(md));
    md.meshlet_base = ctx->n_meshlets;
    md.total_meshlets = total;
    md.bone_count = d->bone_count;
    md.mesh_count = d->mesh_count;
    md.blas_base = ctx->n_blas; md.blas_root = d->blas_nodes ? d->blas_root : 0; md.blas_count = d->blas_nodes ? d->blas_count : 0;
    int rc;
    /* meshlet pools are indexed by meshlet, so they append at exact element offsets */
    if ((rc = pool_reserve(ctx, ctx->ml_attr, ((size_t)ctx->n_meshlets + total) * 2560))) return rc;
    if ((rc = pool_reserve(ctx, ctx->ml_inds, ((size_t)ctx->n_meshlets + total) * 512))) return rc;
    if ((rc = pool_reserve(ctx, ctx->ml_cull, ((size_t)ctx->n_meshlets + total) * 32))) return rc;
    if ((rc = pool_reserve(ctx, ctx->ml_info, ((size_t)ctx->n_meshlets + total) * sizeof(sftg_meshlet_info)))) return rc;
    CK(cudaMemcpyAsync((char*)ctx->ml_attr.ptr + (size_t)ctx->n_meshlets * 2560, attr.data(), (size_t)total * 2560, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync((char*)ctx->ml_inds.ptr + (size_t)ctx->n_meshlets * 512, inds.data(), (size_t)total * 512, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync((char*)ctx->ml_cull.ptr + (size_t)ctx->n_meshlets * 32, cull.data(), (size_t)total * 32, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync((char*)ctx->ml_info.ptr + (size_t)ctx->n_meshlets * sizeof(sftg_meshlet_info), info.data(), (size_t)total * sizeof(sftg_meshlet_info), cudaMemcpyHostToDevice, ctx->stream));
    /* sizes must track the filled bytes: a later growth copies exactly `size` bytes */
    ctx->ml_attr.size = ((size_t)ctx->n_meshlets + total) * 2560;
    ctx->ml_inds.size = ((size_t)ctx->n_meshlets + total) * 512;
    ctx->ml_cull.size = ((size_t)ctx->n_meshlets + total) * 32;
    ctx->ml_info.size = ((size_t)ctx->n_meshlets + total) * sizeof(sftg_meshlet_info);
    if (nskin) {
        if ((rc = pool_reserve(ctx, ctx->skin_j, ((size_t)ctx->n_skin + nskin) * 512))) return rc;
        if ((rc = pool_reserve(ctx, ctx->skin_w, ((size_t)ctx->n_skin + nskin) * 256))) return rc;
        CK(cudaMemcpyAsync((char*)ctx->skin_j.ptr + (size_t)ctx->n_skin * 512, sj.data(), (size_t)nskin * 512, cudaMemcpyHostToDevice, ctx->stream));
        CK(cudaMemcpyAsync((char*)ctx->skin_w.ptr + (size_t)ctx->n_skin * 256, sw.data(), (size_t)nskin * 256, cudaMemcpyHostToDevice, ctx->stream));
        ctx->skin_j.size = ((size_t)ctx->n_skin + nskin) * 512;
        ctx->skin_w.size = ((size_t)ctx->n_skin + nskin) * 256;
    }
    if (d->blas_count && d->blas_nodes) {
        if ((rc = pool_reserve(ctx, ctx->blas, ((size_t)ctx->n_blas + d->blas_count) * 256))) return rc;
        CK(cudaMemcpyAsync((char*)ctx->blas.ptr + (size_t)ctx->n_blas * 256, d->blas_nodes, (size_t)d->blas_count * 256, cudaMemcpyHostToDevice, ctx->stream));
        ctx->blas.size = ((size_t)ctx->n_blas + d->blas_count) * 256;
    } else if (d->build_blas && total) {   /* built from the meshlets just uploaded */
        md.blas_count = 0; md.blas_root = 0;
        sftg_blas_job* job = nullptr;
        uint32_t n_items = 0, n_nodes = 0, status = 0;
        for (int k = 0; k < 2; k++) if (!ctx->ev_blas[k]) CK(cudaEventCreate(&ctx->ev_blas[k]));
        CK(cudaStreamSynchronize(ctx->stream));   /* the meshlets are in place */
        const auto t0 = std::chrono::steady_clock::now();
        CK(cudaEventRecord(ctx->ev_blas[0], ctx->stream));
        cudaError_t e = sftg_blas_begin(&job, (const float*)((const char*)ctx->ml_attr.ptr + (size_t)ctx->n_meshlets * 2560),
                                        (const uint8_t*)ctx->ml_inds.ptr + (size_t)ctx->n_meshlets * 512, total, ctx->stream, &n_items, &n_nodes);
        if (e == cudaSuccess && n_nodes) {
            if ((rc = pool_reserve(ctx, ctx->blas, ((size_t)ctx->n_blas + n_nodes) * 256))) { sftg_blas_end(job); return rc; }
            e = sftg_blas_finish(job, (sftg_bvh_node*)((char*)ctx->blas.ptr + (size_t)ctx->n_blas * 256), &status);
            if (e == cudaSuccess && !status) {
                ctx->blas.size = ((size_t)ctx->n_blas + n_nodes) * 256;
                md.blas_count = n_nodes;
            }
        }
        ctx->blas_launches = sftg_blas_launches(job);
        sftg_blas_end(job);
        float ev_ms = 0.f;
        if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_blas[1], ctx->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(ctx->ev_blas[1]);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ev_ms, ctx->ev_blas[0], ctx->ev_blas[1]);
        ctx->blas_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        ctx->blas_stream_ms = ev_ms;
        ctx->blas_items = n_items;
        if (e != cudaSuccess) return set_err(ctx, SFTG_E_CUDA, "BLAS build: %s", cudaGetErrorString(e));
        if (status) return set_err(ctx, SFTG_E_DEVICE_STATUS, "BLAS build: a device work list overflowed");
    }
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->n_meshlets += total; ctx->n_skin += nskin; ctx->n_blas += md.blas_count;
    ctx->h_models.push_back(md);
    if (ctx->h_job_tmpl.size() >= ctx->h_models.size()) ctx->h_job_tmpl[ctx->h_models.size() - 1].jw = 0;   /* id reused */
    ctx->h_mesh_skinned.push_back(mesh_sk);
    ctx->h_mesh_first.push_back(mesh_first);
    ctx->h_mesh_count.push_back(mesh_cnt);
    ctx->tables_dirty = true;
    *out_model = (int32_t)ctx->h_models.size() - 1;
    return SFTG_OK;
}

extern "C" int sftg_model_upload(sftg_ctx* ctx, const sftg_model_desc* d, int32_t* out_model) {
    return model_upload(ctx, d, out_model, false);
}

extern "C" int sftg_model_blas(sftg_ctx* ctx, int32_t model, uint32_t first, uint32_t count, void* dst, uint32_t* out_count, uint32_t* out_root) {
    if (!ctx || model < 0 || (size_t)model >= ctx->h_models.size()) return SFTG_E_ARG;
    const sftg_model& md = ctx->h_models[model];
    if (out_count) *out_count = md.blas_count;
    if (out_root) *out_root = md.blas_root;
    if (!dst || !count) return SFTG_OK;
    if (first > md.blas_count || count > md.blas_count - first)
        return set_err(ctx, SFTG_E_ARG, "nodes %u..%u of a BLAS of %u", first, first + count, md.blas_count);
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(dst, (const char*)ctx->blas.ptr + ((size_t)md.blas_base + first) * 256, (size_t)count * 256, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SFTG_OK;
}

extern "C" int sftg_model_upload_transient(sftg_ctx* ctx, const sftg_model_desc* d, int32_t* out_model) {
    return model_upload(ctx, d, out_model, true);
}

extern "C" void sftg_transient_reset(sftg_ctx* ctx) {
    if (!ctx || !ctx->tr_live) return;
    if (!ctx->tr_pinned) {   /* drop the transient tail of every pool and table */
        wait_lanes(ctx);     /* a lane in flight may still read it */
        ctx->n_meshlets = ctx->tr_meshlets; ctx->n_skin = ctx->tr_skin; ctx->n_blas = ctx->tr_blas;
        ctx->h_models.resize(ctx->tr_models);
        ctx->h_mesh_skinned.resize(ctx->tr_models); ctx->h_mesh_first.resize(ctx->tr_models); ctx->h_mesh_count.resize(ctx->tr_models);
        ctx->ml_attr.size = (size_t)ctx->n_meshlets * 2560; ctx->ml_inds.size = (size_t)ctx->n_meshlets * 512;
        ctx->ml_cull.size = (size_t)ctx->n_meshlets * 32; ctx->ml_info.size = (size_t)ctx->n_meshlets * sizeof(sftg_meshlet_info);
        ctx->skin_j.size = (size_t)ctx->n_skin * 512; ctx->skin_w.size = (size_t)ctx->n_skin * 256;
        ctx->blas.size = (size_t)ctx->n_blas * 256;
        ctx->tables_dirty = true;
    }
    ctx->tr_live = false; ctx->tr_pinned = false;
}

static int sync_tables(sftg_ctx* ctx) {
    if (!ctx->tables_dirty) return 0;
    int rc;
    if ((rc = pool_reserve(ctx, ctx->texs, (ctx->h_texs.size() + 1) * sizeof(sftg_tex)))) return rc;
    if ((rc = pool_reserve(ctx, ctx->mats, (ctx->h_mats.size() + 1) * sizeof(sftg_mat)))) return rc;
    if ((rc = pool_reserve(ctx, ctx->models, (ctx->h_models.size() + 1) * sizeof(sftg_model)))) return rc;
    if (!ctx->h_texs.empty()) CK(cudaMemcpyAsync(ctx->texs.ptr, ctx->h_texs.data(), ctx->h_texs.size() * sizeof(sftg_tex), cudaMemcpyHostToDevice, ctx->stream));
    if (!ctx->h_mats.empty()) CK(cudaMemcpyAsync(ctx->mats.ptr, ctx->h_mats.data(), ctx->h_mats.size() * sizeof(sftg_mat), cudaMemcpyHostToDevice, ctx->stream));
    if (!ctx->h_models.empty()) CK(cudaMemcpyAsync(ctx->models.ptr, ctx->h_models.data(), ctx->h_models.size() * sizeof(sftg_model), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->tables_dirty = false;
    return 0;
}

/* ------------------------------------------------------------------ frame */
struct bump {
    char* base; size_t off, cap;
    template <class T> T* take(size_t n) {
        off = (off + 255) & ~(size_t)255;
        T* p = (T*)(base + off);
        off += n * sizeof(T);
        return p;
    }
};

/* Placement of one view inside a batch: where its rows start in the batch-wide arrays. */
struct view_plan {
    uint32_t ss_base, total_ss, tile_base, tiles, prox_base, packet_base, n_packets, stile_base, stiles, scols;
    uint32_t inst_off, bone_off, pl_off, dl_off, tl_off;
    uint64_t vis_base, color_off;
    uint32_t* direct;   /* the caller's pinned colour buffer, written by the kernels in place; else null */
    int32_t direct_pitch;   /* its row stride in pixels */
};

struct batch_bufs {
    sftg_frame* frames;  /* device copies of the views' frame blocks */
    const sftg_job* jobs;
    const uint16_t* tile_view; const uint16_t* packet_view; const uint16_t* prox_view; const uint16_t* stile_view;
    uint32_t* stile_count; uint32_t* stile_start; uint32_t* stile_list;   /* super-tile meshlet lists */
    float* ss;
    sftg_batch_rec* recs;
    uint32_t* clip_cnt; uint32_t* clip_base;
    int4* mrect;
    sftg_clip_tri* clips; int4* clip_rect;
    uint32_t* tile_count; uint32_t* tile_start;
    uint32_t* tile_order; uint32_t* order_scratch;
    uint8_t* tile_nlights;   /* per tile: its light list length (debug views) */
    sftg_tile_lights* tile_lights;   /* per tile: lights and selected proxies, shared by its resolve CTAs */
    uint32_t* queue;         /* item counters of the persistent raster and resolve launches, one per launch */
    bool any_overlay;        /* a view asks for a tile overlay (debug modes 2-4) */
    uint64_t* tile_pay;
    uint8_t* light_vis;
    void* packets; uint2* pairs; uint32_t* n_pairs; uint32_t max_pairs;
    uint32_t* scan_tmp;
    uint32_t* status;
    uint32_t* totals;    /* [0] clip total, [1] tile payload total, [2] super-tile list total */
    float* vis_depth; uint32_t* vis_id; float* shadow;
    float2* vis; float2* zrange;
    uint32_t n_views, total_ss, n_jobs, total_tiles, total_prox, total_packets, max_inst, total_stiles;
    uint32_t s_tile0[3], s_tiles[3];   /* batch-wide tile range of the views with 1, 2 and 4 samples */
    uint64_t color_total;              /* pixels over all views */
    std::vector<view_plan> plan;
};

static void scan_u32(const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* tmp, uint32_t* total, cudaStream_t st, int* launches) {
    const uint32_t nb = (n + SFTG_SCAN_ELEMS_PER_BLOCK - 1) / SFTG_SCAN_ELEMS_PER_BLOCK;
    if (!nb) return;
    if (n <= SFTG_SCAN_SMALL) {
        k_scan_small<<<1, 1024, 0, st>>>(in, n, out, total);
        *launches += 1;
        return;
    }
    k_scan_reduce<<<nb, 1024, 0, st>>>(in, n, tmp);
    k_scan_top<<<1, 1024, 0, st>>>(tmp, nb, total);
    k_scan_down<<<nb, 1024, 0, st>>>(in, n, tmp, out);
    *launches += 3;
}

static int sample_slot(int S) { return S == 1 ? 0 : (S == 2 ? 1 : 2); }

/* Plans the views, sizes the arena and colour pool, and uploads every view's frame block with
 * one H2D copy.  Views keep their own instance, light, proxy and TLAS arrays; the shared arrays
 * (screen-space cache, batch records, clip pool, tile lists, light_vis, visibility buffers) are
 * laid out view after view, with tiles numbered by sample count first (1, 2, 4) so that each
 * raster/resolve specialisation covers one contiguous tile range. */
/* The device-visible address of a caller's colour buffer the kernels can write in place: page-
 * locked host memory (registered or allocated by CUDA) with a clearing view and a pitch of whole
 * pixels.  Writes then reach host memory over the chip-to-chip link as the resolve stores them,
 * and the frame needs no device-to-host copy.  Null for any other buffer (copied as before). */
static uint32_t* direct_color(const sftg_frame_desc& fd, uint32_t* host, int32_t pitch_bytes) {
    if (!host || !fd.clear) return nullptr;
    const size_t pitch = pitch_bytes > 0 ? (size_t)pitch_bytes : (size_t)fd.width * 4;
    if (pitch % 4 || pitch < (size_t)fd.width * 4) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
    return (uint32_t*)at.devicePointer;
}

static int build_batch(sftg_ctx* ctx, sftg_lane& ln, const sftg_frame_desc* fds, uint32_t nv, bool want_debug, batch_bufs& B,
                       uint32_t* const* host_color = nullptr, const int32_t* pitch_bytes = nullptr) {
    if (!nv || nv > 65535) return set_err(ctx, SFTG_E_ARG, "a batch holds 1 to 65535 views, not %u", nv);
    if (want_debug && nv != 1) return set_err(ctx, SFTG_E_ARG, "debug capture covers single-view submissions only");
    B.plan.assign(nv, view_plan{});
    B.n_views = nv;
    std::vector<sftg_inst> inst;
    std::vector<sftg_job>& jobs = ctx->tmp_jobs;   /* capacity kept between batches */
    jobs.clear();
    std::vector<float> bones;
    uint32_t total_ss = 0, total_prox = 0, total_packets = 0, max_inst = 0, n_pl = 0, n_dl = 0, n_tl = 0;
    uint64_t max_pairs = 0, color_total = 0;
    for (uint32_t v = 0; v < nv; v++) {
        const sftg_frame_desc* fd = &fds[v];
        view_plan& P = B.plan[v];
        const int W = fd->width, H = fd->height, S = fd->samples;
        if (W <= 0 || H <= 0 || !(S == 1 || S == 2 || S == 4)) return set_err(ctx, SFTG_E_ARG, "view %u: bad frame size or samples", v);
        if (fd->n_instances > SFTG_MAX_INSTANCES) return set_err(ctx, SFTG_E_LIMIT, "view %u: more than %d instances in one frame", v, SFTG_MAX_INSTANCES);
        P.ss_base = total_ss; P.inst_off = (uint32_t)inst.size(); P.bone_off = (uint32_t)bones.size();
        P.pl_off = n_pl; P.dl_off = n_dl; P.tl_off = n_tl;
        uint32_t lss = 0;
        for (uint32_t i = 0; i < fd->n_instances; i++) {
            const sftg_instance_desc& id = fd->instances[i];
            if (id.model < 0 || (size_t)id.model >= ctx->h_models.size()) return set_err(ctx, SFTG_E_ARG, "view %u instance %u: bad model", v, i);
            const sftg_model& md = ctx->h_models[id.model];
            sftg_inst I;
            memset(&I, 0, sizeof(I));
            memcpy(I.T, id.transform, 64);
            I.model = (uint32_t)id.model;
            I.ss_offset = lss;
            I.meshlet_base = md.meshlet_base;
            I.bones = -1;
            if (id.bones && id.bone_count) {
                I.bones = (int32_t)((bones.size() - P.bone_off) / 16);
                bones.insert(bones.end(), id.bones, id.bones + (size_t)id.bone_count * 16);
            }
            const uint32_t jw = (uint32_t)ctx->tuning.geom_job_width;
            if (ctx->h_job_tmpl.size() <= (size_t)id.model) ctx->h_job_tmpl.resize((size_t)id.model + 1);
            sftg_ctx::job_tmpl& T = ctx->h_job_tmpl[id.model];
            if (T.jw != jw || T.meshlet_base != md.meshlet_base || T.total != md.total_meshlets) {
                T.jobs.clear();
                for (uint32_t k = 0; k < md.mesh_count; k++) {
                    const uint32_t first = ctx->h_mesh_first[id.model][k], cnt = ctx->h_mesh_count[id.model][k];
                    const uint32_t sk = ctx->h_mesh_skinned[id.model][k];
                    for (uint32_t s = 0; s < cnt; s += 8) {   /* the reference's groups of 8, cut into jobs of jw */
                        const uint32_t gc = (cnt - s) < 8 ? (cnt - s) : 8;
                        for (uint32_t q = 0; q < gc; q += jw) {
                            sftg_job j; j.inst = 0; j.first = first + s + q; j.count = (uint16_t)((gc - q) < jw ? (gc - q) : jw);
                            j.skinned = (uint16_t)sk; j.view = 0; j.group_first = first + s;
                            T.jobs.push_back(j);
                        }
                    }
                }
                T.jw = jw; T.meshlet_base = md.meshlet_base; T.total = md.total_meshlets;
            }
            const size_t j0 = jobs.size();
            jobs.resize(j0 + T.jobs.size());
            sftg_job* jd = jobs.data() + j0;
            const uint16_t has_bones = I.bones >= 0 ? 1 : 0;
            for (size_t q = 0; q < T.jobs.size(); q++) {
                sftg_job j = T.jobs[q];
                j.inst = i; j.view = v; j.skinned = (uint16_t)(j.skinned & has_bones);
                jd[q] = j;
            }
            lss += md.total_meshlets;
            inst.push_back(I);
        }
        inst.push_back(sftg_inst{});   /* keeps every view's instance array non-empty */
        P.total_ss = lss; total_ss += lss;
        P.prox_base = total_prox; total_prox += fd->n_proxies;
        const uint32_t lc = fd->n_point < 64 ? fd->n_point : 64;
        P.n_packets = (fd->shadows && fd->n_point && fd->n_proxies) ? lc * ((fd->n_proxies + 7) / 8) * 3 : 0;
        P.packet_base = total_packets; total_packets += P.n_packets;
        max_pairs += (uint64_t)P.n_packets * (fd->n_instances ? fd->n_instances : 1);
        if (fd->n_instances > max_inst) max_inst = fd->n_instances;
        n_pl += fd->n_point; n_dl += fd->n_dir; n_tl += fd->tlas_count;
        P.color_off = color_total; color_total += (uint64_t)W * H;
        P.direct = direct_color(*fd, host_color ? host_color[v] : nullptr, pitch_bytes ? pitch_bytes[v] : 0);
        P.direct_pitch = P.direct ? (pitch_bytes && pitch_bytes[v] > 0 ? pitch_bytes[v] / 4 : W) : W;
    }
    if (max_pairs * (1 + SFTG_OCC_ITEMS_PER_PAIR) > 0xFFFFFFF0ull || total_ss > (1u << 26)) return set_err(ctx, SFTG_E_LIMIT, "batch too large for one submission");
    uint32_t total_tiles = 0;
    uint64_t vis_total = 0;
    for (int si = 0; si < 3; si++) {
        const int Sv = 1 << si;
        B.s_tile0[si] = total_tiles;
        for (uint32_t v = 0; v < nv; v++) {
            if (fds[v].samples != Sv) continue;
            view_plan& P = B.plan[v];
            P.tiles = (uint32_t)(((fds[v].width + 63) / 64) * ((fds[v].height + 63) / 64));
            P.tile_base = total_tiles; total_tiles += P.tiles;
            P.vis_base = vis_total; vis_total += (uint64_t)P.tiles * Sv * 4096;
        }
        B.s_tiles[si] = total_tiles - B.s_tile0[si];
    }
    uint32_t total_stiles = 0;
    for (uint32_t v = 0; v < nv; v++) {
        view_plan& P = B.plan[v];
        const uint32_t cols = (uint32_t)((fds[v].width + 63) / 64), rows = (uint32_t)((fds[v].height + 63) / 64);
        /* coarse lists pay off once a tile would scan more than four chunks of meshlet slots */
        const bool coarse = P.total_ss > 4u * 256u;
        P.scols = coarse ? (cols + SFTG_STILE - 1) / SFTG_STILE : 0u;
        P.stiles = P.scols * ((rows + SFTG_STILE - 1) / SFTG_STILE);
        P.stile_base = total_stiles; total_stiles += P.stiles;
    }
    B.total_stiles = total_stiles;
    B.total_ss = total_ss; B.n_jobs = (uint32_t)jobs.size(); B.total_tiles = total_tiles; B.total_prox = total_prox;
    B.total_packets = total_packets; B.max_inst = max_inst; B.max_pairs = (uint32_t)max_pairs; B.color_total = color_total;
    const size_t n_rec = (size_t)total_ss * 16;
    /* staging layout */
    size_t so = 0;
    auto stage_take = [&](size_t bytes) { so = (so + 255) & ~(size_t)255; const size_t r = so; so += bytes; return r; };
    const size_t o_F = stage_take((size_t)nv * sizeof(sftg_frame));
    const size_t o_inst = stage_take(inst.size() * sizeof(sftg_inst));
    const size_t o_bones = stage_take(bones.size() * 4 + 64);
    const size_t o_jobs = stage_take(jobs.size() * sizeof(sftg_job) + 16);
    const size_t o_pl = stage_take((size_t)n_pl * sizeof(sftg_point_light) + 16);
    const size_t o_dl = stage_take((size_t)n_dl * sizeof(sftg_dir_light) + 16);
    const size_t o_px = stage_take((size_t)total_prox * sizeof(sftg_proxy) + 16);
    const size_t o_tl = stage_take((size_t)n_tl * 256 + 16);
    const size_t o_tv = stage_take((size_t)total_tiles * 2 + 16);
    const size_t o_pv = stage_take((size_t)total_packets * 2 + 16);
    const size_t o_xv = stage_take((size_t)total_prox * 2 + 16);
    const size_t o_sv = stage_take((size_t)total_stiles * 2 + 16);
    const size_t stage_bytes = so;
    /* device arena layout */
    size_t need = stage_bytes + 4096;
    auto acc = [&](size_t bytes) { need = ((need + 255) & ~(size_t)255) + bytes; };
    acc((size_t)total_ss * SFTG_SS_FLOATS * 4); acc(n_rec * sizeof(sftg_batch_rec)); acc(n_rec * 4); acc(n_rec * 4);
    acc((size_t)total_ss * 16 + 16); acc(ctx->clip_cap * sizeof(sftg_clip_tri)); acc(ctx->clip_cap * 16);
    acc((size_t)total_tiles * 4); acc((size_t)total_tiles * 4); acc((size_t)total_tiles * 4); acc(1024); acc(total_tiles + 16);
    acc(ctx->tile_cap * 8);
    acc((size_t)total_stiles * 4); acc((size_t)total_stiles * 4); acc(ctx->stile_cap * 4);
    acc((size_t)total_prox * 64 + 64); acc((size_t)total_packets * sftg_packet_bytes() + 64);
    acc((max_pairs * (1 + SFTG_OCC_ITEMS_PER_PAIR) + 1) * 8); acc(64); acc(((n_rec + total_tiles + total_stiles) / SFTG_SCAN_ELEMS_PER_BLOCK + 16) * 4); acc(64); acc(64);
    acc(vis_total * 8); acc((size_t)(total_tiles + 1) * sftg_raster_bands() * sizeof(float2));
    acc((size_t)total_tiles * sizeof(sftg_tile_lights)); acc(64);
    const int W0 = fds[0].width, H0 = fds[0].height, S0 = fds[0].samples;
    if (want_debug) { acc((size_t)total_tiles * S0 * 4096 * 4); acc((size_t)total_tiles * S0 * 4096 * 4); acc((size_t)W0 * H0 * 16 * 4); }
    /* growth: the lane's previous batch has finished (a lane takes a batch only once the last
     * one was collected), so its buffers are free; other lanes keep running meanwhile */
    if (need > ln.arena_cap) {
        if (ln.arena) { CK(cudaFreeAsync(ln.arena, ln.stream)); ln.arena = nullptr; }
        size_t nc = need + need / 4;
        if (cudaMallocFromPoolAsync(&ln.arena, nc, ctx->lane_pool, ln.stream) != cudaSuccess) {
            ln.arena = nullptr; ln.arena_cap = 0; cudaGetLastError();
            return set_err(ctx, SFTG_E_NOMEM, "frame arena of %zu bytes", nc);
        }
        ln.arena_cap = nc;
    }
    if (color_total * 4 > ln.d_color_cap) {
        if (ln.d_color) { CK(cudaFreeAsync(ln.d_color, ln.stream)); ln.d_color = nullptr; }
        const size_t nc = color_total * 4 + color_total;
        if (cudaMallocFromPoolAsync((void**)&ln.d_color, nc, ctx->lane_pool, ln.stream) != cudaSuccess) {
            ln.d_color = nullptr; ln.d_color_cap = 0; cudaGetLastError();
            return set_err(ctx, SFTG_E_NOMEM, "colour buffers");
        }
        ln.d_color_cap = nc;
    }
    if (stage_bytes > ln.h_stage_cap) {
        if (ln.h_stage) ctx->retired_stage.push_back(ln.h_stage);
        size_t nc = 2 * stage_bytes + 4096;
        if (cudaMallocHost(&ln.h_stage, nc) != cudaSuccess) { ln.h_stage = nullptr; ln.h_stage_cap = 0; return set_err(ctx, SFTG_E_NOMEM, "pinned staging"); }
        ln.h_stage_cap = nc;
    }
    char* hs = (char*)ln.h_stage;
    char* ds = (char*)ln.arena;
    bump bp{ ds, stage_bytes, ln.arena_cap };
    B.ss = bp.take<float>((size_t)total_ss * SFTG_SS_FLOATS);
    B.recs = bp.take<sftg_batch_rec>(n_rec);
    B.clip_cnt = bp.take<uint32_t>(n_rec);
    B.clip_base = bp.take<uint32_t>(n_rec);
    B.mrect = bp.take<int4>((size_t)total_ss + 1);
    B.clips = bp.take<sftg_clip_tri>(ctx->clip_cap);
    B.clip_rect = bp.take<int4>(ctx->clip_cap);
    B.tile_count = bp.take<uint32_t>(total_tiles);
    B.tile_start = bp.take<uint32_t>(total_tiles);
    B.tile_order = bp.take<uint32_t>(total_tiles);
    B.order_scratch = bp.take<uint32_t>(256);
    B.tile_nlights = bp.take<uint8_t>((size_t)total_tiles + 16);
    B.any_overlay = false;
    for (uint32_t v = 0; v < nv; v++) if (fds[v].debug_mode >= 2 && fds[v].debug_mode <= 4) B.any_overlay = true;
    B.tile_pay = bp.take<uint64_t>(ctx->tile_cap);
    B.stile_count = bp.take<uint32_t>(total_stiles);
    B.stile_start = bp.take<uint32_t>(total_stiles);
    B.stile_list = bp.take<uint32_t>(ctx->stile_cap);
    B.light_vis = bp.take<uint8_t>((size_t)total_prox * 64 + 64);
    B.packets = bp.take<char>((size_t)total_packets * sftg_packet_bytes() + 64);
    B.pairs = bp.take<uint2>((size_t)max_pairs * (1 + SFTG_OCC_ITEMS_PER_PAIR) + 1);   /* pairs, then BLAS sub-walk items */
    B.n_pairs = bp.take<uint32_t>(16);
    B.scan_tmp = bp.take<uint32_t>((n_rec + total_tiles + total_stiles) / SFTG_SCAN_ELEMS_PER_BLOCK + 16);
    B.status = bp.take<uint32_t>(16);
    B.totals = bp.take<uint32_t>(16);
    B.vis = bp.take<float2>(vis_total);
    B.zrange = bp.take<float2>((size_t)(total_tiles + 1) * sftg_raster_bands());   /* per raster band of each tile */
    B.tile_lights = bp.take<sftg_tile_lights>(total_tiles);
    B.queue = bp.take<uint32_t>(16);
    B.vis_depth = nullptr; B.vis_id = nullptr; B.shadow = nullptr;
    if (want_debug) {
        B.vis_depth = bp.take<float>((size_t)total_tiles * S0 * 4096);
        B.vis_id = bp.take<uint32_t>((size_t)total_tiles * S0 * 4096);
        B.shadow = bp.take<float>((size_t)W0 * H0 * 16);
    }
    if (bp.off > ln.arena_cap)   /* the sizing above and these takes disagree: refuse rather than overrun */
        return set_err(ctx, SFTG_E_NOMEM, "frame arena layout of %zu bytes exceeds its %zu-byte sizing", bp.off, ln.arena_cap);
    /* fill the staging block */
    uint16_t* tv = (uint16_t*)(hs + o_tv);
    uint16_t* pv = (uint16_t*)(hs + o_pv);
    uint16_t* xv = (uint16_t*)(hs + o_xv);
    uint16_t* sv = (uint16_t*)(hs + o_sv);
    for (uint32_t v = 0; v < nv; v++) {
        const sftg_frame_desc* fd = &fds[v];
        const view_plan& P = B.plan[v];
        const int W = fd->width, H = fd->height;
        sftg_frame* F = (sftg_frame*)(hs + o_F) + v;
        memset(F, 0, sizeof(*F));
        F->width = W; F->height = H; F->samples = fd->samples; F->pitch = P.direct_pitch;
        F->hw = (float)W * 0.5f; F->hh = (float)H * 0.5f; F->vpx = 0.f; F->vpy = 0.f;
        F->cols = (W + 63) / 64; F->rows = (H + 63) / 64; F->tiles = (int32_t)P.tiles; F->debug_mode = (int32_t)fd->debug_mode;
        F->clear = fd->clear; F->clear_color = fd->clear_color; F->shadows = fd->shadows;
        F->debug_tex = fd->debug_texture;
        memcpy(F->cam, fd->cam_pos, 12);
        memcpy(F->vp, fd->view_proj, 64);
        for (int p = 0; p < 6; p++) {
            for (int a = 0; a < 3; a++) { F->fn[p][a] = fd->frustum_n[p][a]; F->fan[p][a] = fabsf(fd->frustum_n[p][a]); }
            F->fd[p] = fd->frustum_d[p];
        }
        memcpy(F->ambient, fd->ambient, 12);
        F->lightmap_brightness = fd->lightmap_brightness;
        F->n_point = fd->n_point; F->n_dir = fd->n_dir; F->n_proxies = fd->n_proxies; F->n_inst = fd->n_instances;
        F->total_ss = P.total_ss; F->n_jobs = B.n_jobs; F->tlas_root = fd->tlas_root; F->tlas_count = fd->tlas_count;
        F->clip_cap = (uint32_t)ctx->clip_cap; F->tile_cap = (uint32_t)ctx->tile_cap; F->stile_cap = (uint32_t)ctx->stile_cap;
        F->stile_base = P.stile_base; F->scols = P.scols;
        F->view = v; F->ss_base = P.ss_base; F->tile_base = P.tile_base; F->prox_base = P.prox_base;
        F->packet_base = P.packet_base; F->n_packets = P.n_packets; F->vis_base = P.vis_base;
        F->color_dev = P.direct ? P.direct : ln.d_color + P.color_off;
        F->inst = (const sftg_inst*)(ds + o_inst) + P.inst_off;
        F->bones = (const float*)(ds + o_bones) + P.bone_off;
        F->jobs = (const sftg_job*)(ds + o_jobs);
        F->point = (const sftg_point_light*)(ds + o_pl) + P.pl_off;
        F->dir = (const sftg_dir_light*)(ds + o_dl) + P.dl_off;
        F->proxies = (const sftg_proxy*)(ds + o_px) + P.prox_base;
        F->tlas = (const sftg_bvh_node*)(ds + o_tl) + P.tl_off;
        F->models = (const sftg_model*)ctx->models.ptr;
        F->texs = (const sftg_tex*)ctx->texs.ptr;
        F->texels = (const uint32_t*)ctx->texels.ptr;
        F->mats = (const sftg_mat*)ctx->mats.ptr;
        F->ml_attr = (const float*)ctx->ml_attr.ptr;
        F->ml_inds = (const uint8_t*)ctx->ml_inds.ptr;
        F->ml_cull = (const float*)ctx->ml_cull.ptr;
        F->ml_info = (const sftg_meshlet_info*)ctx->ml_info.ptr;
        F->skin_j = (const uint16_t*)ctx->skin_j.ptr;
        F->skin_w = (const uint8_t*)ctx->skin_w.ptr;
        F->blas = (const sftg_bvh_node*)ctx->blas.ptr;
        for (uint32_t l = 0; l < fd->n_point; l++) memcpy(hs + o_pl + (P.pl_off + l) * sizeof(sftg_point_light), fd->point_lights + 8 * l, 32);
        for (uint32_t l = 0; l < fd->n_dir; l++) memcpy(hs + o_dl + (P.dl_off + l) * sizeof(sftg_dir_light), fd->dir_lights + 6 * l, 24);
        for (uint32_t p = 0; p < fd->n_proxies; p++) memcpy(hs + o_px + (P.prox_base + p) * sizeof(sftg_proxy), fd->proxies + 8 * p, 32);
        if (fd->tlas_count) memcpy(hs + o_tl + (size_t)P.tl_off * 256, fd->tlas_nodes, (size_t)fd->tlas_count * 256);
        for (uint32_t t = 0; t < P.tiles; t++) tv[P.tile_base + t] = (uint16_t)v;
        for (uint32_t k = 0; k < P.n_packets; k++) pv[P.packet_base + k] = (uint16_t)v;
        for (uint32_t p = 0; p < fd->n_proxies; p++) xv[P.prox_base + p] = (uint16_t)v;
        for (uint32_t t = 0; t < P.stiles; t++) sv[P.stile_base + t] = (uint16_t)v;
    }
    memcpy(hs + o_inst, inst.data(), inst.size() * sizeof(sftg_inst));
    if (!bones.empty()) memcpy(hs + o_bones, bones.data(), bones.size() * 4);
    if (!jobs.empty()) memcpy(hs + o_jobs, jobs.data(), jobs.size() * sizeof(sftg_job));
    B.frames = (sftg_frame*)(ds + o_F);
    B.jobs = (const sftg_job*)(ds + o_jobs);
    B.tile_view = (const uint16_t*)(ds + o_tv);
    B.packet_view = (const uint16_t*)(ds + o_pv);
    B.prox_view = (const uint16_t*)(ds + o_xv);
    B.stile_view = (const uint16_t*)(ds + o_sv);
    CK(cudaMemcpyAsync(ds, hs, stage_bytes, cudaMemcpyHostToDevice, ln.stream));
    return 0;
}

/* Phase events: inside a stream capture they must become event-record nodes of the graph
 * (cudaEventRecordExternal) so that replays still time the phases. */
static cudaError_t record_event(cudaEvent_t ev, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) return e;
    return cs == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal) : cudaEventRecord(ev, st);
}

static int launch_batch(sftg_ctx* ctx, sftg_lane& ln, const batch_bufs& B) {
    const uint32_t n_rec = B.total_ss * 16;
    cudaStream_t st = ln.stream;
    ln.launches = 0;
    CK(cudaGetLastError());   /* nothing pending from earlier calls: every launch below is checked */
    CK(cudaMemsetAsync(B.status, 0, 64, st));
    CK(record_event(ln.ev[0], st));
    /* proxy occlusion only feeds the resolve: it runs on the second stream, forked here and
     * joined before the resolve, overlapping geometry, binning and raster */
    const bool occl = B.total_prox || B.total_packets;
    if (occl) {
        cudaStream_t so = ln.stream2;
        CK(cudaEventRecord(ln.ev_fork, st));
        CK(cudaStreamWaitEvent(so, ln.ev_fork, 0));
        if (B.total_prox) CK(cudaMemsetAsync(B.light_vis, 0, (size_t)B.total_prox * 64, so));   /* columns past the lights stay 0 */
        if (B.total_packets) {
            sftg_launch_occlusion(B.frames, B.packet_view, B.total_packets, B.prox_view, B.total_prox, B.max_inst, B.packets,
                                  B.pairs, B.n_pairs, B.max_pairs, SFTG_OCC_ITEMS_PER_PAIR, B.light_vis, B.status,
                                  ctx->tuning.occl_ray_prune, so);
            ln.launches += 4;
            CK(cudaGetLastError());
        }
        CK(record_event(ln.ev[1], so));
        CK(cudaEventRecord(ln.ev_join, so));
    } else {
        CK(record_event(ln.ev[1], st));
    }
    CK(record_event(ln.ev_geo, st));
    if (B.n_jobs) {
        k_geometry<<<(B.n_jobs + 3) / 4, 128, 0, st>>>(B.frames, B.jobs, B.n_jobs, B.ss, B.recs, B.clip_cnt, B.mrect);
        ln.launches++;
        CK(cudaGetLastError());
    }
    if (n_rec) {
        scan_u32(B.clip_cnt, B.clip_base, n_rec, B.scan_tmp, B.totals + 0, st, &ln.launches);
        k_clip<<<(n_rec + 255) / 256, 256, 0, st>>>(B.frames, B.n_views, B.ss, B.clip_cnt, B.clip_base, B.clips, B.clip_rect, B.mrect, n_rec);
        ln.launches++;
        CK(cudaGetLastError());
    } else {
        CK(cudaMemsetAsync(B.totals, 0, 8, st));
    }
    CK(record_event(ln.ev[2], st));
    if (B.total_stiles) {
        k_coarse<<<B.total_stiles, 1024, 0, st>>>(B.frames, B.stile_view, B.mrect, B.stile_count, nullptr, nullptr);
        scan_u32(B.stile_count, B.stile_start, B.total_stiles, B.scan_tmp, B.totals + 2, st, &ln.launches);
        k_coarse<<<B.total_stiles, 1024, 0, st>>>(B.frames, B.stile_view, B.mrect, B.stile_count, B.stile_start, B.stile_list);
        ln.launches += 2;
    } else {
        CK(cudaMemsetAsync(B.totals + 2, 0, 4, st));
    }
    k_bin<<<B.total_tiles, 256, 0, st>>>(B.frames, B.tile_view, B.recs, B.clip_cnt, B.clip_base, B.clip_rect, B.mrect,
                                         B.stile_count, B.stile_start, B.stile_list, B.tile_count, nullptr, nullptr);
    scan_u32(B.tile_count, B.tile_start, B.total_tiles, B.scan_tmp, B.totals + 1, st, &ln.launches);
    k_bin<<<B.total_tiles, 256, 0, st>>>(B.frames, B.tile_view, B.recs, B.clip_cnt, B.clip_base, B.clip_rect, B.mrect,
                                         B.stile_count, B.stile_start, B.stile_list, B.tile_count, B.tile_start, B.tile_pay);
    ln.launches += 2 + sftg_launch_tile_order(B.frames, B.tile_view, B.tile_count, B.total_tiles, B.order_scratch, B.tile_order, st);
    CK(cudaGetLastError());
    CK(record_event(ln.ev[3], st));
    if (B.shadow) CK(cudaMemsetAsync(B.shadow, 0, B.color_total * 16 * 4, st));
    sftg_tile_args A;
    A.frames = B.frames; A.tile_view = B.tile_view; A.ss = B.ss; A.clips = B.clips; A.clip_base = B.clip_base;
    A.tile_order = B.tile_order; A.tile_nlights = B.tile_nlights; A.tile_lights = B.tile_lights;
    A.tile_start = B.tile_start; A.tile_count = B.tile_count; A.tile_pay = B.tile_pay; A.light_vis = B.light_vis;
    A.vis = B.vis; A.zrange = B.zrange; A.vis_depth = B.vis_depth; A.vis_id = B.vis_id; A.shadow_out = B.shadow;
    /* With views of several sample counts, the 4x tile range runs on the main stream and the 1x
     * and 2x ranges beside it on a third stream, so that one range's tail overlaps the others. */
    const bool split_s = B.s_tiles[2] && (B.s_tiles[0] || B.s_tiles[1]);
    auto per_range = [&](int k, auto&& launch) -> int {
        if (!split_s) {
            for (int si = 0; si < 3; si++) if (B.s_tiles[si]) { launch(si, st); ln.launches++; }
            return 0;
        }
        CK(cudaEventRecord(ln.ev_split[k], st));
        CK(cudaStreamWaitEvent(ln.stream3, ln.ev_split[k], 0));
        launch(2, st); ln.launches++;
        for (int si = 0; si < 2; si++) if (B.s_tiles[si]) { launch(si, ln.stream3); ln.launches++; }
        CK(cudaEventRecord(ln.ev_merge[k], ln.stream3));
        CK(cudaStreamWaitEvent(st, ln.ev_merge[k], 0));
        return 0;
    };
    const bool queue_raster = (ctx->tuning.tile_queue & 1) != 0, queue_resolve = (ctx->tuning.tile_queue & 2) != 0;
    if (ctx->tuning.tile_queue) CK(cudaMemsetAsync(B.queue, 0, 64, st));   /* counters: raster 0-2, resolve 3-5 */
    int prc = per_range(0, [&](int si, cudaStream_t s) {
        sftg_launch_raster(1 << si, B.s_tile0[si], B.s_tiles[si], ctx->tuning.raster_slab_rows[si], ctx->tuning.raster_bands[si],
                           queue_raster ? B.queue + si : nullptr, s, A);
    });
    if (prc) return prc;
    CK(cudaGetLastError());
    CK(record_event(ln.ev[4], st));
    if (occl) CK(cudaStreamWaitEvent(st, ln.ev_join, 0));
    /* per sample count: the tiles' light lists and proxy selections made once per tile (one more
     * launch on the critical path) or by every resolve CTA of the tile (split-fold work) */
    bool records[3];
    for (int si = 0; si < 3; si++) {
        const int m = ctx->tuning.tile_lights[si];
        records[si] = m == 2 || (m == 0 && ctx->tuning.resolve_split[si] >= 16 && B.s_tiles[si] >= 256);
        if (records[si] && B.s_tiles[si]) {   /* on st: every range's resolve waits for it (per_range forks after it) */
            sftg_launch_tile_lights(B.s_tile0[si], B.s_tiles[si], st, A);
            ln.launches++;
        }
    }
    prc = per_range(1, [&](int si, cudaStream_t s) {
        sftg_launch_resolve(1 << si, B.s_tile0[si], B.s_tiles[si], ctx->tuning.resolve_split[si], records[si],
                            queue_resolve ? B.queue + 3 + si : nullptr, s, A);
    });
    if (prc) return prc;
    if (B.any_overlay) { sftg_launch_debug_overlay(B.total_tiles, st, A); ln.launches++; }
    CK(cudaGetLastError());
    CK(record_event(ln.ev[5], st));
    return 0;
}

static uint64_t fnv(uint64_t h, const void* p, size_t n) {
    const unsigned char* c = (const unsigned char*)p;
    for (size_t i = 0; i < n; i++) { h ^= c[i]; h *= 1099511628211ull; }
    return h;
}

/* Every value launch_batch passes to a launch: arena pointers, counts, ranges and knobs. */
static uint64_t batch_key(const sftg_ctx* ctx, const batch_bufs& B) {
    uint64_t h = 1469598103934665603ull;
    const uint32_t ov = B.any_overlay ? 1u : 0u;
    h = fnv(h, &ov, sizeof(ov));
    const void* ptrs[] = { B.frames, B.jobs, B.tile_view, B.packet_view, B.prox_view, B.stile_view, B.stile_count, B.stile_start,
                           B.stile_list, B.ss, B.recs, B.clip_cnt, B.clip_base, B.tile_nlights, B.tile_lights, B.queue,
                           B.mrect, B.clips, B.clip_rect, B.tile_count, B.tile_start, B.tile_order, B.order_scratch, B.tile_pay,
                           B.light_vis, B.packets, B.pairs, B.n_pairs, B.scan_tmp, B.status, B.totals, B.vis, B.zrange,
                           B.vis_depth, B.vis_id, B.shadow };
    h = fnv(h, ptrs, sizeof(ptrs));
    const uint32_t cnt[] = { B.max_pairs, B.n_views, B.total_ss, B.n_jobs, B.total_tiles, B.total_prox, B.total_packets, B.max_inst,
                             B.total_stiles,
                             B.s_tile0[0], B.s_tile0[1], B.s_tile0[2], B.s_tiles[0], B.s_tiles[1], B.s_tiles[2] };
    h = fnv(h, cnt, sizeof(cnt));
    h = fnv(h, &B.color_total, sizeof(B.color_total));
    h = fnv(h, &ctx->tuning, sizeof(ctx->tuning));
    return h;
}

/* launch_batch through a CUDA graph: captured when a batch repeats the previous batch's layout,
 * replayed while the layout stays.  A layout seen once (a served batch of new requests) is
 * launched directly, without the cost of a capture it would not reuse. */
static int launch_batch_graph(sftg_ctx* ctx, sftg_lane& ln, const batch_bufs& B) {
    const uint64_t key = batch_key(ctx, B);
    const uint64_t prev = ln.seen_key;
    ln.seen_key = key;
    if ((!ln.graph || key != ln.graph_key) && key != prev) return launch_batch(ctx, ln, B);
    if (!ln.graph || key != ln.graph_key) {
        if (ln.graph) { cudaGraphExecDestroy(ln.graph); ln.graph = nullptr; }
        CK(cudaStreamBeginCapture(ln.stream, cudaStreamCaptureModeThreadLocal));
        const int rc = launch_batch(ctx, ln, B);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(ln.stream, &g);
        if (rc || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return rc ? rc : set_err(ctx, SFTG_E_CUDA, "graph capture: %s", cudaGetErrorString(e));
        }
        const cudaError_t ie = cudaGraphInstantiate(&ln.graph, g, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) { ln.graph = nullptr; return set_err(ctx, SFTG_E_CUDA, "graph instantiate: %s", cudaGetErrorString(ie)); }
        ln.graph_key = key;
        ln.graph_launches = ln.launches;
    }
    CK(cudaGraphLaunch(ln.graph, ln.stream));
    ln.launches = ln.graph_launches;
    return 0;
}

/* Queues a batch on a lane: the frame block, the caller's pixels for views that keep them, the
 * launches (one graph replay unless debug capture or graphs are off), the status read-back, the
 * colour read-back (deferred to finish_batch when a view keeps the caller's pixels, so that a
 * re-render still starts from them) and the lane's completion event. */
static int submit_batch(sftg_ctx* ctx, sftg_lane& ln, const sftg_frame_desc* fds, uint32_t nv, uint32_t* const* host_color,
                        const int32_t* pitch_bytes, sftg_debug_out* dbg, batch_bufs& B, bool& defer_colors) {
    auto pitch_of = [&](uint32_t v) { return (pitch_bytes && pitch_bytes[v] > 0) ? (size_t)pitch_bytes[v] : (size_t)fds[v].width * 4; };
    if (&ln != &ctx->lanes[0]) {   /* after every upload queued so far on lane 0's stream */
        CK(cudaEventRecord(ctx->ev_upload, ctx->stream));
        CK(cudaStreamWaitEvent(ln.stream, ctx->ev_upload, 0));
    }
    int rc;
    if ((rc = build_batch(ctx, ln, fds, nv, dbg != nullptr, B, host_color, pitch_bytes))) return rc;
    defer_colors = false;
    for (uint32_t v = 0; v < nv; v++)   /* the reference blends over / keeps the caller's pixels */
        if (!fds[v].clear && host_color && host_color[v] && !B.plan[v].direct) {
            defer_colors = true;
            CK(cudaMemcpy2DAsync(ln.d_color + B.plan[v].color_off, (size_t)fds[v].width * 4, host_color[v], pitch_of(v),
                                 (size_t)fds[v].width * 4, fds[v].height, cudaMemcpyHostToDevice, ln.stream));
        }
    if ((rc = (dbg || !ctx->use_graphs) ? launch_batch(ctx, ln, B) : launch_batch_graph(ctx, ln, B))) return rc;
    CK(cudaMemcpyAsync(ln.h_status, B.status, 4, cudaMemcpyDeviceToHost, ln.stream));
    CK(cudaMemcpyAsync(ln.h_status + 2, B.totals, 12, cudaMemcpyDeviceToHost, ln.stream));
    if (!defer_colors)
        for (uint32_t v = 0; v < nv; v++)
            if (host_color && host_color[v] && !B.plan[v].direct)
                CK(cudaMemcpy2DAsync(host_color[v], pitch_of(v), ln.d_color + B.plan[v].color_off, (size_t)fds[v].width * 4,
                                     (size_t)fds[v].width * 4, fds[v].height, cudaMemcpyDeviceToHost, ln.stream));
    CK(cudaEventRecord(ln.ev_done, ln.stream));
    return 0;
}

#define BATCH_REDO 1   /* finish_batch: a capacity was exceeded and has been grown; queue the batch again */

/* Waits for the lane's batch and checks it: capacities, phase timings, deferred colour
 * read-back, debug buffers, device colour pointers and the device status word. */
static int finish_batch(sftg_ctx* ctx, sftg_lane& ln, const sftg_frame_desc* fds, uint32_t nv, uint32_t* const* host_color,
                        const int32_t* pitch_bytes, const batch_bufs& B, bool defer_colors, sftg_debug_out* dbg,
                        const uint32_t** out_dev) {
    CK(cudaEventSynchronize(ln.ev_done));
    const uint32_t clip_total = ln.h_status[2], pay_total = ln.h_status[3], stile_total = ln.h_status[4];
    if (clip_total > ctx->clip_cap || pay_total > ctx->tile_cap || stile_total > ctx->stile_cap) {   /* capacity exceeded: grow and redo */
        while (ctx->clip_cap < clip_total) ctx->clip_cap *= 2;
        while (ctx->tile_cap < pay_total) ctx->tile_cap *= 2;
        while (ctx->stile_cap < stile_total) ctx->stile_cap *= 2;
        return BATCH_REDO;
    }
    for (int k = 0; k < 5; k++) {   /* geometry is timed from its own start: occlusion runs beside it */
        float t = 0.f;
        if (cudaEventElapsedTime(&t, k == 1 ? ln.ev_geo : ln.ev[k], ln.ev[k + 1]) != cudaSuccess) { t = 0.f; cudaGetLastError(); }
        ln.timings[k] = t;
        ctx->timings[k] = t;
    }
    ctx->launches = ln.launches;
    ctx->launch_total += (uint64_t)ln.launches;
    if (defer_colors) {
        auto pitch_of = [&](uint32_t v) { return (pitch_bytes && pitch_bytes[v] > 0) ? (size_t)pitch_bytes[v] : (size_t)fds[v].width * 4; };
        for (uint32_t v = 0; v < nv; v++)
            if (host_color && host_color[v] && !B.plan[v].direct)
                CK(cudaMemcpy2DAsync(host_color[v], pitch_of(v), ln.d_color + B.plan[v].color_off, (size_t)fds[v].width * 4,
                                     (size_t)fds[v].width * 4, fds[v].height, cudaMemcpyDeviceToHost, ln.stream));
        CK(cudaStreamSynchronize(ln.stream));
    }
    if (dbg) {
        const sftg_frame_desc* fd = &fds[0];
        const int W = fd->width, H = fd->height, S = fd->samples, tiles = (int)B.total_tiles;
        if (dbg->vis_depth) CK(cudaMemcpy(dbg->vis_depth, B.vis_depth, (size_t)tiles * S * 4096 * 4, cudaMemcpyDeviceToHost));
        if (dbg->vis_id) CK(cudaMemcpy(dbg->vis_id, B.vis_id, (size_t)tiles * S * 4096 * 4, cudaMemcpyDeviceToHost));
        if (dbg->tile_counts) CK(cudaMemcpy(dbg->tile_counts, B.tile_count, (size_t)tiles * 4, cudaMemcpyDeviceToHost));
        if (dbg->tile_payload_total) *dbg->tile_payload_total = pay_total;
        if (dbg->tile_payloads && pay_total <= dbg->tile_payload_cap) CK(cudaMemcpy(dbg->tile_payloads, B.tile_pay, (size_t)pay_total * 8, cudaMemcpyDeviceToHost));
        if (dbg->ss_cache) {   /* back to the reference's rows: sx sy inv_w wx wy wz wnx wny wnz, 64 each */
            std::vector<float> all((size_t)B.total_ss * SFTG_SS_FLOATS + 1);
            CK(cudaMemcpy(all.data(), B.ss, (size_t)B.total_ss * SFTG_SS_FLOATS * 4, cudaMemcpyDeviceToHost));
            for (uint32_t k = 0; k < B.total_ss; k++) {
                const float* rec = all.data() + (size_t)k * SFTG_SS_FLOATS;
                float* r = dbg->ss_cache + (size_t)k * 576;
                for (int v = 0; v < 64; v++) {
                    for (int c = 0; c < 4; c++) r[c * 64 + v] = rec[SFTG_SS_A + v * 4 + c];
                    for (int c = 0; c < 4; c++) r[(4 + c) * 64 + v] = rec[SFTG_SS_B + v * 4 + c];
                    r[8 * 64 + v] = rec[SFTG_SS_C + v * 4];
                }
            }
        }
        if (dbg->light_vis && fd->n_proxies) CK(cudaMemcpy(dbg->light_vis, B.light_vis, (size_t)fd->n_proxies * 64, cudaMemcpyDeviceToHost));
        if (dbg->clip_total) *dbg->clip_total = clip_total;
        if (dbg->clip_tris && clip_total <= dbg->clip_cap) CK(cudaMemcpy(dbg->clip_tris, B.clips, (size_t)clip_total * sizeof(sftg_clip_tri), cudaMemcpyDeviceToHost));
        if (dbg->shadow && S == 1) CK(cudaMemcpy(dbg->shadow, B.shadow, (size_t)W * H * 16 * 4, cudaMemcpyDeviceToHost));
        if (dbg->status) *dbg->status = ln.h_status[0];
    }
    if (out_dev) for (uint32_t v = 0; v < nv; v++) out_dev[v] = B.plan[v].direct ? B.plan[v].direct : ln.d_color + B.plan[v].color_off;
    if (ln.h_status[0] & 1u) return set_err(ctx, SFTG_E_DEVICE_STATUS, "occlusion traversal exceeded its stack bound");
    return SFTG_OK;
}

/* Renders a batch of views on lane 0 and waits for it.  host_color[v] (optional) receives view
 * v's colour with pitch pitch_bytes[v]; out_dev[v] (optional) its device colour buffer, valid
 * until the next synchronous call. */
static int batch_common(sftg_ctx* ctx, const sftg_frame_desc* fds, uint32_t nv, uint32_t* const* host_color, const int32_t* pitch_bytes,
                        sftg_debug_out* dbg, const uint32_t** out_dev) {
    if (!ctx || !fds) return SFTG_E_ARG;
    CK(cudaSetDevice(ctx->device));
    int rc = sync_tables(ctx);
    if (rc) return rc;
    sftg_lane& ln = ctx->lanes[0];
    for (int attempt = 0; attempt < 4; attempt++) {
        batch_bufs B;
        bool defer = false;
        if ((rc = submit_batch(ctx, ln, fds, nv, host_color, pitch_bytes, dbg, B, defer))) return rc;
        rc = finish_batch(ctx, ln, fds, nv, host_color, pitch_bytes, B, defer, dbg, out_dev);
        if (rc != BATCH_REDO) return rc;
    }
    return set_err(ctx, SFTG_E_NOMEM, "frame capacities did not converge");
}

extern "C" int sftg_frame_render(sftg_ctx* ctx, const sftg_frame_desc* fd, uint32_t* color, int32_t pitch_bytes, sftg_debug_out* dbg) {
    uint32_t* hc[1] = { color };
    const int32_t pb[1] = { pitch_bytes };
    return batch_common(ctx, fd, 1, color ? hc : nullptr, pb, dbg, nullptr);
}

extern "C" int sftg_frame_render_device(sftg_ctx* ctx, const sftg_frame_desc* fd, const uint32_t** out_device_color) {
    return batch_common(ctx, fd, 1, nullptr, nullptr, nullptr, out_device_color);
}

extern "C" int sftg_frames_render(sftg_ctx* ctx, const sftg_frame_desc* fds, uint32_t n_views, uint32_t* const* colors,
                                  const int32_t* pitch_bytes, const uint32_t** out_device_colors) {
    return batch_common(ctx, fds, n_views, colors, pitch_bytes, nullptr, out_device_colors);
}

/* ------------------------------------------------------------------ overlapping batches */
extern "C" int sftg_frames_submit(sftg_ctx* ctx, uint32_t lane, const sftg_frame_desc* fds, uint32_t n_views, uint32_t* const* colors,
                                  const int32_t* pitch_bytes) {
    if (!ctx || !fds || !n_views) return SFTG_E_ARG;
    if (lane == 0 || lane >= SFTG_MAX_LANES) return set_err(ctx, SFTG_E_ARG, "lane %u: lanes 1 to %d take submissions", lane, SFTG_MAX_LANES - 1);
    sftg_lane& ln = ctx->lanes[lane];
    if (ln.busy) return set_err(ctx, SFTG_E_ARG, "lane %u has a batch in flight", lane);
    CK(cudaSetDevice(ctx->device));
    int rc = sync_tables(ctx);
    if (rc) return rc;
    ln.fds = fds; ln.nv = n_views;
    ln.colors.assign(n_views, nullptr);
    ln.pitch.assign(n_views, 0);
    for (uint32_t v = 0; v < n_views; v++) {
        if (colors) ln.colors[v] = colors[v];
        if (pitch_bytes) ln.pitch[v] = pitch_bytes[v];
    }
    batch_bufs B;
    bool defer = false;
    if ((rc = submit_batch(ctx, ln, fds, n_views, ln.colors.data(), ln.pitch.data(), nullptr, B, defer))) return rc;
    ln.busy = true;
    if (defer) {   /* a view keeps the caller's pixels: finish now, so that a re-render can start from them */
        ln.busy = false;
        rc = finish_batch(ctx, ln, fds, n_views, ln.colors.data(), ln.pitch.data(), B, true, nullptr, nullptr);
        for (int attempt = 0; rc == BATCH_REDO && attempt < 4; attempt++) {
            batch_bufs B2;
            if ((rc = submit_batch(ctx, ln, fds, n_views, ln.colors.data(), ln.pitch.data(), nullptr, B2, defer))) return rc;
            rc = finish_batch(ctx, ln, fds, n_views, ln.colors.data(), ln.pitch.data(), B2, defer, nullptr, nullptr);
        }
        if (rc == BATCH_REDO) return set_err(ctx, SFTG_E_NOMEM, "frame capacities did not converge");
        ln.busy = rc == SFTG_OK;   /* sftg_lane_wait then returns at once */
        ln.fds = nullptr;
        return rc;
    }
    return SFTG_OK;
}

extern "C" int sftg_lane_done(sftg_ctx* ctx, uint32_t lane) {
    if (!ctx || lane >= SFTG_MAX_LANES) return SFTG_E_ARG;
    sftg_lane& ln = ctx->lanes[lane];
    if (!ln.busy || !ln.fds) return 1;
    const cudaError_t e = cudaEventQuery(ln.ev_done);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    return set_err(ctx, SFTG_E_CUDA, "lane %u: %s", lane, cudaGetErrorString(e));
}

extern "C" int sftg_lane_wait(sftg_ctx* ctx, uint32_t lane) {
    if (!ctx || lane == 0 || lane >= SFTG_MAX_LANES) return SFTG_E_ARG;
    sftg_lane& ln = ctx->lanes[lane];
    if (!ln.busy) return SFTG_OK;
    ln.busy = false;
    if (!ln.fds) return SFTG_OK;   /* finished inside sftg_frames_submit */
    CK(cudaSetDevice(ctx->device));
    const sftg_frame_desc* fds = ln.fds;
    ln.fds = nullptr;
    batch_bufs none;
    int rc = finish_batch(ctx, ln, fds, ln.nv, ln.colors.data(), ln.pitch.data(), none, false, nullptr, nullptr);
    for (int attempt = 0; rc == BATCH_REDO && attempt < 4; attempt++) {
        batch_bufs B;
        bool defer = false;
        if ((rc = submit_batch(ctx, ln, fds, ln.nv, ln.colors.data(), ln.pitch.data(), nullptr, B, defer))) return rc;
        rc = finish_batch(ctx, ln, fds, ln.nv, ln.colors.data(), ln.pitch.data(), B, defer, nullptr, nullptr);
    }
    if (rc == BATCH_REDO) return set_err(ctx, SFTG_E_NOMEM, "frame capacities did not converge");
    return rc;
}

/* ------------------------------------------------------------------ skeletal poses */
/* appends n records of T to a pool whose element count is tracked in count (pool_append aligns
 * byte offsets to 256, so element arrays are appended at exact element offsets instead) */
template <class T>
static int pool_push(sftg_ctx* ctx, dpool& p, uint32_t& count, const T* src, size_t n) {
    const size_t off = (size_t)count * sizeof(T);
    int rc = pool_reserve(ctx, p, off + n * sizeof(T) + 16);
    if (rc) return rc;
    if (n) CK(cudaMemcpyAsync((char*)p.ptr + off, src, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
    p.size = off + n * sizeof(T);
    count += (uint32_t)n;
    return 0;
}

extern "C" int sftg_skeleton_upload(sftg_ctx* ctx, const sftg_bone_desc* bones, uint32_t bone_count, const sftg_animation_desc* anims,
                                    uint32_t anim_count, int32_t* out_skeleton) {
    if (!ctx || !bones || !bone_count || (anim_count && !anims)) return SFTG_E_ARG;
    if (bone_count > SFTG_MAX_BONES) return set_err(ctx, SFTG_E_LIMIT, "skeleton of %u bones (at most %d)", bone_count, SFTG_MAX_BONES);
    CK(cudaSetDevice(ctx->device));
    /* parents first, level by level; parent indices must be in range and acyclic */
    std::vector<int> depth(bone_count, -1);
    for (uint32_t b = 0; b < bone_count; b++) {
        if (bones[b].parent >= (int32_t)bone_count) return set_err(ctx, SFTG_E_ARG, "bone %u: parent %d out of range", b, bones[b].parent);
        int d = 0, q = (int)b;
        while (bones[q].parent >= 0) { q = bones[q].parent; if (++d > (int)bone_count) return set_err(ctx, SFTG_E_ARG, "bone hierarchy has a cycle"); }
        depth[b] = d;
    }
    const int levels = *std::max_element(depth.begin(), depth.end()) + 1;
    std::vector<uint16_t> order, lv;
    for (int L = 0; L < levels; L++) {
        lv.push_back((uint16_t)order.size());
        for (uint32_t b = 0; b < bone_count; b++) if (depth[b] == L) order.push_back((uint16_t)b);
    }
    lv.push_back((uint16_t)order.size());
    std::vector<sftg_bone_dev> bd(bone_count);
    for (uint32_t b = 0; b < bone_count; b++) {
        memcpy(bd[b].inverse_bind, bones[b].inverse_bind, 64); memcpy(bd[b].local_bind, bones[b].local_bind, 64);
        bd[b].parent = bones[b].parent;
        memcpy(bd[b].base_t, bones[b].base_t, 12); memcpy(bd[b].base_r, bones[b].base_r, 16); memcpy(bd[b].base_s, bones[b].base_s, 12);
    }
    sftg_skel_dev sk;
    memset(&sk, 0, sizeof(sk));
    sk.bone_base = ctx->n_bones; sk.bone_count = bone_count;
    sk.anim_base = ctx->n_anims; sk.anim_count = anim_count;
    sk.order_base = ctx->n_order; sk.level_base = ctx->n_levels; sk.level_count = (uint32_t)levels;
    std::vector<sftg_anim_dev> ad(anim_count);
    std::vector<sftg_sampler_dev> sd;
    std::vector<sftg_channel_desc> cd;
    std::vector<float> keys;
    for (uint32_t a = 0; a < anim_count; a++) {
        const sftg_animation_desc& A = anims[a];
        if (A.sampler_count < 0 || A.channel_count < 0 || (A.sampler_count && !A.samplers) || (A.channel_count && !A.channels))
            return set_err(ctx, SFTG_E_ARG, "animation %u: bad arrays", a);
        ad[a].sampler_base = ctx->n_samplers + (uint32_t)sd.size(); ad[a].channel_base = ctx->n_channels + (uint32_t)cd.size();
        ad[a].sampler_count = A.sampler_count; ad[a].channel_count = A.channel_count; ad[a].duration = A.duration;
        for (int k = 0; k < A.sampler_count; k++) {
            const sftg_sampler_desc& S = A.samplers[k];
            if (S.count < 1 || !S.inputs || !S.outputs) return set_err(ctx, SFTG_E_ARG, "animation %u sampler %d: no keyframes", a, k);
            sftg_sampler_dev d;
            d.input_base = ctx->n_keys + (uint32_t)keys.size(); keys.insert(keys.end(), S.inputs, S.inputs + S.count);
            d.output_base = ctx->n_keys + (uint32_t)keys.size(); keys.insert(keys.end(), S.outputs, S.outputs + (size_t)S.count * 4);
            d.count = S.count; d.is_step = S.is_step;
            sd.push_back(d);
        }
        for (int k = 0; k < A.channel_count; k++) {
            const sftg_channel_desc& C = A.channels[k];
            if (C.sampler < 0 || C.sampler >= A.sampler_count || C.path < 0 || C.path > 2)
                return set_err(ctx, SFTG_E_ARG, "animation %u channel %d: bad sampler or path", a, k);
            cd.push_back(C);
        }
    }
    int rc;
    if ((rc = pool_push(ctx, ctx->p_bones, ctx->n_bones, bd.data(), bd.size())) ||
        (rc = pool_push(ctx, ctx->p_anims, ctx->n_anims, ad.data(), ad.size())) ||
        (rc = pool_push(ctx, ctx->p_samplers, ctx->n_samplers, sd.data(), sd.size())) ||
        (rc = pool_push(ctx, ctx->p_channels, ctx->n_channels, cd.data(), cd.size())) ||
        (rc = pool_push(ctx, ctx->p_keys, ctx->n_keys, keys.data(), keys.size())) ||
        (rc = pool_push(ctx, ctx->p_order, ctx->n_order, order.data(), order.size())) ||
        (rc = pool_push(ctx, ctx->p_levels, ctx->n_levels, lv.data(), lv.size())))
        return rc;
    ctx->h_skels.push_back(sk);
    uint32_t ns = (uint32_t)ctx->h_skels.size() - 1;
    if ((rc = pool_push(ctx, ctx->p_skels, ns, &sk, 1))) return rc;
    CK(cudaStreamSynchronize(ctx->stream));
    if (out_skeleton) *out_skeleton = (int32_t)ctx->h_skels.size() - 1;
    return SFTG_OK;
}

static sftg_pose_tables pose_tables(const sftg_ctx* ctx) {
    sftg_pose_tables T;
    T.n_skels = (uint32_t)ctx->h_skels.size();
    T.skels = (const sftg_skel_dev*)ctx->p_skels.ptr; T.bones = (const sftg_bone_dev*)ctx->p_bones.ptr;
    T.anims = (const sftg_anim_dev*)ctx->p_anims.ptr; T.samplers = (const sftg_sampler_dev*)ctx->p_samplers.ptr;
    T.channels = (const sftg_channel_desc*)ctx->p_channels.ptr; T.keys = (const float*)ctx->p_keys.ptr;
    T.order = (const uint16_t*)ctx->p_order.ptr; T.levels = (const uint16_t*)ctx->p_levels.ptr;
    return T;
}

extern "C" int sftg_pose_eval_device(sftg_ctx* ctx, const sftg_pose_request* d_reqs, const uint32_t* d_off, uint32_t n, float* d_posed,
                                     float* d_global) {
    if (!ctx || (n && (!d_reqs || !d_off || !d_posed))) return SFTG_E_ARG;
    if (!n) return SFTG_OK;
    CK(cudaSetDevice(ctx->device));
    if (ctx->h_skels.empty()) return set_err(ctx, SFTG_E_ARG, "no skeleton uploaded");
    sftg_launch_pose(pose_tables(ctx), d_reqs, d_off, n, d_posed, d_global, ctx->stream);
    CK(cudaGetLastError());
    return SFTG_OK;
}

extern "C" int sftg_pose_eval(sftg_ctx* ctx, const sftg_pose_request* reqs, uint32_t n, float* posed, float* global) {
    if (!ctx || (n && (!reqs || !posed))) return SFTG_E_ARG;
    if (!n) return SFTG_OK;
    CK(cudaSetDevice(ctx->device));
    std::vector<uint32_t> off(n);
    uint32_t total = 0;
    for (uint32_t k = 0; k < n; k++) {
        if (reqs[k].skeleton < 0 || (size_t)reqs[k].skeleton >= ctx->h_skels.size())
            return set_err(ctx, SFTG_E_ARG, "pose request %u: bad skeleton %d", k, reqs[k].skeleton);
        off[k] = total;
        total += ctx->h_skels[reqs[k].skeleton].bone_count;
    }
    /* device io: requests, offsets, posed, global */
    const size_t b_req = ((size_t)n * sizeof(sftg_pose_request) + 255) & ~(size_t)255, b_off = ((size_t)n * 4 + 255) & ~(size_t)255;
    const size_t b_mat = (size_t)total * 64;
    int rc = pool_reserve(ctx, ctx->p_pose_io, b_req + b_off + 2 * b_mat + 256);
    if (rc) return rc;
    char* io = (char*)ctx->p_pose_io.ptr;
    sftg_pose_request* d_req = (sftg_pose_request*)io;
    uint32_t* d_off = (uint32_t*)(io + b_req);
    float* d_posed = (float*)(io + b_req + b_off);
    float* d_global = global ? d_posed + (size_t)total * 16 : nullptr;
    CK(cudaMemcpyAsync(d_req, reqs, (size_t)n * sizeof(sftg_pose_request), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(d_off, off.data(), (size_t)n * 4, cudaMemcpyHostToDevice, ctx->stream));
    sftg_launch_pose(pose_tables(ctx), d_req, d_off, n, d_posed, d_global, ctx->stream);
    CK(cudaGetLastError());
    /* a request with an out-of-range animation leaves its matrices as they were: those are saved,
     * the whole result is copied straight into the caller's arrays, and the saved ones put back */
    std::vector<uint32_t> keep;
    size_t keep_floats = 0;
    for (uint32_t k = 0; k < n; k++) {
        const sftg_skel_dev& sk = ctx->h_skels[reqs[k].skeleton];
        if (reqs[k].animation < 0 || (uint32_t)reqs[k].animation >= sk.anim_count) { keep.push_back(k); keep_floats += (size_t)sk.bone_count * 16; }
    }
    std::vector<float> saved(keep_floats * (global ? 2 : 1));
    size_t q = 0;
    for (uint32_t k : keep) {
        const size_t c = (size_t)ctx->h_skels[reqs[k].skeleton].bone_count * 16;
        memcpy(saved.data() + q, posed + (size_t)off[k] * 16, c * 4); q += c;
        if (global) { memcpy(saved.data() + q, global + (size_t)off[k] * 16, c * 4); q += c; }
    }
    CK(cudaMemcpyAsync(posed, d_posed, b_mat, cudaMemcpyDeviceToHost, ctx->stream));
    if (global) CK(cudaMemcpyAsync(global, d_global, b_mat, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    q = 0;
    for (uint32_t k : keep) {
        const size_t c = (size_t)ctx->h_skels[reqs[k].skeleton].bone_count * 16;
        memcpy(posed + (size_t)off[k] * 16, saved.data() + q, c * 4); q += c;
        if (global) { memcpy(global + (size_t)off[k] * 16, saved.data() + q, c * 4); q += c; }
    }
    return SFTG_OK;
}

/* ------------------------------------------------------------------ ray queries */
extern "C" int sftg_raycast_device(sftg_ctx* ctx, const sftg_ray* d_rays, uint32_t n, sftg_ray_hit* d_hits) {
    if (!ctx || (n && (!d_rays || !d_hits))) return SFTG_E_ARG;
    if (!n) return SFTG_OK;
    CK(cudaSetDevice(ctx->device));
    int rc = sync_tables(ctx);   /* the device model table follows uploads lazily */
    if (rc) return rc;
    sftg_launch_raycast(d_rays, n, (const sftg_model*)ctx->models.ptr, (uint32_t)ctx->h_models.size(), (const sftg_bvh_node*)ctx->blas.ptr,
                        (const float*)ctx->ml_attr.ptr, (const uint8_t*)ctx->ml_inds.ptr, d_hits, ctx->stream);
    CK(cudaGetLastError());
    return SFTG_OK;
}

extern "C" int sftg_raycast(sftg_ctx* ctx, const sftg_ray* rays, uint32_t n, sftg_ray_hit* hits) {
    if (!ctx || (n && (!rays || !hits))) return SFTG_E_ARG;
    if (!n) return SFTG_OK;
    CK(cudaSetDevice(ctx->device));
    const size_t b_ray = ((size_t)n * sizeof(sftg_ray) + 255) & ~(size_t)255;
    int rc = pool_reserve(ctx, ctx->p_ray_io, b_ray + (size_t)n * sizeof(sftg_ray_hit) + 256);
    if (rc) return rc;
    sftg_ray* d_rays = (sftg_ray*)ctx->p_ray_io.ptr;
    sftg_ray_hit* d_hits = (sftg_ray_hit*)((char*)ctx->p_ray_io.ptr + b_ray);
    CK(cudaMemcpyAsync(d_rays, rays, (size_t)n * sizeof(sftg_ray), cudaMemcpyHostToDevice, ctx->stream));
    if ((rc = sftg_raycast_device(ctx, d_rays, n, d_hits))) return rc;
    CK(cudaMemcpyAsync(hits, d_hits, (size_t)n * sizeof(sftg_ray_hit), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (uint32_t k = 0; k < n; k++)
        if (hits[k].hit == 2) return set_err(ctx, SFTG_E_DEVICE_STATUS, "ray %u: BLAS walk overflowed its stack", k);
    return SFTG_OK;
}

/* ------------------------------------------------------------------ tuning */
static bool tuning_valid(const sftg_tuning* t) {
    for (int k = 0; k < 3; k++) {
        const int sp = t->resolve_split[k], sl = t->raster_slab_rows[k];
        if (!(sp == 1 || sp == 2 || sp == 4 || sp == 8 || sp == 16)) return false;
        if (sl < 4 || sl > 64) return false;
        const int rb = t->raster_bands[k];
        if (!(rb == 0 || rb == 1 || rb == 2 || rb == 4)) return false;
        if (t->tile_lights[k] < 0 || t->tile_lights[k] > 2) return false;
    }
    return t->geom_job_width >= 1 && t->geom_job_width <= 8 && (t->occl_ray_prune == 0 || t->occl_ray_prune == 1) &&
           t->tile_queue >= 0 && t->tile_queue <= 3;
}

extern "C" int sftg_get_tuning(const sftg_ctx* ctx, sftg_tuning* out) {
    if (!ctx || !out) return SFTG_E_ARG;
    *out = ctx->tuning;
    return SFTG_OK;
}

extern "C" int sftg_set_tuning(sftg_ctx* ctx, const sftg_tuning* t) {
    if (!ctx || !t) return SFTG_E_ARG;
    if (!tuning_valid(t)) return set_err(ctx, SFTG_E_ARG, "tuning out of range (split 1/2/4/8/16, slab rows 4..64, job width 1..8, raster bands 0/1/2/4, tile lights 0/1/2, tile queue 0-3)");
    ctx->tuning = *t;
    return SFTG_OK;
}

/* median over reps renders of one phase's device time (ms) */
static int time_phase(sftg_ctx* ctx, const sftg_frame_desc* fds, uint32_t n, int reps, int phase, float* out) {
    std::vector<float> t;
    for (int r = 0; r < reps; r++) {
        const int rc = batch_common(ctx, fds, n, nullptr, nullptr, nullptr, nullptr);
        if (rc) return rc;
        t.push_back(phase < 0 ? ctx->timings[3] + ctx->timings[4] : ctx->timings[phase]);   /* -1: raster + resolve */
    }
    std::sort(t.begin(), t.end());
    *out = t[t.size() / 2];
    return 0;
}

/* Coordinate search over the knobs that change only scheduling, never results: the geometry
 * job width against the geometry phase, then per sample count the raster slab height and the
 * raster bands against the raster phase and the resolve split with the tile light lists against
 * the resolve phase, each measured on the views with that sample count, then the persistent tile
 * queue against raster + resolve of all views.  Leaves the best setting in the context. */
extern "C" int sftg_autotune(sftg_ctx* ctx, const sftg_frame_desc* fds, uint32_t n_views, int32_t reps, sftg_tuning* out) {
    if (!ctx || !fds || !n_views) return SFTG_E_ARG;
    if (reps < 1) reps = 5;
    sftg_tuning best = ctx->tuning;
    int rc;
    if ((rc = batch_common(ctx, fds, n_views, nullptr, nullptr, nullptr, nullptr))) return rc;   /* warm: arena, tables */
    {
        const int widths[4] = { 1, 2, 4, 8 };
        float bt = 1e30f;
        for (int k = 0; k < 4; k++) {
            ctx->tuning = best; ctx->tuning.geom_job_width = widths[k];
            float t;
            if ((rc = time_phase(ctx, fds, n_views, reps, 1, &t))) { ctx->tuning = best; return rc; }
            if (t < bt) { bt = t; best.geom_job_width = widths[k]; }
        }
    }
    for (int si = 0; si < 3; si++) {
        std::vector<sftg_frame_desc> sub;
        for (uint32_t v = 0; v < n_views; v++) if (fds[v].samples == (1 << si)) sub.push_back(fds[v]);
        if (sub.empty()) continue;
        const int slabs[5] = { 4, 8, 16, 32, 64 };
        float bt = 1e30f;
        for (int k = 0; k < 5; k++) {
            ctx->tuning = best; ctx->tuning.raster_slab_rows[si] = slabs[k];
            float t;
            if ((rc = time_phase(ctx, sub.data(), (uint32_t)sub.size(), reps, 3, &t))) { ctx->tuning = best; return rc; }
            if (t < bt) { bt = t; best.raster_slab_rows[si] = slabs[k]; }
        }
        const int bands[4] = { 0, 1, 2, 4 };
        bt = 1e30f;
        for (int k = 0; k < 4; k++) {
            ctx->tuning = best; ctx->tuning.raster_bands[si] = bands[k];
            float t;
            if ((rc = time_phase(ctx, sub.data(), (uint32_t)sub.size(), reps, 3, &t))) { ctx->tuning = best; return rc; }
            if (t < bt) { bt = t; best.raster_bands[si] = bands[k]; }
        }
        /* resolve split and where the tile light lists are made, jointly: per-tile lists take the
         * split-fold selection work out of every CTA, which favours higher splits */
        const int splits[5] = { 4, 8, 16, 2, 1 };
        bt = 1e30f;
        for (int k = 0; k < 5; k++)
            for (int m = 1; m <= 2; m++) {
                ctx->tuning = best; ctx->tuning.resolve_split[si] = splits[k]; ctx->tuning.tile_lights[si] = m;
                float t;
                if ((rc = time_phase(ctx, sub.data(), (uint32_t)sub.size(), reps, 4, &t))) { ctx->tuning = best; return rc; }
                if (t < bt) { bt = t; best.resolve_split[si] = splits[k]; best.tile_lights[si] = m; }
            }
    }
    {   /* the persistent tile queue, against raster + resolve of all views */
        float bt = 1e30f;
        for (int q = 0; q <= 3; q++) {
            ctx->tuning = best; ctx->tuning.tile_queue = q;
            float t;
            if ((rc = time_phase(ctx, fds, n_views, reps, -1, &t))) { ctx->tuning = best; return rc; }
            if (t < bt) { bt = t; best.tile_queue = q; }
        }
    }
    ctx->tuning = best;
    if (out) *out = best;
    return SFTG_OK;
}

extern "C" int sftg_last_timings(const sftg_ctx* ctx, float* out5) {
    if (!ctx || !out5) return SFTG_E_ARG;
    for (int k = 0; k < 5; k++) out5[k] = ctx->timings[k];
    return SFTG_OK;
}

extern "C" int sftg_last_launch_count(const sftg_ctx* ctx) { return ctx ? ctx->launches : 0; }
extern "C" uint64_t sftg_launch_total(const sftg_ctx* ctx) { return ctx ? ctx->launch_total : 0; }
extern "C" int sftg_last_blas_build(const sftg_ctx* ctx, double* wall_ms, double* stream_ms, uint32_t* items, uint32_t* launches) {
    if (!ctx) return SFTG_E_ARG;
    if (wall_ms) *wall_ms = ctx->blas_ms;
    if (stream_ms) *stream_ms = ctx->blas_stream_ms;
    if (items) *items = ctx->blas_items;
    if (launches) *launches = ctx->blas_launches;
    return SFTG_OK;
}

extern "C" void* sftg_stream(const sftg_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

/* ------------------------------------------------------------------ allocation-free light visibility
 *
 * sftg_light_vis_noalloc runs the proxy-occlusion pass (sft_present's light visibility,
 * sofren2.c:8163-8280) without touching any allocator.  It is for callers that must not
 * allocate while they run: a serving loop whose admission control has already committed the
 * device-memory budget (a cudaMalloc there can fail, or take memory promised to a resident
 * scene), and per-frame code on a latency deadline (cudaMalloc / cudaFree can synchronise the
 * whole device).  The context's frame arena and pinned staging may need to grow and so are
 * not used; all scratch lives in one file-scope device array of SFTG_NOALLOC_SCRATCH_BYTES
 * whose address is looked up once per device.
 *
 * Scratch layout (each part 256-byte aligned): frame block, instances, point lights (first 64),
 * proxies, TLAS nodes, shadow packets, (packet, instance) pairs, pair counter, status word,
 * light_vis rows, packet -> view and proxy -> view maps.  What must start at zero, and is
 * cleared by this call with cudaMemsetAsync: the pair counter, the status word, the light_vis
 * rows (columns at or beyond the light count are never written) and both maps (one view).
 *
 * The scratch is shared by every context on the device: two calls that overlap in time, from
 * any threads or contexts, race on it.  Callers serialise them.
 *
 * The array's device address is looked up when a context is created on the device
 * (noalloc_scratch_setup, from sftg_create).  The lookup loads the module that holds the array,
 * which is when the 4 MiB are committed on the device: with CUDA's lazy module loading that
 * would otherwise happen inside the first allocation-free call. */
#define SFTG_NOALLOC_MAX_DEVICES 64
static __device__ __align__(256) unsigned char g_noalloc_scratch[SFTG_NOALLOC_SCRATCH_BYTES];
static void* g_noalloc_addr[SFTG_NOALLOC_MAX_DEVICES];

/* with `device` current: the host-side name g_noalloc_scratch is only a stand-in, the kernels
 * need the address the runtime gives for it on this device */
static cudaError_t noalloc_scratch_setup(int device) {
    if (device < 0 || device >= SFTG_NOALLOC_MAX_DEVICES) return cudaSuccess;   /* the entry point refuses such devices */
    if (g_noalloc_addr[device]) return cudaSuccess;
    void* a = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&a, g_noalloc_scratch);
    if (e == cudaSuccess) g_noalloc_addr[device] = a;
    return e;
}

extern "C" int sftg_light_vis_noalloc(sftg_ctx* ctx, const sftg_frame_desc* fd, uint8_t* light_vis) {
    if (!ctx || !fd) return SFTG_E_ARG;
    if (ctx->device < 0 || ctx->device >= SFTG_NOALLOC_MAX_DEVICES) return set_err(ctx, SFTG_E_ARG, "device %d out of range", ctx->device);
    if (fd->n_proxies && !light_vis) return set_err(ctx, SFTG_E_ARG, "light_vis output is NULL");
    if (fd->n_instances > SFTG_MAX_INSTANCES) return set_err(ctx, SFTG_E_LIMIT, "more than %d instances in one frame", SFTG_MAX_INSTANCES);
    if (ctx->tables_dirty)   /* copying the model table may have to grow its device pool */
        return set_err(ctx, SFTG_E_ARG, "models changed since the last render: render one frame first");
    for (uint32_t i = 0; i < fd->n_instances; i++)
        if (fd->instances[i].model < 0 || (size_t)fd->instances[i].model >= ctx->h_models.size())
            return set_err(ctx, SFTG_E_ARG, "instance %u: bad model", i);
    const uint32_t np = fd->n_proxies, lc = fd->n_point < 64 ? fd->n_point : 64, nbatch = (np + 7) / 8;
    const uint32_t n_packets = (fd->shadows && lc && np) ? lc * nbatch * 3 : 0;
    const uint64_t max_pairs = (uint64_t)n_packets * (fd->n_instances ? fd->n_instances : 1);
    size_t off = 0;
    auto take = [&](uint64_t bytes) { off = (off + 255) & ~(size_t)255; const size_t r = off; off += (size_t)bytes; return r; };
    const size_t o_F = take(sizeof(sftg_frame)), o_inst = take((uint64_t)(fd->n_instances + 1) * sizeof(sftg_inst));
    const size_t o_pl = take((uint64_t)lc * sizeof(sftg_point_light)), o_px = take((uint64_t)np * sizeof(sftg_proxy));
    const size_t o_tl = take((uint64_t)fd->tlas_count * 256), o_pk = take((uint64_t)n_packets * sftg_packet_bytes());
    const size_t o_pr = take(max_pairs * (1 + SFTG_OCC_ITEMS_PER_PAIR_NOALLOC) * 8 + 8), o_np = take(16), o_st = take(16), o_lv = take((uint64_t)np * 64);
    const size_t o_pv = take((uint64_t)n_packets * 2), o_xv = take((uint64_t)np * 2);
    if (off > SFTG_NOALLOC_SCRATCH_BYTES)
        return set_err(ctx, SFTG_E_LIMIT, "frame needs %zu bytes of occlusion scratch; the static scratch holds %u (%u proxies, %u lights, %u instances)",
                       off, (unsigned)SFTG_NOALLOC_SCRATCH_BYTES, np, fd->n_point, fd->n_instances);
    if (!np) return SFTG_OK;
    CK(cudaSetDevice(ctx->device));
    CK(noalloc_scratch_setup(ctx->device));   /* done by sftg_create; a no-op here */
    char* d = (char*)g_noalloc_addr[ctx->device];
    cudaStream_t st = ctx->stream;
    sftg_frame F;
    memset(&F, 0, sizeof(F));
    F.width = fd->width; F.height = fd->height; F.samples = fd->samples; F.shadows = fd->shadows;
    F.n_point = lc; F.n_proxies = np; F.n_inst = fd->n_instances;
    F.tlas_root = fd->tlas_root; F.tlas_count = fd->tlas_count;
    F.n_packets = n_packets;
    F.inst = (const sftg_inst*)(d + o_inst);
    F.point = (const sftg_point_light*)(d + o_pl);
    F.proxies = (const sftg_proxy*)(d + o_px);
    F.tlas = (const sftg_bvh_node*)(d + o_tl);
    F.models = (const sftg_model*)ctx->models.ptr;
    F.ml_attr = (const float*)ctx->ml_attr.ptr;
    F.ml_inds = (const uint8_t*)ctx->ml_inds.ptr;
    F.ml_info = (const sftg_meshlet_info*)ctx->ml_info.ptr;
    F.blas = (const sftg_bvh_node*)ctx->blas.ptr;
    sftg_inst inst[SFTG_MAX_INSTANCES + 1];
    memset(inst, 0, sizeof(inst));
    for (uint32_t i = 0; i < fd->n_instances; i++) {
        const sftg_instance_desc& id = fd->instances[i];
        memcpy(inst[i].T, id.transform, 64);
        inst[i].model = (uint32_t)id.model;
        inst[i].bones = -1;
        inst[i].meshlet_base = ctx->h_models[id.model].meshlet_base;
    }
    /* pageable sources: each copy returns once its source has been read */
    CK(cudaMemcpyAsync(d + o_F, &F, sizeof(F), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d + o_inst, inst, (size_t)(fd->n_instances + 1) * sizeof(sftg_inst), cudaMemcpyHostToDevice, st));
    if (lc) CK(cudaMemcpyAsync(d + o_pl, fd->point_lights, (size_t)lc * 32, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(d + o_px, fd->proxies, (size_t)np * 32, cudaMemcpyHostToDevice, st));
    if (fd->tlas_count) CK(cudaMemcpyAsync(d + o_tl, fd->tlas_nodes, (size_t)fd->tlas_count * 256, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(d + o_st, 0, 16, st));
    CK(cudaMemsetAsync(d + o_lv, 0, (size_t)np * 64, st));
    if (n_packets) {
        CK(cudaMemsetAsync(d + o_pv, 0, (size_t)n_packets * 2, st));
        CK(cudaMemsetAsync(d + o_xv, 0, (size_t)np * 2, st));
        sftg_launch_occlusion((const sftg_frame*)(d + o_F), (const uint16_t*)(d + o_pv), n_packets, (const uint16_t*)(d + o_xv), np,
                              fd->n_instances, d + o_pk, (uint2*)(d + o_pr), (uint32_t*)(d + o_np), (uint32_t)max_pairs, SFTG_OCC_ITEMS_PER_PAIR_NOALLOC,
                              (uint8_t*)(d + o_lv), (uint32_t*)(d + o_st), 0, st);
        CK(cudaGetLastError());
    }
    uint32_t status = 0;
    CK(cudaMemcpyAsync(light_vis, d + o_lv, (size_t)np * 64, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&status, d + o_st, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (status & 1u) return set_err(ctx, SFTG_E_DEVICE_STATUS, "occlusion traversal exceeded its stack bound");
    return SFTG_OK;
}
