/*
 * Served rendering: a native request loop over resident scenes.
 *
 * Requests arrive on a schedule (arrival times relative to the start of the run).  The loop
 * runs on one host thread and keeps no request waiting while the GPU is idle: whenever it is
 * free it takes every request that has arrived, in arrival order, as long as the batch stays
 * within max_batch requests and the memory budget (the sum of the requests' estimated device
 * bytes), and renders them as one batched submission (sft_batch_begin / sft_present per request
 * / sft_batch_submit, one launch per pipeline stage for the whole batch).  A request's latency
 * runs from its arrival to the moment its pixels are in its host colour buffer.  With plain
 * set, every request is rendered on its own with sft_present instead, for comparison.
 *
 * No counterpart in the reference, which renders one view per sft_present call.
 */
#define SFT_FUNC __attribute__((visibility("default")))
#include "../../include/sofren2.h"

#include <stdint.h>
#include <string.h>
#include <time.h>

#define SFTX_EXPORT __attribute__((visibility("default")))

SFTX_EXPORT int sftx_scene_render_ex(void* p, uint32_t frame, uint32_t* color, int32_t pitch_bytes, uint32_t max_point_lights);

typedef struct sftx_request {
    uint64_t arrival_ns;       /* from the start of the run */
    uint64_t device_bytes;     /* estimated device memory while in flight (admission) */
    uint32_t scene;            /* index into the scenes array */
    uint32_t frame;            /* frame of that scene: camera, size, pose */
    int32_t samples;           /* MSAA 1, 2 or 4 */
    uint32_t max_point_lights;
} sftx_request;

typedef struct sftx_serve_stats {
    uint64_t batches;
    uint64_t max_batch;        /* largest batch formed */
    uint64_t peak_bytes;       /* largest admitted batch, estimated device bytes */
    uint64_t errors;
} sftx_serve_stats;

static uint64_t sftx_now_ns(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (uint64_t)ts.tv_sec * 1000000000ull + (uint64_t)ts.tv_nsec;
}

static void sftx_wait_until(uint64_t t0, uint64_t at) {
    for (;;) {
        const uint64_t now = sftx_now_ns() - t0;
        if (now >= at) return;
        const uint64_t left = at - now;
        if (left > 200000u) {   /* sleep through all but the last 0.1 ms, then spin */
            struct timespec d = { 0, (long)(left - 100000u) };
            nanosleep(&d, NULL);
        }
    }
}

/* Serves n requests sorted by arrival.  colors[k % n_colors] (pitch: the request's width * 4)
 * receives request k's pixels; n_colors must be at least max_batch.  done_ns[k] is the
 * completion time of request k from the start of the run, batch_of[k] (optional) its batch. */
SFTX_EXPORT int sftx_serve(void* const* scenes, const sftx_request* reqs, uint32_t n, uint32_t max_batch, uint64_t budget_bytes,
                           int plain, uint32_t* const* colors, uint32_t n_colors, uint64_t* done_ns, uint32_t* batch_of,
                           sftx_serve_stats* stats) {
    if (!scenes || (!reqs && n) || !colors || !done_ns || max_batch == 0 || n_colors < max_batch) return -1;
    sftx_serve_stats st;
    memset(&st, 0, sizeof(st));
    const uint64_t t0 = sftx_now_ns();
    uint32_t next = 0;
    while (next < n) {
        if (reqs[next].arrival_ns > sftx_now_ns() - t0) sftx_wait_until(t0, reqs[next].arrival_ns);
        const uint64_t now = sftx_now_ns() - t0;
        /* admission: arrived requests in order, within the batch size and the memory budget */
        uint32_t end = next;
        uint64_t bytes = 0;
        const uint32_t cap = plain ? 1u : max_batch;
        while (end < n && end - next < cap && reqs[end].arrival_ns <= now) {
            if (end > next && bytes + reqs[end].device_bytes > budget_bytes) break;
            bytes += reqs[end].device_bytes;
            end++;
        }
        if (plain) {
            const sftx_request* r = &reqs[next];
            sft_set_msaa_samples(r->samples);
            if (sftx_scene_render_ex(scenes[r->scene], r->frame, colors[next % n_colors], 0, r->max_point_lights)) st.errors++;
        } else {
            sft_batch_begin();
            for (uint32_t k = next; k < end; k++) {
                const sftx_request* r = &reqs[k];
                sft_set_msaa_samples(r->samples);
                if (sftx_scene_render_ex(scenes[r->scene], r->frame, colors[k % n_colors], 0, r->max_point_lights)) st.errors++;
            }
            if (sft_batch_submit()) st.errors++;
        }
        const uint64_t done = sftx_now_ns() - t0;
        for (uint32_t k = next; k < end; k++) {
            done_ns[k] = done;
            if (batch_of) batch_of[k] = (uint32_t)st.batches;
        }
        st.batches++;
        if (end - next > st.max_batch) st.max_batch = end - next;
        if (bytes > st.peak_bytes) st.peak_bytes = bytes;
        next = end;
    }
    if (stats) *stats = st;
    return st.errors ? -2 : 0;
}
