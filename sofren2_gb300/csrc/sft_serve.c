/*
 * Served rendering: a native request loop over resident scenes.
 *
 * Requests arrive on a schedule (arrival times relative to the start of the run).  The loop
 * runs on one host thread.  A request's latency runs from its arrival to the moment its pixels
 * are in its host colour buffer.  Three modes:
 *   SFTX_SERVE_OVERLAP  continuous batching: up to SFTG_MAX_LANES - 1 batches in flight, one per
 *                       submission lane.  Whenever a lane is free, the requests that have
 *                       arrived, in arrival order, within max_batch and the memory budget
 *                       (estimated device bytes of every request in flight), are recorded
 *                       (sft_batch_begin / sft_present per request) and queued on that lane
 *                       (sft_batch_submit_async); they run on the GPU beside the batches
 *                       already there.  Finished lanes are collected as they complete.
 *   SFTX_SERVE_BATCHED  one batch at a time: formed as above whenever the GPU is free, rendered
 *                       with sft_batch_submit and waited for.
 *   SFTX_SERVE_PLAIN    every request on its own with sft_present, for comparison.
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
    uint64_t max_inflight;     /* most batches on the GPU at once (SFTX_SERVE_OVERLAP) */
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

#define SFTX_SERVE_BATCHED 0
#define SFTX_SERVE_PLAIN 1
#define SFTX_SERVE_OVERLAP 2

/* the requests that have arrived by `now`, from `next` on, within max_batch and the budget
 * left after `inflight` bytes; at least one when the GPU holds nothing else */
static uint32_t sftx_admit(const sftx_request* reqs, uint32_t n, uint32_t next, uint64_t now, uint32_t cap, uint64_t budget,
                           uint64_t inflight, uint64_t* bytes_out) {
    uint32_t end = next;
    uint64_t bytes = 0;
    while (end < n && end - next < cap && reqs[end].arrival_ns <= now) {
        if ((end > next || inflight) && inflight + bytes + reqs[end].device_bytes > budget) break;
        bytes += reqs[end].device_bytes;
        end++;
    }
    *bytes_out = bytes;
    return end;
}

static int sftx_serve_overlap(void* const* scenes, const sftx_request* reqs, uint32_t n, uint32_t max_batch, uint64_t budget,
                              uint32_t lanes, uint32_t* const* colors, uint32_t n_colors, uint64_t* done_ns, uint32_t* batch_of,
                              sftx_serve_stats* st) {
    uint32_t first[SFTG_MAX_LANES] = { 0 }, last[SFTG_MAX_LANES] = { 0 };
    uint64_t lbytes[SFTG_MAX_LANES] = { 0 }, lbatch[SFTG_MAX_LANES] = { 0 };
    int busy[SFTG_MAX_LANES] = { 0 };
    uint64_t inflight = 0;
    uint32_t next = 0, finished = 0;
    const uint64_t t0 = sftx_now_ns();
    while (finished < n) {
        int progressed = 0;
        for (uint32_t l = 1; l < SFTG_MAX_LANES; l++) {   /* collect finished lanes */
            if (!busy[l] || sft_batch_done(l) == 0) continue;
            if (sft_batch_wait(l)) st->errors++;
            const uint64_t done = sftx_now_ns() - t0;
            for (uint32_t k = first[l]; k < last[l]; k++) {
                done_ns[k] = done;
                if (batch_of) batch_of[k] = (uint32_t)lbatch[l];
            }
            finished += last[l] - first[l];
            inflight -= lbytes[l];
            busy[l] = 0;
            progressed = 1;
        }
        uint32_t lane = 0;
        for (uint32_t l = 1; l <= lanes && !lane; l++) if (!busy[l]) lane = l;
        const uint64_t now = sftx_now_ns() - t0;
        if (lane && next < n && reqs[next].arrival_ns <= now) {
            uint64_t bytes = 0;
            /* colour buffers: request k uses colors[k % n_colors]; those of the oldest request in
             * flight onwards are taken */
            uint32_t oldest = next;
            for (uint32_t l = 1; l < SFTG_MAX_LANES; l++) if (busy[l] && first[l] < oldest) oldest = first[l];
            uint32_t cap = max_batch;
            if (oldest + n_colors - next < cap) cap = oldest + n_colors - next;
            const uint32_t end = cap ? sftx_admit(reqs, n, next, now, cap, budget, inflight, &bytes) : next;
            if (end > next) {
                sft_batch_begin();
                for (uint32_t k = next; k < end; k++) {
                    const sftx_request* r = &reqs[k];
                    sft_set_msaa_samples(r->samples);
                    if (sftx_scene_render_ex(scenes[r->scene], r->frame, colors[k % n_colors], 0, r->max_point_lights)) st->errors++;
                }
                if (sft_batch_submit_async(lane)) st->errors++;
                first[lane] = next; last[lane] = end; lbytes[lane] = bytes; lbatch[lane] = st->batches; busy[lane] = 1;
                inflight += bytes;
                uint64_t lanes_busy = 0;
                for (uint32_t q = 1; q < SFTG_MAX_LANES; q++) lanes_busy += (uint64_t)busy[q];
                if (lanes_busy > st->max_inflight) st->max_inflight = lanes_busy;
                if (end - next > st->max_batch) st->max_batch = end - next;
                if (inflight > st->peak_bytes) st->peak_bytes = inflight;
                st->batches++;
                next = end;
                progressed = 1;
            }
        }
        if (progressed) continue;
        int any_busy = 0;
        for (uint32_t l = 1; l < SFTG_MAX_LANES; l++) any_busy |= busy[l];
        if (!any_busy && next < n) sftx_wait_until(t0, reqs[next].arrival_ns);   /* idle until the next arrival */
        /* otherwise poll the lanes again: completions and arrivals are both due soon */
    }
    return 0;
}

/* Serves n requests sorted by arrival.  colors[k % n_colors] (pitch: the request's width * 4)
 * receives request k's pixels; n_colors must be at least max_batch (in SFTX_SERVE_OVERLAP, the
 * requests in flight are also limited to n_colors).  done_ns[k] is the completion time of
 * request k from the start of the run, batch_of[k] (optional) its batch.  In SFTX_SERVE_OVERLAP,
 * at most `lanes` batches (1 to SFTG_MAX_LANES - 1) are on the GPU at once. */
SFTX_EXPORT int sftx_serve_ex(void* const* scenes, const sftx_request* reqs, uint32_t n, uint32_t max_batch, uint64_t budget_bytes,
                              int mode, uint32_t lanes, uint32_t* const* colors, uint32_t n_colors, uint64_t* done_ns,
                              uint32_t* batch_of, sftx_serve_stats* stats) {
    if (!scenes || (!reqs && n) || !colors || !done_ns || max_batch == 0 || n_colors < max_batch) return -1;
    if (mode != SFTX_SERVE_BATCHED && mode != SFTX_SERVE_PLAIN && mode != SFTX_SERVE_OVERLAP) return -1;
    if (mode == SFTX_SERVE_OVERLAP && (lanes < 1 || lanes > SFTG_MAX_LANES - 1)) return -1;
    sftx_serve_stats st;
    memset(&st, 0, sizeof(st));
    if (mode == SFTX_SERVE_OVERLAP) {
        sftx_serve_overlap(scenes, reqs, n, max_batch, budget_bytes, lanes, colors, n_colors, done_ns, batch_of, &st);
        if (stats) *stats = st;
        return st.errors ? -2 : 0;
    }
    const int plain = mode == SFTX_SERVE_PLAIN;
    const uint64_t t0 = sftx_now_ns();
    uint32_t next = 0;
    while (next < n) {
        if (reqs[next].arrival_ns > sftx_now_ns() - t0) sftx_wait_until(t0, reqs[next].arrival_ns);
        const uint64_t now = sftx_now_ns() - t0;
        /* admission: arrived requests in order, within the batch size and the memory budget */
        uint64_t bytes = 0;
        const uint32_t end = sftx_admit(reqs, n, next, now, plain ? 1u : max_batch, budget_bytes, 0, &bytes);
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

/* Grows every lane's buffers before a run, so that no lane first grows its frame arena, colour
 * pool or pinned staging while requests are being timed.  The largest batch admission can form
 * from reqs (the max_batch requests with the largest device estimates, taken in that order while
 * they fit the budget) is rendered once on each of lanes 1..lanes, all queued before any is waited
 * for, and once on lane 0 (SFTX_SERVE_BATCHED and SFTX_SERVE_PLAIN render there).  Its i-th view
 * goes to colors[i % n_colors].  Returns 0, -1 for bad arguments, -2 when a render, submission or
 * wait failed. */
SFTX_EXPORT int sftx_serve_warm(void* const* scenes, const sftx_request* reqs, uint32_t n, uint32_t max_batch, uint64_t budget_bytes,
                                uint32_t lanes, uint32_t* const* colors, uint32_t n_colors) {
    if (!scenes || !reqs || !n || !colors || max_batch == 0 || n_colors < max_batch || max_batch > 4096) return -1;
    if (lanes > SFTG_MAX_LANES - 1) return -1;
    uint32_t pick[4096];
    uint32_t np = 0;
    for (uint32_t k = 0; k < n; k++) {   /* the max_batch largest estimates, largest first (earliest on ties) */
        if (np == max_batch && reqs[k].device_bytes <= reqs[pick[np - 1]].device_bytes) continue;
        uint32_t j = np < max_batch ? np++ : np - 1;
        while (j > 0 && reqs[pick[j - 1]].device_bytes < reqs[k].device_bytes) { pick[j] = pick[j - 1]; j--; }
        pick[j] = k;
    }
    uint32_t take = 0;
    uint64_t bytes = 0;
    while (take < np && (take == 0 || bytes + reqs[pick[take]].device_bytes <= budget_bytes)) bytes += reqs[pick[take++]].device_bytes;
    int errors = 0;
    for (uint32_t l = 0; l <= lanes; l++) {
        const uint32_t lane = l < lanes ? l + 1 : 0;   /* the submission lanes first, lane 0 last */
        sft_batch_begin();
        for (uint32_t i = 0; i < take; i++) {
            const sftx_request* r = &reqs[pick[i]];
            sft_set_msaa_samples(r->samples);
            if (sftx_scene_render_ex(scenes[r->scene], r->frame, colors[i % n_colors], 0, r->max_point_lights)) errors++;
        }
        if (lane) { if (sft_batch_submit_async(lane)) errors++; }
        else {
            for (uint32_t q = 1; q <= lanes; q++) if (sft_batch_wait(q)) errors++;
            if (sft_batch_submit()) errors++;
        }
    }
    return errors ? -2 : 0;
}

SFTX_EXPORT int sftx_serve(void* const* scenes, const sftx_request* reqs, uint32_t n, uint32_t max_batch, uint64_t budget_bytes,
                           int mode, uint32_t* const* colors, uint32_t n_colors, uint64_t* done_ns, uint32_t* batch_of,
                           sftx_serve_stats* stats) {
    return sftx_serve_ex(scenes, reqs, n, max_batch, budget_bytes, mode, SFTG_MAX_LANES - 1, colors, n_colors, done_ns, batch_of,
                         stats);
}
