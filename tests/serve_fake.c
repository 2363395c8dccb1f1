/* Fakes of the library calls made by the serving loop (sofren2_gb300/csrc/sft_serve.c), so that its
 * host logic runs on the CPU: a queued batch "runs" until its lane has been polled a set number of
 * times; a render, a submission or a wait can be made to fail at a chosen call.  The fakes record
 * what the loop did: batch sizes, submissions onto a lane that was still busy, renders outside a
 * batch, the most lanes busy at once. */
#include <stdint.h>
#include <string.h>

#define FK_LANES 8
#define FK_MAX_BATCHES 65536

static int recording, cur_n;
static int busy[FK_LANES], polls_left[FK_LANES];
static uint32_t renders, submits, waits, fail_render, fail_submit, fail_wait, done_polls;
static uint32_t busy_submit, max_busy, nbatches, sizes[FK_MAX_BATCHES];

void fk_reset(uint32_t polls, uint32_t f_render, uint32_t f_submit, uint32_t f_wait) {
    recording = 0; cur_n = 0;
    memset(busy, 0, sizeof(busy)); memset(polls_left, 0, sizeof(polls_left));
    renders = submits = waits = busy_submit = max_busy = nbatches = 0;
    done_polls = polls; fail_render = f_render; fail_submit = f_submit; fail_wait = f_wait;
}

/* renders, submissions, waits, submissions onto a busy lane, most lanes busy, batches */
void fk_stats(uint32_t* out) {
    out[0] = renders; out[1] = submits; out[2] = waits; out[3] = busy_submit; out[4] = max_busy; out[5] = nbatches;
}

uint32_t fk_batch_size(uint32_t i) { return i < FK_MAX_BATCHES ? sizes[i] : 0; }

void sft_batch_begin(void) { recording = 1; cur_n = 0; }
void sft_set_msaa_samples(int32_t samples) { (void)samples; }

int sftx_scene_render_ex(void* scene, uint32_t frame, uint32_t* color, int32_t pitch_bytes, uint32_t max_point_lights) {
    (void)scene; (void)pitch_bytes; (void)max_point_lights;
    if (recording) cur_n++;
    color[0] = frame + 1;
    return renders++ == fail_render ? -1 : 0;
}

static int32_t end_batch(void) {
    recording = 0;
    if (nbatches < FK_MAX_BATCHES) sizes[nbatches] = (uint32_t)cur_n;
    nbatches++;
    return submits++ == fail_submit ? -3 : 0;
}

int32_t sft_batch_submit(void) { return end_batch(); }

int32_t sft_batch_submit_async(uint32_t lane) {
    if (lane == 0 || lane >= FK_LANES) return -1;
    if (busy[lane]) busy_submit++;
    const int32_t rc = end_batch();
    busy[lane] = 1; polls_left[lane] = (int)done_polls;
    uint32_t nb = 0;
    for (int l = 1; l < FK_LANES; l++) nb += (uint32_t)busy[l];
    if (nb > max_busy) max_busy = nb;
    return rc;
}

int32_t sft_batch_done(uint32_t lane) {
    if (lane >= FK_LANES || !busy[lane]) return 1;
    return polls_left[lane]-- <= 0;
}

int32_t sft_batch_wait(uint32_t lane) {
    if (lane < FK_LANES) busy[lane] = 0;
    return waits++ == fail_wait ? -4 : 0;
}
