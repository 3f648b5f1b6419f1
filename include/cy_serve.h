/*
 * cy_serve.h -- a continuous-batching render server on one GPU.
 *
 * No reference counterpart: the reference renders one canvas at a time on
 * the calling thread.  A request is a recorded call list (cy_trace.h) whose
 * get_image_data reads are its result.  Worker threads (one CUDA stream
 * each) repeatedly admit every waiting request that fits the device memory
 * budget, oldest first, render them together as one frame (cy_batch.h) and
 * return each request's reads.  Requests that arrive while frames are on
 * the GPU join the next frame formed as budget frees up, so frames overlap
 * on the device.  A request's canvas and clip masks stay on the device for
 * the life of its frame.  The admission estimate is 184 B per canvas pixel
 * plus 16 B per call-list byte; a request above the whole budget runs alone.
 */
#ifndef CY_SERVE_H
#define CY_SERVE_H

#include <stddef.h>

#include "cy_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cy_server cy_server;

/* Start `workers` (1..16) worker threads on the current device with an
 * admission budget in bytes, `host_threads` threads per call-list replay
 * (0: one per core), and at most `max_batch` requests and `max_pixels`
 * canvas pixels per frame (a single larger request still runs). */
int cy_server_create(long long budget_bytes, int workers, int host_threads, int max_batch, long long max_pixels,
                     cy_server **out);

/* Queue a request (the call list is copied); its arrival time is now. */
int cy_server_submit(cy_server *server, const void *trace, size_t trace_len, unsigned long long *id);

/* Take one finished request: waits up to wait_ms (-1: forever, 0: no wait).
 * Returns 0 with its id, status (0 or an engine code), reads (copied to
 * images, *len bytes) and latency from submission to completion in ms; 1 if
 * none finished in time; -2 if cap < *len (the result stays queued). */
int cy_server_poll(cy_server *server, int wait_ms, unsigned long long *id, int *status, unsigned char *images,
                   size_t cap, size_t *len, double *latency_ms);

/* Counters: frames, requests finished, pixels finished, requests waiting,
 * bytes admitted now, most bytes admitted at once, largest frame (requests),
 * budget.  Returns how many were written. */
int cy_server_stats(cy_server *server, long long *stats, int n);

/* Finish every queued request, then stop the workers and free the server. */
void cy_server_destroy(cy_server *server);

#ifdef __cplusplus
}
#endif

#endif /* CY_SERVE_H */
