/*
 * ophpc serving — continuous batching of hologram jobs on one GPU.
 *
 * No counterpart in the reference (its generateHologram runs one object's
 * job to completion, ophgen/src/ophPointCloud.cpp:151-191). A server owns a
 * worker thread, a device memory budget and `max_in_flight` slots. Jobs of
 * any resolution, point count, wavelength set and method are submitted at
 * any time; the worker admits them as soon as a slot is free and their
 * device memory fits both the budget and the free HBM reported by
 * cudaMemGetInfo, then runs every admitted job as a sequence of steps of
 * ~step_ms of GPU time on its own stream, so that admitted jobs overlap on
 * the device. The policy orders admission and the streams' priorities:
 *   OPHPC_SERVE_EARLIEST_DEADLINE (default, 0): every job by earliest
 *     deadline, a job's deadline being its submission time + 2 x its
 *     estimated isolated service time (interactions at the kernels' rate +
 *     copies + a fixed per-job cost) + 20 ms. A long job's priority rises as
 *     its deadline nears, so it is not kept waiting by a stream of short
 *     ones; the lowest tail of the three on mixed streams;
 *   OPHPC_SERVE_SHORTEST_REMAINING: admission in arrival order, priority by
 *     remaining work (best median latency, worst tail);
 *   OPHPC_SERVE_DEADLINE: jobs whose estimated isolated service time is
 *     under 20 ms first, least remaining work first among them; then the
 *     others by earliest deadline (submission + 2 x estimated isolated
 *     time). Short jobs always overtake long ones.
 * Admission never skips the first job in policy order that does not fit, so
 * a large job cannot be starved of memory by smaller ones behind it.
 * A job's result does not depend on the other jobs: its chunking is fixed
 * by the job and its FP64 field is accumulated in the same order whatever
 * else runs.
 *
 * Host buffers (vertices in, field / codes out) must stay valid until the
 * job is waited for; page-locked buffers let the copies overlap with other
 * jobs' kernels.
 */
#ifndef OPHPC_SERVE_H
#define OPHPC_SERVE_H

#include "ophpc.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ophpc_server ophpc_server;

#define OPHPC_SERVE_EARLIEST_DEADLINE 0u
#define OPHPC_SERVE_SHORTEST_REMAINING 1u
#define OPHPC_SERVE_DEADLINE 2u

typedef struct ophpc_server_options {
    uint32_t max_in_flight;    /* admitted jobs at once (0 = 16) */
    uint32_t policy;           /* OPHPC_SERVE_EARLIEST_DEADLINE (0), _SHORTEST_REMAINING or _DEADLINE */
    uint64_t memory_budget;    /* bytes of device memory for jobs (0 = half the free memory) */
    uint64_t reserve_bytes;    /* free device memory always left untouched (0 = 512 MiB) */
    double step_ms;            /* target GPU time of one scheduling step (<= 0: 2 ms) */
} ophpc_server_options;

/* One hologram job: generateHologram (RS or Fresnel, on the FP32 cores or,
 * by mode, on the tensor cores) and, when h_codes is set, encoding +
 * normalize. */
typedef struct ophpc_job {
    ophpc_config cfg;
    const ophpc_vertex* h_vertices;  /* host, n_points records */
    uint64_t n_points;
    uint32_t diff_flag;              /* OPHPC_DIFF_RS / OPHPC_DIFF_FRESNEL */
    uint32_t mode;                   /* OPHPC_MODE_*: RS with OPHPC_MODE_TENSOR_BF16X3, and Fresnel
                                        with OPHPC_MODE_TENSOR_BF16X3 or OPHPC_MODE_TENSOR_FP16, run
                                        on the tensor cores; RS with OPHPC_MODE_TENSOR_FP16, or both
                                        tensor bits at once, is rejected */
    double* h_field;                 /* optional host output [ch][pnY][pnX][re, im] */
    uint8_t* h_codes;                /* optional host output [ch][pnY][pnX] */
    uint32_t encode_flag;            /* OPHPC_ENCODE_* for h_codes */
    uint32_t pad;
} ophpc_job;

/* Host timestamps (seconds since the server was created). */
typedef struct ophpc_job_stats {
    double t_submit;
    double t_admit;
    double t_done;
} ophpc_job_stats;

ophpc_status ophpc_server_create(int32_t device, const ophpc_server_options* options, ophpc_server** out);

/* Queues a job; returns OPHPC_ERROR_INVALID_ARGUMENT for a malformed job and
 * OPHPC_ERROR_OUT_OF_MEMORY when it alone exceeds the memory budget. */
ophpc_status ophpc_server_submit(ophpc_server* server, const ophpc_job* job, uint64_t* ticket);

/* Waits for a job (timeout_s < 0: no limit) and forgets its ticket. Returns
 * the job's status, or OPHPC_ERROR_TIMEOUT (the ticket stays valid).
 * timeout_s = 0 polls: it never blocks on the job. */
ophpc_status ophpc_server_wait(ophpc_server* server, uint64_t ticket, double timeout_s, ophpc_job_stats* stats);

/* Finishes every queued job, then stops the worker and frees the server. */
ophpc_status ophpc_server_destroy(ophpc_server* server);

#ifdef __cplusplus
}
#endif

#endif /* OPHPC_SERVE_H */
