// Hologram serving engine (declared in include/ophpc_serve.h).
//
// Continuous batching of independent hologram jobs on one GPU. A worker
// thread admits queued jobs while device memory (a fixed budget, checked
// against cudaMemGetInfo) and in-flight slots allow, splits every job into
// steps of bounded GPU time — upload + per-point prep, point-range chunks of
// the RS / Fresnel kernel accumulating into the job's FP64 field, encode +
// download — and keeps one step of every admitted job in flight on its own
// stream. Jobs therefore overlap on the device; a job that arrives while
// others run is admitted as soon as a slot and memory free up and its
// kernels interleave with theirs at CTA granularity. Steps are issued on
// streams whose priority follows the policy's order: by default every job
// by earliest deadline (submission + 2 x estimated isolated time + 20 ms);
// or short jobs first, then the others by earliest deadline; or purely
// shortest remaining work. Short jobs are not stuck behind long ones and
// long ones are not starved by a stream of short ones.
//
// RS jobs submitted with OPHPC_MODE_TENSOR_BF16X3 run their point-range
// steps on the tensor-core RS kernel (plus its CUDA-core complement for the
// same range); Fresnel jobs with OPHPC_MODE_TENSOR_BF16X3 run point-range
// steps of the tensor-core Fresnel tile kernel (factors generated on chip,
// adding into the job's FP64 field); Fresnel jobs with OPHPC_MODE_TENSOR_FP16
// run one channel's chunk of points per step on the table path (factor
// tables + GEMM into FP64 sums, the channel's field written after its last
// chunk). Steps are sized by each path's rate.
//
// A job's result does not depend on what else runs: its chunking is fixed
// by the job alone and every chunk adds into the FP64 field in order.
#include "ophpc_serve.h"

#include "pc_common.cuh"
#include "pc_tc.cuh"
#include "pc_tcrs.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace ophpc {
namespace {

using Clock = std::chrono::steady_clock;

constexpr int kPrioLevels = 6;   // CUDA exposes six stream priorities on this GPU family
constexpr double kDeadlineFactor = 2.0;
constexpr double kShortJobS = 20e-3;     // estimated isolated time below which a job goes first
constexpr double kEdfSlackS = 20e-3;     // added to every deadline under OPHPC_SERVE_EARLIEST_DEADLINE
constexpr double kJobFixedS = 3e-3;      // per-job launch, sync and bookkeeping time
constexpr double kCopyBytesPerS = 20e9;  // host <-> device copies, page-locked

struct ServeJob {
    uint64_t ticket = 0;
    ophpc_job desc{};
    JobGeom jg{};
    int64_t chunk_points = 0;
    int64_t next_point = 0;
    int stage = 0;              // 0 upload+prep, 1 chunks, 2 encode+download, 3 done
    bool in_flight = false;
    cudaEvent_t ev = nullptr;
    int slot = -1;
    size_t bytes = 0;
    unsigned char* dmem = nullptr;
    ophpc_vertex* d_v = nullptr;
    PointRec* d_recs = nullptr;
    double* d_field = nullptr;
    uint8_t* d_codes = nullptr;
    unsigned long long* d_mm = nullptr;
    bool tc = false;            // RS on the tensor cores (OPHPC_MODE_TENSOR_BF16X3)
    bool tcf = false;           // Fresnel on the tensor cores, factor tables (OPHPC_MODE_TENSOR_FP16)
    bool tcft = false;          // Fresnel on the tensor cores, on-chip factors (OPHPC_MODE_TENSOR_BF16X3)
    float* d_amax = nullptr;    // tensor cores: per-channel amplitude bound
    int32_t* d_left = nullptr;  // tensor-core RS: per-tile pair counts for the complement
    uint32_t* d_mask = nullptr; // tensor-core RS: per-tile bits of the pairs left to the complement
    int* d_err = nullptr;       // tensor cores: kernel timeout word
    double* d_sum = nullptr;    // tensor-core Fresnel: [channel][re plane, im plane] FP64 sums
    TcFresnelPlan plan{};       // tensor-core Fresnel: factor tables of one step's points
    int cur_ch = 0;             // tensor-core Fresnel: channel being stepped
    double t_submit = 0, t_admit = 0, t_done = 0;
    double remaining = 0;       // interactions left
    double est_s = 0;           // estimated isolated service time
    double deadline = 0;        // t_submit + kDeadlineFactor * est_s
    double edf_deadline = 0;    // deadline + kEdfSlackS (OPHPC_SERVE_EARLIEST_DEADLINE)
    ophpc_status status = OPHPC_SUCCESS;
    bool finished = false;
};

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Policy order. OPHPC_SERVE_EARLIEST_DEADLINE (default): earliest deadline
// + kEdfSlackS first. OPHPC_SERVE_SHORTEST_REMAINING: least remaining work
// first. OPHPC_SERVE_DEADLINE: short jobs (estimated isolated time under
// kShortJobS) first, least remaining work first among them; then the others
// by earliest deadline.
bool before(uint32_t policy, const ServeJob* a, const ServeJob* b) {
    if (policy == OPHPC_SERVE_SHORTEST_REMAINING) return a->remaining < b->remaining;
    if (policy == OPHPC_SERVE_EARLIEST_DEADLINE) return a->edf_deadline < b->edf_deadline;
    const bool sa = a->est_s < kShortJobS, sb = b->est_s < kShortJobS;
    if (sa != sb) return sa;
    return sa ? a->remaining < b->remaining : a->deadline < b->deadline;
}

}  // namespace
}  // namespace ophpc

using namespace ophpc;

struct ophpc_server {
    int device = 0;
    ophpc_server_options opt{};
    cudaMemPool_t pool = nullptr;
    std::vector<std::vector<cudaStream_t>> streams;   // [slot][priority level]
    int prio_hi = 0, prio_lo = 0;
    Clock::time_point t0;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<ServeJob*> queue;
    std::vector<ServeJob*> active;
    std::unordered_map<uint64_t, std::unique_ptr<ServeJob>> jobs;
    std::vector<int> free_slots;
    uint64_t next_ticket = 1;
    size_t mem_in_use = 0;
    bool stop = false;
    double rate_rs = 2.0e12, rate_fresnel = 2.6e12;   // interactions/s used to size steps
    double rate_tc_rs = 2.2e13;                        // tensor-core RS
    double rate_tcf_fp16 = 9e13;                       // tensor-core Fresnel, tables
    double rate_tcf_tile = 4.5e13;                     // tensor-core Fresnel, on-chip factors
    int* h_err = nullptr;                              // [slot]: page-locked copies of the jobs' error words
};

namespace {

double now_s(const ophpc_server* s) {
    return std::chrono::duration<double>(Clock::now() - s->t0).count();
}

bool job_ok(const ophpc_job* j) {
    const ophpc_config& c = j->cfg;
    if (c.pixel_number[0] <= 0 || c.pixel_number[1] <= 0) return false;
    if ((int64_t)c.pixel_number[0] * c.pixel_number[1] > (int64_t)1 << 31) return false;
    if ((int64_t)c.pixel_number[1] > (int64_t)65535 * kTileH) return false;
    if (!(c.pixel_pitch[0] > 0) || !(c.pixel_pitch[1] > 0)) return false;
    if (c.n_channels < 1 || c.n_channels > OPHPC_MAX_CHANNELS) return false;
    for (uint32_t i = 0; i < c.n_channels; ++i)
        if (!(c.wave_length[i] > 0) || c.wave_length[i] >= 2 * c.pixel_pitch[0] || c.wave_length[i] >= 2 * c.pixel_pitch[1])
            return false;
    if (j->diff_flag > 1) return false;
    // tensor cores: RS with split-BF16, Fresnel with split-BF16 or FP16
    if ((j->mode & OPHPC_MODE_TENSOR_FP16) && (j->mode & OPHPC_MODE_TENSOR_BF16X3)) return false;
    if ((j->mode & OPHPC_MODE_TENSOR_FP16) && j->diff_flag == OPHPC_DIFF_RS) return false;
    if (j->n_points > 0 && !j->h_vertices) return false;
    if (j->n_points > (uint64_t)INT32_MAX) return false;
    if (j->encode_flag > OPHPC_ENCODE_IMAGINARY) return false;
    return true;
}

JobGeom make_job_geom(const ophpc_config* cfg, int64_t n) {
    JobGeom jg;
    std::memset(&jg, 0, sizeof(jg));
    jg.n_channels = (int32_t)cfg->n_channels;
    jg.n_points = n;
    for (uint32_t ch = 0; ch < cfg->n_channels; ++ch) {
        ChannelGeom& g = jg.ch[ch];
        g.pnX = cfg->pixel_number[0];
        g.pnY = cfg->pixel_number[1];
        g.offX = cfg->offset[0];
        g.offY = cfg->offset[1];
        g.ppX = cfg->pixel_pitch[0];
        g.ppY = cfg->pixel_pitch[1];
        const double ssX = g.pnX * g.ppX, ssY = g.pnY * g.ppY;
        g.x0 = -ssX / 2;
        g.y0 = -ssY / 2;
        g.lambda = cfg->wave_length[ch];
        g.inv_lambda = 1.0 / g.lambda;
        const double tx = g.lambda / (2 * g.ppX), ty = g.lambda / (2 * g.ppY);
        g.detx = tx / std::sqrt(1 - (tx * tx));
        g.dety = ty / std::sqrt(1 - (ty * ty));
    }
    jg.tiles_x = (cfg->pixel_number[0] + kTileW - 1) / kTileW;
    jg.tiles_y = (cfg->pixel_number[1] + kTileH - 1) / kTileH;
    jg.ksplit = 1;
    return jg;
}

bool uses_tc(const ophpc_job* j) { return j->diff_flag == OPHPC_DIFF_RS && (j->mode & OPHPC_MODE_TENSOR_BF16X3); }
bool uses_tcf(const ophpc_job* j) { return j->diff_flag == OPHPC_DIFF_FRESNEL && (j->mode & OPHPC_MODE_TENSOR_FP16); }
bool uses_tcft(const ophpc_job* j) {
    return j->diff_flag == OPHPC_DIFF_FRESNEL && (j->mode & OPHPC_MODE_TENSOR_BF16X3);
}

// Points per tensor-core Fresnel step: ~step_ms of GPU time for one
// channel, a multiple of the tables' K granularity, at most 65,536.
int64_t tcf_step_points(const ophpc_job* j, double step_ms, double rate) {
    const double plane = (double)j->cfg.pixel_number[0] * j->cfg.pixel_number[1];
    const int64_t m = tc_fresnel_chunk_multiple();
    int64_t kc = (int64_t)(step_ms * 1e-3 * rate / plane);
    kc = std::max<int64_t>(m, std::min<int64_t>(kc, 65536)) / m * m;
    const int64_t nup = ((int64_t)j->n_points + m - 1) / m * m;
    return std::max<int64_t>(m, std::min<int64_t>(kc, nup));
}

size_t tc_tiles(const ophpc_job* j) {
    return (size_t)((j->cfg.pixel_number[0] + kRsTcTile - 1) / kRsTcTile) *
           ((j->cfg.pixel_number[1] + kRsTcTile - 1) / kRsTcTile) * j->cfg.n_channels;
}
size_t tc_left_bytes(const ophpc_job* j) { return align256(sizeof(int32_t) * tc_tiles(j)); }
size_t tc_mask_bytes(const ophpc_job* j) {
    return align256(sizeof(uint32_t) * tc_tiles(j) * (size_t)tc_rs_mask_words((int64_t)j->n_points));
}

size_t tcf_bytes(const ophpc_job* j, int64_t kc) {
    const size_t px = (size_t)j->cfg.pixel_number[0] * j->cfg.pixel_number[1] * j->cfg.n_channels;
    return 1024 + tc_fresnel_table_bytes(j->cfg.pixel_number[0], j->cfg.pixel_number[1], (int)kc,
                                         (j->mode & OPHPC_MODE_TENSOR_BF16X3) != 0) +
           align256(sizeof(double) * 2 * px);
}

size_t job_bytes(const ophpc_job* j, int64_t tcf_kc) {
    const size_t px = (size_t)j->cfg.pixel_number[0] * j->cfg.pixel_number[1] * j->cfg.n_channels;
    return align256(sizeof(ophpc_vertex) * j->n_points) + align256(sizeof(PointRec) * j->n_points * j->cfg.n_channels) +
           align256(sizeof(double2) * px) + align256(px) + 256 + (uses_tc(j) || uses_tcf(j) || uses_tcft(j) ? 256 : 0) +
           (uses_tc(j) ? tc_left_bytes(j) + tc_mask_bytes(j) : 0) + (uses_tcf(j) ? tcf_bytes(j, tcf_kc) : 0);
}

// Enqueues the job's next step on the stream of its slot at the priority
// its remaining work earns. Called with the server lock held.
void enqueue_step(ophpc_server* s, ServeJob* j, int prio_index) {
    cudaStream_t st = s->streams[j->slot][prio_index];
    const ophpc_job& d = j->desc;
    const int64_t n = (int64_t)d.n_points;
    const int64_t px = (int64_t)d.cfg.pixel_number[0] * d.cfg.pixel_number[1];
    cudaError_t e = cudaSuccess;
    if (j->stage == 0) {
        if (j->tc || j->tcf || j->tcft) e = cudaMemsetAsync(j->d_amax, 0, 32, st);   // amax[0..3], error word
        if (n > 0) {
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(j->d_v, d.h_vertices, sizeof(ophpc_vertex) * n, cudaMemcpyHostToDevice, st);
            launch_prep(j->d_v, n, d.cfg.scale, d.cfg.distance, d.cfg.field_length, d.cfg.viewing_window,
                        (int)d.diff_flag, j->jg, j->d_recs, st);
            if (j->tc)
                launch_rs_amax(j->d_recs, n, (int)d.cfg.n_channels, d.cfg.pixel_number[0], d.cfg.pixel_number[1],
                               j->d_amax, st);
            if (j->tcft) launch_fresnel_amax(j->d_recs, n, (int)d.cfg.n_channels, j->d_amax, st);
            if (j->tcf)
                for (uint32_t c = 0; c < d.cfg.n_channels; ++c)
                    launch_tc_fresnel_cmax(j->d_recs + (int64_t)c * n, n, j->d_amax + c, st);
        } else if (e == cudaSuccess) {
            e = cudaMemsetAsync(j->d_field, 0, sizeof(double2) * px * d.cfg.n_channels, st);
        }
        j->stage = n > 0 ? 1 : 2;
    } else if (j->stage == 1 && j->tcf) {
        // one chunk of one channel: tables + GEMM into the channel's FP64
        // sums; the channel's last chunk also writes its field
        const int c = j->cur_ch;
        const int64_t k0 = j->next_point, kc = std::min<int64_t>(j->chunk_points, n - k0);
        double* sre = j->d_sum + (int64_t)c * 2 * px;
        e = launch_tc_fresnel_chunk(j->plan, j->d_recs + (int64_t)c * n, n, j->jg.ch[c], k0, (int)kc, j->d_amax + c,
                                    sre, sre + px, k0 > 0, j->d_err, st);
        j->remaining -= (double)kc * px;
        j->next_point = k0 + kc;
        if (j->next_point >= n) {
            launch_tc_fresnel_finalize(sre, sre + px, j->d_amax + c, px,
                                       reinterpret_cast<double2*>(j->d_field) + (int64_t)c * px, st);
            j->next_point = 0;
            if (++j->cur_ch >= (int)d.cfg.n_channels) j->stage = 2;
        }
    } else if (j->stage == 1) {
        JobGeom g = j->jg;
        g.p0 = j->next_point;
        g.p1 = std::min<int64_t>(n, j->next_point + j->chunk_points);
        g.accumulate = j->next_point > 0 ? 1 : 0;
        g.points_per_split = std::max<int64_t>(kChunk, ((g.p1 - g.p0 + kChunk - 1) / kChunk) * kChunk);
        if (j->tc)
            e = launch_tc_rs_range(j->jg, j->d_recs, g.p0, g.p1, g.accumulate != 0,
                                   reinterpret_cast<double2*>(j->d_field), j->d_amax, j->d_left, j->d_mask,
                                   tc_rs_mask_words((int64_t)d.n_points), j->d_err, st);
        else if (j->tcft)
            e = launch_tc_fresnel_range(j->jg, j->d_recs, g.p0, g.p1, g.accumulate != 0,
                                        reinterpret_cast<double2*>(j->d_field), j->d_amax, j->d_err, st);
        else if (d.diff_flag == OPHPC_DIFF_RS)
            launch_rs(j->d_recs, g, reinterpret_cast<double2*>(j->d_field), nullptr, st);
        else
            launch_fresnel(j->d_recs, g, reinterpret_cast<double2*>(j->d_field), nullptr, st);
        j->remaining -= (double)(g.p1 - g.p0) * px * d.cfg.n_channels;
        j->next_point = g.p1;
        if (j->next_point >= n) j->stage = 2;
    } else if (j->stage == 2) {
        if (d.h_codes) {
            launch_encode(reinterpret_cast<const double2*>(j->d_field), (int)d.cfg.n_channels, px, (int)d.encode_flag,
                          nullptr, j->d_codes, j->d_mm, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(d.h_codes, j->d_codes, (size_t)px * d.cfg.n_channels,
                                                      cudaMemcpyDeviceToHost, st);
        }
        if (d.h_field && e == cudaSuccess)
            e = cudaMemcpyAsync(d.h_field, j->d_field, sizeof(double2) * px * d.cfg.n_channels, cudaMemcpyDeviceToHost, st);
        if ((j->tc || j->tcf || j->tcft) && e == cudaSuccess)
            e = cudaMemcpyAsync(&s->h_err[j->slot], j->d_err, sizeof(int), cudaMemcpyDeviceToHost, st);
        j->stage = 3;
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(j->ev, st);
    if (e != cudaSuccess) {
        j->status = e == cudaErrorMemoryAllocation ? OPHPC_ERROR_OUT_OF_MEMORY : OPHPC_ERROR_CUDA;
        j->stage = 3;
    }
    j->in_flight = true;
}

bool admit(ophpc_server* s, ServeJob* j) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return false;
    if (j->bytes + s->opt.reserve_bytes > free_b) return false;
    if (s->mem_in_use + j->bytes > s->opt.memory_budget) return false;
    if (s->free_slots.empty()) return false;
    j->slot = s->free_slots.back();
    cudaStream_t st = s->streams[j->slot][0];
    if (cudaMallocFromPoolAsync((void**)&j->dmem, j->bytes, s->pool, st) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    s->free_slots.pop_back();
    const ophpc_job& d = j->desc;
    const size_t px = (size_t)d.cfg.pixel_number[0] * d.cfg.pixel_number[1] * d.cfg.n_channels;
    unsigned char* q = j->dmem;
    j->d_v = (ophpc_vertex*)q;
    q += align256(sizeof(ophpc_vertex) * d.n_points);
    j->d_recs = (PointRec*)q;
    q += align256(sizeof(PointRec) * d.n_points * d.cfg.n_channels);
    j->d_field = (double*)q;
    q += align256(sizeof(double2) * px);
    j->d_codes = q;
    q += align256(px);
    j->d_mm = (unsigned long long*)q;
    if (j->tc || j->tcf || j->tcft) {
        q += 256;
        j->d_amax = (float*)q;   // [4] floats, then the error word
        j->d_err = (int*)(q + 16);
        q += 256;
        s->h_err[j->slot] = 0;
    }
    if (j->tc) {
        j->d_left = (int32_t*)q;
        j->d_mask = (uint32_t*)(q + tc_left_bytes(&d));
    }
    if (j->tcf) {
        unsigned char* tq = (unsigned char*)(((uintptr_t)q + 1023) & ~(uintptr_t)1023);
        const size_t tb = tc_fresnel_table_bytes(d.cfg.pixel_number[0], d.cfg.pixel_number[1], (int)j->chunk_points,
                                                 (d.mode & OPHPC_MODE_TENSOR_BF16X3) != 0);
        if (!tc_fresnel_plan(&j->plan, tq, d.cfg.pixel_number[0], d.cfg.pixel_number[1], (int)j->chunk_points,
                             (d.mode & OPHPC_MODE_TENSOR_BF16X3) != 0)) {
            j->status = OPHPC_ERROR_UNSUPPORTED;
            j->stage = 3;
        }
        j->d_sum = (double*)(tq + tb);
    }
    s->mem_in_use += j->bytes;
    j->t_admit = now_s(s);
    return true;
}

void release(ophpc_server* s, ServeJob* j) {
    cudaFreeAsync(j->dmem, s->streams[j->slot][0]);
    s->mem_in_use -= j->bytes;
    s->free_slots.push_back(j->slot);
    j->dmem = nullptr;
}

void worker_main(ophpc_server* s) {
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true) {
        // admission in policy order; the first job that does not fit blocks
        // the ones behind it
        const uint32_t pol = s->opt.policy;
        while (!s->queue.empty()) {
            auto it = s->queue.begin();   // shortest-remaining: arrival order
            if (pol != OPHPC_SERVE_SHORTEST_REMAINING)
                it = std::min_element(s->queue.begin(), s->queue.end(),
                                      [pol](const ServeJob* a, const ServeJob* b) { return before(pol, a, b); });
            ServeJob* j = *it;
            if (!admit(s, j)) break;
            s->queue.erase(it);
            s->active.push_back(j);
        }
        if (s->stop && s->queue.empty() && s->active.empty()) break;
        bool progressed = false;
        // completions
        for (size_t i = 0; i < s->active.size();) {
            ServeJob* j = s->active[i];
            if (j->in_flight) {
                const cudaError_t q = cudaEventQuery(j->ev);
                if (q == cudaErrorNotReady) {
                    ++i;
                    continue;
                }
                j->in_flight = false;
                progressed = true;
                if (q != cudaSuccess) {
                    j->status = OPHPC_ERROR_CUDA;
                    j->stage = 3;
                } else if ((j->tc || j->tcf || j->tcft) && j->stage == 3 && s->h_err[j->slot] != 0 &&
                           j->status == OPHPC_SUCCESS) {
                    j->status = OPHPC_ERROR_TIMEOUT;   // a tensor-core wait gave up
                }
            }
            if (!j->in_flight && j->stage == 3) {
                j->t_done = now_s(s);
                j->finished = true;
                release(s, j);
                s->active.erase(s->active.begin() + (long)i);
                s->cv_done.notify_all();
                progressed = true;
                continue;
            }
            ++i;
        }
        // issue: rank active jobs in policy order (earliest deadline or
        // least remaining work first)
        std::vector<ServeJob*> idle;
        for (ServeJob* j : s->active)
            if (!j->in_flight && j->stage < 3) idle.push_back(j);
        if (!idle.empty()) {
            std::vector<ServeJob*> ranked(s->active.begin(), s->active.end());
            std::sort(ranked.begin(), ranked.end(),
                      [pol](const ServeJob* a, const ServeJob* b) { return before(pol, a, b); });
            for (ServeJob* j : idle) {
                // rank among admitted jobs -> priority bucket
                const size_t r = (size_t)(std::find(ranked.begin(), ranked.end(), j) - ranked.begin());
                const int prio = (int)(r * kPrioLevels / ranked.size());
                enqueue_step(s, j, std::min(prio, kPrioLevels - 1));
            }
            progressed = true;
        }
        if (!progressed) {
            if (s->active.empty()) {
                s->cv_work.wait_for(lk, std::chrono::milliseconds(5));
            } else {
                lk.unlock();
                std::this_thread::sleep_for(std::chrono::microseconds(20));
                lk.lock();
            }
        }
    }
}

}  // namespace

extern "C" {

ophpc_status ophpc_server_create(int32_t device, const ophpc_server_options* options, ophpc_server** out) {
    if (!out) return OPHPC_ERROR_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return OPHPC_ERROR_NO_DEVICE;
    }
    if (device < 0 || device >= ndev) return OPHPC_ERROR_INVALID_ARGUMENT;
    if (cudaSetDevice(device) != cudaSuccess) return OPHPC_ERROR_CUDA;
    std::unique_ptr<ophpc_server> s(new ophpc_server());
    s->device = device;
    if (options) s->opt = *options;
    if (s->opt.max_in_flight == 0) s->opt.max_in_flight = 16;
    if (s->opt.policy != OPHPC_SERVE_EARLIEST_DEADLINE && s->opt.policy != OPHPC_SERVE_SHORTEST_REMAINING &&
        s->opt.policy != OPHPC_SERVE_DEADLINE)
        return OPHPC_ERROR_INVALID_ARGUMENT;
    if (s->opt.step_ms <= 0) s->opt.step_ms = 2.0;
    if (s->opt.reserve_bytes == 0) s->opt.reserve_bytes = (size_t)512 << 20;
    if (s->opt.memory_budget == 0) {
        size_t f = 0, t = 0;
        cudaMemGetInfo(&f, &t);
        s->opt.memory_budget = f / 2;
    }
    rs_blocks_per_sm();        // kernels' shared-memory limits
    fresnel_blocks_per_sm();
    cudaMemPoolProps pp;
    std::memset(&pp, 0, sizeof(pp));
    pp.allocType = cudaMemAllocationTypePinned;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = device;
    if (cudaMemPoolCreate(&s->pool, &pp) != cudaSuccess) return OPHPC_ERROR_CUDA;
    if (cudaHostAlloc((void**)&s->h_err, sizeof(int) * s->opt.max_in_flight, cudaHostAllocDefault) != cudaSuccess)
        return OPHPC_ERROR_CUDA;
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);   // hi is the numerically smallest (highest) priority
    s->streams.resize(s->opt.max_in_flight);
    for (uint32_t slot = 0; slot < s->opt.max_in_flight; ++slot) {
        for (int p = 0; p < kPrioLevels; ++p) {
            const int prio = hi + (int)((double)(lo - hi) * p / (kPrioLevels - 1) + 0.5);
            cudaStream_t st;
            if (cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio) != cudaSuccess) return OPHPC_ERROR_CUDA;
            s->streams[slot].push_back(st);
        }
        s->free_slots.push_back((int)slot);
    }
    s->t0 = Clock::now();
    ophpc_server* raw = s.release();
    raw->worker = std::thread(worker_main, raw);
    *out = raw;
    return OPHPC_SUCCESS;
}

ophpc_status ophpc_server_submit(ophpc_server* s, const ophpc_job* job, uint64_t* ticket) {
    if (!s || !job || !ticket) return OPHPC_ERROR_INVALID_ARGUMENT;
    if (!job_ok(job)) return OPHPC_ERROR_INVALID_ARGUMENT;
    std::unique_ptr<ServeJob> j(new ServeJob());
    j->desc = *job;
    j->tc = uses_tc(job);
    j->tcf = uses_tcf(job);
    j->tcft = uses_tcft(job);
    const double tcf_rate = s->rate_tcf_fp16;
    const int64_t tcf_kc = j->tcf ? tcf_step_points(job, s->opt.step_ms, tcf_rate) : 0;
    j->bytes = job_bytes(job, tcf_kc);
    if (j->bytes > s->opt.memory_budget) return OPHPC_ERROR_OUT_OF_MEMORY;
    j->jg = make_job_geom(&job->cfg, (int64_t)job->n_points);
    const double px = (double)job->cfg.pixel_number[0] * job->cfg.pixel_number[1] * job->cfg.n_channels;
    const double rate = j->tc     ? s->rate_tc_rs
                        : j->tcft ? s->rate_tcf_tile
                        : j->tcf  ? tcf_rate
                                  : (job->diff_flag == OPHPC_DIFF_RS ? s->rate_rs : s->rate_fresnel);
    int64_t cp = (int64_t)(s->opt.step_ms * 1e-3 * rate / px);
    cp = std::max<int64_t>(kChunk, cp / kChunk * kChunk);
    j->chunk_points = j->tcf ? tcf_kc : cp;
    j->remaining = (double)job->n_points * px;
    const double copy_bytes = (double)sizeof(ophpc_vertex) * job->n_points +
                              (job->h_codes ? px : 0.0) + (job->h_field ? 16.0 * px : 0.0);
    j->est_s = kJobFixedS + j->remaining / rate + copy_bytes / kCopyBytesPerS;
    if (cudaEventCreateWithFlags(&j->ev, cudaEventDisableTiming) != cudaSuccess) return OPHPC_ERROR_CUDA;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) {
        cudaEventDestroy(j->ev);
        return OPHPC_ERROR_INVALID_ARGUMENT;
    }
    j->ticket = s->next_ticket++;
    j->t_submit = now_s(s);
    j->deadline = j->t_submit + kDeadlineFactor * j->est_s;
    j->edf_deadline = j->deadline + kEdfSlackS;
    *ticket = j->ticket;
    s->queue.push_back(j.get());
    s->jobs.emplace(j->ticket, std::move(j));
    s->cv_work.notify_all();
    return OPHPC_SUCCESS;
}

ophpc_status ophpc_server_wait(ophpc_server* s, uint64_t ticket, double timeout_s, ophpc_job_stats* stats) {
    if (!s) return OPHPC_ERROR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end()) return OPHPC_ERROR_INVALID_ARGUMENT;
    ServeJob* j = it->second.get();
    const auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(timeout_s));
    while (!j->finished) {
        if (timeout_s >= 0 && s->cv_done.wait_until(lk, deadline) == std::cv_status::timeout && !j->finished)
            return OPHPC_ERROR_TIMEOUT;
        if (timeout_s < 0) s->cv_done.wait(lk);
    }
    if (stats) {
        stats->t_submit = j->t_submit;
        stats->t_admit = j->t_admit;
        stats->t_done = j->t_done;
    }
    const ophpc_status st = j->status;
    cudaEventDestroy(j->ev);
    s->jobs.erase(it);
    return st;
}

ophpc_status ophpc_server_destroy(ophpc_server* s) {
    if (!s) return OPHPC_ERROR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->device);
    for (auto& v : s->streams)
        for (cudaStream_t st : v) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    for (auto& kv : s->jobs)
        if (kv.second->ev) cudaEventDestroy(kv.second->ev);
    cudaMemPoolDestroy(s->pool);
    if (s->h_err) cudaFreeHost(s->h_err);
    delete s;
    return OPHPC_SUCCESS;
}

}  // extern "C"
