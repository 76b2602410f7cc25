// jobs.cu — the job queue behind gbrt_job_submit / poll / wait.
//
// One scheduler thread per context owns the context's stream while jobs are
// outstanding.  Each loop it
//   1. admits queued jobs in submission order while fewer than kMaxWaveJobs
//      are active and the job's device memory fits the HBM budget (a job that
//      carries skins also waits until no active job renders its scene, then
//      its scene is skinned and rebuilt);
//   2. packs one wave: active jobs ordered by the policy (shortest remaining
//      paths first, or submission order) contribute segments -- k samples of
//      a pixel chunk -- until the wave's kMaxWavePaths paths are used;
//   3. launches it (wavefront.cu), and for every job whose last segment it
//      carried, the job's resolve (accumulate + tone map);
//   4. retires waves whose completion event has fired: finished jobs get
//      their image and counters downloaded and their device memory freed.
// Up to two waves are in flight so that packing overlaps the GPU.  A job's
// per-pixel sums run in sample order whatever waves its segments land in, so
// its results equal the same frame rendered alone.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <thread>
#include <unordered_map>

#include "api_internal.h"

using namespace gbrt;

namespace gbrt_host {

namespace {

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// paths per batched wave: 2^22 while little work is queued, so that a wave,
// and the wait of a job that joins the batch, stays short; growing to a
// quarter of the queued paths on a deep queue, at most 2^24 (latency: 200
// Poisson jobs over 8 scenes gave p50 2.5 s with 2^24, 3.3 s with 2^26) or
// 2^26 with GBRT_JOB_LARGE_WAVES (throughput: 32 frames of 1.0G paths gave
// 1257 Mrays/s with 2^24, 1312 with 2^26)
constexpr uint32_t kWaveCap = kMaxWavePaths < (1u << 22) ? kMaxWavePaths : (1u << 22);
constexpr uint32_t kWaveCapDeep = kMaxWavePaths < (1u << 24) ? kMaxWavePaths : (1u << 24);
constexpr uint32_t kWaveCapLarge = kMaxWavePaths < (1u << 26) ? kMaxWavePaths : (1u << 26);
// With GBRT_JOB_LARGE_WAVES, a job of at least this many paths that no wave
// has touched runs alone, through the single-frame kernels (a frame this
// large fills the GPU by itself; the batched form's job table and partition
// cost it about 5%)
constexpr uint64_t kSoloPaths = 1ull << 24;
constexpr uint32_t kChunkDiv = 8;             // pixel chunk = wave / 8 (finer packing)
constexpr int kMaxInFlight = 2;

// Stream-ordered device buffer: cudaFree would wait for the whole device,
// stalling the waves in flight.
struct AsyncBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaStream_t st = nullptr;
    cudaError_t alloc(size_t n, cudaStream_t s) {
        st = s;
        cudaError_t e = cudaMallocAsync(&p, n, s);
        if (e == cudaSuccess) bytes = n;
        else p = nullptr;
        return e;
    }
    void release() {
        if (p) cudaFreeAsync(p, st);
        p = nullptr;
        bytes = 0;
    }
    ~AsyncBuf() { release(); }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

struct Job {
    uint64_t id = 0;
    gbrt_scene* scene = nullptr;
    gbrt_accum* acc = nullptr;
    gbrt_ubo ubo{};
    uint8_t* out_rgba8 = nullptr;
    std::vector<gbrt_skin_raw> skins;
    bool has_skins = false;
    gbrt_nrc* cache = nullptr;  // rendered alone through the cache (nrc_frame)
    bool cancelled = false;
    gbrt_nrc_render_opts copts{};
    // progress
    uint32_t npix = 0, ns = 0, sbase = 0, chunk = 0;
    uint32_t px0 = 0, s0 = 0;
    uint64_t paths_left = 0;
    // device memory (allocated at admission)
    AsyncBuf frame_sum, img, counters;
    size_t dev_bytes = 0;
    // status
    uint32_t state = GBRT_JOB_QUEUED;
    int status = GBRT_OK;
    double t_submit = 0, t_admit = 0, t_done = 0;
    gbrt_stats stats{};
    std::string err;
};

struct Wave {
    cudaEvent_t ev = nullptr;
    std::vector<Job*> finishing;  // jobs whose last segment this wave carried
    bool cancel = false;          // a marker after a cancelled job's waves: it ends with GBRT_E_CANCELLED
};

}  // namespace

struct JobQueue {
    gbrt_ctx* ctx = nullptr;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Job*> queued;
    std::vector<Job*> active;
    std::unordered_map<uint64_t, std::unique_ptr<Job>> jobs;
    std::deque<Wave> inflight;
    std::vector<cudaEvent_t> free_events;
    uint64_t next_id = 1;
    uint32_t outstanding = 0;  // submitted and not finished
    uint64_t budget = 0, used = 0;
    uint32_t policy = GBRT_JOB_POLICY_SRPT;
    uint32_t deep_cap = kWaveCapDeep;  // kWaveCapLarge with GBRT_JOB_LARGE_WAVES
    bool stop = false;
    std::thread worker;
    cudaStream_t dl = nullptr;  // downloads of finished jobs (non-blocking stream)

    void run();
    bool admit_one(std::unique_lock<std::mutex>& lk);
    int pack_and_launch();
    int run_cache_job(Job* j, std::unique_lock<std::mutex>& lk);
    int run_solo_job(Job* j);
    bool solo(const Job* j) const {
        return deep_cap == kWaveCapLarge && j->paths_left >= kSoloPaths && j->paths_left == (uint64_t)j->npix * j->ns;
    }
    int launch_next(std::unique_lock<std::mutex>& lk);
    void retire(Wave& w);
    void fail_active(int code, const std::string& msg);
};

namespace {

// The binary traversal form (the wave kernels' kTraceBinary): chosen by the
// autotuner, or the only one a world BVH without its 8-wide copy has.
bool binary_traversal(const DevScene& s) { return s.prefer_binary || (s.has_world && !s.cw_nodes); }

uint32_t scene_active(const JobQueue& q, const gbrt_scene* s) {
    uint32_t n = 0;
    for (const Job* j : q.active) n += j->scene == s;
    return n;
}

void finish_job(JobQueue& q, Job* j, int status, const std::string& msg) {
    if (j->dev_bytes) q.used -= j->dev_bytes;
    j->dev_bytes = 0;
    j->frame_sum.release();
    j->img.release();
    j->counters.release();
    j->status = status;
    j->err = msg;
    j->state = GBRT_JOB_DONE;
    j->t_done = now_ms();
    j->stats.device_ms = j->t_admit > 0 ? j->t_done - j->t_admit : 0.0;
    j->scene->jobs_pending.fetch_sub(1);
    j->acc->jobs_pending.fetch_sub(1);
    --q.outstanding;
}

}  // namespace

// Admission of the job at the head of the queue (lock held on entry and exit;
// released around device work).  Returns false when it has to wait.
bool JobQueue::admit_one(std::unique_lock<std::mutex>& lk) {
    if (queued.empty() || active.size() >= (size_t)kMaxWaveJobs) return false;
    Job* j = queued.front();
    const size_t need = (size_t)j->npix * (sizeof(float4) + (j->out_rgba8 ? 4 : 0)) + sizeof(DeviceCounters);
    if (used + need > budget && !active.empty()) return false;  // wait for memory to free up
    if (j->has_skins && scene_active(*this, j->scene)) return false;
    queued.pop_front();
    used += need;
    j->dev_bytes = need;
    j->state = GBRT_JOB_RUNNING;
    j->t_admit = now_ms();
    lk.unlock();
    cudaStream_t st = ctx->stream;
    int rc = GBRT_OK;
    std::string msg;
    cudaError_t e = cudaSuccess;
    uint32_t inject = ctx->inject_admit_oom.load();
    while (inject && !ctx->inject_admit_oom.compare_exchange_weak(inject, inject - 1)) {
    }
    if (inject) e = cudaErrorMemoryAllocation;  // injected (host side): as if the allocation had failed
    if (e == cudaSuccess) e = j->frame_sum.alloc((size_t)j->npix * sizeof(float4), st);
    if (e == cudaSuccess && j->out_rgba8) e = j->img.alloc((size_t)j->npix * 4, st);
    if (e == cudaSuccess) e = j->counters.alloc(sizeof(DeviceCounters), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(j->frame_sum.p, 0, j->frame_sum.bytes, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(j->counters.p, 0, sizeof(DeviceCounters), st);
    if (e != cudaSuccess) {
        if (!inject) cudaGetLastError();
        rc = e == cudaErrorMemoryAllocation ? GBRT_E_OOM : GBRT_E_CUDA;
        msg = std::string("job admission: ") + cudaGetErrorString(e) + (inject ? " (injected)" : "");
    } else if (j->has_skins) {
        rc = skin_scene(j->scene, j->skins.data(), (uint32_t)j->skins.size());
        if (rc != GBRT_OK) msg = ctx->err;
        j->skins.clear();
        j->skins.shrink_to_fit();
    }
    lk.lock();
    if (rc != GBRT_OK) {
        finish_job(*this, j, rc, msg);
        cv_done.notify_all();
    } else {
        active.push_back(j);
    }
    return true;
}

// Packs one wave from the active jobs and launches it.  Returns GBRT_OK, or 1
// when no active job has paths left.  Called with the lock held.
int JobQueue::pack_and_launch() {
    std::vector<Job*> order;
    for (Job* j : active)
        if (j->paths_left && !j->cache && !solo(j)) order.push_back(j);
    if (order.empty()) return 1;
    if (policy == GBRT_JOB_POLICY_SRPT)
        std::stable_sort(order.begin(), order.end(),
                         [](const Job* a, const Job* b) { return a->paths_left < b->paths_left; });
    else
        std::stable_sort(order.begin(), order.end(), [](const Job* a, const Job* b) { return a->id < b->id; });
    WaveDesc* w = nullptr;
    cudaError_t e = wave_acquire(ctx->ring, &w);
    if (e != cudaSuccess) {
        fail_active(GBRT_E_CUDA, std::string("wave descriptor: ") + cudaGetErrorString(e));
        return GBRT_E_CUDA;
    }
    w->njobs = w->nsegs = w->npaths = w->nfin = w->nb = 0;
    std::vector<Job*> finishing;
    uint64_t queued = 0;
    for (const Job* j : order) queued += j->paths_left;
    const uint32_t cap = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(queued / 4, kWaveCap), deep_cap);
    uint32_t room = std::min(cap, ctx->wf.cap);
    // a wave runs one traversal form for all its jobs: it packs only the jobs
    // whose scenes traverse like the first one's (binary, or 8-wide with or
    // without a TLAS), so a scene tuned for one form never runs in the other
    const bool binary0 = binary_traversal(order.front()->scene->view);
    for (Job* j : order) {
        if (w->njobs == (uint32_t)kMaxWaveJobs || w->nsegs == (uint32_t)kMaxWaveSegs || room == 0) break;
        if (binary_traversal(j->scene->view) != binary0) continue;
        const uint32_t slot = w->njobs, path0 = w->npaths;
        while (j->paths_left && room && w->nsegs < (uint32_t)kMaxWaveSegs) {
            const uint32_t npw = std::min(j->chunk, j->npix - j->px0);
            const uint32_t k = std::min(j->ns - j->s0, room / npw);
            if (k == 0) break;
            w->segs[w->nsegs++] = WaveSeg{w->npaths, slot, j->px0, npw, j->sbase + j->s0, j->s0, k, w->nfin};
            w->npaths += k * npw;
            w->nfin += npw;
            room -= k * npw;
            j->paths_left -= (uint64_t)k * npw;
            j->s0 += k;
            if (j->s0 == j->ns) {
                j->s0 = 0;
                j->px0 += npw;
            }
        }
        if (w->npaths == path0) continue;
        WaveJob& J = w->jobs[slot];
        J.s = j->scene->view;
        J.ubo = j->ubo;
        J.out = RenderOut{};
        J.out.width = j->acc->w;
        J.out.height = j->acc->h;
        J.out.accum = j->acc->buf.as<float4>();
        J.out.rgba8 = j->out_rgba8 ? j->img.as<uchar4>() : nullptr;
        J.out.counters = j->counters.as<DeviceCounters>();
        J.frame_sum = j->frame_sum.as<float4>();
        J.ns = j->ns;
        J.flags = j->ubo.fully_opaque ? GBRT_RAY_OPAQUE : 0u;
        J.tfar = j->ubo.orthographic_fov_dis > 0.0f ? 100000.0f : 10000.0f;
        J.path0 = path0;
        J.npaths = w->npaths - path0;
        w->nb = std::max(w->nb, j->ubo.number_of_bounces);
        ++w->njobs;
        if (!j->paths_left) finishing.push_back(j);
    }
    if (w->njobs == 0) return 1;
    if ((e = wave_partition(*w)) == cudaSuccess) e = launch_wave(ctx->ring, ctx->wf, ctx->stream, nullptr);
    for (Job* j : finishing) {
        if (e != cudaSuccess) break;
        RenderOut out{};
        out.width = j->acc->w;
        out.height = j->acc->h;
        out.accum = j->acc->buf.as<float4>();
        out.rgba8 = j->out_rgba8 ? j->img.as<uchar4>() : nullptr;
        out.counters = j->counters.as<DeviceCounters>();
        e = launch_resolve(j->ubo, out, j->frame_sum.as<float4>(), ctx->stream);
    }
    Wave wv;
    if (e == cudaSuccess) {
        if (free_events.empty()) {
            cudaEvent_t ev;
            e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
            if (e == cudaSuccess) free_events.push_back(ev);
        }
    }
    if (e == cudaSuccess) {
        wv.ev = free_events.back();
        free_events.pop_back();
        e = cudaEventRecord(wv.ev, ctx->stream);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail_active(GBRT_E_CUDA, std::string("wave launch: ") + cudaGetErrorString(e));
        return GBRT_E_CUDA;
    }
    wv.finishing = std::move(finishing);
    inflight.push_back(std::move(wv));
    return GBRT_OK;
}

// Renders a cache job's whole frame and its training on the context stream
// (lock released meanwhile; one host wait, for the training sample count),
// then queues its completion like a wave's.  Called with the lock held.
int JobQueue::run_cache_job(Job* j, std::unique_lock<std::mutex>& lk) {
    j->paths_left = 0;
    RenderOut out{};
    out.width = j->acc->w;
    out.height = j->acc->h;
    out.accum = j->acc->buf.as<float4>();
    out.rgba8 = j->out_rgba8 ? j->img.as<uchar4>() : nullptr;
    out.counters = j->counters.as<DeviceCounters>();
    WfState wf = ctx->wf;
    wf.frame_sum = j->frame_sum.as<float4>();
    const char* what = "";
    lk.unlock();
    cudaError_t e = nrc_frame(j->cache, j->scene->view, j->ubo, out, wf, j->copts, ctx->stream, nullptr, &what);
    const uint32_t qstatus = e == cudaSuccess ? nrc_status(j->cache, ctx->stream) : 0u;
    lk.lock();
    if (e == cudaSuccess && qstatus) {
        active.erase(std::find(active.begin(), active.end(), j));
        finish_job(*this, j, GBRT_E_DEVICE_LIMIT, "a tensor-core wait of the cache query timed out");
        cv_done.notify_all();
        return GBRT_OK;
    }
    Wave wv;
    if (e == cudaSuccess && free_events.empty()) {
        cudaEvent_t ev;
        e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e == cudaSuccess) free_events.push_back(ev);
    }
    if (e == cudaSuccess) {
        wv.ev = free_events.back();
        free_events.pop_back();
        e = cudaEventRecord(wv.ev, ctx->stream);
        if (e != cudaSuccess) free_events.push_back(wv.ev);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail_active(GBRT_E_CUDA, std::string("cache job (") + what + "): " + cudaGetErrorString(e));
        return GBRT_E_CUDA;
    }
    wv.finishing.push_back(j);
    inflight.push_back(std::move(wv));
    return GBRT_OK;
}

// Renders a large untouched job alone with the single-frame kernels, like
// gbrt_render_ex, and queues its completion like a wave's.  Lock held (no
// host wait: the frame is only enqueued).
int JobQueue::run_solo_job(Job* j) {
    j->paths_left = 0;
    RenderOut out{};
    out.width = j->acc->w;
    out.height = j->acc->h;
    out.accum = j->acc->buf.as<float4>();
    out.rgba8 = j->out_rgba8 ? j->img.as<uchar4>() : nullptr;
    out.counters = j->counters.as<DeviceCounters>();
    WfState wf = ctx->wf;
    wf.frame_sum = j->frame_sum.as<float4>();
    cudaError_t e = launch_wavefront(j->scene->view, j->ubo, out, wf, ctx->stream, nullptr, nullptr, nullptr, &ctx->side);
    Wave wv;
    if (e == cudaSuccess && free_events.empty()) {
        cudaEvent_t ev;
        e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (e == cudaSuccess) free_events.push_back(ev);
    }
    if (e == cudaSuccess) {
        wv.ev = free_events.back();
        free_events.pop_back();
        e = cudaEventRecord(wv.ev, ctx->stream);
        if (e != cudaSuccess) free_events.push_back(wv.ev);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail_active(GBRT_E_CUDA, std::string("solo job launch: ") + cudaGetErrorString(e));
        return GBRT_E_CUDA;
    }
    wv.finishing.push_back(j);
    inflight.push_back(std::move(wv));
    return GBRT_OK;
}

// Launches the next unit of work: a cache job when one comes first in the
// policy's order, else a batched wave of the other jobs.  Returns GBRT_OK,
// or 1 when no active job has paths left.  Lock held.
int JobQueue::launch_next(std::unique_lock<std::mutex>& lk) {
    Job* first = nullptr;
    for (Job* j : active) {
        if (!j->paths_left) continue;
        const bool before = !first || (policy == GBRT_JOB_POLICY_SRPT
                                           ? (j->paths_left < first->paths_left ||
                                              (j->paths_left == first->paths_left && j->id < first->id))
                                           : j->id < first->id);
        if (before) first = j;
    }
    if (!first) return 1;
    if (first->cache) return run_cache_job(first, lk);
    if (solo(first)) return run_solo_job(first);
    const int rc = pack_and_launch();
    if (rc != 1) return rc;
    for (Job* j : active)  // only solo jobs left
        if (j->paths_left && solo(j)) return run_solo_job(j);
    return 1;
}

// A wave's event has fired: finish the jobs it completed.  Lock held.
void JobQueue::retire(Wave& w) {
    if (w.cancel) {
        for (Job* j : w.finishing) {
            active.erase(std::find(active.begin(), active.end(), j));
            finish_job(*this, j, GBRT_E_CANCELLED, "job cancelled");
        }
        free_events.push_back(w.ev);
        cv_done.notify_all();
        return;
    }
    for (Job* j : w.finishing) {
        DeviceCounters dc{};
        cudaError_t e = cudaMemcpyAsync(&dc, j->counters.p, sizeof(dc), cudaMemcpyDeviceToHost, dl);
        if (e == cudaSuccess && j->out_rgba8)
            e = cudaMemcpyAsync(j->out_rgba8, j->img.p, (size_t)j->npix * 4, cudaMemcpyDeviceToHost, dl);
        if (e == cudaSuccess) e = cudaStreamSynchronize(dl);
        fill_stats(&j->stats, dc, 0.0, 0);
        active.erase(std::find(active.begin(), active.end(), j));
        if (e != cudaSuccess) {
            cudaGetLastError();
            finish_job(*this, j, GBRT_E_CUDA, std::string("job download: ") + cudaGetErrorString(e));
        } else if (dc.status) {
            finish_job(*this, j, GBRT_E_DEVICE_LIMIT,
                       "a kernel reported a traversal limit (status " + std::to_string(dc.status) + ")");
        } else {
            finish_job(*this, j, GBRT_OK, "");
        }
    }
    free_events.push_back(w.ev);
    cv_done.notify_all();
}

void JobQueue::fail_active(int code, const std::string& msg) {
    cudaStreamSynchronize(ctx->stream);
    cudaGetLastError();
    for (Wave& w : inflight) free_events.push_back(w.ev);
    inflight.clear();
    for (Job* j : active) finish_job(*this, j, code, msg);
    active.clear();
    cv_done.notify_all();
}

void JobQueue::run() {
    cudaSetDevice(ctx->device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        while (admit_one(lk)) {
        }
        // retire completed waves (in order)
        while (!inflight.empty() && cudaEventQuery(inflight.front().ev) == cudaSuccess) {
            Wave w = std::move(inflight.front());
            inflight.pop_front();
            retire(w);
        }
        if ((int)inflight.size() < kMaxInFlight && launch_next(lk) == GBRT_OK) continue;
        if (!inflight.empty()) {
            cudaEvent_t ev = inflight.front().ev;
            lk.unlock();
            cudaEventSynchronize(ev);
            lk.lock();
            continue;
        }
        if (stop && queued.empty() && active.empty()) break;
        if (!queued.empty() && active.empty()) continue;  // admission retries at once
        cv_work.wait(lk);
    }
}

void jobs_shutdown(gbrt_ctx* c) {
    JobQueue* q = c->jobs;
    if (!q) return;
    {
        std::lock_guard<std::mutex> lk(q->mu);
        q->stop = true;
    }
    q->cv_work.notify_all();
    if (q->worker.joinable()) q->worker.join();
    {
        DeviceGuard g(c->device);
        for (cudaEvent_t ev : q->free_events) cudaEventDestroy(ev);
        if (q->dl) cudaStreamDestroy(q->dl);
    }
    delete q;
    c->jobs = nullptr;
}

uint32_t jobs_outstanding(const gbrt_ctx* c) {
    JobQueue* q = c->jobs;
    if (!q) return 0;
    std::lock_guard<std::mutex> lk(q->mu);
    return q->outstanding;
}

}  // namespace gbrt_host

using namespace gbrt_host;

namespace {

int job_result(JobQueue* q, gbrt_ctx* c, uint64_t id, gbrt_job_info* info, std::unique_lock<std::mutex>& lk,
               bool wait, uint32_t timeout_ms) {
    auto it = q->jobs.find(id);
    if (it == q->jobs.end()) return fail(c, GBRT_E_INVALID, "unknown job id");
    Job* j = it->second.get();
    if (wait && j->state != GBRT_JOB_DONE) {
        auto done = [&] { return j->state == GBRT_JOB_DONE; };
        if (timeout_ms == 0xFFFFFFFFu) q->cv_done.wait(lk, done);
        else q->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), done);
    }
    if (info) {
        info->state = j->state;
        info->status = j->status;
        info->queue_ms = j->t_admit > 0 ? j->t_admit - j->t_submit : 0.0;
        info->latency_ms = j->state == GBRT_JOB_DONE ? j->t_done - j->t_submit : 0.0;
        info->stats = j->stats;
    }
    if (j->state != GBRT_JOB_DONE) return GBRT_E_BUSY;
    const int st = j->status;
    const std::string msg = j->err;
    q->jobs.erase(it);
    if (st != GBRT_OK) return fail(c, st, msg);
    return GBRT_OK;
}

}  // namespace

extern "C" {

int gbrt_jobs_configure(gbrt_ctx* c, uint64_t budget, uint32_t policy) {
    if (!c) return GBRT_E_INVALID;
    if ((policy & ~GBRT_JOB_LARGE_WAVES) > GBRT_JOB_POLICY_FIFO) return fail(c, GBRT_E_INVALID, "unknown job policy");
    std::lock_guard<std::mutex> lk(c->mu);
    if (c->jobs) {
        std::lock_guard<std::mutex> lq(c->jobs->mu);
        if (budget) c->jobs->budget = budget;
        c->jobs->policy = policy & ~GBRT_JOB_LARGE_WAVES;
        // the wave buffers were sized at the first submit: larger waves only up to them
        c->jobs->deep_cap = std::min((policy & GBRT_JOB_LARGE_WAVES) ? kWaveCapLarge : kWaveCapDeep, c->wf.cap);
        return GBRT_OK;
    }
    c->jobs_budget = budget;
    c->jobs_policy = policy;
    return GBRT_OK;
}

int gbrt_job_submit(gbrt_ctx* c, const gbrt_job_desc* d, uint64_t* job_id) {
    if (!c) return GBRT_E_INVALID;
    if (!d || !job_id || !d->scene || !d->ubo || !d->accum) return fail(c, GBRT_E_INVALID, "NULL argument");
    gbrt_scene* s = d->scene;
    const gbrt_ubo& u = *d->ubo;
    if (s->ctx != c || d->accum->ctx != c) return fail(c, GBRT_E_INVALID, "scene or accumulation of another context");
    if (!s->built) return fail(c, GBRT_E_NOT_BUILT, "build the BLAS and TLAS before submitting");
    if (u.number_of_samples == 0 || u.total_number_of_samples < u.number_of_samples)
        return fail(c, GBRT_E_INVALID, "need 0 < number_of_samples <= total_number_of_samples");
    if (u.number_of_bounces > 31) return fail(c, GBRT_E_INVALID, "jobs trace at most 31 bounces");
    if (d->skins && d->nskin == 0) return fail(c, GBRT_E_INVALID, "skins given with nskin = 0");
    if (d->cache && (!d->cache_opts || nrc_ctx(d->cache) != c))
        return fail(c, GBRT_E_INVALID, "a cache job needs cache_opts and a cache of this context");
    const uint64_t npix = (uint64_t)d->accum->w * d->accum->h;
    if (npix > kWaveCap) return fail(c, GBRT_E_INVALID, "job image larger than " + std::to_string(kWaveCap) + " pixels");
    auto j = std::make_unique<Job>();
    j->scene = s;
    j->acc = d->accum;
    j->ubo = u;
    j->out_rgba8 = d->out_rgba8;
    if (d->skins) {
        j->skins.assign(d->skins, d->skins + d->nskin);
        j->has_skins = true;
    }
    if (d->cache) {
        j->cache = d->cache;
        j->copts = *d->cache_opts;
    }
    j->npix = (uint32_t)npix;
    j->ns = u.number_of_samples;
    j->sbase = u.total_number_of_samples - u.number_of_samples;
    j->chunk = std::max<uint32_t>(1, std::min<uint32_t>(j->npix, kWaveCap / kChunkDiv));
    j->paths_left = npix * j->ns;
    j->t_submit = now_ms();
    {
        std::lock_guard<std::mutex> lk(c->mu);
        if (!c->jobs) {
            DeviceGuard g(c->device);
            auto q = std::make_unique<JobQueue>();
            q->ctx = c;
            q->policy = c->jobs_policy & ~GBRT_JOB_LARGE_WAVES;
            q->deep_cap = (c->jobs_policy & GBRT_JOB_LARGE_WAVES) ? kWaveCapLarge : kWaveCapDeep;
            size_t fr = 0, tot = 0;
            cudaError_t e = cudaMemGetInfo(&fr, &tot);
            const uint64_t gib = 1ull << 30;
            q->budget = c->jobs_budget ? c->jobs_budget : (fr > gib ? fr - gib : fr / 2);
            if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&q->dl, cudaStreamNonBlocking);
            if (e == cudaSuccess) e = wavefront_reserve(c, q->deep_cap, 0) == cudaSuccess ? cudaSuccess : cudaErrorMemoryAllocation;
            if (e != cudaSuccess) {
                if (q->dl) cudaStreamDestroy(q->dl);
                return cuda_fail(c, e, "job scheduler setup");
            }
            c->jobs = q.release();
            c->jobs->worker = std::thread([q = c->jobs] { q->run(); });
        }
    }
    JobQueue* q = c->jobs;
    {
        std::lock_guard<std::mutex> lk(q->mu);
        j->id = q->next_id++;
        *job_id = j->id;
        s->jobs_pending.fetch_add(1);
        d->accum->jobs_pending.fetch_add(1);
        ++q->outstanding;
        q->queued.push_back(j.get());
        q->jobs.emplace(j->id, std::move(j));
    }
    q->cv_work.notify_all();
    return GBRT_OK;
}

int gbrt_job_cancel(gbrt_ctx* c, uint64_t id) {
    if (!c) return GBRT_E_INVALID;
    if (!c->jobs) return fail(c, GBRT_E_INVALID, "unknown job id");
    JobQueue* q = c->jobs;
    {
        std::lock_guard<std::mutex> lk(q->mu);
        auto it = q->jobs.find(id);
        if (it == q->jobs.end()) return fail(c, GBRT_E_INVALID, "unknown job id");
        Job* j = it->second.get();
        if (j->state == GBRT_JOB_DONE) return fail(c, GBRT_E_INVALID, "the job has finished");
        if (j->state == GBRT_JOB_QUEUED) {
            q->queued.erase(std::find(q->queued.begin(), q->queued.end(), j));
            finish_job(*q, j, GBRT_E_CANCELLED, "job cancelled");
            q->cv_done.notify_all();
            return GBRT_OK;
        }
        if (!j->paths_left || j->cancelled)
            return fail(c, GBRT_E_INVALID, "every path of the job is already on the stream");
        // running: no further segments; a marker after the waves already on the stream ends it
        DeviceGuard g(c->device);
        cudaEvent_t ev = nullptr;
        if (!q->free_events.empty()) {
            ev = q->free_events.back();
            q->free_events.pop_back();
        } else if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return fail(c, GBRT_E_CUDA, "event for the cancellation");
        }
        if (cudaEventRecord(ev, c->stream) != cudaSuccess) {
            cudaGetLastError();
            q->free_events.push_back(ev);
            return fail(c, GBRT_E_CUDA, "event for the cancellation");
        }
        j->paths_left = 0;
        j->cancelled = true;
        Wave w;
        w.ev = ev;
        w.cancel = true;
        w.finishing.push_back(j);
        q->inflight.push_back(std::move(w));
    }
    q->cv_work.notify_all();
    return GBRT_OK;
}

int gbrt_jobs_inject(gbrt_ctx* c, uint32_t kind, uint32_t count) {
    if (!c) return GBRT_E_INVALID;
    if (kind != GBRT_INJECT_ADMIT_OOM) return fail(c, GBRT_E_INVALID, "unknown injection");
    c->inject_admit_oom.store(count);
    return GBRT_OK;
}

int gbrt_job_poll(gbrt_ctx* c, uint64_t id, gbrt_job_info* info) {
    if (!c) return GBRT_E_INVALID;
    if (!c->jobs) return fail(c, GBRT_E_INVALID, "unknown job id");
    std::unique_lock<std::mutex> lk(c->jobs->mu);
    return job_result(c->jobs, c, id, info, lk, false, 0);
}

int gbrt_job_wait(gbrt_ctx* c, uint64_t id, uint32_t timeout_ms, gbrt_job_info* info) {
    if (!c) return GBRT_E_INVALID;
    if (!c->jobs) return fail(c, GBRT_E_INVALID, "unknown job id");
    std::unique_lock<std::mutex> lk(c->jobs->mu);
    return job_result(c->jobs, c, id, info, lk, true, timeout_ms);
}

}  // extern "C"
