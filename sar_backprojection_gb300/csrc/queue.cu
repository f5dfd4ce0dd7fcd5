// queue.cu -- continuous-batching focusing queue behind the C ABI
// (sarbp_queue_create / submit / poll / wait / destroy).
//
// A worker thread owns two streams and two batch workspaces.  Submitted jobs
// (device-resident scenes, caller-owned buffers) wait in FIFO order; the
// worker admits them into free scene slots (chunk tables prepared, the
// scene's record written into both batch workspaces), then runs the device
// in waves: each wave is one launch of the persistent batch kernel over up
// to `wave_items` (slot, tile) items taken from the admitted jobs in arrival
// order, alternating streams so one wave's tail overlaps the next.  A job is
// done when the last wave holding its tiles has finished; the batch status
// of that wave tells whether a bounded device wait gave up.
#include <algorithm>
#include <condition_variable>
#include <chrono>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "sarbp_internal.cuh"

namespace sarbp {
namespace {

struct QJob {
    int64_t id = 0;
    SceneParams P{};
    double *out = nullptr;
    int slot = -1;
    void *ws = nullptr;
    size_t ws_bytes = 0;
    int64_t ntiles = 0;
    int64_t next_tile = 0;
    int waves_in_flight = 0;
    int status = SARBP_OK;
    bool done = false;
};

struct Wave {
    cudaEvent_t ev;
    int turn;
    std::vector<int64_t> jobs;   // jobs with items in this wave
};

}  // namespace

struct Queue {
    int device = 0;
    sarbp_tuning T{};
    int max_slots = 0;
    int64_t wave_items = 0;
    size_t bws_bytes = 0;
    void *bws[2] = {nullptr, nullptr};
    cudaStream_t stream[2] = {nullptr, nullptr};
    int turn = 0;

    std::mutex mu;
    std::condition_variable cv;       // worker wake-up
    std::condition_variable done_cv;  // job completion
    std::deque<int64_t> pending;      // submitted, not admitted
    std::vector<int64_t> active;      // admitted, not done
    std::unordered_map<int64_t, std::unique_ptr<QJob>> jobs;
    std::vector<int> free_slots;
    std::deque<Wave> waves;
    int64_t next_id = 0;
    bool stopping = false;
    int fatal = SARBP_OK;
    std::thread worker;

    void run();
    int admit(QJob &j);
    int launch_wave(bool *launched);
    int retire_waves(bool block);
    void finish(QJob &j);
};

static int queue_cuda(cudaError_t e, const char *what)
{
    return cuda_status(e, what);
}

int Queue::admit(QJob &j)
{
    const MixedLayout L = mixed_layout(j.P, T);
    j.ws_bytes = L.total;
    int rc = queue_cuda(cudaMalloc(&j.ws, j.ws_bytes), "queue: scene workspace");
    if (rc) return rc;
    rc = launch_mixed_prepare(j.P, T, j.ws, j.ws_bytes, stream[0]);
    if (rc) return rc;
    rc = tile_count(j.P, T, &j.ntiles);
    if (rc) return rc;
    for (int b = 0; b < 2; ++b) {
        rc = batch_set_scene(bws[b], bws_bytes, j.slot, max_slots, j.P, T, j.ws, j.ws_bytes,
                             j.out, nullptr, nullptr, stream[b]);
        if (rc) return rc;
    }
    // the second stream's waves must see the tables the first stream prepared
    cudaEvent_t ready;
    rc = queue_cuda(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming), "queue: event");
    if (rc) return rc;
    cudaEventRecord(ready, stream[0]);
    cudaStreamWaitEvent(stream[1], ready, 0);
    cudaEventDestroy(ready);
    return SARBP_OK;
}

void Queue::finish(QJob &j)
{
    if (j.ws) cudaFree(j.ws);
    j.ws = nullptr;
    if (j.slot >= 0) free_slots.push_back(j.slot);
    j.slot = -1;
    j.done = true;
}

// One wave over the admitted jobs' next tiles, in arrival order.
int Queue::launch_wave(bool *launched)
{
    *launched = false;
    std::vector<int32_t> items;
    Wave w;
    for (int64_t id : active) {
        QJob &j = *jobs[id];
        if (j.next_tile >= j.ntiles) continue;
        bool used = false;
        while (j.next_tile < j.ntiles && (int64_t)items.size() / 2 < wave_items) {
            items.push_back(j.slot);
            items.push_back((int32_t)j.next_tile++);
            used = true;
        }
        if (used) {
            ++j.waves_in_flight;
            w.jobs.push_back(id);
        }
        if ((int64_t)items.size() / 2 >= wave_items) break;
    }
    if (items.empty()) return SARBP_OK;
    const int64_t n = (int64_t)items.size() / 2;
    w.turn = turn;
    turn ^= 1;
    cudaStream_t s = stream[w.turn];
    int rc = batch_set_items(bws[w.turn], bws_bytes, max_slots, items.data(), n, s);
    if (!rc) rc = batch_focus(bws[w.turn], bws_bytes, max_slots, T, n, false, nullptr, s);
    if (!rc) rc = queue_cuda(cudaEventCreateWithFlags(&w.ev, cudaEventDisableTiming),
                             "queue: wave event");
    if (!rc) rc = queue_cuda(cudaEventRecord(w.ev, s), "queue: wave record");
    if (rc) return rc;
    waves.push_back(std::move(w));
    *launched = true;
    return SARBP_OK;
}

// Retire finished waves (in launch order); with `block`, wait for the oldest.
int Queue::retire_waves(bool block)
{
    while (!waves.empty()) {
        Wave &w = waves.front();
        cudaError_t q = block ? cudaEventSynchronize(w.ev) : cudaEventQuery(w.ev);
        if (q == cudaErrorNotReady) return SARBP_OK;
        int rc = queue_cuda(q, "queue: wave");
        if (rc) return rc;
        // batch status of this wave: a bounded device wait gave up?
        StatusBlock st;
        rc = queue_cuda(cudaMemcpy(&st, bws[w.turn], sizeof(st), cudaMemcpyDeviceToHost),
                        "queue: batch status");
        if (rc) return rc;
        if (st.error) cudaMemsetAsync(bws[w.turn], 0, sizeof(StatusBlock), stream[w.turn]);
        cudaEventDestroy(w.ev);
        {
            std::lock_guard<std::mutex> lk(mu);
            for (int64_t id : w.jobs) {
                QJob &j = *jobs[id];
                if (st.error) j.status = SARBP_ETIMEOUT;
                if (--j.waves_in_flight == 0 && j.next_tile >= j.ntiles) {
                    finish(j);
                    active.erase(std::find(active.begin(), active.end(), id));
                }
            }
        }
        done_cv.notify_all();
        waves.pop_front();
        block = false;
    }
    return SARBP_OK;
}

void Queue::run()
{
    cudaSetDevice(device);
    for (;;) {
        std::vector<int64_t> admit_now;
        {
            std::unique_lock<std::mutex> lk(mu);
            const bool work = !pending.empty() || !active.empty() || !waves.empty();
            if (!work) {
                if (stopping) break;
                cv.wait_for(lk, std::chrono::milliseconds(5));
                continue;
            }
            while (!pending.empty() && !free_slots.empty()) {
                const int64_t id = pending.front();
                pending.pop_front();
                QJob &j = *jobs[id];
                j.slot = free_slots.back();
                free_slots.pop_back();
                admit_now.push_back(id);
            }
        }
        int rc = SARBP_OK;
        for (int64_t id : admit_now) {
            QJob *j;
            {
                std::lock_guard<std::mutex> lk(mu);
                j = jobs[id].get();
            }
            rc = admit(*j);
            std::lock_guard<std::mutex> lk(mu);
            if (rc) {
                j->status = rc;
                finish(*j);
                done_cv.notify_all();
                rc = SARBP_OK;   // this job failed; the queue goes on
            } else {
                active.push_back(id);
            }
        }
        // keep at most two waves in flight (one per stream); with nothing new
        // to launch, wait for the oldest
        bool launched = false;
        if (waves.size() < 2) {
            std::lock_guard<std::mutex> lk(mu);
            rc = launch_wave(&launched);
        }
        if (!rc) rc = retire_waves(waves.size() >= 2 || (!launched && !waves.empty()));
        if (rc) {
            std::lock_guard<std::mutex> lk(mu);
            fatal = rc;
            for (auto &kv : jobs)
                if (!kv.second->done) {
                    kv.second->status = rc;
                    finish(*kv.second);
                }
            pending.clear();
            active.clear();
            done_cv.notify_all();
            break;
        }
    }
}

}  // namespace sarbp

using namespace sarbp;

struct sarbp_queue {
    Queue q;
};

extern "C" {

SARBP_API int sarbp_queue_create(sarbp_queue **queue, const sarbp_tuning *tuning,
                                 int32_t max_slots, int64_t wave_items)
{
    if (!queue || max_slots <= 0 || max_slots > 1024 || wave_items < 0) {
        set_error("sarbp_queue_create: bad arguments (max_slots %d, wave_items %lld)",
                  max_slots, (long long)wave_items);
        return SARBP_EINVAL;
    }
    sarbp_tuning T;
    if (tuning) {
        T = *tuning;
    } else {
        memset(&T, 0, sizeof(T));
    }
    if (!valid_tuning(&T)) return SARBP_EINVAL;
    if (T.staged != 1) {
        set_error("sarbp_queue_create: the queue runs the batch kernel (tuning.staged = 1)");
        return SARBP_EINVAL;
    }
    auto *h = new (std::nothrow) sarbp_queue;
    if (!h) {
        set_error("sarbp_queue_create: out of host memory");
        return SARBP_EINVAL;
    }
    Queue &q = h->q;
    cudaGetDevice(&q.device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, q.device);
    q.T = T;
    q.max_slots = max_slots;
    q.wave_items = wave_items > 0 ? wave_items : (int64_t)6 * sms;
    q.bws_bytes = (size_t)batch_workspace_size(max_slots, q.wave_items);
    int rc = SARBP_OK;
    for (int b = 0; b < 2 && !rc; ++b) {
        rc = cuda_status(cudaMalloc(&q.bws[b], q.bws_bytes), "sarbp_queue_create: workspace");
        if (!rc) rc = cuda_status(cudaMemset(q.bws[b], 0, q.bws_bytes), "sarbp_queue_create");
        if (!rc)
            rc = cuda_status(cudaStreamCreateWithFlags(&q.stream[b], cudaStreamNonBlocking),
                             "sarbp_queue_create: stream");
    }
    if (rc) {
        for (int b = 0; b < 2; ++b) {
            if (q.bws[b]) cudaFree(q.bws[b]);
            if (q.stream[b]) cudaStreamDestroy(q.stream[b]);
        }
        delete h;
        return rc;
    }
    for (int s = max_slots - 1; s >= 0; --s) q.free_slots.push_back(s);
    q.worker = std::thread([&q] { q.run(); });
    *queue = h;
    return SARBP_OK;
}

SARBP_API int64_t sarbp_queue_submit(sarbp_queue *queue, const sarbp_scene *scene, double *out)
{
    if (!queue || !out) {
        set_error("sarbp_queue_submit: queue or out is NULL");
        return SARBP_EINVAL;
    }
    auto j = std::make_unique<QJob>();
    if (!build_params(scene, &j->P)) return SARBP_EINVAL;
    j->P.wait_polls = queue->q.T.wait_polls > 0 ? (uint32_t)queue->q.T.wait_polls : (1u << 22);
    j->out = out;
    Queue &q = queue->q;
    int64_t id;
    {
        std::lock_guard<std::mutex> lk(q.mu);
        if (q.fatal) {
            set_error("sarbp_queue_submit: the queue stopped after an error");
            return q.fatal;
        }
        id = q.next_id++;
        j->id = id;
        q.jobs.emplace(id, std::move(j));
        q.pending.push_back(id);
    }
    q.cv.notify_one();
    return id;
}

static int job_state(Queue &q, int64_t job, bool *done)
{
    auto it = q.jobs.find(job);
    if (it == q.jobs.end()) {
        set_error("sarbp_queue: unknown job %lld", (long long)job);
        return SARBP_EINVAL;
    }
    *done = it->second->done;
    const int st = it->second->status;
    if (*done) q.jobs.erase(it);   // completion is reported once: the id is released
    if (*done && st) {
        set_error("sarbp_queue: job %lld failed (status %d)", (long long)job, st);
        return st;
    }
    return SARBP_OK;
}

SARBP_API int sarbp_queue_poll(sarbp_queue *queue, int64_t job)
{
    if (!queue) return SARBP_EINVAL;
    std::lock_guard<std::mutex> lk(queue->q.mu);
    bool done = false;
    const int rc = job_state(queue->q, job, &done);
    return rc ? rc : (done ? 1 : 0);
}

SARBP_API int sarbp_queue_wait(sarbp_queue *queue, int64_t job)
{
    if (!queue) return SARBP_EINVAL;
    Queue &q = queue->q;
    std::unique_lock<std::mutex> lk(q.mu);
    for (;;) {
        bool done = false;
        const int rc = job_state(q, job, &done);
        if (rc || done) return rc;
        q.done_cv.wait_for(lk, std::chrono::milliseconds(50));
    }
}

SARBP_API int sarbp_queue_destroy(sarbp_queue *queue)
{
    if (!queue) return SARBP_OK;
    Queue &q = queue->q;
    {
        std::lock_guard<std::mutex> lk(q.mu);
        q.stopping = true;
    }
    q.cv.notify_all();
    if (q.worker.joinable()) q.worker.join();
    for (auto &kv : q.jobs)
        if (kv.second->ws) cudaFree(kv.second->ws);
    for (int b = 0; b < 2; ++b) {
        if (q.stream[b]) cudaStreamDestroy(q.stream[b]);
        if (q.bws[b]) cudaFree(q.bws[b]);
    }
    const int rc = q.fatal;
    delete queue;
    return rc;
}

}  // extern "C"
