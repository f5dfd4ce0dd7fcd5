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
//
// Host-memory jobs (sarbp_queue_submit_host) take the whole request path
// without the caller: admitted when a slot is free and their device copies
// fit in the queue's reserved device memory (first fit, in arrival order),
// their small inputs go up, their chunk tables and the bound of the range
// bins their apertures can reach are computed on a setup stream (the bound
// lands in pinned memory); only the reachable bins of each pulse row are
// then copied on a copy stream, queued at admission behind the set-up (a
// device-side wait) by a copy kernel that reads the bound itself, so no
// host round trip separates one job's bound from its upload (layouts that
// kernel cannot take wait for the bound on the host instead); once the rows
// have landed the job's tiles join waves; after its last wave its image
// goes back to the caller's host buffer on a read-back stream.  Sources and
// destinations the device can reach (page-locked memory, and on GB300 any
// host memory) are copied by SM loads and stores, so no step makes the
// worker wait for the GPU; it polls events between steps.  Device-resident
// jobs take their chunk-table workspace from the reserved memory too when
// it is reserved.
#include <algorithm>
#include <condition_variable>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "sarbp_internal.cuh"

namespace sarbp {
namespace {

enum HostStage { kQueued, kSetup, kUpload, kActive, kReadback };

// CTAs of a host job's raw-row copy (four rows, 64 KB of loads in flight
// each).  Saturated 500-job serving from host memory: 48 CTAs 93.5
// Gpix-pulse/s (0.66 of the link), 152: 87.8, 608: 78.6 -- the copy shares
// the SMs with the waves, and fewer, deeper copy CTAs leave them more room
constexpr int kRowCopyCtas = 48;

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
    double done_s = 0.0;          // completion time, steady clock seconds
    // host-memory jobs: the caller's host arrays (scene H), its host image,
    // the job's share of the reserved device memory and its current step
    bool host = false;
    SceneParams H{};
    double *host_out = nullptr;
    size_t arena_off = 0, arena_bytes = 0;
    HostStage stage = kQueued;
    cudaEvent_t ev = nullptr;
    bool rows_queued = false;     // raw rows enqueued behind the bound (no host wait)
};

// Device copies of a host job, carved from the queue's reserved memory
// (offsets 256-byte aligned): DEM x/y/z, mask, index, Sint, trajectory,
// raw rows (even pitch), image, chunk-table workspace.
struct HostLayout {
    size_t x, y, z, mask, index, sint, tx, ty, tz, raw, out, ws, total;
    int64_t pitch;
    size_t ws_bytes;
};

static size_t up256(size_t v) { return (v + 255) & ~(size_t)255; }

static HostLayout host_layout(const SceneParams &P, const sarbp_tuning &T)
{
    HostLayout h{};
    const size_t npix = (size_t)P.npix, naz = (size_t)P.naz;
    h.pitch = P.nra + (P.nra & 1);
    size_t o = 0;
    auto take = [&o](size_t bytes) {
        const size_t at = o;
        o = up256(o + bytes);
        return at;
    };
    h.x = take(8 * npix);
    h.y = take(8 * npix);
    h.z = take(8 * npix);
    h.mask = take(npix);
    h.index = take(4 * npix);
    h.sint = take(4 * npix);
    h.tx = take(8 * naz);
    h.ty = take(8 * naz);
    h.tz = take(8 * naz);
    h.raw = take(8 * (size_t)h.pitch * naz);
    h.out = take(16 * npix);
    h.ws_bytes = mixed_layout(P, T).total;
    h.ws = take(h.ws_bytes);
    h.total = o;
    return h;
}

// First-fit allocator over one reserved device allocation.
struct Arena {
    char *base = nullptr;
    size_t bytes = 0;
    std::map<size_t, size_t> free_;   // offset -> size, coalesced

    void reset(char *b, size_t n)
    {
        base = b;
        bytes = n;
        free_.clear();
        if (n) free_[0] = n;
    }
    bool alloc(size_t n, size_t *off)
    {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            *off = it->first;
            const size_t rest = it->second - n;
            const size_t at = it->first + n;
            free_.erase(it);
            if (rest) free_[at] = rest;
            return true;
        }
        return false;
    }
    void release(size_t off, size_t n)
    {
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
};

static double steady_seconds()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct Wave {
    cudaEvent_t ev;
    int turn;
    std::vector<int64_t> jobs;   // jobs with items in this wave
};

// The batch status word of a wave into mapped page-locked host memory (an
// SM store: the worker reads it once the wave's event has completed, with no
// copy or synchronisation of its own).
__global__ void wave_status_kernel(const StatusBlock *st, unsigned *host_word)
{
    *host_word = st->error;
}

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
    // totals since creation: completed jobs, waves, kernel launches, bytes
    // copied host -> device and device -> host
    int64_t stat_jobs = 0, stat_waves = 0, stat_launches = 0, stat_h2d = 0, stat_d2h = 0;
    unsigned *wave_error = nullptr;   // mapped pinned: batch status per turn
    unsigned *wave_error_dev = nullptr;
    int64_t next_id = 0;
    bool stopping = false;
    int fatal = SARBP_OK;
    std::thread worker;
    // host-memory jobs
    Arena arena;                      // reserved device memory (sarbp_queue_reserve)
    int32_t *bounds = nullptr;        // pinned: reachable-bin bound per slot
    cudaStream_t setup = nullptr, copy = nullptr, readback = nullptr;
    std::vector<int64_t> staging;     // host jobs in set-up, upload or read-back (worker)
    std::deque<int64_t> completions;  // finished jobs, reported by sarbp_queue_completed

    void run();
    int admit(QJob &j);
    int admit_host(QJob &j);
    bool advance_host();
    int launch_wave(bool *launched);
    int retire_waves(bool *retired);
    void finish(QJob &j);
    void fail(QJob &j, int rc);
};

static int queue_cuda(cudaError_t e, const char *what)
{
    return cuda_status(e, what);
}

int Queue::admit(QJob &j)
{
    const MixedLayout L = mixed_layout(j.P, T);
    j.ws_bytes = L.total;
    int rc = SARBP_OK;
    if (j.arena_bytes) {
        // carved from the reserved memory at admission: no cudaMalloc, and
        // no device-wide synchronisation of a cudaFree when it retires
        j.ws = arena.base + j.arena_off;
    } else {
        rc = queue_cuda(cudaMalloc(&j.ws, j.ws_bytes), "queue: scene workspace");
        if (rc) return rc;
    }
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

// Upload a host job's small inputs, prepare its chunk tables and batch slot,
// and bound its reachable range bins, all on the setup stream (no wait).
int Queue::admit_host(QJob &j)
{
    const HostLayout h = host_layout(j.H, T);
    char *b = arena.base + j.arena_off;
    SceneParams D = j.H;
    D.x = reinterpret_cast<const double *>(b + h.x);
    D.y = reinterpret_cast<const double *>(b + h.y);
    D.z = reinterpret_cast<const double *>(b + h.z);
    D.mask = reinterpret_cast<const uint8_t *>(b + h.mask);
    D.index = reinterpret_cast<const int32_t *>(b + h.index);
    D.sint = reinterpret_cast<const int32_t *>(b + h.sint);
    D.tx = reinterpret_cast<const double *>(b + h.tx);
    D.ty = reinterpret_cast<const double *>(b + h.ty);
    D.tz = reinterpret_cast<const double *>(b + h.tz);
    D.raw = reinterpret_cast<const float2 *>(b + h.raw);
    D.pitch = h.pitch;
    j.P = D;
    j.out = reinterpret_cast<double *>(b + h.out);
    j.ws = b + h.ws;
    j.ws_bytes = h.ws_bytes;
    const int64_t npix = j.H.npix, naz = j.H.naz;
    struct Part {
        const void *dst, *src;
        int64_t bytes;
    } parts[9] = {{D.x, j.H.x, 8 * npix},     {D.y, j.H.y, 8 * npix},
                  {D.z, j.H.z, 8 * npix},     {D.mask, j.H.mask, npix},
                  {D.index, j.H.index, 4 * npix}, {D.sint, j.H.sint, 4 * npix},
                  {D.tx, j.H.tx, 8 * naz},    {D.ty, j.H.ty, 8 * naz},
                  {D.tz, j.H.tz, 8 * naz}};
    int rc = SARBP_OK;
    for (const Part &p : parts) {
        rc = h2d_bytes(const_cast<void *>(p.dst), p.src, p.bytes, setup);
        if (rc) return rc;
    }
    rc = launch_mixed_prepare(D, T, j.ws, j.ws_bytes, setup);
    if (rc) return rc;
    rc = tile_count(D, T, &j.ntiles);
    if (rc) return rc;
    for (int k = 0; k < 2; ++k) {
        rc = batch_set_scene(bws[k], bws_bytes, j.slot, max_slots, D, T, j.ws, j.ws_bytes, j.out,
                             nullptr, nullptr, setup);
        if (rc) return rc;
    }
    rc = raw_bin_range_async(D, T, j.ws, j.ws_bytes, bounds + 2 * j.slot, setup);
    if (rc) return rc;
    // the reachable raw rows straight behind the bound, the copy kernel
    // reading the bound from page-locked memory: no host round trip between
    // one job's bound and its upload (layouts the 16-byte copy cannot take
    // wait for the bound on the host, then h2d_rows)
    rc = queue_cuda(cudaEventCreateWithFlags(&j.ev, cudaEventDisableTiming), "queue: job event");
    if (rc) return rc;
    rc = queue_cuda(cudaEventRecord(j.ev, setup), "queue: set-up record");
    if (rc) return rc;
    // on the copy stream, behind this job's set-up (a device-side wait), so
    // the next jobs' set-up overlaps this upload
    rc = queue_cuda(cudaStreamWaitEvent(copy, j.ev, 0), "queue: upload wait");
    if (rc) return rc;
    j.rows_queued = h2d_rows_bound(const_cast<float2 *>(D.raw), D.pitch, j.H.raw, j.H.pitch,
                                   bounds + 2 * j.slot, naz, kRowCopyCtas, copy) == SARBP_OK;
    cudaGetLastError();
    if (j.rows_queued) {
        rc = queue_cuda(cudaEventRecord(j.ev, copy), "queue: upload record");
        if (rc) return rc;
    }
    {
        std::lock_guard<std::mutex> lk(mu);
        stat_launches += 9 + 1 + 3 + 2 + (j.rows_queued ? 1 : 0);
        stat_h2d += 33 * npix + 24 * naz;
    }
    j.stage = j.rows_queued ? kUpload : kSetup;
    return SARBP_OK;
}

// Move host jobs along when their last step has completed: set-up -> raw
// upload of the reachable bins -> waves; read-back -> done.
bool Queue::advance_host()
{
    bool progress = false;
    std::vector<int64_t> keep;
    for (int64_t id : staging) {
        QJob *jp;
        {
            std::lock_guard<std::mutex> lk(mu);
            jp = jobs[id].get();
        }
        QJob &j = *jp;
        const cudaError_t q = cudaEventQuery(j.ev);
        if (q == cudaErrorNotReady) {
            keep.push_back(id);
            continue;
        }
        progress = true;
        int rc = queue_cuda(q, "queue: job step");
        if (!rc && j.stage == kSetup) {
            const int32_t lo = bounds[2 * j.slot], hi = bounds[2 * j.slot + 1];
            if (hi >= lo) {
                rc = h2d_rows(const_cast<float2 *>(j.P.raw), j.P.pitch, j.H.raw, j.H.pitch, lo,
                              (int64_t)hi - lo + 1, j.H.naz, copy);
                std::lock_guard<std::mutex> lk(mu);
                stat_launches += 1;
                stat_h2d += 8 * ((int64_t)hi - lo + 1) * j.H.naz;
            }
            if (!rc) rc = queue_cuda(cudaEventRecord(j.ev, copy), "queue: upload record");
            if (!rc) {
                j.stage = kUpload;
                keep.push_back(id);
            }
        } else if (!rc && j.stage == kUpload) {
            j.stage = kActive;                      // its tiles join the next waves
            std::lock_guard<std::mutex> lk(mu);
            if (j.rows_queued) {
                const int32_t lo = bounds[2 * j.slot], hi = bounds[2 * j.slot + 1];
                if (hi >= lo) stat_h2d += 8 * ((int64_t)hi - lo + 1) * j.H.naz;
            }
            active.push_back(id);
        } else if (!rc && j.stage == kReadback) {
            std::lock_guard<std::mutex> lk(mu);
            finish(j);
            done_cv.notify_all();
        }
        if (rc) {
            std::lock_guard<std::mutex> lk(mu);
            fail(j, rc);
        }
    }
    staging.swap(keep);
    return progress;
}

void Queue::finish(QJob &j)
{
    if (j.arena_bytes) arena.release(j.arena_off, j.arena_bytes);
    if (j.host) {
        j.ws = nullptr;
        if (j.ev) cudaEventDestroy(j.ev);
        j.ev = nullptr;
    } else if (j.ws && !j.arena_bytes) {
        cudaFree(j.ws);
    }
    j.arena_bytes = 0;
    j.ws = nullptr;
    if (j.slot >= 0) free_slots.push_back(j.slot);
    j.slot = -1;
    j.done = true;
    j.done_s = steady_seconds();
    stat_jobs += 1;
    // ids already reported through poll/wait are dropped from the front
    while (completions.size() > 4096 && !jobs.count(completions.front())) completions.pop_front();
    completions.push_back(j.id);
}

void Queue::fail(QJob &j, int rc)
{
    j.status = rc;
    auto it = std::find(active.begin(), active.end(), j.id);
    if (it != active.end()) active.erase(it);
    finish(j);
    done_cv.notify_all();
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
    if (!rc) {
        wave_status_kernel<<<1, 1, 0, s>>>(reinterpret_cast<const StatusBlock *>(bws[w.turn]),
                                           wave_error_dev + w.turn);
        rc = queue_cuda(cudaGetLastError(), "queue: wave status");
    }
    if (!rc) rc = queue_cuda(cudaEventCreateWithFlags(&w.ev, cudaEventDisableTiming),
                             "queue: wave event");
    if (!rc) rc = queue_cuda(cudaEventRecord(w.ev, s), "queue: wave record");
    if (rc) return rc;
    waves.push_back(std::move(w));
    *launched = true;
    stat_waves += 1;
    stat_launches += 2;   // persistent batch kernel, status word
    return SARBP_OK;
}

// Retire finished waves (in launch order).
int Queue::retire_waves(bool *retired)
{
    *retired = false;
    while (!waves.empty()) {
        Wave &w = waves.front();
        cudaError_t q = cudaEventQuery(w.ev);
        if (q == cudaErrorNotReady) return SARBP_OK;
        *retired = true;
        int rc = queue_cuda(q, "queue: wave");
        if (rc) return rc;
        // batch status of this wave: a bounded device wait gave up?
        struct {
            unsigned error;
        } st{((volatile unsigned *)wave_error)[w.turn]};
        if (st.error) cudaMemsetAsync(bws[w.turn], 0, sizeof(StatusBlock), stream[w.turn]);
        cudaEventDestroy(w.ev);
        {
            std::lock_guard<std::mutex> lk(mu);
            for (int64_t id : w.jobs) {
                QJob &j = *jobs[id];
                if (st.error) j.status = SARBP_ETIMEOUT;
                if (--j.waves_in_flight == 0 && j.next_tile >= j.ntiles) {
                    active.erase(std::find(active.begin(), active.end(), id));
                    if (!j.host) {
                        finish(j);
                        continue;
                    }
                    // the image goes back to the caller's host buffer
                    int rc2 = d2h_bytes(j.host_out, j.out, 16 * j.P.npix, readback);
                    stat_launches += 1;
                    stat_d2h += 16 * j.P.npix;
                    if (!rc2) rc2 = queue_cuda(cudaEventRecord(j.ev, readback),
                                               "queue: read-back record");
                    if (rc2) {
                        fail(j, rc2);
                        continue;
                    }
                    j.stage = kReadback;
                    staging.push_back(id);
                }
            }
        }
        done_cv.notify_all();
        waves.pop_front();
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
            const bool work = !pending.empty() || !active.empty() || !waves.empty() ||
                              !staging.empty();
            if (!work) {
                if (stopping) break;
                cv.wait_for(lk, std::chrono::milliseconds(5));
                continue;
            }
            // arrival order: a host job that does not fit the reserved
            // memory yet holds the jobs behind it
            while (!pending.empty() && !free_slots.empty()) {
                QJob &j = *jobs[pending.front()];
                if (j.host && !arena.alloc(j.arena_bytes, &j.arena_off)) break;
                if (!j.host && arena.base) {
                    // a device job's workspace comes from the reserved memory
                    // when it fits there (else from cudaMalloc at admission)
                    const size_t need = up256(mixed_layout(j.P, T).total);
                    if (need <= arena.bytes) {
                        if (!arena.alloc(need, &j.arena_off)) break;
                        j.arena_bytes = need;
                    }
                }
                pending.pop_front();
                j.slot = free_slots.back();
                free_slots.pop_back();
                admit_now.push_back(j.id);
            }
        }
        bool progress = !admit_now.empty();
        int rc = SARBP_OK;
        for (int64_t id : admit_now) {
            QJob *j;
            {
                std::lock_guard<std::mutex> lk(mu);
                j = jobs[id].get();
            }
            rc = j->host ? admit_host(*j) : admit(*j);
            std::lock_guard<std::mutex> lk(mu);
            if (rc) {
                fail(*j, rc);    // this job failed; the queue goes on
                rc = SARBP_OK;
            } else if (j->host) {
                staging.push_back(id);
            } else {
                active.push_back(id);
            }
        }
        if (advance_host()) progress = true;
        // keep at most two waves in flight (one per stream)
        bool launched = false;
        if (waves.size() < 2) {
            std::lock_guard<std::mutex> lk(mu);
            rc = launch_wave(&launched);
        }
        bool retired = false;
        if (!rc) rc = retire_waves(&retired);
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
            staging.clear();
            done_cv.notify_all();
            break;
        }
        // nothing moved: the device is busy with what is queued; poll again soon
        if (!(progress || launched || retired))
            std::this_thread::sleep_for(std::chrono::microseconds(20));
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
    if (!rc)
        rc = cuda_status(cudaHostAlloc((void **)&q.wave_error, 2 * sizeof(unsigned),
                                       cudaHostAllocMapped),
                         "sarbp_queue_create: status words");
    if (!rc)
        rc = cuda_status(cudaHostGetDevicePointer((void **)&q.wave_error_dev, q.wave_error, 0),
                         "sarbp_queue_create: status words");
    if (rc) {
        for (int b = 0; b < 2; ++b) {
            if (q.bws[b]) cudaFree(q.bws[b]);
            if (q.stream[b]) cudaStreamDestroy(q.stream[b]);
        }
        if (q.wave_error) cudaFreeHost(q.wave_error);
        delete h;
        return rc;
    }
    q.wave_error[0] = q.wave_error[1] = 0;
    for (int s = max_slots - 1; s >= 0; --s) q.free_slots.push_back(s);
    q.worker = std::thread([&q] { q.run(); });
    *queue = h;
    return SARBP_OK;
}

SARBP_API int sarbp_queue_reserve(sarbp_queue *queue, size_t bytes)
{
    if (!queue || bytes == 0) {
        set_error("sarbp_queue_reserve: queue is NULL or no bytes asked for");
        return SARBP_EINVAL;
    }
    Queue &q = queue->q;
    {
        std::lock_guard<std::mutex> lk(q.mu);
        if (q.arena.base) {
            set_error("sarbp_queue_reserve: device memory is already reserved");
            return SARBP_EINVAL;
        }
    }
    int dev = 0;
    int rc = cuda_status(cudaGetDevice(&dev), "sarbp_queue_reserve: device");
    if (rc) return rc;
    rc = cuda_status(cudaSetDevice(q.device), "sarbp_queue_reserve: device");
    if (rc) return rc;
    void *base = nullptr;
    int32_t *bounds = nullptr;
    cudaStream_t st[3] = {nullptr, nullptr, nullptr};
    rc = cuda_status(cudaMalloc(&base, bytes), "sarbp_queue_reserve: device memory");
    if (!rc)
        rc = cuda_status(cudaHostAlloc((void **)&bounds, sizeof(int32_t) * 2 * q.max_slots,
                                       cudaHostAllocDefault),
                         "sarbp_queue_reserve: pinned bounds");
    for (int k = 0; k < 3 && !rc; ++k)
        rc = cuda_status(cudaStreamCreateWithFlags(&st[k], cudaStreamNonBlocking),
                         "sarbp_queue_reserve: stream");
    cudaSetDevice(dev);
    if (rc) {
        if (base) cudaFree(base);
        if (bounds) cudaFreeHost(bounds);
        for (cudaStream_t x : st)
            if (x) cudaStreamDestroy(x);
        return rc;
    }
    std::lock_guard<std::mutex> lk(q.mu);
    q.arena.reset(static_cast<char *>(base), bytes);
    q.bounds = bounds;
    q.setup = st[0];
    q.copy = st[1];
    q.readback = st[2];
    return SARBP_OK;
}

SARBP_API int64_t sarbp_queue_job_bytes(sarbp_queue *queue, const sarbp_scene *scene)
{
    if (!queue) {
        set_error("sarbp_queue_job_bytes: queue is NULL");
        return SARBP_EINVAL;
    }
    SceneParams P;
    if (!build_params(scene, &P)) return SARBP_EINVAL;
    return (int64_t)host_layout(P, queue->q.T).total;
}

SARBP_API int64_t sarbp_queue_submit_host(sarbp_queue *queue, const sarbp_scene *host_scene,
                                          double *host_out)
{
    if (!queue || !host_out) {
        set_error("sarbp_queue_submit_host: queue or host_out is NULL");
        return SARBP_EINVAL;
    }
    auto j = std::make_unique<QJob>();
    if (!build_params(host_scene, &j->H)) return SARBP_EINVAL;
    Queue &q = queue->q;
    j->H.wait_polls = q.T.wait_polls > 0 ? (uint32_t)q.T.wait_polls : (1u << 22);
    j->host = true;
    j->host_out = host_out;
    j->arena_bytes = host_layout(j->H, q.T).total;
    int64_t id;
    {
        std::lock_guard<std::mutex> lk(q.mu);
        if (!q.arena.base) {
            set_error("sarbp_queue_submit_host: no device memory reserved "
                      "(sarbp_queue_reserve)");
            return SARBP_EINVAL;
        }
        if (j->arena_bytes > q.arena.bytes) {
            set_error("sarbp_queue_submit_host: the job needs %zu bytes of device memory, the "
                      "queue reserved %zu",
                      j->arena_bytes, q.arena.bytes);
            return SARBP_ERANGE;
        }
        if (q.fatal) {
            set_error("sarbp_queue_submit_host: the queue stopped after an error");
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

SARBP_API int sarbp_queue_cancel(sarbp_queue *queue, int64_t job)
{
    if (!queue) {
        set_error("sarbp_queue_cancel: queue is NULL");
        return SARBP_EINVAL;
    }
    Queue &q = queue->q;
    std::lock_guard<std::mutex> lk(q.mu);
    auto it = q.jobs.find(job);
    if (it == q.jobs.end()) {
        set_error("sarbp_queue_cancel: unknown job %lld", (long long)job);
        return SARBP_EINVAL;
    }
    auto pit = std::find(q.pending.begin(), q.pending.end(), job);
    if (pit == q.pending.end()) {
        set_error("sarbp_queue_cancel: job %lld is already admitted or done", (long long)job);
        return SARBP_EINVAL;
    }
    q.pending.erase(pit);
    QJob &j = *it->second;
    j.status = SARBP_ECANCELED;
    j.arena_bytes = 0;                 // nothing was carved for it
    q.finish(j);
    q.done_cv.notify_all();
    return SARBP_OK;
}

SARBP_API int sarbp_queue_stats(sarbp_queue *queue, int64_t *stats)
{
    if (!queue || !stats) {
        set_error("sarbp_queue_stats: queue or stats is NULL");
        return SARBP_EINVAL;
    }
    Queue &q = queue->q;
    std::lock_guard<std::mutex> lk(q.mu);
    stats[0] = q.stat_jobs;
    stats[1] = q.stat_waves;
    stats[2] = q.stat_launches;
    stats[3] = q.stat_h2d;
    stats[4] = q.stat_d2h;
    return SARBP_OK;
}

SARBP_API int64_t sarbp_queue_completed(sarbp_queue *queue, int64_t *ids, double *done_s,
                                        int32_t *status, int64_t max)
{
    if (!queue || !ids || max < 0) {
        set_error("sarbp_queue_completed: queue or ids is NULL");
        return SARBP_EINVAL;
    }
    Queue &q = queue->q;
    std::lock_guard<std::mutex> lk(q.mu);
    int64_t n = 0;
    while (n < max && !q.completions.empty()) {
        const int64_t id = q.completions.front();
        q.completions.pop_front();
        auto it = q.jobs.find(id);
        if (it == q.jobs.end()) continue;          // reported through poll/wait already
        ids[n] = id;
        if (done_s) done_s[n] = it->second->done_s;
        if (status) status[n] = it->second->status;
        q.jobs.erase(it);
        ++n;
    }
    return n;
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
        if (kv.second->ws && !kv.second->host && !kv.second->arena_bytes)
            cudaFree(kv.second->ws);
    for (int b = 0; b < 2; ++b) {
        if (q.stream[b]) cudaStreamDestroy(q.stream[b]);
        if (q.bws[b]) cudaFree(q.bws[b]);
    }
    for (cudaStream_t x : {q.setup, q.copy, q.readback})
        if (x) cudaStreamDestroy(x);
    if (q.arena.base) cudaFree(q.arena.base);
    if (q.bounds) cudaFreeHost(q.bounds);
    if (q.wave_error) cudaFreeHost(q.wave_error);
    const int rc = q.fatal;
    delete queue;
    return rc;
}

}  // extern "C"
