// lsgb_server.cpp -- continuous-batching request loop over the engine (lsgb_server_* ABI).
//
// The reference has no serving path: every LombScarglePy call is one synchronous
// batch (source/main.cu:742-941). Here objects are submitted one at a time as they
// arrive; a dispatcher thread packs whatever has arrived into the next free slot,
// admits it only while the in-flight device footprint stays under an HBM budget,
// and launches it on that slot's own stream and engine, so several batches overlap
// on the GPU. Results (best frequency index and power) are published with their
// completion times; per-object results do not depend on which batch an object
// joined, because every (object, frequency tile) unit is computed the same way in
// any batch.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/lsgb.h"

namespace lsgb {
void set_last_error(const char *msg);
}

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

struct Pending {
    uint64_t id;
    double t_submit;
    std::vector<double> t, y, dy;
};

struct Done {
    uint64_t id;
    uint32_t idx;
    double power;
    double t_submit, t_done;
};

template <typename T>
struct Pinned {
    T *p = nullptr;
    size_t cap = 0;
    Pinned() = default;
    Pinned(const Pinned &) = delete;
    Pinned &operator=(const Pinned &) = delete;
    bool ensure(size_t n) {
        if (n <= cap && p) return true;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        if (cudaHostAlloc((void **)&p, sizeof(T) * std::max<size_t>(n, 1), cudaHostAllocDefault) !=
            cudaSuccess)
            return false;
        cap = std::max<size_t>(n, 1);
        return true;
    }
    ~Pinned() {
        if (p) cudaFreeHost(p);
    }
};

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    bool ensure(size_t bytes) {
        if (bytes <= cap && p) return true;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        if (cudaMalloc(&p, std::max<size_t>(bytes, 256)) != cudaSuccess) return false;
        cap = std::max<size_t>(bytes, 256);
        return true;
    }
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

struct Slot {
    lsgb_engine *eng = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    bool busy = false;
    size_t footprint = 0;
    std::vector<Pending> objs;
    std::vector<uint64_t> offsets;
    Pinned<double> h_t, h_y, h_dy, h_power;
    Pinned<uint32_t> h_idx, h_status;  // h_status: the batch's status word (LSGB_STATUS_*)
    DevBuf d_t, d_y, d_dy, d_idx, d_power;
};

}  // namespace

struct lsgb_server {
    int device = 0;
    int variant = 0, precision = 1, normalize = 1;
    double fmin = 0, df = 0;
    uint32_t n_freq = 0, max_batch = 0;
    size_t budget = 0, inflight_bytes = 0, peak_inflight_bytes = 0;
    std::vector<std::unique_ptr<Slot>> slots;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Pending> pending;
    std::deque<Done> done;
    std::atomic<bool> stop{false};
    std::thread worker;
    std::string error;
    uint64_t batches = 0, objects_done = 0, max_batch_seen = 0;
    uint64_t peak_busy_slots = 0, peak_waiting = 0;  // lsgb_server_peaks
    uint64_t budget_deferrals = 0;  // admissions that stopped at the HBM budget
};

namespace {

// Device bytes a batch holds while in flight: inputs, engine records and tables.
size_t batch_footprint(const lsgb_server *s, size_t rows, size_t objs) {
    const size_t tiles = (s->n_freq + 2047) / 2048;  // smallest mixed tile, upper bound
    return rows * (3 * 8 + 32) + objs * (72 + 8 + 4 + 8 + 4 + 16 * tiles);
}

void publish(lsgb_server *s, Slot &sl) {
    const double t = now_s();
    std::lock_guard<std::mutex> lk(s->mu);
    if (sl.h_status.p[0] != 0) {
        // the batch's results are invalid: stop with an error instead of publishing them
        s->error = sl.h_status.p[0] & LSGB_STATUS_BAD_INPUT
                       ? "server: a submitted object has a non-finite t / y or an invalid dy"
                       : "server: a pipeline wait of the tensor-form kernel timed out";
        s->stop = true;
        s->inflight_bytes -= sl.footprint;
        sl.busy = false;
        sl.objs.clear();
        return;
    }
    for (size_t i = 0; i < sl.objs.size(); ++i)
        s->done.push_back(Done{sl.objs[i].id, sl.h_idx.p[i], sl.h_power.p[i], sl.objs[i].t_submit, t});
    s->objects_done += sl.objs.size();
    s->inflight_bytes -= sl.footprint;
    sl.busy = false;
    sl.objs.clear();
}

// Packs, copies and launches one batch on its slot; returns "" or an error message.
std::string launch(lsgb_server *s, Slot &sl) {
    const size_t n_obj = sl.objs.size();
    size_t rows = 0;
    for (auto &o : sl.objs) rows += o.t.size();
    if (!sl.h_t.ensure(rows) || !sl.h_y.ensure(rows) || !sl.h_dy.ensure(rows) ||
        !sl.h_idx.ensure(n_obj) || !sl.h_power.ensure(n_obj) || !sl.h_status.ensure(1) ||
        !sl.d_t.ensure(8 * rows) ||
        !sl.d_y.ensure(8 * rows) || !sl.d_dy.ensure(8 * rows) || !sl.d_idx.ensure(4 * n_obj) ||
        !sl.d_power.ensure(8 * n_obj))
        return "server: staging allocation failed";
    sl.offsets.assign(1, 0);
    size_t r = 0;
    for (auto &o : sl.objs) {
        memcpy(sl.h_t.p + r, o.t.data(), 8 * o.t.size());
        memcpy(sl.h_y.p + r, o.y.data(), 8 * o.y.size());
        if (s->variant == LSGB_GENERALIZED) memcpy(sl.h_dy.p + r, o.dy.data(), 8 * o.dy.size());
        r += o.t.size();
        sl.offsets.push_back(r);
    }
    cudaStream_t st = sl.stream;
    cudaMemcpyAsync(sl.d_t.p, sl.h_t.p, 8 * rows, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(sl.d_y.p, sl.h_y.p, 8 * rows, cudaMemcpyHostToDevice, st);
    if (s->variant == LSGB_GENERALIZED)
        cudaMemcpyAsync(sl.d_dy.p, sl.h_dy.p, 8 * rows, cudaMemcpyHostToDevice, st);
    int rc = lsgb_periodogram_device(
        sl.eng, s->variant, s->precision, LSGB_F64, sl.d_t.p, sl.d_y.p,
        s->variant == LSGB_GENERALIZED ? sl.d_dy.p : nullptr, sl.offsets.data(), (uint32_t)n_obj,
        s->fmin, s->df, s->n_freq, s->normalize, nullptr, (uint32_t *)sl.d_idx.p, sl.d_power.p,
        (void *)st);
    if (rc != LSGB_OK) return std::string("server: ") + lsgb_last_error();
    cudaMemcpyAsync(sl.h_idx.p, sl.d_idx.p, 4 * n_obj, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(sl.h_power.p, sl.d_power.p, 8 * n_obj, cudaMemcpyDeviceToHost, st);
    // what the batch's kernels recorded arrives with its results; publish() checks it
    if (lsgb_status_async(sl.eng, sl.h_status.p, (void *)st) != LSGB_OK)
        return std::string("server: ") + lsgb_last_error();
    if (cudaEventRecord(sl.done, st) != cudaSuccess) return "server: cudaEventRecord failed";
    return "";
}

void dispatcher(lsgb_server *s) {
    cudaSetDevice(s->device);
    while (true) {
        // 1. retire finished batches
        bool any_busy = false;
        for (auto &slp : s->slots) {
            Slot &sl = *slp;
            if (!sl.busy) continue;
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaSuccess) {
                publish(s, sl);
            } else if (q != cudaErrorNotReady) {
                std::lock_guard<std::mutex> lk(s->mu);
                s->error = std::string("server: ") + cudaGetErrorString(q);
                s->stop = true;
                sl.busy = false;  // its results are lost; the error is reported by poll
            } else {
                any_busy = true;
            }
        }
        // 2. admit arrived objects into a free slot while the HBM budget allows
        Slot *free_slot = nullptr;
        for (auto &slp : s->slots)
            if (!slp->busy) {
                free_slot = slp.get();
                break;
            }
        bool launched = false;
        if (free_slot && !s->stop) {
            std::unique_lock<std::mutex> lk(s->mu);
            size_t rows = 0, take = 0;
            bool over_budget = false;
            while (take < s->pending.size() && take < s->max_batch) {
                const size_t r2 = rows + s->pending[take].t.size();
                const size_t fp = batch_footprint(s, r2, take + 1);
                over_budget = s->inflight_bytes + fp > s->budget &&
                              (take > 0 || s->inflight_bytes > 0);
                if (over_budget) break;
                rows = r2;
                ++take;
            }
            if (over_budget) s->budget_deferrals++;  // objects left waiting for memory
            if (take > 0) {
                Slot &sl = *free_slot;
                sl.objs.assign(std::make_move_iterator(s->pending.begin()),
                               std::make_move_iterator(s->pending.begin() + take));
                s->pending.erase(s->pending.begin(), s->pending.begin() + take);
                sl.footprint = batch_footprint(s, rows, take);
                s->inflight_bytes += sl.footprint;
                s->peak_inflight_bytes = std::max(s->peak_inflight_bytes, s->inflight_bytes);
                sl.busy = true;
                s->batches++;
                s->max_batch_seen = std::max<uint64_t>(s->max_batch_seen, take);
                uint64_t busy = 0;
                for (auto &sp : s->slots) busy += sp->busy ? 1 : 0;
                s->peak_busy_slots = std::max(s->peak_busy_slots, busy);
                lk.unlock();
                const std::string err = launch(s, sl);
                if (!err.empty()) {
                    std::lock_guard<std::mutex> lk2(s->mu);
                    s->error = err;
                    s->stop = true;
                    sl.busy = false;
                    s->inflight_bytes -= sl.footprint;
                } else {
                    launched = true;
                    any_busy = true;
                }
            }
        }
        if (s->stop) {
            bool busy = false;
            for (auto &slp : s->slots) busy |= slp->busy;
            if (!busy) break;
        }
        if (!launched) {
            if (any_busy) {
                // a batch is on the GPU: poll its event again at once, so that its completion
                // time is taken when it completes (a timed sleep here overshoots by tens of
                // microseconds, the size of a small batch's whole latency)
                std::this_thread::yield();
            } else {
                std::unique_lock<std::mutex> lk(s->mu);
                s->cv.wait_for(lk, std::chrono::milliseconds(2),
                               [&] { return !s->pending.empty() || s->stop.load(); });
            }
        }
    }
}

}  // namespace

extern "C" {

LSGB_API int lsgb_server_create(int device, int variant, int precision, double fmin, double df,
                                uint32_t n_freq, int normalize, uint32_t slots,
                                uint32_t max_batch_objects, uint64_t hbm_budget_bytes,
                                lsgb_server **out) {
    if (!out || slots == 0 || slots > 16 || max_batch_objects == 0 || n_freq == 0 ||
        (variant != LSGB_STANDARD && variant != LSGB_GENERALIZED) ||
        (precision != LSGB_PLAIN_FP64 && precision != LSGB_MIXED)) {
        lsgb::set_last_error("lsgb_server_create: bad argument");
        return LSGB_ERR_INVALID;
    }
    lsgb_server *s = new lsgb_server();
    s->device = device;
    s->variant = variant;
    s->precision = precision;
    s->fmin = fmin;
    s->df = df;
    s->n_freq = n_freq;
    s->normalize = normalize;
    s->max_batch = max_batch_objects;
    s->budget = hbm_budget_bytes;
    for (uint32_t i = 0; i < slots; ++i) s->slots.emplace_back(new Slot());
    for (auto &slp : s->slots) {
        Slot &sl = *slp;
        int rc = lsgb_engine_create(device, &sl.eng);
        if (rc != LSGB_OK || cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) {
            for (auto &xp : s->slots) {
                if (xp->eng) lsgb_engine_destroy(xp->eng);
                if (xp->stream) cudaStreamDestroy(xp->stream);
                if (xp->done) cudaEventDestroy(xp->done);
            }
            delete s;
            lsgb::set_last_error("lsgb_server_create: engine or stream set-up failed");
            return rc != LSGB_OK ? rc : LSGB_ERR_CUDA;
        }
    }
    s->worker = std::thread(dispatcher, s);
    *out = s;
    return LSGB_OK;
}

LSGB_API int lsgb_server_submit(lsgb_server *s, uint64_t id, const double *t, const double *y,
                                const double *dy, uint32_t n) {
    if (!s || !t || !y || n == 0 || (s->variant == LSGB_GENERALIZED && !dy)) {
        lsgb::set_last_error("lsgb_server_submit: bad argument");
        return LSGB_ERR_INVALID;
    }
    Pending p;
    p.id = id;
    p.t.assign(t, t + n);
    p.y.assign(y, y + n);
    if (s->variant == LSGB_GENERALIZED) p.dy.assign(dy, dy + n);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) {
            lsgb::set_last_error(s->error.empty() ? "server stopped" : s->error.c_str());
            return LSGB_ERR_CUDA;
        }
        p.t_submit = now_s();
        s->pending.push_back(std::move(p));
        s->peak_waiting = std::max<uint64_t>(s->peak_waiting, s->pending.size());
    }
    s->cv.notify_one();
    return LSGB_OK;
}

// Completed objects, up to max: ids, best index, best power, submit and completion
// times (seconds on a monotonic clock). Returns how many were written.
LSGB_API int lsgb_server_poll(lsgb_server *s, uint32_t max, uint64_t *ids, uint32_t *idx,
                              double *power, double *t_submit, double *t_done) {
    if (!s) return LSGB_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    uint32_t n = 0;
    while (n < max && !s->done.empty()) {
        const Done &d = s->done.front();
        if (ids) ids[n] = d.id;
        if (idx) idx[n] = d.idx;
        if (power) power[n] = d.power;
        if (t_submit) t_submit[n] = d.t_submit;
        if (t_done) t_done[n] = d.t_done;
        s->done.pop_front();
        ++n;
    }
    if (n == 0 && !s->error.empty()) {
        lsgb::set_last_error(s->error.c_str());
        return LSGB_ERR_CUDA;
    }
    return (int)n;
}

// Counters: [batches, objects completed, largest batch, pending, peak in-flight bytes].
LSGB_API int lsgb_server_stats(lsgb_server *s, uint64_t *out5) {
    if (!s || !out5) return LSGB_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    out5[0] = s->batches;
    out5[1] = s->objects_done;
    out5[2] = s->max_batch_seen;
    out5[3] = s->pending.size();
    out5[4] = s->peak_inflight_bytes;
    return LSGB_OK;
}

// Peaks: [device bytes in flight, batches (slots) in flight at once, objects waiting for
// admission, admissions stopped at the HBM budget].
LSGB_API int lsgb_server_peaks(lsgb_server *s, uint64_t *out4) {
    if (!s || !out4) return LSGB_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    out4[0] = s->peak_inflight_bytes;
    out4[1] = s->peak_busy_slots;
    out4[2] = s->peak_waiting;
    out4[3] = s->budget_deferrals;
    return LSGB_OK;
}

LSGB_API double lsgb_server_now(void) { return now_s(); }

// Drains submitted work, stops the dispatcher and frees everything.
LSGB_API void lsgb_server_destroy(lsgb_server *s) {
    if (!s) return;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        while (!s->pending.empty() && s->error.empty()) {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(200));
            lk.lock();
        }
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->device);
    for (auto &slp : s->slots) {
        Slot &sl = *slp;
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.eng) lsgb_engine_destroy(sl.eng);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
    }
    delete s;
}

}  // extern "C"
