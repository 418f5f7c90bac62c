// server.cpp -- continuous batching of shot requests on one GPU.
//
// The reference's programs run a fixed list of shots, one after another
// (acforward's shot loop).  A server instead takes requests of any kind (aps,
// vaps, artm, qrtm) and grid at any time and keeps the GPU shared among them:
//   * admission: queued requests enter in arrival order while a slot and the
//     device-memory budget allow; an RTM request gets the largest revolve
//     snapshot count, up to its own snaps, that fits what is left (at least
//     min(snaps, 4) while other shots run);
//   * execution: every admitted shot has its own stream and advances in slices
//     (modeling: steps with the gather kept on the device; RTM: revolve actions
//     of a bounded number of steps), at most two slices in flight per shot, so
//     shots admitted later overlap with the running ones on the device;
//   * retirement: once a shot's last slice has completed, its result is copied
//     to the caller's buffers and its memory returns to the server's arena (no
//     cudaFree, which would wait for every other shot's work).
// One worker thread drives all of it; submit / status / wait are thread-safe.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/qpstd.h"
#include "arena.h"
#include "shot.h"

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Req {
    qpstd_shot_desc d{};
    const float* obs = nullptr;
    float* out0 = nullptr;
    float* out1 = nullptr;
    int state = 0;  // 0 queued, 1 running, 2 done, < 0 failed (status code)
    double t_submit = 0.0, t_done = 0.0;
    int snaps_used = 0;
    bool plain = false;  // served in the plain form
    size_t bytes = 0;
    // while running
    qpstd_shot* shot = nullptr;
    int t_next = 0;
    bool all_enqueued = false;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    bool ev_live[2] = {false, false};
    int ev_next = 0;
};

const int kModelSlice = 32;    // modeling steps per slice
const int kRtmSteps = 16;      // steps per revolve advance action
const int kRtmActions = 4;     // actions per RTM slice

}  // namespace

struct qpstd_server {
    int device = 0;
    qp::Arena arena;
    size_t budget = 0, reserved = 0;
    int max_active = 64;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<long long> queue;
    std::unordered_map<long long, std::unique_ptr<Req>> reqs;  // stable addresses
    std::vector<long long> active;
    long long next_id = 0;
    bool stop = false;
    std::thread worker;
};

namespace {

bool is_rtm(const qpstd_shot_desc& d) { return d.kind == QPSTD_ARTM || d.kind == QPSTD_QRTM; }

int inflight(Req& r) {
    int n = 0;
    for (int k = 0; k < 2; k++)
        if (r.ev_live[k]) {
            if (cudaEventQuery(r.ev[k]) == cudaSuccess) r.ev_live[k] = false;
            else n++;
        }
    return n;
}

void release(qpstd_server* sv, Req& r) {
    for (int k = 0; k < 2; k++)
        if (r.ev[k]) cudaEventDestroy(r.ev[k]);
    r.ev[0] = r.ev[1] = nullptr;
    if (r.shot) qpstd_shot_destroy(r.shot);
    r.shot = nullptr;
    sv->reserved -= std::min(sv->reserved, r.bytes);
}

// Enqueue one slice of r's work; returns a status code.
int feed(Req& r) {
    int rc = QPSTD_OK;
    if (!is_rtm(r.d)) {
        const int n = std::min(kModelSlice, r.d.nt - r.t_next);
        rc = model_slice(r.shot, r.t_next, n);
        r.t_next += n;
        if (r.t_next >= r.d.nt) r.all_enqueued = true;
    } else {
        for (int a = 0; a < kRtmActions && !r.all_enqueued && rc == QPSTD_OK; a++) {
            const int q = rtm_action(r.shot);
            if (q < 0) rc = q;
            else if (q == 1) r.all_enqueued = true;
        }
    }
    if (rc) return rc;
    const int k = r.ev_next;
    r.ev_next ^= 1;
    if (cudaEventRecord(r.ev[k], r.shot->stream) != cudaSuccess) return QPSTD_ECUDA;
    r.ev_live[k] = true;
    return QPSTD_OK;
}

// Copy the finished shot's result to the caller (its stream is idle by now).
int collect(Req& r) {
    qpstd_shot* s = r.shot;
    if (is_rtm(r.d)) return qpstd_shot_get_image(s, r.out0, r.out1);
    if (r.d.nr > 0 && r.out0) {
        const size_t bytes = sizeof(float) * (size_t)r.d.nt * r.d.nr;
        if (cudaMemcpyAsync(r.out0, s->gather, bytes, cudaMemcpyDeviceToHost, s->stream) != cudaSuccess)
            return QPSTD_ECUDA;
    }
    return cudaStreamSynchronize(s->stream) == cudaSuccess ? QPSTD_OK : QPSTD_ECUDA;
}

// Admit r if memory allows; returns 1 admitted, 0 not now, < 0 failed.
int admit(qpstd_server* sv, Req& r, bool alone) {
    qpstd_shot_desc d = r.d;
    // windows whose transforms the fused passes cannot plan (x lines beyond the
    // compiled long plans, about 4600 points; z lines beyond about 2800) run in
    // the plain cuFFT form
    if (qpstd_shot_bytes(&d) < 0) d.method = QPSTD_PLAIN;
    r.plain = d.method == QPSTD_PLAIN;
    const size_t avail = sv->budget > sv->reserved ? sv->budget - sv->reserved : 0;
    size_t need = 0;
    if (is_rtm(d)) {
        const double N = (double)d.nxx * d.nzz;
        const size_t per_snap = (size_t)(32.0 * N) + 256;
        qpstd_shot_desc d0 = d;
        d0.snaps = 0;
        const long long base = qpstd_shot_bytes(&d0);
        if (base < 0) return QPSTD_EINVAL;
        const int want = d.snaps;
        const int floor_snaps = alone ? 1 : std::min(want, 4);
        int fit = (avail > (size_t)base) ? (int)((avail - (size_t)base) / per_snap) : 0;
        fit = std::min(fit, want);
        // the snapshot pool is one block: it must fit the arena's largest hole too
        while (fit >= floor_snaps && (size_t)fit * per_snap > sv->arena.largest_free()) fit--;
        if (fit < floor_snaps) return alone ? QPSTD_ENOMEM : 0;
        d.snaps = fit;
        need = (size_t)base + (size_t)fit * per_snap;
    } else {
        const long long b = qpstd_shot_bytes(&d);
        if (b < 0) return QPSTD_EINVAL;
        need = (size_t)b;
        if (need > avail) return alone ? QPSTD_ENOMEM : 0;
    }
    qpstd_shot* s = nullptr;
    int rc = shot_create_ex(&d, &s, false, &sv->arena);
    if (rc == QPSTD_ENOMEM && !alone) return 0;  // fragmentation: wait for running shots
    if (rc) return rc;
    r.shot = s;
    r.bytes = need;
    r.snaps_used = is_rtm(d) ? d.snaps : 0;
    sv->reserved += need;
    for (int k = 0; k < 2; k++)
        if (cudaEventCreateWithFlags(&r.ev[k], cudaEventDisableTiming) != cudaSuccess) return QPSTD_ECUDA;
    if (is_rtm(d)) {
        if ((rc = qpstd_shot_set_obs(s, r.obs))) return rc;
        if ((rc = rtm_begin(s))) return rc;
        s->run.slice = kRtmSteps;
    }
    return 1;
}

Req* lookup(qpstd_server* sv, long long id) {
    std::lock_guard<std::mutex> lk(sv->mu);
    return sv->reqs[id].get();
}

void finish(qpstd_server* sv, long long id, Req& r, int code) {
    // the library's error text is per thread: report it from here
    if (code) fprintf(stderr, "qpstd_server: request %lld failed (%d): %s\n", id, code, qpstd_last_error());
    release(sv, r);
    std::lock_guard<std::mutex> lk(sv->mu);
    r.state = code ? code : 2;
    r.t_done = now_s();
    sv->cv.notify_all();
}

void worker_main(qpstd_server* sv) {
    cudaSetDevice(sv->device);
    for (;;) {
        bool busy = false;
        // retire finished shots, feed running ones
        for (size_t i = 0; i < sv->active.size();) {
            const long long id = sv->active[i];
            Req& r = *lookup(sv, id);
            int code = QPSTD_OK;
            bool done = false;
            int n = inflight(r);
            if (r.all_enqueued && n == 0) {
                code = collect(r);
                done = true;
            } else {
                while (!r.all_enqueued && n < 2 && code == QPSTD_OK) {
                    code = feed(r);
                    n++;
                    busy = true;
                }
                if (code) done = true;
            }
            if (done) {
                if (code && r.shot) cudaStreamSynchronize(r.shot->stream);
                finish(sv, id, r, code);
                sv->active.erase(sv->active.begin() + i);
                busy = true;
                continue;
            }
            i++;
        }
        // admit queued requests in arrival order
        for (;;) {
            long long id = -1;
            {
                std::lock_guard<std::mutex> lk(sv->mu);
                if (sv->queue.empty() || (int)sv->active.size() >= sv->max_active) break;
                id = sv->queue.front();
            }
            Req& r = *lookup(sv, id);
            const int a = admit(sv, r, sv->active.empty());
            if (a == 0) break;
            {
                std::lock_guard<std::mutex> lk(sv->mu);
                sv->queue.pop_front();
                if (a > 0) r.state = 1;
            }
            busy = true;
            if (a < 0) {
                finish(sv, id, r, a);
                continue;
            }
            sv->active.push_back(id);
        }
        std::unique_lock<std::mutex> lk(sv->mu);
        if (sv->stop && sv->queue.empty() && sv->active.empty()) return;
        if (!busy) sv->cv.wait_for(lk, std::chrono::microseconds(200));
    }
}

}  // namespace

extern "C" int qpstd_server_create(long long mem_budget, int max_active, qpstd_server** out) {
    if (!out) return QPSTD_EINVAL;
    *out = nullptr;
    qpstd_server* sv = new qpstd_server();
    cudaGetDevice(&sv->device);
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        delete sv;
        return QPSTD_ECUDA;
    }
    size_t b = mem_budget > 0 ? (size_t)mem_budget : (size_t)(0.85 * (double)fr);
    b = std::min(b, (size_t)(0.95 * (double)fr));
    if (sv->arena.init(b) != cudaSuccess) {
        delete sv;
        return QPSTD_ENOMEM;
    }
    sv->budget = b;
    sv->max_active = max_active > 0 ? max_active : 64;
    sv->worker = std::thread(worker_main, sv);
    *out = sv;
    return QPSTD_OK;
}

extern "C" int qpstd_server_destroy(qpstd_server* sv) {
    if (!sv) return QPSTD_OK;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
        sv->cv.notify_all();
    }
    if (sv->worker.joinable()) sv->worker.join();
    delete sv;
    return QPSTD_OK;
}

extern "C" long long qpstd_server_submit(qpstd_server* sv, const qpstd_shot_desc* d, const float* obs, float* out0,
                                         float* out1) {
    if (!sv || !d) return QPSTD_EINVAL;
    if (is_rtm(*d) && (!obs || !out0)) return QPSTD_EINVAL;
    std::unique_ptr<Req> r(new Req());
    r->d = *d;
    r->obs = obs;
    r->out0 = out0;
    r->out1 = out1;
    r->t_submit = now_s();
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->stop) return QPSTD_EINVAL;
    const long long id = sv->next_id++;
    sv->reqs.emplace(id, std::move(r));
    sv->queue.push_back(id);
    sv->cv.notify_all();
    return id;
}

extern "C" int qpstd_server_status(qpstd_server* sv, long long id, double* latency_s, int* snaps_used) {
    if (!sv) return QPSTD_EINVAL;
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(id);
    if (it == sv->reqs.end()) return QPSTD_EINVAL;
    const Req& r = *it->second;
    if (latency_s) *latency_s = (r.state == 2 || r.state < 0) ? r.t_done - r.t_submit : now_s() - r.t_submit;
    if (snaps_used) *snaps_used = r.snaps_used;
    return r.state;
}

extern "C" int qpstd_server_wait(qpstd_server* sv, long long id) {
    if (!sv) return QPSTD_EINVAL;
    std::unique_lock<std::mutex> lk(sv->mu);
    if (id >= 0) {
        auto it = sv->reqs.find(id);
        if (it == sv->reqs.end()) return QPSTD_EINVAL;
        const Req* r = it->second.get();
        sv->cv.wait(lk, [&] { return r->state == 2 || r->state < 0; });
        return r->state < 0 ? r->state : QPSTD_OK;
    }
    sv->cv.wait(lk, [&] {
        for (auto& kv : sv->reqs)
            if (kv.second->state == 0 || kv.second->state == 1) return false;
        return true;
    });
    for (auto& kv : sv->reqs)
        if (kv.second->state < 0) return kv.second->state;
    return QPSTD_OK;
}
