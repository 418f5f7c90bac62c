// batch.cu -- many shots advancing together on one GPU.
//
// The reference processes the shots of a rank one after another
// (acforward's shot loop, sgpstd-qrtm/acsglw.cu:304).  Here a batch keeps every
// shot resident in HBM with its own CUDA stream; the host interleaves the
// shots' revolve actions (advances in slices of a few steps), so the kernels of
// different shots overlap on the device and small windows fill the GPU
// together.  Shots may have different windows (nxx), nt and snapshot counts.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/qpstd.h"
#include "shot.h"

struct qpstd_batch {
    std::vector<qpstd_shot*> shots;
};

extern "C" int qpstd_batch_create(const qpstd_shot_desc* d, int n, qpstd_batch** out) {
    if (!d || n < 1 || !out) return QPSTD_EINVAL;
    *out = nullptr;
    qpstd_batch* b = new qpstd_batch();
    for (int i = 0; i < n; i++) {
        qpstd_shot* s = nullptr;
        const int rc = qpstd_shot_create(&d[i], &s);
        if (rc) {
            qpstd_batch_destroy(b);
            return rc;
        }
        b->shots.push_back(s);
    }
    *out = b;
    return QPSTD_OK;
}

extern "C" int qpstd_batch_destroy(qpstd_batch* b) {
    if (!b) return QPSTD_OK;
    for (qpstd_shot* s : b->shots) qpstd_shot_destroy(s);
    delete b;
    return QPSTD_OK;
}

extern "C" int qpstd_batch_size(const qpstd_batch* b) { return b ? (int)b->shots.size() : 0; }

extern "C" qpstd_shot* qpstd_batch_shot(qpstd_batch* b, int i) {
    if (!b || i < 0 || i >= (int)b->shots.size()) return nullptr;
    return b->shots[i];
}

extern "C" int qpstd_batch_sync(qpstd_batch* b) {
    if (!b) return QPSTD_EINVAL;
    for (qpstd_shot* s : b->shots) {
        const int rc = qpstd_shot_sync(s);
        if (rc) return rc;
    }
    return QPSTD_OK;
}

// Stream priorities by work: every shot gets the same number of kernel
// launches per round, but a wide window's kernels run longer, so with equal
// priorities the narrow shots finish first and the last part of the batch
// runs a few wide shots on a partly idle GPU.  The widest shots get the
// highest priority (the CTA scheduler then serves them first), in as many
// classes as the device has priorities.
static int prioritise_by_work(qpstd_batch* b) {
    int least = 0, greatest = 0;
    if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) return QPSTD_OK;
    const int levels = least - greatest + 1;
    const int n = (int)b->shots.size();
    if (levels < 2 || n < 2) return QPSTD_OK;
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    auto work = [&](int i) {
        const qpstd_shot_desc& d = b->shots[i]->d;
        return (double)d.nxx * d.nzz * d.nt;
    };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return work(x) < work(y); });
    for (int r = 0; r < n; r++) {
        const int cls = (int)((long long)r * levels / n);  // 0: least work
        const int rc = shot_set_priority(b->shots[order[r]], least - cls);
        if (rc) return rc;
    }
    return QPSTD_OK;
}

// All shots' RTM, their revolve actions interleaved round-robin; advances are
// enqueued `slice` steps at a time.  Returns after enqueueing everything (the
// results are ready after qpstd_batch_sync / qpstd_shot_get_image).
extern "C" int qpstd_batch_rtm_device(qpstd_batch* b, int slice) {
    if (!b) return QPSTD_EINVAL;
    if (const int rc = prioritise_by_work(b)) return rc;
    for (qpstd_shot* s : b->shots) {
        const int rc = rtm_begin(s);
        if (rc) return rc;
        s->run.slice = std::max(1, slice);
    }
    size_t left = b->shots.size();
    std::vector<char> done(b->shots.size(), 0);
    while (left > 0) {
        for (size_t i = 0; i < b->shots.size(); i++) {
            if (done[i]) continue;
            const int rc = rtm_action(b->shots[i]);
            if (rc < 0) return rc;
            if (rc == 1) {
                done[i] = 1;
                left--;
            }
        }
    }
    return QPSTD_OK;
}

// Pipelined steps of every shot's source wavefield (benchmarking / modeling
// without gathers): begin, step(t) for each t, end.
extern "C" int qpstd_batch_pipeline_begin(qpstd_batch* b) {
    if (!b) return QPSTD_EINVAL;
    for (qpstd_shot* s : b->shots) {
        const int rc = qpstd_shot_pipeline_begin(s);
        if (rc) return rc;
    }
    return QPSTD_OK;
}

extern "C" int qpstd_batch_pipeline_step(qpstd_batch* b, int t, int last) {
    if (!b) return QPSTD_EINVAL;
    for (qpstd_shot* s : b->shots) {
        const int rc = qpstd_shot_pipeline_step(s, t, last);
        if (rc) return rc;
    }
    return QPSTD_OK;
}

extern "C" int qpstd_batch_pipeline_end(qpstd_batch* b) {
    if (!b) return QPSTD_EINVAL;
    for (qpstd_shot* s : b->shots) {
        const int rc = qpstd_shot_pipeline_end(s);
        if (rc) return rc;
    }
    return QPSTD_OK;
}

// One call for a batch of RTM shots with host buffers (upload, concurrent
// revolve-driven RTM, download).  obs[i]: nt_i*nr_i; img[i], ssg[i]: nx_i*nz_i.
extern "C" int qpstd_rtm_batch(const qpstd_shot_desc* d, int n, const float* const* obs, float* const* img,
                               float* const* ssg) {
    if (!d || n < 1 || !obs || !img) return QPSTD_EINVAL;
    qpstd_batch* b = nullptr;
    int rc = qpstd_batch_create(d, n, &b);
    if (rc) return rc;
    for (int i = 0; i < n && !rc; i++) rc = qpstd_shot_set_obs(b->shots[i], obs[i]);
    if (!rc) rc = qpstd_batch_rtm_device(b, 8);
    for (int i = 0; i < n && !rc; i++) rc = qpstd_shot_get_image(b->shots[i], img[i], ssg ? ssg[i] : nullptr);
    qpstd_batch_destroy(b);
    return rc;
}
