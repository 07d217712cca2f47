// Many scenes on one GPU: the batched and served forms of the FLIP step.
//
// Each scene is an ordinary context (flip_create) with its own CUDA stream.
// A pool of host worker threads takes step requests from a FIFO queue; a
// request runs update(dt) on its scene `steps` times.  Requests for the
// same scene run in submission order, one at a time (a context is not
// re-entrant); requests for different scenes run on different workers, so
// their kernels overlap on the GPU.  That is where the throughput comes
// from: one scene's pressure solve is a latency-bound wavefront that keeps
// a fraction of the SMs busy, and other scenes fill the rest.  Every scene
// computes exactly what it computes alone: its kernels and their order do
// not depend on the other scenes.
//
// Batched: flip_runtime_update_all steps a set of scenes once each and
// returns when all are done.  Served: flip_runtime_submit / _wait enqueue
// requests as they arrive and report each one's latency (submission to
// completion, queueing included); flip_runtime_admit tells whether a new
// scene of a given size fits in the free device memory.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/flip3d.h"

namespace flip {
int record_error(int code, const std::string &msg);
}

struct flip_runtime {
    struct Request {
        long long id;
        flip_ctx *scene;
        double dt;
        int steps;
        std::chrono::steady_clock::time_point submitted;
    };
    struct Result {
        int status;
        double latencyMs;
    };
    int device = 0;
    long long reserveBytes = 0;
    std::vector<std::thread> workers;
    std::mutex mu;
    std::condition_variable cvWork, cvDone;
    std::deque<Request> queue;
    std::unordered_set<flip_ctx *> busy;
    std::unordered_map<long long, Result> results;
    std::unordered_set<long long> outstanding;   // submitted, not yet waited for
    long long nextId = 1;
    int running = 0;
    bool stopping = false;

    void work() {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lock(mu);
        for (;;) {
            // the oldest request whose scene is idle
            auto it = queue.end();
            cvWork.wait(lock, [&] {
                it = std::find_if(queue.begin(), queue.end(), [&](const Request &r) { return !busy.count(r.scene); });
                return stopping || it != queue.end();
            });
            if (it == queue.end()) return;   // stopping and nothing runnable
            Request r = *it;
            queue.erase(it);
            busy.insert(r.scene);
            running++;
            lock.unlock();
            int status = FLIP_OK;
            for (int s = 0; s < r.steps; s++) {
                int rc = flip_update(r.scene, r.dt);
                if (rc != FLIP_OK && status == FLIP_OK) status = rc;
                if (rc != FLIP_OK && rc != FLIP_E_SOLVER_NOCONV) break;
            }
            const double ms =
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - r.submitted).count();
            lock.lock();
            busy.erase(r.scene);
            running--;
            results[r.id] = Result{status, ms};
            cvDone.notify_all();
            cvWork.notify_all();   // a later request of this scene may be runnable now
        }
    }
};

extern "C" {

int flip_runtime_create(int workers, long long reserve_bytes, flip_runtime **out) {
    if (!out) return flip::record_error(FLIP_E_NULL, "null output pointer");
    *out = nullptr;
    if (workers < 1 || workers > 1024 || reserve_bytes < 0)
        return flip::record_error(FLIP_E_DOMAIN, "workers must be in [1, 1024] and the reserve non-negative");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    int ndev = 0;
    if (e == cudaSuccess) e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return flip::record_error(FLIP_E_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    flip_runtime *rt = new flip_runtime();
    rt->device = dev;
    rt->reserveBytes = reserve_bytes;
    for (int w = 0; w < workers; w++) rt->workers.emplace_back([rt] { rt->work(); });
    *out = rt;
    return FLIP_OK;
}

int flip_runtime_destroy(flip_runtime *rt) {
    if (!rt) return FLIP_E_NULL;
    {
        std::unique_lock<std::mutex> lock(rt->mu);
        rt->cvDone.wait(lock, [&] { return rt->queue.empty() && rt->running == 0; });   // finish what was submitted
        rt->stopping = true;
    }
    rt->cvWork.notify_all();
    for (auto &t : rt->workers) t.join();
    delete rt;
    return FLIP_OK;
}

int flip_runtime_submit(flip_runtime *rt, flip_ctx *scene, double dt, int steps, long long *request_id) {
    if (!rt || !scene || !request_id) return flip::record_error(FLIP_E_NULL, "null runtime, scene or id pointer");
    if (steps < 1) return flip::record_error(FLIP_E_DOMAIN, "steps must be at least 1");
    if (!(dt >= 0.0)) return flip::record_error(FLIP_E_DOMAIN, "Error: delta time must be greater than or equal to 0");
    std::lock_guard<std::mutex> lock(rt->mu);
    if (rt->stopping) return flip::record_error(FLIP_E_RUNTIME, "runtime is shutting down");
    const long long id = rt->nextId++;
    rt->outstanding.insert(id);
    rt->queue.push_back(flip_runtime::Request{id, scene, dt, steps, std::chrono::steady_clock::now()});
    *request_id = id;
    rt->cvWork.notify_one();
    return FLIP_OK;
}

int flip_runtime_wait(flip_runtime *rt, long long request_id, double *latency_ms, int *status) {
    if (!rt) return FLIP_E_NULL;
    std::unique_lock<std::mutex> lock(rt->mu);
    if (!rt->outstanding.count(request_id))
        return flip::record_error(FLIP_E_DOMAIN, "unknown request id, or one already waited for");
    rt->cvDone.wait(lock, [&] { return rt->results.count(request_id) > 0 || !rt->outstanding.count(request_id); });
    auto it = rt->results.find(request_id);
    if (it == rt->results.end())   // another thread waited for it first
        return flip::record_error(FLIP_E_DOMAIN, "request already waited for");
    if (latency_ms) *latency_ms = it->second.latencyMs;
    if (status) *status = it->second.status;
    rt->results.erase(it);
    rt->outstanding.erase(request_id);
    rt->cvDone.notify_all();
    return FLIP_OK;
}

int flip_runtime_update_all(flip_runtime *rt, flip_ctx **scenes, int n, double dt) {
    if (!rt || (n > 0 && !scenes)) return flip::record_error(FLIP_E_NULL, "null runtime or scene list");
    if (n < 0) return flip::record_error(FLIP_E_DOMAIN, "negative scene count");
    // largest scenes first (longest-processing-time order), so that the big
    // steps do not start last and stretch the round
    std::vector<std::pair<long long, int>> order(n);
    for (int q = 0; q < n; q++) {
        int np = 0;
        flip_get_num_marker_particles(scenes[q], &np);
        order[q] = {-(long long)np, q};
    }
    std::stable_sort(order.begin(), order.end());
    std::vector<long long> ids(n);
    for (int o = 0; o < n; o++) {
        const int q = order[o].second;
        int rc = flip_runtime_submit(rt, scenes[q], dt, 1, &ids[q]);
        if (rc) {
            for (int p = 0; p < o; p++) flip_runtime_wait(rt, ids[order[p].second], nullptr, nullptr);
            return rc;
        }
    }
    int first = FLIP_OK;
    for (int q = 0; q < n; q++) {
        int status = FLIP_OK;
        int rc = flip_runtime_wait(rt, ids[q], nullptr, &status);
        if (rc == FLIP_OK) rc = status;
        if (rc != FLIP_OK && first == FLIP_OK) first = rc;
    }
    return first;
}

int flip_runtime_admit(flip_runtime *rt, long long bytes, int *admitted) {
    if (!rt || !admitted) return FLIP_E_NULL;
    if (bytes < 0) return flip::record_error(FLIP_E_DOMAIN, "negative byte count");
    size_t freeB = 0, totalB = 0;
    cudaSetDevice(rt->device);
    cudaError_t e = cudaMemGetInfo(&freeB, &totalB);
    if (e != cudaSuccess) return flip::record_error(FLIP_E_CUDA, std::string("cudaMemGetInfo: ") + cudaGetErrorString(e));
    *admitted = (long long)freeB - rt->reserveBytes >= bytes ? 1 : 0;
    return FLIP_OK;
}

int flip_runtime_pending(flip_runtime *rt, int *queued, int *running) {
    if (!rt) return FLIP_E_NULL;
    std::lock_guard<std::mutex> lock(rt->mu);
    if (queued) *queued = (int)rt->queue.size();
    if (running) *running = rt->running;
    return FLIP_OK;
}

}  // extern "C"
