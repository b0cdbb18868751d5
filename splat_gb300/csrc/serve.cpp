// serve.cpp -- the continuous-batching render server (the served form) on
// top of the batch engine: requests wait in arrival order, are admitted while
// the engine has a slot and pool room and their light maps fit the map
// budget, join the engine's next tick, and complete on the device.  Scenes
// are caller-owned (the caller keeps geometry resident and evicts it); the
// server owns the engine, the queue, the tick events and the bookkeeping.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <deque>
#include <new>
#include <string>
#include <vector>

#include "kernels.h"

using splat::set_error;

namespace {

struct Request {
    int64_t id = 0;
    const splat_scene_t* scene = nullptr;
    splat_trace_params_t params;
    void* map = nullptr;
    int64_t map_bytes = 0;
};

struct Completion {
    int64_t id;
    int32_t slot;
    int64_t map_bytes;
    cudaEvent_t ev;  // recorded after the tick that ran the request's last bounce
};

// rays of a frame: its range of the light's grid
int64_t rays_of(const splat_trace_params_t& p) {
    if (p.upscale < 1) return 0;
    const int64_t n_grid = (p.light.res1 / p.upscale) * (p.light.res2 / p.upscale);
    const int64_t rb = p.ray_begin < 0 ? 0 : p.ray_begin;
    const int64_t re = (p.ray_end <= 0 || p.ray_end > n_grid) ? n_grid : p.ray_end;
    return re - rb;
}

int64_t map_bytes_of(const splat_trace_params_t& p) {
    const int64_t planes = p.n_lambda > 0 ? p.n_lambda : 1;
    return p.map_w * p.map_h * planes * 4;
}

splat_status_t cuda_error(cudaError_t e, const char* what) {
    return set_error(SPLAT_ERR_CUDA, std::string("server: ") + what + ": " + cudaGetErrorString(e));
}

}  // namespace

struct splat_server {
    splat_batch_t* engine = nullptr;
    int32_t max_items = 0;
    int64_t map_budget = 0, map_in_use = 0, pool_rays = 0;
    int32_t max_ahead = 4;
    int64_t next_id = 1;
    std::deque<Request> pending;
    std::vector<Request> in_flight;      // by slot
    std::vector<uint8_t> slot_used;
    std::deque<cudaEvent_t> ahead;        // tick events the host has not waited for
    std::vector<cudaEvent_t> free_events;
    std::vector<Completion> completing;
    std::vector<std::pair<int64_t, double>> done;  // (id, device ms since the first step)
    cudaEvent_t t0 = nullptr;
    bool started = false;
    std::vector<int32_t> done_slots;
};

namespace {

cudaError_t take_event(splat_server* s, cudaEvent_t* ev) {
    if (!s->free_events.empty()) {
        *ev = s->free_events.back();
        s->free_events.pop_back();
        return cudaSuccess;
    }
    return cudaEventCreate(ev);
}

// An event goes back to the pool once neither the run-ahead queue nor a
// pending completion refers to it.
void maybe_free(splat_server* s, cudaEvent_t ev) {
    for (cudaEvent_t e : s->ahead)
        if (e == ev) return;
    for (const Completion& c : s->completing)
        if (c.ev == ev) return;
    for (cudaEvent_t e : s->free_events)
        if (e == ev) return;
    s->free_events.push_back(ev);
}

// Moves completions whose event has passed (or every one, when block) to the
// done list and frees their slots and map budget.
splat_status_t collect(splat_server* s, bool block) {
    std::vector<Completion> keep, gone;
    for (const Completion& c : s->completing) {
        cudaError_t q = block ? cudaEventSynchronize(c.ev) : cudaEventQuery(c.ev);
        if (q == cudaErrorNotReady) {
            keep.push_back(c);
            continue;
        }
        if (q != cudaSuccess) return cuda_error(q, "completion event");
        float ms = 0.f;
        cudaError_t e = cudaEventElapsedTime(&ms, s->t0, c.ev);
        if (e != cudaSuccess) return cuda_error(e, "completion time");
        splat_status_t rc = splat_batch_release(s->engine, c.slot);
        if (rc != SPLAT_OK) return rc;
        s->slot_used[(size_t)c.slot] = 0;
        s->map_in_use -= c.map_bytes;
        s->done.emplace_back(c.id, (double)ms);
        gone.push_back(c);
    }
    s->completing.swap(keep);
    for (const Completion& c : gone) maybe_free(s, c.ev);
    return SPLAT_OK;
}

}  // namespace

extern "C" {

splat_status_t splat_server_create(int32_t max_items, int64_t max_pool_rays, int64_t map_budget_bytes,
                                   int32_t max_ticks_ahead, splat_server_t** out) {
    if (!out) return set_error(SPLAT_ERR_INVALID, "server_create: out is null");
    *out = nullptr;
    if (map_budget_bytes < 0 || max_ticks_ahead < 1 || max_ticks_ahead > 64)
        return set_error(SPLAT_ERR_INVALID, "server_create: bad budget or run-ahead");
    splat_server* s = new (std::nothrow) splat_server();
    if (!s) return set_error(SPLAT_ERR_ALLOC, "server_create: host allocation");
    splat_status_t rc = splat_batch_create(max_items, max_pool_rays, &s->engine);
    if (rc != SPLAT_OK) {
        delete s;
        return rc;
    }
    s->max_items = max_items;
    s->pool_rays = max_pool_rays;
    s->map_budget = map_budget_bytes;
    s->max_ahead = max_ticks_ahead;
    s->in_flight.resize((size_t)max_items);
    s->slot_used.assign((size_t)max_items, 0);
    s->done_slots.resize((size_t)max_items);
    cudaError_t e = cudaEventCreate(&s->t0);
    if (e != cudaSuccess) {
        splat_batch_destroy(s->engine);
        delete s;
        return cuda_error(e, "create");
    }
    *out = s;
    return SPLAT_OK;
}

splat_status_t splat_server_destroy(splat_server_t* s) {
    if (!s) return set_error(SPLAT_ERR_INVALID, "server_destroy: null server");
    cudaDeviceSynchronize();
    std::vector<cudaEvent_t> all(s->ahead.begin(), s->ahead.end());
    all.insert(all.end(), s->free_events.begin(), s->free_events.end());
    for (const Completion& c : s->completing) all.push_back(c.ev);
    std::sort(all.begin(), all.end());
    all.erase(std::unique(all.begin(), all.end()), all.end());
    for (cudaEvent_t e : all) cudaEventDestroy(e);
    if (s->t0) cudaEventDestroy(s->t0);
    splat_status_t rc = splat_batch_destroy(s->engine);
    delete s;
    return rc;
}

splat_status_t splat_server_submit(splat_server_t* s, const splat_scene_t* scene, const splat_trace_params_t* params,
                                   void* d_map, int64_t* request_id) {
    if (!s || !scene || !params || !d_map || !request_id)
        return set_error(SPLAT_ERR_INVALID, "server_submit: null argument");
    Request r;
    r.id = s->next_id++;
    r.scene = scene;
    std::memcpy(&r.params, params, sizeof(r.params));
    r.map = d_map;
    r.map_bytes = map_bytes_of(*params);
    if (r.map_bytes > s->map_budget)
        return set_error(SPLAT_ERR_WORKSPACE, "server_submit: the light map alone exceeds the budget");
    if (rays_of(*params) > s->pool_rays)
        return set_error(SPLAT_ERR_WORKSPACE, "server_submit: more rays than the engine's pool holds");
    s->pending.push_back(r);
    *request_id = r.id;
    return SPLAT_OK;
}

splat_status_t splat_server_step(splat_server_t* s, void* stream, int32_t* in_flight, int32_t* queued) {
    if (!s) return set_error(SPLAT_ERR_INVALID, "server_step: null server");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (!s->started) {
        cudaError_t e = cudaEventRecord(s->t0, st);
        if (e != cudaSuccess) return cuda_error(e, "start event");
        s->started = true;
    }
    splat_status_t rc = collect(s, false);
    if (rc != SPLAT_OK) return rc;
    // admission, in arrival order
    while (!s->pending.empty()) {
        Request& r = s->pending.front();
        if (s->map_in_use + r.map_bytes > s->map_budget) break;
        int32_t slot = -1;
        rc = splat_batch_admit(s->engine, r.scene, &r.params, r.map, &slot);
        if (rc == SPLAT_ERR_WORKSPACE) break;  // no slot or pool room until a request leaves
        if (rc != SPLAT_OK) return rc;
        s->in_flight[(size_t)slot] = r;
        s->slot_used[(size_t)slot] = 1;
        s->map_in_use += r.map_bytes;
        s->pending.pop_front();
    }
    int32_t n_in = 0;
    rc = splat_batch_status(s->engine, &n_in, nullptr, nullptr);
    if (rc != SPLAT_OK) return rc;
    if (n_in > 0) {
        // keep the host at most max_ahead ticks ahead of the device
        while ((int32_t)s->ahead.size() >= s->max_ahead) {
            cudaEvent_t e = s->ahead.front();
            s->ahead.pop_front();
            cudaError_t q = cudaEventSynchronize(e);
            if (q != cudaSuccess) return cuda_error(q, "run-ahead wait");
            maybe_free(s, e);
        }
        int32_t nd = 0;
        rc = splat_batch_tick(s->engine, stream, s->done_slots.data(), s->max_items, &nd);
        if (rc != SPLAT_OK) return rc;
        cudaEvent_t ev;
        cudaError_t e = take_event(s, &ev);
        if (e == cudaSuccess) e = cudaEventRecord(ev, st);
        if (e != cudaSuccess) return cuda_error(e, "tick event");
        s->ahead.push_back(ev);
        for (int32_t i = 0; i < nd; ++i) {
            const int32_t slot = s->done_slots[(size_t)i];
            const Request& r = s->in_flight[(size_t)slot];
            s->completing.push_back(Completion{r.id, slot, r.map_bytes, ev});
        }
        rc = collect(s, false);
        if (rc != SPLAT_OK) return rc;
    }
    if (in_flight) *in_flight = n_in;
    if (queued) *queued = (int32_t)s->pending.size();
    return SPLAT_OK;
}

splat_status_t splat_server_poll(splat_server_t* s, int32_t block, int64_t* ids, double* device_ms, int32_t max,
                                 int32_t* n) {
    if (!s || !n || max < 0 || (max > 0 && !ids))
        return set_error(SPLAT_ERR_INVALID, "server_poll: bad arguments");
    splat_status_t rc = collect(s, block != 0);
    if (rc != SPLAT_OK) return rc;
    const int32_t k = (int32_t)std::min<size_t>((size_t)max, s->done.size());
    for (int32_t i = 0; i < k; ++i) {
        ids[i] = s->done[(size_t)i].first;
        if (device_ms) device_ms[i] = s->done[(size_t)i].second;
    }
    s->done.erase(s->done.begin(), s->done.begin() + k);
    *n = k;
    return SPLAT_OK;
}

splat_status_t splat_server_status(const splat_server_t* s, int32_t* queued, int32_t* in_flight,
                                   int64_t* map_bytes_in_use) {
    if (!s) return set_error(SPLAT_ERR_INVALID, "server_status: null server");
    int32_t n_in = 0;
    splat_status_t rc = splat_batch_status(s->engine, &n_in, nullptr, nullptr);
    if (rc != SPLAT_OK) return rc;
    if (queued) *queued = (int32_t)s->pending.size();
    if (in_flight) *in_flight = n_in;
    if (map_bytes_in_use) *map_bytes_in_use = s->map_in_use;
    return SPLAT_OK;
}

}  // extern "C"
