// serve.cu -- native request server (pgeof_server_*) for
// compute_features_selected (include/pgeof.hpp:325-375); the reference has no
// serving layer.
//
// Continuous batching: `slots` worker threads, each with its own CUDA stream
// (the host-pointer API keeps one stream per host thread), take requests from
// one FIFO queue as soon as a slot is free and the request's device-memory
// footprint fits next to what is in flight, so requests that arrive while
// others run start at once and their kernels overlap on the GPU. A request
// runs exactly the synchronous host call (upload, radius grid, fused radius
// search, PCA, selected features, download); results do not depend on what
// else is in flight. No Python and no GIL on this path: submit() enqueues and
// returns, wait() blocks on the request alone.
//
// Resident clouds: a cloud added to the server stays on the device with its
// grid; requests that name it skip the upload and the grid build (repeated
// queries with other radii, k or feature lists). Its bytes are reserved from
// the budget until it is removed.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "kernels.cuh"

namespace pgeof {
namespace {

using Clock = std::chrono::steady_clock;

struct CloudEntry {
    ResidentCloud cloud;
    uint64_t bytes = 0;
    int users = 0;  // queued or running requests on it
    bool removing = false;
};

struct ServeRequest {
    std::shared_ptr<CloudEntry> cloud;  // resident cloud, or null (xyz below)
    uint64_t id = 0;
    bool f64 = false;
    const void* xyz = nullptr;
    int64_t n = 0;
    double radius = 0.0;
    uint32_t max_knn = 0;
    std::vector<int32_t> ids;
    void* out = nullptr;
    uint64_t footprint = 0;
    int slot = -1;
    Clock::time_point t_submit, t_admit, t_done;
    int status = PGEOF_OK;
    std::string msg;
    bool done = false;
};

// Device bytes a request holds while in flight (upper bound): input, the
// cell-sorted copy, the grid build's keys and cell table, the neighbour table,
// the counts and the output, plus 1 MiB of fixed scratch.
uint64_t footprint(int64_t n, uint32_t max_knn, int64_t n_ids, bool f64) {
    const uint64_t real = f64 ? 8 : 4;
    const uint64_t per_point = 3 * real + (f64 ? 32 : 16) + 16 + 20 + 4ull * std::max<uint32_t>(max_knn, 1) + 4 +
                               real * (uint64_t)n_ids;
    return (uint64_t)n * per_point + (1ull << 20);
}

// Device bytes of a resident cloud (upper bound): xyz, the cell-sorted copy
// and a cell table of at most max(4n, 65536) + 1 entries.
uint64_t resident_bytes_of(int64_t n) { return (uint64_t)n * (12 + 16 + 16) + (1ull << 20); }

// A request on a resident cloud holds only its neighbour table, counts and
// output while in flight.
uint64_t resident_footprint(int64_t n, uint32_t max_knn, int64_t n_ids) {
    return (uint64_t)n * (4ull * std::max<uint32_t>(max_knn, 1) + 4 + 4 * (uint64_t)n_ids) + (1ull << 20);
}

struct Server {
    int device = 0;
    uint64_t budget = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<ServeRequest>> queue;
    std::unordered_map<uint64_t, std::shared_ptr<ServeRequest>> table;
    std::unordered_map<uint64_t, std::shared_ptr<CloudEntry>> clouds;
    std::vector<int> free_slots;
    uint64_t next_id = 1, next_cloud = 1, in_use = 0, resident = 0, peak_bytes = 0, completed = 0;
    int in_flight = 0, peak_in_flight = 0;
    bool stopping = false;
    std::vector<std::thread> workers;

    void worker() {
        cudaSetDevice(device);
        for (;;) {
            std::shared_ptr<ServeRequest> r;
            uint64_t fp = 0;
            {
                std::unique_lock<std::mutex> lk(mu);
                // FIFO admission: the oldest request runs as soon as a slot and
                // its footprint are free (a request larger than the budget runs
                // alone)
                cv_work.wait(lk, [&] {
                    if (queue.empty()) return stopping;
                    const uint64_t avail = budget - resident;  // resident clouds hold the rest
                    fp = std::min(queue.front()->footprint, avail);
                    return !free_slots.empty() && in_use + fp <= avail;
                });
                if (queue.empty()) return;
                r = queue.front();
                queue.pop_front();
                r->slot = free_slots.back();
                free_slots.pop_back();
                in_use += fp;
                ++in_flight;
                peak_bytes = std::max(peak_bytes, in_use + resident);
                peak_in_flight = std::max(peak_in_flight, in_flight);
                r->t_admit = Clock::now();
            }
            int st;
            if (r->cloud)
                st = host_selected_resident(r->cloud->cloud, (float)r->radius, r->max_knn, r->ids.data(),
                                            (int64_t)r->ids.size(), static_cast<float*>(r->out));
            else if (r->f64)
                st = pgeof_host_compute_features_selected_f64(static_cast<const double*>(r->xyz), r->n, r->radius,
                                                              r->max_knn, r->ids.data(), (int64_t)r->ids.size(),
                                                              static_cast<double*>(r->out));
            else
                st = pgeof_host_compute_features_selected_f32(static_cast<const float*>(r->xyz), r->n,
                                                              (float)r->radius, r->max_knn, r->ids.data(),
                                                              (int64_t)r->ids.size(), static_cast<float*>(r->out));
            {
                std::lock_guard<std::mutex> lk(mu);
                r->status = st;
                if (st != PGEOF_OK) r->msg = pgeof_last_error_message();
                r->t_done = Clock::now();
                r->done = true;
                in_use -= fp;
                --in_flight;
                free_slots.push_back(r->slot);
                ++completed;
                if (r->cloud) --r->cloud->users;
                r->cloud.reset();
            }
            cv_work.notify_all();
            cv_done.notify_all();
        }
    }
};

int submit(Server* sv, bool f64, const void* xyz, int64_t n, double radius, uint32_t max_knn, const int32_t* ids,
           int64_t n_ids, void* out, uint64_t* request_id, uint64_t cloud_id = 0) {
    if (!sv || !request_id) return fail(PGEOF_ERR_INVALID_ARGUMENT, "invalid server or NULL request_id");
    std::shared_ptr<CloudEntry> cloud;
    if (cloud_id) {
        std::lock_guard<std::mutex> lk(sv->mu);
        auto it = sv->clouds.find(cloud_id);
        if (it == sv->clouds.end() || it->second->removing)
            return fail(PGEOF_ERR_INVALID_ARGUMENT, "unknown resident cloud id");
        cloud = it->second;
        n = (int64_t)cloud->cloud.n;  // the request runs on the resident copy
    }
    if (n < 0 || n_ids < 0) return fail(PGEOF_ERR_INVALID_ARGUMENT, "negative size");
    if ((n > 0 && ((!xyz && !cloud) || (n_ids > 0 && !out))) || (n_ids > 0 && !ids))
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "NULL buffer");
    auto r = std::make_shared<ServeRequest>();
    r->cloud = cloud;
    r->f64 = f64;
    r->xyz = xyz;
    r->n = n;
    r->radius = radius;
    r->max_knn = max_knn;
    r->ids.assign(ids, ids + n_ids);
    r->out = out;
    r->footprint = cloud ? resident_footprint(n, max_knn, n_ids) : footprint(n, max_knn, n_ids, f64);
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (sv->stopping) return fail(PGEOF_ERR_INVALID_ARGUMENT, "the server is shutting down");
        if (cloud) {
            if (cloud->removing) return fail(PGEOF_ERR_INVALID_ARGUMENT, "unknown resident cloud id");
            ++cloud->users;
        }
        r->id = sv->next_id++;
        sv->table.emplace(r->id, r);
        sv->queue.push_back(r);
        *request_id = r->id;
    }
    sv->cv_work.notify_all();
    return PGEOF_OK;
}

}  // namespace
}  // namespace pgeof

using namespace pgeof;

extern "C" {

int pgeof_server_create(int slots, uint64_t budget_bytes, pgeof_server* out) {
    if (!out) return fail(PGEOF_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (slots < 1 || slots > 256) return fail(PGEOF_ERR_INVALID_ARGUMENT, "slots must be in [1, 256]");
    if (budget_bytes == 0) return fail(PGEOF_ERR_INVALID_ARGUMENT, "budget_bytes must be > 0");
    Server* sv = new Server();
    if (cudaGetDevice(&sv->device) != cudaSuccess) {
        delete sv;
        return fail(PGEOF_ERR_CUDA, "cudaGetDevice");
    }
    sv->budget = budget_bytes;
    for (int i = slots - 1; i >= 0; --i) sv->free_slots.push_back(i);
    for (int i = 0; i < slots; ++i) sv->workers.emplace_back([sv] { sv->worker(); });
    *out = reinterpret_cast<pgeof_server>(sv);
    return PGEOF_OK;
}

int pgeof_server_submit_selected_f32(pgeof_server server, const float* xyz, int64_t n, float search_radius,
                                     uint32_t max_knn, const int32_t* selected, int64_t n_selected, float* features,
                                     uint64_t* request_id) {
    return submit(reinterpret_cast<Server*>(server), false, xyz, n, search_radius, max_knn, selected, n_selected,
                  features, request_id);
}

int pgeof_server_submit_selected_f64(pgeof_server server, const double* xyz, int64_t n, double search_radius,
                                     uint32_t max_knn, const int32_t* selected, int64_t n_selected, double* features,
                                     uint64_t* request_id) {
    return submit(reinterpret_cast<Server*>(server), true, xyz, n, search_radius, max_knn, selected, n_selected,
                  features, request_id);
}

int pgeof_server_add_cloud_f32(pgeof_server server, const float* xyz, int64_t n, float radius_hint,
                               uint32_t k_hint, uint64_t* cloud_id) {
    Server* sv = reinterpret_cast<Server*>(server);
    if (!sv || !cloud_id) return fail(PGEOF_ERR_INVALID_ARGUMENT, "invalid server or NULL cloud_id");
    if (n < 1 || !xyz) return fail(PGEOF_ERR_INVALID_ARGUMENT, "a resident cloud needs at least one point");
    const uint64_t bytes = resident_bytes_of(n);
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (sv->stopping) return fail(PGEOF_ERR_INVALID_ARGUMENT, "the server is shutting down");
        if (sv->resident + bytes > sv->budget)
            return fail(PGEOF_ERR_INVALID_ARGUMENT, "resident clouds would exceed the server's device budget");
        sv->resident += bytes;  // reserved now, so concurrent additions cannot overshoot
    }
    auto e = std::make_shared<CloudEntry>();
    e->bytes = bytes;
    cudaSetDevice(sv->device);
    const int st = resident_cloud_build(xyz, (uint64_t)n, radius_hint, k_hint, e->cloud);
    std::lock_guard<std::mutex> lk(sv->mu);
    if (st != PGEOF_OK) {
        sv->resident -= bytes;
        sv->cv_work.notify_all();
        return st;
    }
    *cloud_id = sv->next_cloud++;
    sv->clouds.emplace(*cloud_id, e);
    return PGEOF_OK;
}

int pgeof_server_remove_cloud(pgeof_server server, uint64_t cloud_id) {
    Server* sv = reinterpret_cast<Server*>(server);
    if (!sv) return fail(PGEOF_ERR_INVALID_ARGUMENT, "invalid server");
    std::shared_ptr<CloudEntry> e;
    {
        std::unique_lock<std::mutex> lk(sv->mu);
        auto it = sv->clouds.find(cloud_id);
        if (it == sv->clouds.end() || it->second->removing)
            return fail(PGEOF_ERR_INVALID_ARGUMENT, "unknown resident cloud id");
        e = it->second;
        e->removing = true;  // no new requests; the queued ones finish first
        sv->cv_done.wait(lk, [&] { return e->users == 0; });
        sv->clouds.erase(cloud_id);
        sv->resident -= e->bytes;
    }
    sv->cv_work.notify_all();
    return PGEOF_OK;  // the device memory goes with the last reference
}

int pgeof_server_submit_selected_resident_f32(pgeof_server server, uint64_t cloud_id, float search_radius,
                                              uint32_t max_knn, const int32_t* selected, int64_t n_selected,
                                              float* features, uint64_t* request_id) {
    if (!cloud_id) return fail(PGEOF_ERR_INVALID_ARGUMENT, "unknown resident cloud id");
    return submit(reinterpret_cast<Server*>(server), false, nullptr, 0, search_radius, max_knn, selected, n_selected,
                  features, request_id, cloud_id);
}

int pgeof_server_wait(pgeof_server server, uint64_t request_id, double* latency_ms, double* queue_ms, int* slot) {
    Server* sv = reinterpret_cast<Server*>(server);
    if (!sv) return fail(PGEOF_ERR_INVALID_ARGUMENT, "invalid server");
    std::shared_ptr<ServeRequest> r;
    {
        std::unique_lock<std::mutex> lk(sv->mu);
        auto it = sv->table.find(request_id);
        if (it == sv->table.end()) return fail(PGEOF_ERR_INVALID_ARGUMENT, "unknown request id");
        r = it->second;
        sv->cv_done.wait(lk, [&] { return r->done; });
        sv->table.erase(it);
    }
    using ms = std::chrono::duration<double, std::milli>;
    if (latency_ms) *latency_ms = ms(r->t_done - r->t_submit).count();
    if (queue_ms) *queue_ms = ms(r->t_admit - r->t_submit).count();
    if (slot) *slot = r->slot;
    if (r->status != PGEOF_OK) return fail(r->status, r->msg);
    return PGEOF_OK;
}

int pgeof_server_stats(pgeof_server server, uint64_t* peak_bytes, int* peak_in_flight, uint64_t* completed) {
    Server* sv = reinterpret_cast<Server*>(server);
    if (!sv) return fail(PGEOF_ERR_INVALID_ARGUMENT, "invalid server");
    std::lock_guard<std::mutex> lk(sv->mu);
    if (peak_bytes) *peak_bytes = sv->peak_bytes;
    if (peak_in_flight) *peak_in_flight = sv->peak_in_flight;
    if (completed) *completed = sv->completed;
    return PGEOF_OK;
}

int pgeof_server_destroy(pgeof_server server) {
    Server* sv = reinterpret_cast<Server*>(server);
    if (!sv) return PGEOF_OK;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stopping = true;
    }
    sv->cv_work.notify_all();
    for (auto& t : sv->workers) t.join();  // queued requests finish first
    delete sv;
    return PGEOF_OK;
}

}  // extern "C"
